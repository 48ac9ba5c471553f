// Basic3DObject.h — analytic scene objects of the drop-in API (Sphere, Box, Plane, BallPlane).
// Same classes and construction semantics as the reference's Basic3DObject.h:5-72; the
// per-ray intersect() virtuals are replaced by the device kernels (raytrace_gb300/csrc).
#pragma once
#include "3DElement.h"

class Sphere : public DrawObject
{
private:
    float radius, radius_sqr;
public:
    Sphere(const float r = 1.0f, unsigned int lnum = 0);
    float getRadius() const { return radius; }
    float getRadiusSqr() const { return radius_sqr; }
};

class Box : public DrawObject
{
private:
    float width, height, length;
    Vertex min, max;
public:
    Box(const float len = 2.0, unsigned int lnum = 0);
    // kept as in the reference: this constructor sets max to -(l,w,h)/2 and leaves min at 0
    Box(const float l, const float w, const float h, unsigned int lnum = 0);
    const Vertex &getMin() const { return min; }
    const Vertex &getMax() const { return max; }
};

class Plane : public DrawObject
{
private:
    Vertex ang;
    Normal axisx, axisy;
    Texture tex;
public:
    Normal normal;
    Plane(unsigned int lnum = 0);
    void rotate(const Vertex &v);
    void setTex(const Texture &t) { this->tex = t; }
    const Texture &getTex() const { return tex; }
    const Normal &getAxisX() const { return axisx; }
    const Normal &getAxisY() const { return axisy; }
};

class BallPlane : public DrawObject
{
private:
    Vertex ang;
    Normal axisx, axisy;
    float radius, radius_sqr;
public:
    Normal normal;
    BallPlane(const float r = 0.3f, unsigned int lnum = 0);
    void rotate(const Vertex &v);
    float getRadius() const { return radius; }
    const Normal &getAxisX() const { return axisx; }
    const Normal &getAxisY() const { return axisy; }
    // centres of the 4x4 spheres in the order the reference visits them
    // (cx outer, cy inner, both from -6r stepping 4r while < 8r; Basic3DObject.cpp:492-497)
    std::vector<Vertex> sphereCentres() const;
};
