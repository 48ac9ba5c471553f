// Basic3DObject.h — analytic scene objects of the drop-in API (Sphere, Box, Plane, BallPlane).
// Same classes and construction semantics as the reference's Basic3DObject.h:5-72. Rendering
// runs in the device kernels (raytrace_gb300/csrc); intersect() is the reference's per-ray
// test on the host, for tools that query the scene one ray at a time.
#pragma once
#include "3DElement.h"

class Sphere : public DrawObject
{
private:
    float radius, radius_sqr;
public:
    Sphere(const float r = 1.0f, unsigned int lnum = 0);
    HitRes intersect(const Ray &ray, const HitRes &hr, const float min = 0) override;
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
    HitRes intersect(const Ray &ray, const HitRes &hr, const float dmin = 0) override;
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
    HitRes intersect(const Ray &ray, const HitRes &hr, const float min = 0) override;
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
    HitRes intersect(const Ray &ray, const HitRes &hr, const float min = 0) override;
    void rotate(const Vertex &v);
    float getRadius() const { return radius; }
    const Normal &getAxisX() const { return axisx; }
    const Normal &getAxisY() const { return axisy; }
    // centres of the 4x4 spheres in the order the reference visits them
    // (cx outer, cy inner, both from -6r stepping 4r while < 8r; Basic3DObject.cpp:492-497)
    std::vector<Vertex> sphereCentres() const;
};

// the slab test of an axis-aligned box: entry distance (at least 0), or 1e20 when the ray
// misses it; *getMax receives the exit distance on a hit (Basic3DObject.cpp:44-81 of the reference)
float BorderTest(const Ray &ray, const Vertex &Min, const Vertex &Max, float *getMax);
