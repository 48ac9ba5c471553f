// Basic3DObject.cpp — construction and frame math of the analytic objects.
#include "Basic3DObject.h"

#include <cmath>

Sphere::Sphere(const float r, unsigned int lnum) : DrawObject(lnum)
{
    type = MY_OBJECT_SPHERE;
    radius = r;
    radius_sqr = r * r;
}

Box::Box(const float len, unsigned int lnum) : DrawObject(lnum)
{
    type = MY_OBJECT_CUBE;
    width = height = length = len;
    float l = len / 2;
    max = Vertex(l, l, l);
    min = max * -1;
}

Box::Box(const float l, const float w, const float h, unsigned int lnum) : DrawObject(lnum)
{
    type = MY_OBJECT_CUBE;
    length = l, width = w, height = h;
    max = Vertex(l / 2, w / 2, h / 2);
    max = max * -1;
}

// Plane frame from spherical angles: ang.x/ang.y step by 5 degrees per unit, ang.z is the
// offset along the normal (Basic3DObject.cpp:312-330 of the reference).
static void plane_frame(Vertex &ang, Vertex &position, Normal &normal, Normal &axisx, Normal &axisy, const Vertex &v)
{
    bool fix = false;
    ang.x = mod(360 + ang.x - v.y * 5, 360.0f);
    ang.y = mod(360 + ang.y - v.x * 5, 360.0f);
    ang.z += v.z;
    if (ang.z < 0.0f)
        ang.z = 0.0f;
    if (std::fabs(ang.z) < 1e-5f)
        fix = true, ang.z = 1;
    Coord_sph2car2(ang.x, ang.y, ang.z, position);
    normal = Normal(position * -1);
    if (fix)
        ang.z = 0, position = Vertex();
    float tangy = mod(90 + ang.x, 360.0f);
    Vertex ay = axisy;
    Coord_sph2car2(tangy, ang.y, 1, ay);
    axisy.x = ay.x, axisy.y = ay.y, axisy.z = ay.z, axisy.w = ay.w;
    axisx = Normal(axisy * normal);
}

Plane::Plane(unsigned int lnum) : DrawObject(lnum), tex(true)
{
    type = MY_OBJECT_PLANE;
    rotate(Vertex(0, 36, 0));
}

void Plane::rotate(const Vertex &v) { plane_frame(ang, position, normal, axisx, axisy, v); }

BallPlane::BallPlane(const float r, unsigned int lnum) : DrawObject(lnum)
{
    type = MY_OBJECT_BALLPLANE;
    radius = r;
    radius_sqr = r * r;
    rotate(Vertex(0, 36, 0));
}

void BallPlane::rotate(const Vertex &v) { plane_frame(ang, position, normal, axisx, axisy, v); }

std::vector<Vertex> BallPlane::sphereCentres() const
{
    std::vector<Vertex> c;
    for (float cx = radius * -6; cx < radius * 8; cx += radius * 4)
        for (float cy = radius * -6; cy < radius * 8; cy += radius * 4) {
            Vertex tmp = axisx * cx + axisy * cy;
            c.push_back(tmp + position);
        }
    return c;
}
