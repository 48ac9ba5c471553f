// Basic3DObject.cpp — construction and frame math of the analytic objects.
#include "Basic3DObject.h"

#include <algorithm>
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

// ---- per-ray tests on the host (the reference's intersect(), Basic3DObject.cpp:44-81, 135-190,
// 274-300, 376-410, 486-551). Same float operations in the same order as the device kernels
// (raytrace_gb300/csrc/rt_trace.cuh); comparisons the reference writes against double
// constants (1e-6) are made in double here too.

float BorderTest(const Ray &ray, const Vertex &Min, const Vertex &Max, float *getMax)
{
    const Vertex &o = ray.origin;
    const Vertex &d = ray.direction;
    const Vertex rrd(1.0f / d.x, 1.0f / d.y, 1.0f / d.z, 1.0f / d.w);
    const Vertex t0 = (Min - o).mixmul(rrd), t1 = (Max - o).mixmul(rrd);
    // MINPS / MAXPS: the second operand when the comparison fails (NaN included)
    auto lo = [](float a, float b) { return a < b ? a : b; };
    auto hi = [](float a, float b) { return a > b ? a : b; };
    float nx = lo(t0.x, t1.x), ny = lo(t0.y, t1.y), nz = lo(t0.z, t1.z);
    float fx = hi(t0.x, t1.x), fy = hi(t0.y, t1.y), fz = hi(t0.z, t1.z);
    // a direction parallel to a slab: the origin must lie between its planes
    if (std::fabs(d.y) < 1e-6) {
        if (o.y > Max.y || o.y < Min.y) return 1e20f;
        ny = -1, fy = 1e10f;
    }
    if (std::fabs(d.x) < 1e-6) {
        if (o.x > Max.x || o.x < Min.x) return 1e20f;
        nx = -1, fx = 1e10f;
    }
    if (std::fabs(d.z) < 1e-6) {
        if (o.z > Max.z || o.z < Min.z) return 1e20f;
        nz = -1, fz = 1e10f;
    }
    const float entry = std::max(std::max(nx, ny), std::max(nz, 0.0f));
    const float exit = std::min(std::min(fx, fy), fz);
    if (exit < entry) return 1e20f;
    *getMax = exit;
    return entry;
}

// inside branch of a sphere test: the far root, for a ray that starts on the sphere's surface
// and travels inside it
static float sphere_far_root(const Ray &ray, const Vertex &centre, float r2)
{
    const Vertex s2r = ray.origin - centre;
    const float b = ray.direction & s2r;
    const float disc = b * b - s2r.length_sqr() + r2;
    return -(ray.direction & s2r) + std::sqrt(disc);
}

// outside branch: the near root, or a negative value when the sphere is behind the ray (b > 0)
// or missed (negative discriminant)
static float sphere_near_root(const Ray &ray, const Vertex &centre, float r2)
{
    const Vertex s2r = ray.origin - centre;
    const float b = ray.direction & s2r;
    if (b > 0) return -1.0f;
    const float disc = b * b - s2r.length_sqr() + r2;
    if (disc < 0) return -1.0f;
    return -((ray.direction & s2r) + std::sqrt(disc));
}

HitRes Sphere::intersect(const Ray &ray, const HitRes &hr, const float)
{
    const bool own = hr.obj == (intptr_t)this;
    if (own && !ray.isInside) return hr;   // a ray leaving the outside of its own sphere
    if (own && ray.type == MY_RAY_SHADOWRAY) return HitRes(radius);
    const float t = own ? sphere_far_root(ray, position, radius_sqr) : sphere_near_root(ray, position, radius_sqr);
    if (!(t < hr.distance && t > 1e-6)) return hr;
    HitRes h(t);
    h.position = ray.origin + ray.direction * t;
    h.normal = own ? Normal(position - h.position) : Normal(h.position - position);
    h.mtl = &mtl;
    h.obj = (intptr_t)this;
    h.isInside = (uint8_t)~ray.isInside;
    // a refracted ray leaving its sphere goes back to rfr 1
    h.rfr = own && ray.type == MY_RAY_REFRACTRAY ? 1.0f : mtl.rfr;
    return h;
}

HitRes Box::intersect(const Ray &ray, const HitRes &hr, const float)
{
    if (hr.obj == (intptr_t)this) return hr;
    float exit;
    const float t = BorderTest(ray, min + position, max + position, &exit);
    if (!(t < hr.distance && t > 1e-6)) return hr;
    HitRes h(t);
    h.position = ray.origin + ray.direction * t;
    const Vertex b2p = h.position - position;
    Vertex face;   // the face(s) the point lies on, z then y then x
    if (std::fabs(std::fabs(b2p.z) - max.z) < 1e-6) face.z = b2p.z > 0 ? 1.0f : -1.0f;
    if (std::fabs(std::fabs(b2p.y) - max.y) < 1e-6) face.y = b2p.y > 0 ? 1.0f : -1.0f;
    if (std::fabs(std::fabs(b2p.x) - max.x) < 1e-6) face.x = b2p.x > 0 ? 1.0f : -1.0f;
    h.normal = Normal(face);
    h.mtl = &mtl;
    h.obj = (intptr_t)this;
    return h;
}

HitRes Plane::intersect(const Ray &ray, const HitRes &hr, const float)
{
    if (hr.obj == (intptr_t)this) return hr;
    const float a = ray.direction & normal;
    if (std::fabs(a) < 1e-6) return hr;
    const Vertex p2r = ray.origin - position;
    const float t = -(p2r & normal) / a;
    if (t < 0 || !(t < hr.distance)) return hr;
    // checker coordinates in the plane's frame, scaled by 1/5
    const Vertex dy = ray.direction * axisy;
    const float f = 1.0f / (axisx & dy) / 5;
    HitRes h(t);
    h.normal = normal;
    h.mtl = &mtl;
    h.tex = &tex;
    h.position = ray.origin + ray.direction * t;
    h.tcoord = Coord2D((p2r & dy) * f, (ray.direction & (p2r * axisx)) * f);
    h.obj = (intptr_t)this;
    return h;
}

HitRes BallPlane::intersect(const Ray &ray, const HitRes &hr, const float)
{
    // the 16 spheres in the reference's order; sphere k (1..16) has the token this + k
    const std::vector<Vertex> centres = sphereCentres();
    HitRes best = hr;
    for (size_t k = 0; k < centres.size(); ++k) {
        const intptr_t token = (intptr_t)this + (intptr_t)(k + 1);
        const bool own = hr.obj == token;
        if (own && !ray.isInside) continue;
        if (own && ray.type == MY_RAY_SHADOWRAY) return HitRes(radius);
        const Vertex &c = centres[k];
        const float t = own ? sphere_far_root(ray, c, radius_sqr) : sphere_near_root(ray, c, radius_sqr);
        if (!(t < best.distance && t > 1e-6)) continue;
        best = HitRes(t);
        best.position = ray.origin + ray.direction * t;
        best.normal = own ? Normal(c - best.position) : Normal(best.position - c);
        best.mtl = &mtl;
        best.obj = token;
        best.isInside = (uint8_t)~ray.isInside;
        best.rfr = own && ray.type == MY_RAY_REFRACTRAY ? 1.0f : mtl.rfr;
    }
    return best.distance < hr.distance ? best : hr;
}
