// rt_trace.cuh — per-ray intersection of the GB300 renderer.
//
// Primitive tests reproduce the reference's arithmetic exactly (same operations, same order,
// same thresholds), so a ray that hits the same primitive gets the same distance bit for bit:
//   Sphere   Basic3DObject.cpp:135-190 (outside branch; inside branch for the ray's own sphere)
//   Plane    Basic3DObject.cpp:376-410
//   Box      Basic3DObject.cpp:274-300 with BorderTest :44-81
//   Triangle Model.cpp:720-744 (Moller-Trumbore, t > 1e-5)
// Which primitive wins follows the reference's object loop (RayTracer.cpp:458-465): the
// smallest distance, ties to the earlier object in Scene::Objects, and `newobj` (the exclude
// key handed to the children) is the last improving object whose key differs from the ray's
// own exclude key. Triangles are found through the LBVH instead of the reference's octant
// lists; its boxes are padded so that traversal never rejects a triangle the exact test hits.
#pragma once
#include "rt_device.cuh"

namespace rtg {

struct Best {
    float t;
    int key;     // primitive key (analytic index, or kTriFlag | sorted triangle)
    int ord;     // object order (tie-break)
    float u, v;  // triangle barycentrics
};

__device__ __forceinline__ bool better(float t, int ord, float bt, int bord)
{
    return t < bt || (t == bt && ord < bord);
}

// Sphere, outside branch: `b > 0` misses even when the origin is inside the sphere.
__device__ __forceinline__ bool sphere_outside(V3 O, V3 D, float4 cr2, float &t)
{
    V3 s = vsub(O, mk(cr2));
    float b = dot3(D, s);
    if (b > 0) return false;
    float disc = __fadd_rn(__fsub_rn(__fmul_rn(b, b), dot3(s, s)), cr2.w);
    if (disc < 0) return false;
    t = -__fadd_rn(b, __fsqrt_rn(disc));
    return t > kEps6;
}
// Sphere, inside branch for the ray's own sphere (refracted ray travelling inside it)
__device__ __forceinline__ bool sphere_inside(V3 O, V3 D, float4 cr2, float &t)
{
    V3 s = vsub(O, mk(cr2));
    float b = dot3(D, s);
    float disc = __fadd_rn(__fsub_rn(__fmul_rn(b, b), dot3(s, s)), cr2.w);
    t = __fadd_rn(-b, __fsqrt_rn(disc));
    return t > kEps6;
}
__device__ __forceinline__ bool plane_hit(V3 O, V3 D, const DevPrim &p, float &t)
{
    V3 N = mk(p.b);
    float a = dot3(D, N);
    if (fabsf(a) <= kEps6) return false;
    V3 p2r = vsub(O, mk(p.a));
    float b = dot3(p2r, N);
    t = __fdiv_rn(-b, a);
    return !(t < 0);
}
// BorderTest: slab entry distance or 1e20
__device__ __forceinline__ float border_test(V3 O, V3 D, V3 mn, V3 mx)
{
    V3 tmin = vsub(mn, O), tmax = vsub(mx, O);
    V3 rrd = mk(__fdiv_rn(1.0f, D.x), __fdiv_rn(1.0f, D.y), __fdiv_rn(1.0f, D.z));
    tmin = vmul(tmin, rrd);
    tmax = vmul(tmax, rrd);
    V3 dmin = mk(minps(tmin.x, tmax.x), minps(tmin.y, tmax.y), minps(tmin.z, tmax.z));
    V3 dmax = mk(maxps(tmin.x, tmax.x), maxps(tmin.y, tmax.y), maxps(tmin.z, tmax.z));
    if (fabsf(D.y) <= kEps6) {
        if (O.y > mx.y || O.y < mn.y) return kMiss;
        dmin.y = -1, dmax.y = 1e10f;
    }
    if (fabsf(D.x) <= kEps6) {
        if (O.x > mx.x || O.x < mn.x) return kMiss;
        dmin.x = -1, dmax.x = 1e10f;
    }
    if (fabsf(D.z) <= kEps6) {
        if (O.z > mx.z || O.z < mn.z) return kMiss;
        dmin.z = -1, dmax.z = 1e10f;
    }
    float dn = stdmax(stdmax(dmin.x, dmin.y), stdmax(dmin.z, 0.0f));
    float dx = stdmin(stdmin(dmax.x, dmax.y), dmax.z);
    if (dx < dn) return kMiss;
    return dn;
}
__device__ __forceinline__ bool box_hit(V3 O, V3 D, const DevPrim &p, float &t)
{
    t = border_test(O, D, mk(p.a), mk(p.b));
    return t > kEps6;
}
// TriangleTest (live branch): returns true and t,u,v when t > 1e-5
__device__ __forceinline__ bool tri_test(V3 O, V3 D, V3 p0, V3 e1, V3 e2, float &t, float &u, float &v)
{
    V3 tmp1 = cross3(D, e2);
    V3 t2r = vsub(O, p0);
    float f = __fdiv_rn(1.0f, dot3(e1, tmp1));
    u = __fmul_rn(dot3(t2r, tmp1), f);
    if (u < 0.0f || u > 1.0f) return false;
    V3 tmp2 = cross3(t2r, e1);
    v = __fmul_rn(dot3(D, tmp2), f);
    float duv = __fsub_rn(__fsub_rn(1.0f, u), v);
    if (v < 0.0f || duv < 0.0f) return false;
    t = __fmul_rn(dot3(e2, tmp2), f);
    return t > 1e-5f;
}

// ---- padded-box slab test used by the LBVH traversal (fast path, FMA allowed) ---------------
struct RayInv {
    float ix, iy, iz, ox, oy, oz;   // 1/d and o/d
};
__device__ __forceinline__ RayInv make_inv(V3 O, V3 D)
{
    auto safe = [](float d) { return fabsf(d) < 1e-30f ? copysignf(1e-30f, d) : d; };
    RayInv r;
    r.ix = __frcp_rn(safe(D.x));   // the correctly rounded 1/d, as 1.0f / d
    r.iy = __frcp_rn(safe(D.y));
    r.iz = __frcp_rn(safe(D.z));
    r.ox = O.x * r.ix;
    r.oy = O.y * r.iy;
    r.oz = O.z * r.iz;
    return r;
}
__device__ __forceinline__ float slab(const RayInv &r, float4 lo, float4 hi, float tmax, bool &hit)
{
    float tx0 = fmaf(lo.x, r.ix, -r.ox), tx1 = fmaf(hi.x, r.ix, -r.ox);
    float ty0 = fmaf(lo.y, r.iy, -r.oy), ty1 = fmaf(hi.y, r.iy, -r.oy);
    float tz0 = fmaf(lo.z, r.iz, -r.oz), tz1 = fmaf(hi.z, r.iz, -r.oz);
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    hit = tn <= tf;
    return tn;
}

struct WorkCount {
    unsigned nodes, tris, spheres;
    int err;   // 1: a child index outside the node array, 2: visit limit reached
};

// a valid LBVH is at most 64 deep and is visited at most once per node; these bounds turn a
// corrupt tree into an error flag instead of a fault or an endless loop
constexpr unsigned kMaxVisits = 1u << 22;

// ---- LBVH leaf tests -------------------------------------------------------------------------
// Leaf k holds a triangle (tag = material >= 0) or a sphere (tag = -1 - primitive index).
struct Leaf {
    float4 a, b, c;
};
// a child reference is an internal node 0..last or a leaf ~k with k < n_leaves
__device__ __forceinline__ bool child_ok(int c, unsigned last, int n_leaves)
{
    return c >= 0 ? (unsigned)c <= last : (unsigned)~c < (unsigned)n_leaves;
}
__device__ __forceinline__ Leaf load_leaf(const float4 *__restrict__ tri, int k)
{
    return Leaf{__ldg(&tri[3 * k]), __ldg(&tri[3 * k + 1]), __ldg(&tri[3 * k + 2])};
}

// ---- closest hit ---------------------------------------------------------------------------
// excl: the ray's exclude key (-1 = none). inside: Ray::isInside != 0. Writes the winner to
// `best` and the exclude key for the children to `newobj`.
template <int STACK, bool COUNT>
__device__ void closest_hit(const DevScene &S, V3 O, V3 D, int excl, bool inside, Best &best, int &newobj, WorkCount &wc)
{
    // "no hit" sits at 1e20 with order -1: a primitive must be strictly closer to replace it,
    // as the reference's `t < hr.distance` (BorderTest reports a box miss as exactly 1e20)
    best.t = kMiss;
    best.key = -1;
    best.ord = -1;
    best.u = best.v = 0.0f;
    // the ray's own sphere uses the inside branch; if it wins, newobj is the best hit among
    // the objects before it (the reference updates newobj only for keys != excl)
    bool self_inside = false;
    int self_ord = 0x7fffffff;
    if (excl >= 0 && !(excl & kTriFlag) && inside) {
        const DevPrim &sp = S.prims[excl];
        if (sp.type == kPrimSphere) self_inside = true, self_ord = sp.obj;
    }
    Best before;
    before.t = kMiss;
    before.key = -1;
    before.ord = -1;
    auto consider = [&](float t, int key, int ord, float u, float v) {
        if (better(t, ord, best.t, best.ord)) best.t = t, best.key = key, best.ord = ord, best.u = u, best.v = v;
        if (self_inside && ord < self_ord && key != excl && better(t, ord, before.t, before.ord))
            before.t = t, before.key = key, before.ord = ord;
    };

    // planes and boxes: unbounded or few, tested linearly
    for (int p = 0; p < S.n_linear; ++p) {
        if (p == excl) continue;
        const DevPrim &P = S.prims[p];
        float t;
        const bool ok = P.type == kPrimPlane ? plane_hit(O, D, P, t) : box_hit(O, D, P, t);
        if (ok) consider(t, p, P.obj, 0.0f, 0.0f);
    }

    if (S.n_leaves > 0) {
        const float4 *__restrict__ tri = S.tri;
        auto test_leaf = [&](int k) {
            const Leaf L = load_leaf(tri, k);
            const int tag = __float_as_int(L.c.w);
            const int ord = __float_as_int(L.b.w);
            float t;
            if (tag >= 0) {   // triangle
                if (COUNT) wc.tris++;
                if ((k | kTriFlag) == excl) return;
                float u, v;
                if (tri_test(O, D, mk(L.a), mk(L.b), mk(L.c), t, u, v)) consider(t, k | kTriFlag, ord, u, v);
            } else {          // sphere
                if (COUNT) wc.spheres++;
                const int p = -1 - tag;
                bool ok;
                if (p == excl) {
                    if (!inside) return;
                    ok = sphere_inside(O, D, L.a, t);
                } else
                    ok = sphere_outside(O, D, L.a, t);
                if (ok) consider(t, p, ord, 0.0f, 0.0f);
            }
        };
        if (S.n_leaves == 1) {
            test_leaf(0);
        } else {
            const float4 *__restrict__ pairs = S.pairs;
            const RayInv ri = make_inv(O, D);
            const unsigned last = (unsigned)S.n_leaves - 2u;   // internal nodes 0..L-2
            int stack[STACK];
            int sp = 0;
            int node = 0;
            for (unsigned visits = 0;; ++visits) {
                if (COUNT) wc.nodes++;
                const float4 l0 = __ldg(&pairs[4 * node]), h0 = __ldg(&pairs[4 * node + 1]);
                const float4 l1 = __ldg(&pairs[4 * node + 2]), h1 = __ldg(&pairs[4 * node + 3]);
                const int c0 = __float_as_int(l0.w), c1 = __float_as_int(l1.w);
                if (!child_ok(c0, last, S.n_leaves) || !child_ok(c1, last, S.n_leaves) || visits >= kMaxVisits) {
                    wc.err |= visits >= kMaxVisits ? 2 : 1;
                    break;
                }
                const float cull = self_inside ? before.t : best.t;
                bool hit0, hit1;
                const float tn0 = slab(ri, l0, h0, cull, hit0);
                const float tn1 = slab(ri, l1, h1, cull, hit1);
                if (hit0 && c0 < 0) {
                    test_leaf(~c0);
                    hit0 = false;
                }
                if (hit1 && c1 < 0) {
                    test_leaf(~c1);
                    hit1 = false;
                }
                if (hit0 && hit1) {
                    const int nearc = tn0 <= tn1 ? c0 : c1, farc = tn0 <= tn1 ? c1 : c0;
                    if (sp < STACK) stack[sp++] = farc;
                    else wc.err |= 4;
                    node = nearc;
                } else if (hit0)
                    node = c0;
                else if (hit1)
                    node = c1;
                else {
                    if (sp == 0) break;
                    node = stack[--sp];
                }
            }
        }
    }
    if (best.key >= 0 && best.key != excl)
        newobj = best.key;
    else if (best.key >= 0)   // own sphere won: last improving key before it, else unchanged
        newobj = before.key >= 0 ? before.key : excl;
    else
        newobj = excl;
}

// ---- any hit (shadow rays) ----------------------------------------------------------------
// true when some primitive other than `excl` is hit at a distance below `dis`
template <int STACK, bool COUNT>
__device__ bool any_hit(const DevScene &S, V3 O, V3 D, float dis, int excl, WorkCount &wc)
{
    for (int p = 0; p < S.n_linear; ++p) {
        if (p == excl) continue;   // shadow rays are never inside: the own primitive is skipped
        const DevPrim &P = S.prims[p];
        float t;
        const bool ok = P.type == kPrimPlane ? plane_hit(O, D, P, t) : box_hit(O, D, P, t);
        if (ok && t < dis) return true;
    }
    if (S.n_leaves == 0) return false;
    const float4 *__restrict__ tri = S.tri;
    auto test_leaf = [&](int k) -> bool {
        const Leaf L = load_leaf(tri, k);
        const int tag = __float_as_int(L.c.w);
        float t;
        if (tag >= 0) {
            if (COUNT) wc.tris++;
            if ((k | kTriFlag) == excl) return false;
            float u, v;
            return tri_test(O, D, mk(L.a), mk(L.b), mk(L.c), t, u, v) && t < dis;
        }
        if (COUNT) wc.spheres++;
        if (-1 - tag == excl) return false;
        return sphere_outside(O, D, L.a, t) && t < dis;
    };
    if (S.n_leaves == 1) return test_leaf(0);
    const float4 *__restrict__ pairs = S.pairs;
    const RayInv ri = make_inv(O, D);
    const unsigned last = (unsigned)S.n_leaves - 2u;
    int stack[STACK];
    int sp = 0;
    int node = 0;
    for (unsigned visits = 0;; ++visits) {
        if (COUNT) wc.nodes++;
        const float4 l0 = __ldg(&pairs[4 * node]), h0 = __ldg(&pairs[4 * node + 1]);
        const float4 l1 = __ldg(&pairs[4 * node + 2]), h1 = __ldg(&pairs[4 * node + 3]);
        const int c0 = __float_as_int(l0.w), c1 = __float_as_int(l1.w);
        if (!child_ok(c0, last, S.n_leaves) || !child_ok(c1, last, S.n_leaves) || visits >= kMaxVisits) {
            wc.err |= visits >= kMaxVisits ? 2 : 1;
            return false;
        }
        bool hit0, hit1;
        const float tn0 = slab(ri, l0, h0, dis, hit0);
        const float tn1 = slab(ri, l1, h1, dis, hit1);
        if (hit0 && c0 < 0) {
            if (test_leaf(~c0)) return true;
            hit0 = false;
        }
        if (hit1 && c1 < 0) {
            if (test_leaf(~c1)) return true;
            hit1 = false;
        }
        if (hit0 && hit1) {
            const int nearc = tn0 <= tn1 ? c0 : c1, farc = tn0 <= tn1 ? c1 : c0;
            if (sp < STACK) stack[sp++] = farc;
            else wc.err |= 4;
            node = nearc;
        } else if (hit0)
            node = c0;
        else if (hit1)
            node = c1;
        else {
            if (sp == 0) return false;
            node = stack[--sp];
        }
    }
}

} // namespace rtg
