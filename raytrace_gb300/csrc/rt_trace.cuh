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
#include "rt_lbvh.cuh"

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

// ---- 4-wide nodes ----------------------------------------------------------------------------
struct Quad {
    float4 lx, hx, ly, hy, lz, hz;
    int4 ref;
};
__device__ __forceinline__ Quad load_quad(const float4 *__restrict__ quads, int node)
{
    const float4 *q = quads + 8ll * node;
    Quad Q;
    Q.lx = __ldg(q), Q.hx = __ldg(q + 1), Q.ly = __ldg(q + 2), Q.hy = __ldg(q + 3);
    Q.lz = __ldg(q + 4), Q.hz = __ldg(q + 5);
    Q.ref = __ldg(reinterpret_cast<const int4 *>(q + 6));
    return Q;
}
__device__ __forceinline__ float slab1(const RayInv &r, float lx, float hx, float ly, float hy, float lz, float hz,
                                       float tmax, bool &hit)
{
    return slab(r, make_float4(lx, ly, lz, 0.0f), make_float4(hx, hy, hz, 0.0f), tmax, hit);
}
// the four slots against one ray: entry distance and hit flag per slot
__device__ __forceinline__ void slab4(const RayInv &r, const Quad &Q, float tmax, float t[4], bool h[4])
{
    t[0] = slab1(r, Q.lx.x, Q.hx.x, Q.ly.x, Q.hy.x, Q.lz.x, Q.hz.x, tmax, h[0]);
    t[1] = slab1(r, Q.lx.y, Q.hx.y, Q.ly.y, Q.hy.y, Q.lz.y, Q.hz.y, tmax, h[1]);
    t[2] = slab1(r, Q.lx.z, Q.hx.z, Q.ly.z, Q.hy.z, Q.lz.z, Q.hz.z, tmax, h[2]);
    t[3] = slab1(r, Q.lx.w, Q.hx.w, Q.ly.w, Q.hy.w, Q.lz.w, Q.hz.w, tmax, h[3]);
}
// order four (distance, ref) pairs by distance (entries not taken carry +inf): 5 exchanges
__device__ __forceinline__ void sort4(float t[4], int c[4])
{
    auto cx = [&](int a, int b) {
        const bool sw = t[b] < t[a];
        const float ta = t[a], tb = t[b];
        const int ca = c[a], cb = c[b];
        t[a] = sw ? tb : ta, t[b] = sw ? ta : tb;
        c[a] = sw ? cb : ca, c[b] = sw ? ca : cb;
    };
    cx(0, 1), cx(2, 3), cx(0, 2), cx(1, 3), cx(1, 2);
}
constexpr float kInf = __builtin_huge_valf();

// ---- traversal stack (kStack entries, rt_device.cuh) --------------------------------------

// the launch's dynamic shared memory: the traversal kernels' short stacks
extern __shared__ int rt_short_stack[];

// A thread's traversal stack. With SS > 0 (a power of two) its top SS entries live in shared
// memory, SS * blockDim.x ints given at launch, entry slot k of thread t at
// [k * blockDim.x + t] so that a warp's accesses fall in 32 different banks; deeper entries go
// to a local-memory array: a push beyond SS moves the entry SS below it out to local memory, a
// pop brings it back. Most paths stay within SS entries and never touch local memory, which
// also holds the node lines in L1. SS = 0 keeps the whole stack in local memory.
template <int SS>
struct TravStack {
    int deep[kStack - SS];
    int sp;
    __device__ __forceinline__ TravStack() : sp(0) {}
    __device__ __forceinline__ bool empty() const { return sp == 0; }
    __device__ __forceinline__ int *slot(int e) const
    {
        return rt_short_stack + (e & (SS - 1)) * (int)blockDim.x + (int)threadIdx.x;
    }
    // false when all kStack entries are taken (the entry is dropped; the caller flags it)
    __device__ __forceinline__ bool push(int v)
    {
        if (sp >= kStack) return false;
        if constexpr (SS == 0) {
            deep[sp] = v;
        } else {
            int *s = slot(sp);
            if (sp >= SS) deep[sp - SS] = *s;
            *s = v;
        }
        ++sp;
        return true;
    }
    __device__ __forceinline__ int pop()
    {
        --sp;
        if constexpr (SS == 0) {
            return deep[sp];
        } else {
            int *s = slot(sp);
            const int v = *s;
            if (sp >= SS) *s = deep[sp - SS];
            return v;
        }
    }
};

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
template <int SS, bool COUNT>
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
            const float4 *__restrict__ quads = S.quads;
            const RayInv ri = make_inv(O, D);
            const unsigned last = (unsigned)S.n_leaves - 2u;   // internal nodes 0..L-2
            TravStack<SS> stack;
            int node = 0;
            for (unsigned visits = 0;; ++visits) {
                if (COUNT) wc.nodes++;
                if ((unsigned)node > last || visits >= kMaxVisits) {
                    wc.err |= visits >= kMaxVisits ? 2 : 1;
                    break;
                }
                const Quad Q = load_quad(quads, node);
                float t[4];
                bool h[4];
                int c[4] = {Q.ref.x, Q.ref.y, Q.ref.z, Q.ref.w};
                slab4(ri, Q, self_inside ? before.t : best.t, t, h);
                // leaves at once (ties resolve by object order, not by visit order), one code copy
                unsigned leaves = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (h[k] && c[k] < 0) {
                        h[k] = false;
                        leaves |= 1u << k;
                    }
                while (leaves) {
                    const int k = __ffs(leaves) - 1;
                    leaves &= leaves - 1u;
                    const int ck = k == 0 ? c[0] : k == 1 ? c[1] : k == 2 ? c[2] : c[3];
                    if ((unsigned)~ck < (unsigned)S.n_leaves) test_leaf(~ck);
                    else wc.err |= 1;
                }
                const float cull = self_inside ? before.t : best.t;   // the leaves may have lowered it
                int n_in = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const bool in = h[k] && t[k] <= cull;
                    t[k] = in ? t[k] : kInf;
                    n_in += in;
                }
                if (n_in == 0) {
                    if (stack.empty()) break;
                    node = stack.pop();
                    continue;
                }
                if (n_in == 1) {
                    node = t[0] < kInf ? c[0] : t[1] < kInf ? c[1] : t[2] < kInf ? c[2] : c[3];
                    continue;
                }
                sort4(t, c);   // nearest next, the others pushed farthest first
                node = c[0];
                for (int k = n_in - 1; k >= 1; --k)
                    if (!stack.push(c[k])) wc.err |= 4;
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
// Written as a start and single node visits so a kernel can advance each lane's ray one node at
// a time and give a finished lane a new ray while the others continue.

// leaf k blocks the segment [0, dis) of the ray (its own primitive `excl` never does)
template <bool COUNT>
__device__ __forceinline__ bool leaf_blocks(const float4 *__restrict__ tri, int k, V3 O, V3 D, float dis, int excl,
                                            WorkCount &wc)
{
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
}

// the linear primitives and the trivial trees: 1 blocked, 0 not blocked, -1 traverse from node 0
template <bool COUNT>
__device__ __forceinline__ int any_hit_begin(const DevScene &S, V3 O, V3 D, float dis, int excl, WorkCount &wc)
{
    for (int p = 0; p < S.n_linear; ++p) {
        if (p == excl) continue;   // shadow rays are never inside: the own primitive is skipped
        const DevPrim &P = S.prims[p];
        float t;
        const bool ok = P.type == kPrimPlane ? plane_hit(O, D, P, t) : box_hit(O, D, P, t);
        if (ok && t < dis) return 1;
    }
    if (S.n_leaves == 0) return 0;
    if (S.n_leaves == 1) return leaf_blocks<COUNT>(S.tri, 0, O, D, dis, excl, wc) ? 1 : 0;
    return -1;
}

// one 4-wide node visit: 1 blocked, 0 not blocked (the stack ran empty), -1 continue at `node`
// (the tree is given by its node and leaf arrays and leaf count, held in registers by the caller)
template <int SS, bool COUNT>
__device__ __forceinline__ int any_hit_step(const float4 *__restrict__ quads, const float4 *__restrict__ tri, int n_leaves,
                                            V3 O, V3 D, const RayInv &ri, float dis, int excl, int &node,
                                            TravStack<SS> &stack, unsigned &visits, WorkCount &wc)
{
    if (COUNT) wc.nodes++;
    if ((unsigned)node > (unsigned)n_leaves - 2u || visits++ >= kMaxVisits) {
        wc.err |= visits > kMaxVisits ? 2 : 1;
        return 0;
    }
    const Quad Q = load_quad(quads, node);
    float t[4];
    bool h[4];
    const int c[4] = {Q.ref.x, Q.ref.y, Q.ref.z, Q.ref.w};
    slab4(ri, Q, dis, t, h);
    int next = -1;
    unsigned leaves = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {   // any blocker ends the ray, so no ordering is needed
        if (!h[k]) continue;
        if (c[k] < 0)
            leaves |= 1u << k;
        else if (next < 0)
            next = c[k];
        else if (!stack.push(c[k]))
            wc.err |= 4;
    }
    while (leaves) {   // one code copy of the leaf test
        const int k = __ffs(leaves) - 1;
        leaves &= leaves - 1u;
        const int ck = k == 0 ? c[0] : k == 1 ? c[1] : k == 2 ? c[2] : c[3];
        if ((unsigned)~ck >= (unsigned)n_leaves) {
            wc.err |= 1;
            return 0;
        }
        if (leaf_blocks<COUNT>(tri, ~ck, O, D, dis, excl, wc)) return 1;
    }
    if (next >= 0) {
        node = next;
        return -1;
    }
    if (stack.empty()) return 0;
    node = stack.pop();
    return -1;
}

// true when some primitive other than `excl` is hit at a distance below `dis`
template <int SS, bool COUNT>
__device__ bool any_hit(const DevScene &S, V3 O, V3 D, float dis, int excl, WorkCount &wc)
{
    int r = any_hit_begin<COUNT>(S, O, D, dis, excl, wc);
    if (r >= 0) return r == 1;
    const RayInv ri = make_inv(O, D);
    TravStack<SS> stack;
    int node = 0;
    unsigned visits = 0;
    while ((r = any_hit_step<SS, COUNT>(S.quads, S.tri, S.n_leaves, O, D, ri, dis, excl, node, stack, visits, wc)) < 0) {
    }
    return r == 1;
}

} // namespace rtg
