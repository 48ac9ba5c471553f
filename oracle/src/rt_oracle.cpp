// rt_oracle.cpp — CPU oracle of the RayTracer per-pixel loop. TEST INFRASTRUCTURE ONLY:
// tests, the smoke check and the CPU-baseline leg of bench.py call it as the checker; the
// renderer never links or calls it.
//
// A restatement of the reference's own algorithm, checked bit-for-bit against the reference
// compiled from its sources (oracle/ref, fixtures in tests/golden):
//   parallelRT   RayTracer.cpp:5-45    64x64 tiles, atomic tile counter, pinhole ray per pixel
//   RTfrac       RayTracer.cpp:450-596 closest hit over Scene::Objects, per-light shadow rays,
//                                      Blinn-Phong, reflect / refract recursion, Beer factor
//   Sphere       Basic3DObject.cpp:135-190    Plane :376-410    Box :274-300 (+ BorderTest :44-81)
//   BallPlane    Basic3DObject.cpp:486-551
//   Model        RTPrepare Model.cpp:402-480 (8 octant lists per part), intersect :748-811,
//                BorderTestEx :482-664 (AVX2 octant slab test), TriangleTest :720-744
//   Vertex math  3DElement.cpp:56-238 (DPPS dot, AVX cross, AVX2 normalise), Color :408-472
// Templated on the scalar type: float reproduces the reference (build with
// -ffp-contract=off), double gives the FP64 re-render used to state FP32 error.
//
// Optional check mode (per ray, brute force over every primitive) marks pixels whose
// reference result rests on a degenerate choice: two primitives within 1e-6 relative
// distance, a shadow blocker within 1e-6 of the light, the reference hitting another octant
// copy of the triangle the ray starts on, or its box pre-tests disagreeing with the exact
// per-primitive tests. Those pixels are "ambiguous" and reported separately by the tests.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/rt_gb300.h"

namespace {

template <class T> struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> add(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> inline V3<T> sub(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> inline V3<T> mul(V3<T> a, V3<T> b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> inline V3<T> scl(V3<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class T> inline T dot(V3<T> a, V3<T> b)   // DPPS 0x71: (p0 + p1) + (p2 + 0)
{
    T p0 = a.x * b.x, p1 = a.y * b.y, p2 = a.z * b.z;
    T s01 = p0 + p1, s23 = p2 + T(0);
    return s01 + s23;
}
template <class T> inline V3<T> cross(V3<T> a, V3<T> b)
{
    T lx = a.y * b.z, ly = a.z * b.x, lz = a.x * b.y;
    T rx = a.z * b.y, ry = a.x * b.z, rz = a.y * b.x;
    return mk(lx - rx, ly - ry, lz - rz);
}
template <class T> inline V3<T> nrm(V3<T> v)
{
    T len = std::sqrt(dot(v, v));
    return mk(v.x / len, v.y / len, v.z / len);
}
template <class T> inline T minps(T a, T b) { return a < b ? a : b; }
template <class T> inline T maxps(T a, T b) { return a > b ? a : b; }
template <class T> inline T smax(T a, T b) { return a < b ? b : a; }   // std::max
template <class T> inline T smin(T a, T b) { return b < a ? b : a; }   // std::min
template <class T> inline V3<T> v3(const float *p) { return mk<T>(T(p[0]), T(p[1]), T(p[2])); }

constexpr int RAY_BASE = 1, RAY_SHADOW = 2, RAY_REFLECT = 3, RAY_REFRACT = 4;
constexpr int64_t NO_KEY = -1;                  // a fresh HitRes points at itself: matches nothing
constexpr int64_t COPY_BIT = int64_t(1) << 62;  // keys of octant-list triangle copies

inline int64_t obj_key(int k, int sub = 0) { return (int64_t)k * 65536 + sub; }

template <class T> struct Ray {
    V3<T> o, d;
    T mtlrfr = T(1);
    int type = 0;
    uint8_t inside = 0;
};

template <class T> struct Hit {
    V3<T> pos{}, n{};
    T tu = 0, tv = 0;
    int mtl = -1, tex = -1;
    int64_t obj = NO_KEY;
    T dist;
    T rfr = T(1);
    uint8_t inside = 0;
    // bookkeeping for the parity outputs
    int obj_index = -1, prim = 0;
    int64_t uid = -1;        // primitive identity (triangle uid shared by its octant copies)
    explicit Hit(T d = T(1e20f)) : dist(d) {}
};

template <class T> struct Tri {   // one octant-list copy (clTri)
    V3<T> e1, e2, p0;
    int part, idx;
    int64_t key, uid;
};

template <class T> struct Obj {
    int kind = 0, index = 0, mtl = 0, tex = -1;
    bool show = true;
    V3<T> pos{};
    T radius = 0, radius_sqr = 0;
    V3<T> normal{}, axisx{}, axisy{};
    V3<T> bmin{}, bmax{};   // cube: local min/max; model: VerMin/VerMax
    // model
    std::vector<std::vector<int64_t>> part_tris;   // scene triangle index per part
    std::vector<int> part_mtl;
    std::vector<V3<T>> borders;                     // per part min, max (untranslated)
    std::vector<std::vector<Tri<T>>> oct;           // 8 lists per part
    int64_t tri_first = 0;
};

template <class T> struct Mtl {
    V3<T> ka, kd, ks;
    T shininess, reflect, refract, rfr;
    int tex;
};

template <class T> struct Lit {
    int type, on;
    V3<T> pos, amb, dif, spec, att;
};

template <class T> struct Color {
    T r, g, b, alpha;
};

struct Tex {
    int w, h;
    const uint8_t *bgr;
};

struct Counts {
    int64_t primary = 0, secondary = 0, shadow = 0;
};

template <class T> struct Scene {
    std::vector<Obj<T>> objs;
    std::vector<Mtl<T>> mtls;
    std::vector<Lit<T>> lights;
    std::vector<Tex> texs;
    V3<T> env;
    const rt_scene_desc *d = nullptr;
    std::vector<int64_t> copy2tri;   // octant copy serial -> scene triangle index
};

// ---- scene build (RTPrepare included) --------------------------------------------------------
template <class T> void build_scene(const rt_scene_desc *d, Scene<T> &S)
{
    S.d = d;
    S.env = v3<T>(d->env_light);
    for (int i = 0; i < d->n_materials; ++i) {
        const rt_material &m = d->materials[i];
        S.mtls.push_back(Mtl<T>{v3<T>(m.ambient), v3<T>(m.diffuse), v3<T>(m.specular), T(m.shininess), T(m.reflect),
                                T(m.refract), T(m.rfr), m.texture});
    }
    for (int i = 0; i < d->n_lights; ++i) {
        const rt_light &l = d->lights[i];
        S.lights.push_back(Lit<T>{l.type, l.on, v3<T>(l.position), v3<T>(l.ambient), v3<T>(l.diffuse),
                                  v3<T>(l.specular), v3<T>(l.attenuation)});
    }
    for (int i = 0; i < d->n_textures; ++i) S.texs.push_back(Tex{d->textures[i].w, d->textures[i].h, d->textures[i].bgr});
    int64_t copy_serial = 0;
    for (int k = 0; k < d->n_objects; ++k) {
        const rt_object &o = d->objects[k];
        Obj<T> ob;
        ob.kind = o.type;
        ob.index = k;
        ob.show = o.show != 0;
        ob.mtl = o.material;
        ob.tex = o.texture;
        ob.pos = v3<T>(o.position);
        ob.radius = T(o.radius);
        ob.radius_sqr = ob.radius * ob.radius;
        ob.normal = v3<T>(o.normal);
        ob.axisx = v3<T>(o.axisx);
        ob.axisy = v3<T>(o.axisy);
        ob.bmin = v3<T>(o.bmin);
        ob.bmax = v3<T>(o.bmax);
        if (o.type == RT_OBJECT_MODEL) {
            ob.tri_first = o.tri_first;
            // parts: runs of triangles with one material (the loader's usemtl groups), at most
            // 32767 per part because clTri numbers triangles with int16_t (3DElement.h:125)
            for (int64_t i = 0; i < o.tri_count; ++i) {
                const int64_t g = o.tri_first + i;
                if (ob.part_tris.empty() || d->tri_mtl[g] != ob.part_mtl.back() || ob.part_tris.back().size() >= 32767) {
                    ob.part_tris.emplace_back();
                    ob.part_mtl.push_back(d->tri_mtl[g]);
                }
                ob.part_tris.back().push_back(g);
            }
            // part borders = box of the part's points (SSE lane min/max)
            for (auto &pt : ob.part_tris) {
                V3<T> mn = v3<T>(d->tri_p + 9 * pt[0]), mx = mn;
                for (int64_t g : pt)
                    for (int j = 0; j < 3; ++j) {
                        V3<T> p = v3<T>(d->tri_p + 9 * g + 3 * j);
                        mn = mk(minps(mn.x, p.x), minps(mn.y, p.y), minps(mn.z, p.z));
                        mx = mk(maxps(mx.x, p.x), maxps(mx.y, p.y), maxps(mx.z, p.z));
                    }
                ob.borders.push_back(mn);
                ob.borders.push_back(mx);
            }
            // RTPrepare: 8 octant lists per part around the part centre (Model.cpp:413-477)
            for (size_t a = 0; a < ob.part_tris.size(); ++a) {
                const V3<T> va = scl(add(ob.borders[2 * a], ob.borders[2 * a + 1]), T(0.5));
                std::vector<Tri<T>> lists[8];
                for (size_t b = 0; b < ob.part_tris[a].size(); ++b) {
                    const int64_t g = ob.part_tris[a][b];
                    const V3<T> p0 = v3<T>(d->tri_p + 9 * g), p1 = v3<T>(d->tri_p + 9 * g + 3), p2 = v3<T>(d->tri_p + 9 * g + 6);
                    Tri<T> t{sub(p1, p0), sub(p2, p0), add(p0, ob.pos), (int)a, (int)b, 0, g};
                    V3<T> tmin = mk(minps(p0.x, minps(p1.x, p2.x)), minps(p0.y, minps(p1.y, p2.y)), minps(p0.z, minps(p1.z, p2.z)));
                    V3<T> tmax = mk(maxps(p0.x, maxps(p1.x, p2.x)), maxps(p0.y, maxps(p1.y, p2.y)), maxps(p0.z, maxps(p1.z, p2.z)));
                    auto put = [&](int oc) {
                        t.key = COPY_BIT | copy_serial++;
                        S.copy2tri.push_back(g);
                        lists[oc].push_back(t);
                    };
                    if (tmin.x <= va.x) {
                        if (tmin.z <= va.z) {
                            if (tmin.y <= va.y) put(0);
                            if (tmax.y >= va.y) put(1);
                        }
                        if (tmax.z >= va.z) {
                            if (tmin.y <= va.y) put(2);
                            if (tmax.y >= va.y) put(3);
                        }
                    }
                    if (tmax.x >= va.x) {
                        if (tmin.z <= va.z) {
                            if (tmin.y <= va.y) put(4);
                            if (tmax.y >= va.y) put(5);
                        }
                        if (tmax.z >= va.z) {
                            if (tmin.y <= va.y) put(6);
                            if (tmax.y >= va.y) put(7);
                        }
                    }
                }
                for (int b = 0; b < 8; ++b) ob.oct.push_back(std::move(lists[b]));
            }
        }
        S.objs.push_back(std::move(ob));
    }
}

// ---- per-thread state ------------------------------------------------------------------------
// reasons a pixel is ambiguous (bit flags)
// 16: the texel lookup ran past the end of the texel array, where the reference reads heap
// bytes beyond its allocation (3DElement.cpp:444-449 with a wrapped coordinate rounding to 1.0)
enum : int { AMB_TIE = 1, AMB_WINNER = 2, AMB_SHADOW_EDGE = 4, AMB_SHADOW = 8, AMB_TEXEL_OOB = 16 };

struct Tls {
    int ambiguous = 0;
    int check = 0;
    Counts counts;
};

// ---- intersections ---------------------------------------------------------------------------------
template <class T> T border_test(const Ray<T> &ray, V3<T> mn, V3<T> mx)
{
    V3<T> tmin = sub(mn, ray.o), tmax = sub(mx, ray.o);
    V3<T> rrd = mk(T(1) / ray.d.x, T(1) / ray.d.y, T(1) / ray.d.z);
    tmin = mul(tmin, rrd);
    tmax = mul(tmax, rrd);
    V3<T> dmin = mk(minps(tmin.x, tmax.x), minps(tmin.y, tmax.y), minps(tmin.z, tmax.z));
    V3<T> dmax = mk(maxps(tmin.x, tmax.x), maxps(tmin.y, tmax.y), maxps(tmin.z, tmax.z));
    if ((double)std::fabs(ray.d.y) < 1e-6) {
        if (ray.o.y > mx.y || ray.o.y < mn.y) return T(1e20f);
        dmin.y = -1, dmax.y = T(1e10f);
    }
    if ((double)std::fabs(ray.d.x) < 1e-6) {
        if (ray.o.x > mx.x || ray.o.x < mn.x) return T(1e20f);
        dmin.x = -1, dmax.x = T(1e10f);
    }
    if ((double)std::fabs(ray.d.z) < 1e-6) {
        if (ray.o.z > mx.z || ray.o.z < mn.z) return T(1e20f);
        dmin.z = -1, dmax.z = T(1e10f);
    }
    T dn = smax(smax(dmin.x, dmin.y), smax(dmin.z, T(0)));
    T dx = smin(smin(dmax.x, dmax.y), dmax.z);
    if (dx < dn) return T(1e20f);
    return dn;
}

// BorderTestEx: slab test of the 8 octants of [mn,mx]; mask bit a set when octant a is hit,
// returns the smallest entry distance of the hit octants (Model.cpp:482-664)
template <class T> T border_test_ex(const Ray<T> &ray, V3<T> Min, V3<T> Max, bool mask[8])
{
    const V3<T> Mid = scl(add(Min, Max), T(0.5));
    const V3<T> rrd = mk(T(1) / ray.d.x, T(1) / ray.d.y, T(1) / ray.d.z);
    const V3<T> tmin = mul(sub(Min, ray.o), rrd), tmax = mul(sub(Max, ray.o), rrd), tmid = mul(sub(Mid, ray.o), rrd);
    T xa[8], xb[8], ya[8], yb[8], za[8], zb[8];
    for (int a = 0; a < 8; ++a) {
        const bool xh = a >> 2, zh = (a >> 1) & 1, yh = a & 1;
        xa[a] = xh ? tmid.x : tmin.x, xb[a] = xh ? tmax.x : tmid.x;
        ya[a] = yh ? tmid.y : tmin.y, yb[a] = yh ? tmax.y : tmid.y;
        za[a] = zh ? tmid.z : tmin.z, zb[a] = zh ? tmax.z : tmid.z;
    }
    T txn[8], txx[8], tyn[8], tyx[8], tzn[8], tzx[8];
    for (int a = 0; a < 8; ++a) {
        txn[a] = minps(xa[a], xb[a]), txx[a] = maxps(xa[a], xb[a]);
        tyn[a] = minps(ya[a], yb[a]), tyx[a] = maxps(ya[a], yb[a]);
        tzn[a] = minps(za[a], zb[a]), tzx[a] = maxps(za[a], zb[a]);
    }
    const T BIG = T(1e20f);
    auto flat = [&](T o, T mn, T mid, T mx, T *lo, T *hi, int bitshift, bool &out) {
        if (o > mx || o < mn) {
            out = true;
            return;
        }
        for (int a = 0; a < 8; ++a) {
            const bool high = (a >> bitshift) & 1;
            if (o > mid) lo[a] = high ? T(0) : BIG, hi[a] = high ? BIG : T(0);
            else if (o < mid) lo[a] = high ? BIG : T(0), hi[a] = high ? T(0) : BIG;
            else lo[a] = T(0), hi[a] = BIG;
        }
    };
    bool out = false;
    if ((double)std::fabs(ray.d.y) < 1e-6) flat(ray.o.y, Min.y, Mid.y, Max.y, tyn, tyx, 0, out);
    if (out) return BIG;
    if ((double)std::fabs(ray.d.x) < 1e-6) flat(ray.o.x, Min.x, Mid.x, Max.x, txn, txx, 2, out);
    if (out) return BIG;
    if ((double)std::fabs(ray.d.z) < 1e-6) flat(ray.o.z, Min.z, Mid.z, Max.z, tzn, tzx, 1, out);
    if (out) return BIG;
    T minist = BIG;
    for (int a = 0; a < 8; ++a) {
        T ansmin = maxps(txn[a], tyn[a]), ansmax = minps(txx[a], tyx[a]);
        const T tt = maxps(tzn[a], T(0));
        ansmin = maxps(ansmin, tt);
        ansmax = minps(ansmax, tzx[a]);
        mask[a] = ansmin <= ansmax;
        if (mask[a]) minist = smin(minist, ansmin);
    }
    return minist;
}

// TriangleTest (live branch, Model.cpp:720-744); 1e20 on a miss
template <class T> T tri_test(const Ray<T> &ray, const Tri<T> &tri, T &u_out, T &v_out)
{
    V3<T> tmp1 = cross(ray.d, tri.e2);
    V3<T> t2r = sub(ray.o, tri.p0);
    T f = dot(tri.e1, tmp1);
    f = T(1) / f;
    T u = dot(t2r, tmp1) * f;
    if (u < T(0) || u > T(1)) return T(1e20f);
    V3<T> tmp2 = cross(t2r, tri.e1);
    T v = dot(ray.d, tmp2) * f, duv = T(1) - u - v;
    if (v < T(0) || duv < T(0)) return T(1e20f);
    T t = dot(tri.e2, tmp2) * f;
    if (t > T(1e-5f)) {
        u_out = u, v_out = v;
        return t;
    }
    return T(1e20f);
}

template <class T> void texture_uv(const Obj<T> &o, const Ray<T> &ray, T &u, T &v)
{
    const V3<T> p2r = sub(ray.o, o.pos);
    const V3<T> tmp1 = cross(ray.d, o.axisy);
    const T f = T(1) / dot(o.axisx, tmp1) / T(5);
    u = dot(p2r, tmp1) * f;
    const V3<T> tmp2 = cross(p2r, o.axisx);
    v = dot(ray.d, tmp2) * f;
}

template <class T>
Hit<T> sphere_hit(const Scene<T> &S, const Obj<T> &o, V3<T> C, int64_t key, int sub_id, const Ray<T> &ray, const Hit<T> &hr)
{
    const Mtl<T> &M = S.mtls[o.mtl];
    if (hr.obj == key) {
        if (!ray.inside) return hr;
        if (ray.type == RAY_SHADOW) return Hit<T>(o.radius);
        V3<T> s2r = sub(ray.o, C);
        T b = dot(ray.d, s2r);
        T dis = b * b - dot(s2r, s2r) + o.radius_sqr;
        T t = -dot(ray.d, s2r) + std::sqrt(dis);
        if (t < hr.dist && (double)t > 1e-6) {
            Hit<T> nh(t);
            nh.pos = add(ray.o, scl(ray.d, t));
            nh.n = nrm(sub(C, nh.pos));
            nh.mtl = o.mtl;
            nh.obj = key;
            nh.inside = (uint8_t)~ray.inside;
            nh.rfr = ray.type == RAY_REFRACT ? T(1) : M.rfr;
            nh.obj_index = o.index, nh.prim = sub_id, nh.uid = key;
            return nh;
        }
        return hr;
    }
    V3<T> s2r = sub(ray.o, C);
    T b = dot(ray.d, s2r);
    if (b > 0) return hr;
    T dis = b * b - dot(s2r, s2r) + o.radius_sqr;
    if (dis < 0) return hr;
    T t = -(dot(ray.d, s2r) + std::sqrt(dis));
    if (t < hr.dist && (double)t > 1e-6) {
        Hit<T> nh(t);
        nh.pos = add(ray.o, scl(ray.d, t));
        nh.n = nrm(sub(nh.pos, C));
        nh.mtl = o.mtl;
        nh.obj = key;
        nh.inside = (uint8_t)~ray.inside;
        nh.rfr = M.rfr;
        nh.obj_index = o.index, nh.prim = sub_id, nh.uid = key;
        return nh;
    }
    return hr;
}

template <class T> std::vector<V3<T>> ballplane_centres(const Obj<T> &o)
{
    std::vector<V3<T>> c;
    const T r = o.radius;
    for (T cx = r * -6; cx < r * 8; cx += r * 4)
        for (T cy = r * -6; cy < r * 8; cy += r * 4) c.push_back(add(add(scl(o.axisx, cx), scl(o.axisy, cy)), o.pos));
    return c;
}

template <class T> Hit<T> intersect(const Scene<T> &S, const Obj<T> &o, const Ray<T> &ray, const Hit<T> &hr, T minv)
{
    const int64_t key = obj_key(o.index);
    switch (o.kind) {
    case RT_OBJECT_SPHERE:
        return sphere_hit(S, o, o.pos, key, 0, ray, hr);
    case RT_OBJECT_PLANE: {
        if (hr.obj == key) return hr;
        T a = dot(ray.d, o.normal);
        if ((double)std::fabs(a) < 1e-6) return hr;
        V3<T> p2r = sub(ray.o, o.pos);
        T b = dot(p2r, o.normal);
        T dis = -b / a;
        if (dis < 0) return hr;
        if (dis < hr.dist) {
            Hit<T> nh(dis);
            texture_uv(o, ray, nh.tu, nh.tv);
            nh.n = o.normal;
            nh.mtl = o.mtl;
            nh.tex = o.tex;
            nh.pos = add(ray.o, scl(ray.d, dis));
            nh.obj = key;
            nh.obj_index = o.index, nh.uid = key;
            return nh;
        }
        return hr;
    }
    case RT_OBJECT_CUBE: {
        if (hr.obj == key) return hr;
        T res = border_test(ray, add(o.bmin, o.pos), add(o.bmax, o.pos));
        if (res < hr.dist && (double)res > 1e-6) {
            Hit<T> nh(res);
            nh.pos = add(ray.o, scl(ray.d, res));
            V3<T> b2p = sub(nh.pos, o.pos), pt = mk(T(0), T(0), T(0));
            if ((double)std::fabs(std::fabs(b2p.z) - o.bmax.z) < 1e-6) pt.z = b2p.z > 0 ? T(1) : T(-1);
            if ((double)std::fabs(std::fabs(b2p.y) - o.bmax.y) < 1e-6) pt.y = b2p.y > 0 ? T(1) : T(-1);
            if ((double)std::fabs(std::fabs(b2p.x) - o.bmax.x) < 1e-6) pt.x = b2p.x > 0 ? T(1) : T(-1);
            nh.n = nrm(pt);
            nh.mtl = o.mtl;
            nh.obj = key;
            nh.obj_index = o.index, nh.uid = key;
            return nh;
        }
        return hr;
    }
    case RT_OBJECT_BALLPLANE: {
        Hit<T> nh = hr;
        const auto cs = ballplane_centres(o);
        for (size_t c = 0; c < cs.size(); ++c) {
            const int cnt = (int)c + 1;
            const int64_t k2 = obj_key(o.index, cnt);
            // the inside branch compares against the incoming hr, then continues with nh
            if (hr.obj == k2) {
                if (!ray.inside) continue;
                if (ray.type == RAY_SHADOW) return Hit<T>(o.radius);
            }
            Hit<T> probe = nh;
            probe.obj = hr.obj;
            Hit<T> r = sphere_hit(S, o, cs[c], k2, cnt, ray, probe);
            if (r.dist < nh.dist) nh = r;
        }
        if (nh.dist < hr.dist) return nh;
        return hr;
    }
    case RT_OBJECT_MODEL: {
        const V3<T> bmn = add(o.bmin, o.pos), bmx = add(o.bmax, o.pos);
        T ans = border_test(ray, bmn, bmx);
        if (ans < hr.dist) {
            ans = hr.dist;
            const Tri<T> *objclt = nullptr;
            T cu = 0, cv = 0;
            bool mask[8];
            for (size_t a = 0; a < o.part_tris.size(); ++a) {
                if (border_test_ex(ray, add(o.borders[2 * a], o.pos), add(o.borders[2 * a + 1], o.pos), mask) < hr.dist) {
                    for (int b = 0; b < 8; ++b) {
                        if (!mask[b]) continue;
                        for (const Tri<T> &t : o.oct[a * 8 + b]) {
                            if (hr.obj == t.key) continue;
                            T u, v;
                            T na = tri_test(ray, t, u, v);
                            if (na < ans) {
                                objclt = &t;
                                ans = na;
                                cu = u, cv = v;
                                if (na < minv) goto eos;
                            }
                        }
                    }
                }
            }
        eos:
            if (ans < hr.dist) {
                Hit<T> nh(ans);
                const int64_t g = objclt->uid;
                const rt_scene_desc *d = S.d;
                const T w = T(1) - cu - cv;
                nh.pos = add(ray.o, scl(ray.d, ans));
                V3<T> n0 = v3<T>(d->tri_n + 9 * g), n1 = v3<T>(d->tri_n + 9 * g + 3), n2 = v3<T>(d->tri_n + 9 * g + 6);
                nh.n = nrm(add(add(scl(n0, w), scl(n1, cu)), scl(n2, cv)));
                if (d->tri_uv) {
                    const float *uv = d->tri_uv + 6 * g;
                    nh.tu = T(uv[0]) * w + T(uv[2]) * cu + T(uv[4]) * cv;
                    nh.tv = T(uv[1]) * w + T(uv[3]) * cu + T(uv[5]) * cv;
                }
                nh.mtl = d->tri_mtl[g];
                nh.rfr = S.mtls[nh.mtl].rfr;
                nh.tex = S.mtls[nh.mtl].tex;
                nh.obj = objclt->key;
                nh.obj_index = o.index;
                nh.prim = d->tri_id ? d->tri_id[g] : (int)(g - o.tri_first);
                nh.uid = COPY_BIT | g;
                return nh;
            }
        }
        return hr;
    }
    }
    return hr;
}

// ---- brute-force check over every primitive (check mode) -----------------------------------------
template <class T> struct Cand {
    T t;
    int ord;
    int64_t uid;
};

// candidates of one ray with the renderer's exclusion rule (the starting triangle by identity,
// the starting sphere through its inside branch); appends every hit
template <class T> void all_hits(const Scene<T> &S, const Ray<T> &ray, int64_t excl_uid, std::vector<Cand<T>> &out)
{
    Hit<T> none(T(1e20f));
    for (const Obj<T> &o : S.objs) {
        if (!o.show) continue;
        if (o.kind == RT_OBJECT_MODEL) {
            for (const auto &pt : o.part_tris)
                for (int64_t g : pt) {
                    if ((COPY_BIT | g) == excl_uid) continue;
                    const rt_scene_desc *d = S.d;
                    const V3<T> p0 = v3<T>(d->tri_p + 9 * g), p1 = v3<T>(d->tri_p + 9 * g + 3), p2 = v3<T>(d->tri_p + 9 * g + 6);
                    Tri<T> t{sub(p1, p0), sub(p2, p0), add(p0, o.pos), 0, 0, 0, g};
                    T u, v;
                    T na = tri_test(ray, t, u, v);
                    if (na < T(1e20f)) out.push_back(Cand<T>{na, o.index, COPY_BIT | g});
                }
        } else if (o.kind == RT_OBJECT_BALLPLANE) {
            const auto cs = ballplane_centres(o);
            for (size_t c = 0; c < cs.size(); ++c) {
                const int64_t k2 = obj_key(o.index, (int)c + 1);
                Hit<T> probe = none;
                probe.obj = excl_uid;
                Hit<T> r = sphere_hit(S, o, cs[c], k2, (int)c + 1, ray, probe);
                if (r.dist < T(1e20f) && r.obj == k2) out.push_back(Cand<T>{r.dist, o.index, k2});
            }
        } else {
            Hit<T> probe = none;
            probe.obj = excl_uid;
            Hit<T> r = intersect(S, o, ray, probe, T(0));
            if (r.dist < T(1e20f) && r.obj == obj_key(o.index)) out.push_back(Cand<T>{r.dist, o.index, r.uid});
        }
    }
}

template <class T> void check_closest(const Scene<T> &S, const Ray<T> &ray, int64_t excl_uid, const Hit<T> &ref, Tls &tls)
{
    std::vector<Cand<T>> c;
    all_hits(S, ray, excl_uid, c);
    const Cand<T> *b1 = nullptr, *b2 = nullptr;
    for (const auto &x : c) {
        if (!b1 || x.t < b1->t || (x.t == b1->t && x.ord < b1->ord)) b2 = b1, b1 = &x;
        else if (!b2 || x.t < b2->t) b2 = &x;
    }
    const int64_t ref_uid = ref.dist < T(1e20f) ? ref.uid : -1;
    const int64_t bf_uid = b1 ? b1->uid : -1;
    if (ref_uid != bf_uid) tls.ambiguous |= AMB_WINNER;
    if (b1 && b2 && (double)(b2->t - b1->t) < 1e-6 * (double)std::fabs(b1->t)) tls.ambiguous |= AMB_TIE;
}

template <class T> void check_shadow(const Scene<T> &S, const Ray<T> &ray, int64_t excl_uid, T dis, bool ref_blocked, Tls &tls)
{
    std::vector<Cand<T>> c;
    all_hits(S, ray, excl_uid, c);
    bool blocked = false;
    for (const auto &x : c) {
        if (x.t < dis) blocked = true;
        if ((double)std::fabs(x.t - dis) < 1e-6 * (double)dis) tls.ambiguous |= AMB_SHADOW_EDGE;
    }
    if (blocked != ref_blocked) tls.ambiguous |= AMB_SHADOW;
}

// uid of the primitive behind an exclude key (octant copies share their triangle's uid)
template <class T> int64_t uid_of(const Scene<T> &S, int64_t key)
{
    if (key < 0) return -1;
    if (key & COPY_BIT) {
        const int64_t serial = key & ~COPY_BIT;
        return serial < (int64_t)S.copy2tri.size() ? (COPY_BIT | S.copy2tri[(size_t)serial]) : -1;
    }
    return key;
}

// ---- RTfrac (RayTracer.cpp:450-596) ----------------------------------------------------------------
template <class T> Color<T> tex_color(const Scene<T> &S, int tex, T u, T v, int &amb)
{
    if (tex < 0) return Color<T>{1, 1, 1, 0};
    const Tex &t = S.texs[tex];
    T ip;
    T nu = std::modf(u, &ip), nv = std::modf(v, &ip);
    if (nu < 0) nu += 1;
    if (nv < 0) nv += 1;
    T fx = nu * T(t.w), fy = nv * T(t.h);
    int x = fx == fx ? (int)(int16_t)(int)fx : 0, y = fy == fy ? (int)(int16_t)(int)fy : 0;
    int64_t off = ((int64_t)y * t.w + x) * 3, last = ((int64_t)t.w * t.h - 1) * 3;
    if (off > last || off < 0) amb |= AMB_TEXEL_OOB;
    off = off > last ? last : (off < 0 ? 0 : off);
    return Color<T>{T(t.bgr[off + 2]) / T(255), T(t.bgr[off + 1]) / T(255), T(t.bgr[off]) / T(255), 0};
}

template <class T> struct Tracer {
    const Scene<T> &S;
    int max_level;
    Tls &tls;
    bool reflect_only = false;   // RTflec (RayTracer.cpp:332-448): RTfrac without the refraction branch

    Color<T> rtfrac(T zNear, T zFar, const Ray<T> &ray, int level, T bwc, int64_t base_obj, Hit<T> *primary)
    {
        if (level > max_level || bwc < T(1e-5f)) return Color<T>{0, 0, 0, T(1e20f)};
        ++(level == 0 ? tls.counts.primary : tls.counts.secondary);
        Hit<T> hr(T(1e20f));
        hr.obj = base_obj;
        int64_t newobj = base_obj;
        for (const Obj<T> &o : S.objs) {
            if (!o.show) continue;
            hr.obj = base_obj;
            hr = intersect(S, o, ray, hr, T(0));
            if (hr.obj != base_obj) newobj = hr.obj;
        }
        if (tls.check) check_closest(S, ray, uid_of(S, base_obj), hr, tls);
        if (primary) *primary = hr;
        if (hr.dist > zFar || hr.dist < zNear) return Color<T>{0, 0, 0, T(1e20f)};
        const Mtl<T> &M = S.mtls[hr.mtl];
        const Color<T> vc = tex_color(S, hr.tex, hr.tu, hr.tv, tls.ambiguous);
        V3<T> mix_vd = mk(T(0), T(0), T(0)), mix_vsc = mk(T(0), T(0), T(0));
        V3<T> mix_va = mul(M.ka, S.env);
        for (const Lit<T> &L : S.lights) {
            if (!L.on) continue;
            V3<T> la, ld, ls, p2l;
            T dis;
            if (L.type == RT_LIGHT_POINT) {
                V3<T> p2l_v = sub(L.pos, hr.pos);
                dis = dot(p2l_v, p2l_v);
                T step = L.att.x + L.att.z * dis;
                dis = std::sqrt(dis);
                step += L.att.y * dis;
                T lum = T(1) / step;
                la = scl(L.amb, lum), ld = scl(L.dif, lum), ls = scl(L.spec, lum);
                p2l = nrm(p2l_v);
            } else {
                dis = T(1e10f);
                la = L.amb, ld = L.dif, ls = L.spec;
                p2l = nrm(L.pos);
            }
            mix_va = add(mix_va, mul(M.ka, la));
            Ray<T> sr{hr.pos, p2l, T(1), RAY_SHADOW, 0};
            Hit<T> shr(dis);
            shr.obj = newobj;
            ++tls.counts.shadow;
            bool blocked = false;
            for (const Obj<T> &o : S.objs) {
                if (o.show) shr = intersect(S, o, sr, shr, dis);
                if (shr.dist < dis) {
                    blocked = true;
                    break;
                }
            }
            if (tls.check) check_shadow(S, sr, uid_of(S, newobj), dis, blocked, tls);
            if (blocked) continue;
            T nn = dot(hr.n, p2l);
            if (nn > 0) mix_vd = add(mix_vd, scl(mul(M.kd, ld), nn));
            V3<T> h = nrm(sub(p2l, ray.d));
            nn = dot(hr.n, h);
            if (nn > 0) {
                V3<T> vs = scl(mul(M.ks, ls), (T)std::pow(nn, M.shininess));
                mix_vsc = add(mix_vsc, mk(T(1) * vs.x, T(1) * vs.y, T(1) * vs.z));
            }
        }
        const V3<T> s = add(mix_vd, mix_va);
        Color<T> c{vc.r * s.x + mix_vsc.x, vc.g * s.y + mix_vsc.y, vc.b * s.z + mix_vsc.z, T(1e20f)};
        if (M.reflect > T(0.01f)) {
            const T r = M.reflect;
            c.r *= (1 - r), c.g *= (1 - r), c.b *= (1 - r);
            T nn = 2 * dot(ray.d, hr.n);
            V3<T> R = nrm(sub(ray.d, scl(hr.n, nn)));
            Ray<T> fr{hr.pos, R, T(1), RAY_REFLECT, 0};
            Color<T> cf = rtfrac(T(0), zFar, fr, level + 1, bwc * r, newobj, nullptr);
            c.r += cf.r * r, c.g += cf.g * r, c.b += cf.b * r;
        }
        if (!reflect_only && M.refract > T(0.01f)) {
            const T f = M.refract;
            c.r *= (1 - f), c.g *= (1 - f), c.b *= (1 - f);
            T n = ray.mtlrfr / hr.rfr;
            T cosIn = -dot(ray.d, hr.n);
            T cosOut2 = T(1) - (n * n) * (T(1) - cosIn * cosIn);
            if (!(cosOut2 < T(0))) {
                V3<T> l2 = scl(ray.d, n), l1 = scl(hr.n, n * cosIn - std::sqrt(cosOut2));
                Ray<T> tr{hr.pos, nrm(add(l1, l2)), hr.rfr, RAY_REFRACT, hr.inside};
                Color<T> cf = rtfrac(T(0), zFar, tr, level + 1, bwc * f, newobj, nullptr);
                Color<T> vf{1, 1, 1, 0};
                if (hr.inside) {
                    V3<T> e = scl(scl(M.kd, T(0.15f)), -cf.alpha);
                    vf = Color<T>{std::exp(e.x), std::exp(e.y), std::exp(e.z), 0};
                }
                c.r += cf.r * vf.r * f, c.g += cf.g * vf.g * f, c.b += cf.b * vf.b * f;
            }
        }
        c.alpha = hr.dist;
        return c;
    }

    // ---- the test modes (RayTracer.cpp:81-444) ----------------------------------------------
    // the first hit over Scene::Objects with a fresh HitRes (its key carried object to object,
    // as those loops do)
    Hit<T> first_hit(const Ray<T> &ray, Hit<T> *primary)
    {
        ++tls.counts.primary;
        Hit<T> hr(T(1e20f));
        for (const Obj<T> &o : S.objs)
            if (o.show) hr = intersect(S, o, ray, hr, T(0));
        if (tls.check) check_closest(S, ray, uid_of(S, NO_KEY), hr, tls);
        if (primary) *primary = hr;
        return hr;
    }

    // RTdepth + Color::set (3DElement.cpp:451-462); log of a float is the float overload
    Color<T> rtdepth(T zNear, T zFar, const Ray<T> &ray, Hit<T> *primary)
    {
        const Hit<T> hr = first_hit(ray, primary);
        const T d = hr.dist;
        if (d <= zNear) return Color<T>{1, 0, 0, 0};
        if (d >= zFar) return Color<T>{0, 0, 0, 0};
        const T after = std::log(d), mx = std::log(zFar);
        const T g = (mx - after) / mx;
        return Color<T>{g, g, g, 0};
    }

    // RTnorm + Color(const Normal&): 0.5 * (n + 1) in double, stored as float
    Color<T> rtnorm(T zNear, T zFar, const Ray<T> &ray, Hit<T> *primary)
    {
        const Hit<T> hr = first_hit(ray, primary);
        if (hr.dist > zFar) return Color<T>{0, 0, 0, 0};
        if (hr.dist < zNear) return Color<T>{1, 1, 1, 0};
        return Color<T>{(T)(0.5 * ((double)hr.n.x + 1)), (T)(0.5 * ((double)hr.n.y + 1)), (T)(0.5 * ((double)hr.n.z + 1)), 0};
    }

    // RTtex
    Color<T> rttex(T zNear, T zFar, const Ray<T> &ray, Hit<T> *primary)
    {
        const Hit<T> hr = first_hit(ray, primary);
        if (hr.dist > zFar) return Color<T>{0, 0, 0, 0};
        if (hr.dist < zNear) return Color<T>{1, 1, 1, 0};
        if (hr.tex >= 0) return tex_color(S, hr.tex, hr.tu, hr.tv, tls.ambiguous);
        return Color<T>{T(0.588f), T(0.588f), T(0.588f), 0};
    }

    // RTmtl: local terms of every light, no shadow test; point light when position.w != 0
    Color<T> rtmtl(T zNear, T zFar, const Ray<T> &ray, Hit<T> *primary)
    {
        const Hit<T> hr = first_hit(ray, primary);
        if (hr.dist > zFar) return Color<T>{0, 0, 0, 0};
        if (hr.dist < zNear) return Color<T>{1, 1, 1, 0};
        const Mtl<T> &M = S.mtls[hr.mtl];
        const Color<T> vc = tex_color(S, hr.tex, hr.tu, hr.tv, tls.ambiguous);
        V3<T> mix_vd = mk(T(0), T(0), T(0)), mix_va = mix_vd, mix_vsc = mix_vd;
        for (const Lit<T> &L : S.lights) {
            if (!L.on) continue;
            T lum;
            V3<T> p2l;
            if (L.type != RT_LIGHT_PARALLEL) {   // position.alpha 1 for point and spot lights
                V3<T> p2l_v = sub(L.pos, hr.pos);
                T dis = dot(p2l_v, p2l_v);
                T step = L.att.x + L.att.y * std::sqrt(dis) + L.att.z * dis;
                lum = T(1) / step;
                p2l = nrm(p2l_v);
            } else {
                lum = T(1);
                p2l = nrm(L.pos);
            }
            const V3<T> la = scl(L.amb, lum), ld = scl(L.dif, lum), ls = scl(L.spec, lum);
            mix_va = add(mix_va, mul(M.ka, la));
            T nn = dot(hr.n, p2l);
            if (nn > 0) mix_vd = add(mix_vd, scl(mul(M.kd, ld), nn));
            V3<T> h = nrm(sub(p2l, ray.d));
            nn = dot(hr.n, h);
            if (nn > 0) {
                V3<T> vs = scl(mul(M.ks, ls), (T)std::pow(nn, M.shininess));
                mix_vsc = add(mix_vsc, mk(T(1) * vs.x, T(1) * vs.y, T(1) * vs.z));
            }
        }
        mix_va = add(mix_va, mul(M.ka, S.env));
        const V3<T> sm = add(mix_vd, mix_va);
        return Color<T>{vc.r * sm.x + mix_vsc.x, vc.g * sm.y + mix_vsc.y, vc.b * sm.z + mix_vsc.z, 0};
    }

    // RTshd: one bounce with shadow rays (the hit excludes itself), environment ambient last
    Color<T> rtshd(T zNear, T zFar, const Ray<T> &ray, Hit<T> *primary)
    {
        const Hit<T> hr = first_hit(ray, primary);
        if (hr.dist > zFar) return Color<T>{0, 0, 0, 0};
        if (hr.dist < zNear) return Color<T>{1, 1, 1, 0};
        const Mtl<T> &M = S.mtls[hr.mtl];
        const Color<T> vc = tex_color(S, hr.tex, hr.tu, hr.tv, tls.ambiguous);
        V3<T> mix_vd = mk(T(0), T(0), T(0)), mix_va = mix_vd, mix_vsc = mix_vd;
        for (const Lit<T> &L : S.lights) {
            if (!L.on) continue;
            T lum, dis;
            V3<T> p2l;
            if (L.type == RT_LIGHT_POINT) {
                V3<T> p2l_v = sub(L.pos, hr.pos);
                dis = dot(p2l_v, p2l_v);
                T step = L.att.x + L.att.z * dis;
                dis = std::sqrt(dis);
                step += L.att.y * dis;
                lum = T(1) / step;
                p2l = nrm(p2l_v);
            } else {
                dis = T(1e10f);
                lum = T(1);
                p2l = nrm(L.pos);
            }
            const V3<T> la = scl(L.amb, lum), ld = scl(L.dif, lum), ls = scl(L.spec, lum);
            mix_va = add(mix_va, mul(M.ka, la));
            Ray<T> sr{hr.pos, p2l, T(1), RAY_SHADOW, 0};
            Hit<T> shr(dis);
            shr.obj = hr.obj;
            ++tls.counts.shadow;
            bool blocked = false;
            for (const Obj<T> &o : S.objs) {
                if (o.show) shr = intersect(S, o, sr, shr, dis);
                if (shr.dist < dis) {
                    blocked = true;
                    break;
                }
            }
            if (tls.check) check_shadow(S, sr, uid_of(S, hr.obj), dis, blocked, tls);
            if (blocked) continue;
            T nn = dot(hr.n, p2l);
            if (nn > 0) mix_vd = add(mix_vd, scl(mul(M.kd, ld), nn));
            V3<T> h = nrm(sub(p2l, ray.d));
            nn = dot(hr.n, h);
            if (nn > 0) {
                V3<T> vs = scl(mul(M.ks, ls), (T)std::pow(nn, M.shininess));
                mix_vsc = add(mix_vsc, mk(T(1) * vs.x, T(1) * vs.y, T(1) * vs.z));
            }
        }
        mix_va = add(mix_va, mul(M.ka, S.env));
        const V3<T> sm = add(mix_vd, mix_va);
        return Color<T>{vc.r * sm.x + mix_vsc.x, vc.g * sm.y + mix_vsc.y, vc.b * sm.z + mix_vsc.z, 0};
    }
};

// Philox4x32-10 (Salmon et al., SC'11), the jitter stream of multi-sample renders
inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)M0 * c[0], p1 = (uint64_t)M1 * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0, c[1] = lo1, c[2] = n2, c[3] = lo0;
        k0 += 0x9E3779B9u, k1 += 0xBB67AE85u;
    }
}

inline uint8_t put_channel(double c)
{
    float f = (float)c;
    if (f > 1.0f) return 255;
    if (f < 0.0f || f != f) return 0;
    return (uint8_t)(int)(f * 255);
}

struct Params {
    int32_t width, height, spp, max_level, ref_tiles, threads, check;
    uint64_t seed;
    const int32_t *tiles;   // 64x64 tile indices to render (NULL = all)
    int32_t n_tiles;
    int32_t block;          // work-unit edge inside a tile for the thread pool (64 = whole tile)
    int32_t mode;           // RT_MODE_* (0 = RT_MODE_RAYTRACE)
    const uint8_t *check_mask;   // with check: only pixels whose byte is non-zero are checked (NULL = all)
    double *tile_seconds;        // per entry of the tile list: thread-seconds spent on it (NULL = not kept)
    int64_t *tile_rays;          // per entry of the tile list: rays traced for it (NULL = not kept)
};

template <class T>
int render(const rt_scene_desc *d, const Params &p, T *rgb, uint8_t *rgb8, int32_t *hobj, int32_t *hprim, float *ht,
           uint8_t *amb, int64_t *counts, double *seconds)
{
    Scene<T> S;
    build_scene<T>(d, S);
    const rt_camera &cam = d->camera;
    const int W = p.width > 0 ? p.width : cam.width, H = p.height > 0 ? p.height : cam.height;
    const int xlim = p.ref_tiles ? (W / 64) * 64 : W, ylim = p.ref_tiles ? (H / 64) * 64 : H;
    const double PIr = 3.1415926535897932384;
    const double dp = std::tan(cam.fovy * PIr / 360) / (H / 2);
    const T zNear = T(cam.znear);
    const T zFar = (T)(std::sqrt(2.0) * (double)cam.zfar);   // float in the reference
    const float zFar32 = (float)(std::sqrt(2.0) * (double)cam.zfar);
    const V3<T> cn = v3<T>(cam.n), cu = v3<T>(cam.u), cv = v3<T>(cam.v), cp = v3<T>(cam.position);
    const int bw = (xlim + 63) / 64, bh = (ylim + 63) / 64;
    std::vector<int32_t> tiles;
    if (p.tiles)
        tiles.assign(p.tiles, p.tiles + p.n_tiles);
    else
        for (int i = 0; i < bw * bh; ++i) tiles.push_back(i);
    // work units: each 64x64 tile, optionally cut into block x block pieces (results do not
    // depend on the split; the timed baseline keeps whole tiles like parallelRT)
    const int blk = (p.block > 0 && p.block < 64 && 64 % p.block == 0) ? p.block : 64;
    const int per_tile = (64 / blk) * (64 / blk);
    std::atomic<int64_t> next(0);
    std::vector<Counts> per((size_t)std::max(1, p.threads));
    // per tile-list entry: thread time and rays of its work units, summed over threads
    std::vector<std::atomic<int64_t>> tile_ns(tiles.size()), tile_rays(tiles.size());
    for (size_t i = 0; i < tiles.size(); ++i) tile_ns[i] = 0, tile_rays[i] = 0;
    auto worker = [&](int tid) {
        Tls tls;
        tls.check = p.check;
        const int mode = p.mode ? p.mode : RT_MODE_RAYTRACE;
        Tracer<T> tr{S, p.max_level, tls};
        tr.reflect_only = mode == RT_MODE_REFLECT;
        while (true) {
            const int64_t k = next.fetch_add(1);
            if (k >= (int64_t)tiles.size() * per_tile) break;
            const size_t entry = (size_t)(k / per_tile);
            const int tile = tiles[entry], sub = (int)(k % per_tile);
            const auto unit_t0 = std::chrono::steady_clock::now();
            const int64_t unit_rays0 = tls.counts.primary + tls.counts.secondary + tls.counts.shadow;
            const int bx = tile % bw, by = tile / bw;
            const int r0 = by * 64 + (sub / (64 / blk)) * blk, c0 = bx * 64 + (sub % (64 / blk)) * blk;
            for (int row = r0; row < std::min(ylim, r0 + blk); ++row)
                for (int col = c0; col < std::min(xlim, c0 + blk); ++col) {
                    const int xcur = col - W / 2, ycur = row - H / 2;
                    const size_t pix = (size_t)row * W + col;
                    tls.ambiguous = 0;
                    tls.check = p.check && (!p.check_mask || p.check_mask[pix]);
                    T acc[3] = {0, 0, 0};
                    for (int s = 0; s < p.spp; ++s) {
                        T a, b;
                        if (p.spp > 1) {
                            uint32_t c[4] = {(uint32_t)pix, 0u, (uint32_t)s, 0u};
                            philox(c, (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
                            double jx = (double)(c[0] >> 8) * (1.0 / 16777216.0), jy = (double)(c[1] >> 8) * (1.0 / 16777216.0);
                            if (sizeof(T) == 4) a = (T)(float)(((double)xcur + jx) * dp), b = (T)(float)(((double)ycur + jy) * dp);
                            else a = (T)(((double)xcur + jx) * dp), b = (T)(((double)ycur + jy) * dp);
                        } else {
                            if (sizeof(T) == 4) a = (T)(float)(xcur * dp), b = (T)(float)(ycur * dp);
                            else a = (T)(xcur * dp), b = (T)(ycur * dp);
                        }
                        V3<T> dir = nrm(add(add(cn, scl(cu, a)), scl(cv, b)));
                        Ray<T> ray{cp, dir, T(1), RAY_BASE, 0};
                        Hit<T> prim;
                        const T zf = sizeof(T) == 4 ? (T)zFar32 : zFar;
                        Hit<T> *pp = s == 0 ? &prim : nullptr;
                        Color<T> c;
                        switch (mode) {
                        case RT_MODE_CHECK: {   // RTcheck: white where the tile row and column parities agree
                            const T wv = ((row >> 6) & 1) == ((col >> 6) & 1) ? T(1) : T(0);
                            c = Color<T>{wv, wv, wv, 0};
                            prim = tr.first_hit(ray, nullptr);
                            break;
                        }
                        case RT_MODE_DEPTH: c = tr.rtdepth(zNear, zf, ray, pp); break;
                        case RT_MODE_NORMAL: c = tr.rtnorm(zNear, zf, ray, pp); break;
                        case RT_MODE_TEXTURE: c = tr.rttex(zNear, zf, ray, pp); break;
                        case RT_MODE_MATERIAL: c = tr.rtmtl(zNear, zf, ray, pp); break;
                        case RT_MODE_SHADOW: c = tr.rtshd(zNear, zf, ray, pp); break;
                        default: c = tr.rtfrac(zNear, zf, ray, 0, T(1), NO_KEY, pp); break;
                        }
                        acc[0] += c.r, acc[1] += c.g, acc[2] += c.b;
                        if (s == 0) {
                            const bool hit = prim.dist < T(1e20f) && prim.obj_index >= 0;
                            if (hobj) hobj[pix] = hit ? prim.obj_index : -1;
                            if (hprim) hprim[pix] = hit ? prim.prim : 0;
                            if (ht) ht[pix] = hit ? (float)prim.dist : 1e20f;
                        }
                    }
                    for (int k2 = 0; k2 < 3; ++k2) {
                        T v = p.spp > 1 ? acc[k2] * (T(1) / T(p.spp)) : acc[k2];
                        if (rgb) rgb[3 * pix + k2] = v;
                        if (rgb8) rgb8[3 * pix + k2] = put_channel((double)v);
                    }
                    if (amb) amb[pix] = (uint8_t)tls.ambiguous;
                }
            tile_ns[entry] += std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - unit_t0)
                                  .count();
            tile_rays[entry] += tls.counts.primary + tls.counts.secondary + tls.counts.shadow - unit_rays0;
        }
        per[(size_t)tid] = tls.counts;
    };
    const auto t0 = std::chrono::steady_clock::now();
    const int nt = std::max(1, p.threads);
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker, i);
    worker(0);
    for (auto &t : th) t.join();
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (size_t i = 0; i < tiles.size(); ++i) {
        if (p.tile_seconds) p.tile_seconds[i] = 1e-9 * (double)tile_ns[i].load();
        if (p.tile_rays) p.tile_rays[i] = tile_rays[i].load();
    }
    if (counts) {
        Counts c;
        for (auto &x : per) c.primary += x.primary, c.secondary += x.secondary, c.shadow += x.shadow;
        counts[0] = c.primary, counts[1] = c.secondary, counts[2] = c.shadow;
    }
    return 0;
}

inline uint32_t expand10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

} // namespace

extern "C" {

typedef struct orc_params {
    int32_t width, height, spp, max_level, ref_tiles, threads, check;
    uint64_t seed;
    const int32_t *tiles;
    int32_t n_tiles;
    int32_t block;
    int32_t mode;
    const uint8_t *check_mask;   // W*H bytes: with check, only the non-zero pixels are checked (NULL = all)
    double *tile_seconds;        // n_tiles entries (all tiles when `tiles` is NULL): thread-seconds per tile
    int64_t *tile_rays;          // the same entries: rays traced per tile
} orc_params;

int orc_render_f32(const rt_scene_desc *d, const orc_params *p, float *rgb, uint8_t *rgb8, int32_t *obj, int32_t *prim,
                   float *t, uint8_t *amb, int64_t *counts, double *seconds)
{
    if (!d || !p) return -1;
    Params q{p->width, p->height, p->spp, p->max_level, p->ref_tiles, p->threads, p->check, p->seed, p->tiles, p->n_tiles,
             p->block, p->mode, p->check_mask, p->tile_seconds, p->tile_rays};
    return render<float>(d, q, rgb, rgb8, obj, prim, t, amb, counts, seconds);
}

int orc_render_f64(const rt_scene_desc *d, const orc_params *p, double *rgb, int32_t *obj, int32_t *prim, float *t,
                   int64_t *counts, double *seconds)
{
    if (!d || !p) return -1;
    Params q{p->width, p->height, p->spp, p->max_level, p->ref_tiles, p->threads, 0, p->seed, p->tiles, p->n_tiles,
             p->block, p->mode, nullptr, p->tile_seconds, p->tile_rays};
    return render<double>(d, q, rgb, nullptr, obj, prim, t, nullptr, counts, seconds);
}

// CPU reference of the device Morton sort: same box, centroid and quantisation arithmetic,
// then std::stable_sort of triangle indices by code
int orc_morton_sort(const float *tri_p, int64_t n, uint32_t *codes, uint32_t *perm)
{
    if (n < 0 || (n > 0 && (!tri_p || !codes || !perm))) return -1;
    std::vector<float> cen((size_t)n * 3);
    float smn[3] = {INFINITY, INFINITY, INFINITY}, smx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; ++i) {
        const float *p = tri_p + 9 * i;
        for (int k = 0; k < 3; ++k) {
            float p0 = p[k] + 0.0f, e1 = p[3 + k] - p[k], e2 = p[6 + k] - p[k];
            float a = p0, b = p0 + e1, c = p0 + e2;
            float mn = std::fmin(a, std::fmin(b, c)), mx = std::fmax(a, std::fmax(b, c));
            cen[(size_t)(3 * i + k)] = (mn + mx) * 0.5f;
            smn[k] = std::fmin(smn[k], mn);
            smx[k] = std::fmax(smx[k], mx);
        }
    }
    // one scale for all axes: the largest extent of the box / 1024 (cubic cells)
    float emax = 0.0f;
    for (int k = 0; k < 3; ++k) emax = std::fmax(emax, smx[k] - smn[k]);
    const float s = emax > 0.0f ? 1024.0f / emax : 0.0f;
    const float scale[3] = {s, s, s};
    std::vector<uint32_t> code((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            float f = (cen[(size_t)(3 * i + k)] - smn[k]) * scale[k];
            int qi = (int)f;
            q[k] = (uint32_t)std::min(std::max(qi, 0), 1023);
        }
        code[(size_t)i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    }
    std::vector<uint32_t> idx((size_t)n);
    for (int64_t i = 0; i < n; ++i) idx[(size_t)i] = (uint32_t)i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });
    for (int64_t i = 0; i < n; ++i) {
        perm[i] = idx[(size_t)i];
        codes[i] = code[idx[(size_t)i]];
    }
    return 0;
}

} // extern "C"
