// rt_device.cuh — device data layout and exact-order arithmetic of the GB300 renderer.
//
// Every quantity that decides a hit (which primitive, at what distance) is computed with the
// reference's FP32 operation order and with explicit round-to-nearest intrinsics, so no
// multiply-add is fused regardless of compiler flags:
//   dot(a,b)   = (a.x*b.x + a.y*b.y) + (a.z*b.z + 0)   DPPS 0x71, 3DElement.cpp:206-214
//   cross(a,b) = (a.y*b.z - a.z*b.y, ...)               AVX branch, 3DElement.cpp:190-197
//   normalise  = v / sqrt(dot(v,v)) per lane            AVX2 branch, 3DElement.cpp:218-223
// Thresholds written against double constants in the reference (`t > 1e-6`, `abs(a) < 1e-6`)
// are turned into the equivalent float comparisons with kEps6 = (float)1e-6, which lies just
// below 1e-6: `x > 1e-6` == `x > kEps6` and `|x| < 1e-6` == `|x| <= kEps6` for every float x.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtg {

constexpr float kEps6 = 9.99999997e-07f;     // float nearest below 1e-6
constexpr float kMiss = 1e20f;               // HitRes() distance
constexpr int kTriFlag = 0x40000000;         // primitive key bit for triangles
constexpr int kMaxLights = 8;                // Scene::AddLight limit
// Traversal stack entries. A Karras node's common prefix grows by at least one bit per level
// over 30 Morton bits plus the index bits that break ties, so a path has at most 63 binary
// levels, i.e. 32 four-wide nodes, each pushing at most 3 entries.
constexpr int kStack = 96;

// ray type codes (MY_RAY_*)
constexpr int kRayBase = 1, kRayShadow = 2, kRayReflect = 3, kRayRefract = 4;
// render modes (RT_MODE_*, the reference's MY_MODEL_* test modes, RayTracer.cpp:631-662)
constexpr int kModeCheck = 0x1, kModeDepth = 0x2, kModeNormal = 0x3, kModeTexture = 0x4, kModeMaterial = 0x5,
              kModeShadow = 0x6, kModeReflect = 0x7, kModeRefract = 0x8, kModeRaytrace = 0x80;
// analytic primitive types (MY_OBJECT_* for the shapes that are intersected analytically)
constexpr int kPrimSphere = 1, kPrimBox = 2, kPrimPlane = 4;

// ---- exact arithmetic ---------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 mk(float4 v) { return V3{v.x, v.y, v.z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ V3 vmul(V3 a, V3 b) { return mk(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return mk(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ float dot3(V3 a, V3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fadd_rn(__fmul_rn(a.z, b.z), 0.0f));
}
__device__ __forceinline__ V3 cross3(V3 a, V3 b)
{
    return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ V3 normalise(V3 v)
{
    float len = __fsqrt_rn(dot3(v, v));
    return mk(__fdiv_rn(v.x, len), __fdiv_rn(v.y, len), __fdiv_rn(v.z, len));
}
// MINPS / MAXPS lane rules and std::min / std::max on floats (NaN handling matters)
__device__ __forceinline__ float minps(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float maxps(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float stdmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float stdmin(float a, float b) { return b < a ? b : a; }

// ---- scene tables in HBM -------------------------------------------------------------------
struct DevMaterial {                  // 64 B
    float ka[3], kd[3], ks[3];
    float shininess, reflect, refract, rfr;
    int tex;                          // texture index or -1
    int pad[2];
};

struct DevLight {                     // 64 B
    int type, on;
    float pos[3];
    float amb[3], dif[3], spec[3], att[3];
    float pad;
};

struct DevTexture {
    int w, h;
    long long offset;                 // byte offset into the texel pool
};

// analytic primitive (96 B): sphere, ballplane sphere, plane or box, in object order
struct DevPrim {
    float4 a;    // sphere: centre, r*r          plane: point, -      box: world min, -
    float4 b;    // sphere: r, -                 plane: normal, -     box: world max, -
    float4 c;    // plane: axisx                                      box: object position
    float4 d;    // plane: axisy                                      box: local max
    int type;    // kPrim*
    int obj;     // index in Scene::Objects (the reported object id and the tie-break order)
    int sub;     // ballplane sphere number 1..16, else 0
    int mtl;     // material index
    int tex;     // plane texture or -1
    int pad[3];
};

struct DevScene {
    const DevPrim *prims;         // planes and boxes first (tested linearly), then spheres
    int n_prims;
    int n_linear;                 // prims [0, n_linear) are outside the LBVH
    int n_tris;                   // triangles
    int n_leaves;                 // LBVH leaves: triangles + spheres
    const float4 *nodes;          // LBVH: (2L-1) nodes x 2 float4 (min|left, max|right)
    const float4 *quads;          // per internal node a 4-wide node of its grandchildren: 8 float4 (see k_quads)
    const float4 *tri;            // per leaf (Morton order): triangle p0|id, e1|obj, e2|mtl; sphere c|r2, 0|obj, 0|-1-prim
    const float4 *trin;           // per leaf: n0, n1, n2
    const float2 *triuv;          // per leaf: uv0, uv1, uv2 (NULL = zero)
    const DevMaterial *mtl;
    const DevLight *lights;
    const DevTexture *tex;
    const uint8_t *texels;
    int n_lights;
    int n_mtl;
    float env[3];
    int pad;
};

// one frame being rendered (a job); the batched path runs many jobs in one wavefront
struct DevJob {
    int scene;                    // index into the scene header array
    int width, height, spp;
    int max_level, flags, mode;
    int xlim, ylim;               // rendered region: cols < xlim, rows < ylim
    long long *acc;               // frame accumulator: 3 x int64 fixed point (2^-32) per pixel
    int *plane_obj;               // primary hit planes of sample 0 (NULL = not written)
    int *plane_prim;
    float *plane_t;
    const float *axis;            // camera offsets per column, then per row (1 sample/pixel; NULL = computed)
    long long sample_base;        // first global sample index of this job
    float cam_pos[3], cam_u[3], cam_v[3], cam_n[3];
    double dp;                    // tan(fovy*pi/360) / (H/2) in double (RayTracer.cpp:14)
    float znear, zfar;            // zfar already multiplied by sqrt(2) (RayTracer.cpp:15)
    unsigned long long seed;
    int slot;                     // serving slot (per-frame ray counter), -1 = none
    int pixel_tile;               // primary rays in pixel tiles of this edge, row-major tiles (0 = rows)
};

// ray queue, structure of arrays, 64 B per ray read as four 128-bit loads
struct RayQueue {
    float4 *o;      // origin xyz, bwc (RTfrac's benefit weight)
    float4 *d;      // direction xyz, mtlrfr (index of the medium the ray travels in)
    float4 *w;      // path weight rgb, pixel index in the frame (int bits)
    int4 *m;        // exclude key (HitRes::obj of the parent), flags, beer material, job
    int capacity;
};
// flags: level (bits 0-7) | type << 8 | isInside << 16 | hit-plane writer << 24
__device__ __forceinline__ int ray_level(int f) { return f & 0xff; }
__device__ __forceinline__ int ray_type(int f) { return (f >> 8) & 0xff; }
__device__ __forceinline__ int ray_inside(int f) { return (f >> 16) & 0xff; }
__device__ __forceinline__ bool ray_plane(int f) { return (f >> 24) & 1; }
__device__ __forceinline__ int ray_flags(int level, int type, int inside, int plane)
{
    return (level & 0xff) | (type & 0xff) << 8 | (inside & 0xff) << 16 | (plane & 1) << 24;
}

// the rays of one bounce that hit something, densely in the order extend found them: the ray
// record as in RayQueue plus the hit, 84 B per hit, read by shading with coalesced loads
struct HitQueue {
    float4 *o, *d, *w;
    int4 *m;
    float4 *h;      // distance, barycentrics u v, primitive key (int bits)
    int *nob;       // exclude key for the children (RTfrac's newobj)
};

// one hit point waiting for its shadow rays, 80 B
struct ShadowQueue {
    float4 *p;      // hit position, pixel index in the frame (int bits)
    float4 *n;      // shading normal, material (int bits)
    float4 *v;      // incoming direction, exclude key (int bits)
    float4 *wc;     // weight * texture colour, job (int bits)
    float4 *ws;     // weight
    int capacity;
};

// device counters of one wavefront pass
struct Counters {
    int q_count[2];                       // ping-pong ray queue sizes
    int pad0;
    int overflow;                         // a queue ran out of space
    int work[16];                         // dynamic work counters (reset per pass)
    int h_count[8];                       // hits listed by extend, per bounce
    unsigned long long rays_primary, rays_secondary, rays_shadow;
    unsigned long long nodes, tris, spheres;            // extend kernels (closest hit)
    unsigned long long s_nodes, s_tris, s_spheres;      // shadow kernels (any hit)
    int error;
    int pad[3];
};

} // namespace rtg
