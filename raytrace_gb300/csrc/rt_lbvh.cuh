// rt_lbvh.cuh — device LBVH build interface (rt_lbvh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtg {

// an unused slot of a 4-wide node (no leaf index reaches ~0x80000000)
constexpr int kEmptySlot = (int)0x80000000;

// inputs of one build, all device pointers; triangle i of the scene has points tri_p[9i..],
// normals tri_n[9i..], optional uvs tri_uv[6i..], material tri_mtl[i], reported id tri_id[i]
// and object index tri_obj[i] (whose position obj_pos[3*obj..] is added to the points)
struct LbvhInput {
    const float *tri_p, *tri_n, *tri_uv;
    const int *tri_mtl, *tri_id, *tri_obj;
    const float *obj_pos;
    int n;                 // triangles
    // spheres as further leaves after the triangles (NULL / 0 when none)
    const float4 *sph;     // centre xyz, r*r (the exact test's data)
    const float *sph_r;    // radius (leaf box half extent)
    const int *sph_prim;   // analytic primitive index = the hit key
    const int *sph_obj;    // object order
    int n_sph;
    // material check of the gather: a triangle material outside [0, n_mtl) sets *bad (NULL =
    // no check); the caller rejects the scene
    int n_mtl;
    int *bad;
    // clustering build instead of the Karras hierarchy when not NULL: a page-locked int the
    // build reads each round's survivor count through (NULL = Karras radix tree)
    int *cluster_count;
};

// leaves = n + n_sph; leaf record k (Morton order), 3 float4:
//   triangle: (p0 | reported id), (e1 | object), (e2 | material >= 0)
//   sphere:   (centre | r*r),     (0 | object),  (0 | -1 - primitive index)
struct LbvhOutput {
    float4 *nodes;   // 2 * (2L-1): own box per node, for refit and inspection
    float4 *quads;   // 8 * (L-1): per internal node its grandchildren (4-wide node), see k_quads
    float4 *tri;     // 3L leaf records
    float4 *trin;    // 3L (vertex normals; zero for spheres)
    float2 *triuv;   // 3L or NULL
};

// name of the build step whose launch failed last (for error messages)
extern const char *g_build_step;

// scratch bytes needed for n leaves (triangles + spheres)
size_t lbvh_scratch_bytes(int n);
// build into `out` using `scratch` (lbvh_scratch_bytes(n) bytes, 256-byte aligned). The boxes,
// codes and sort read only tri_p, tri_obj, obj_pos and the sphere arrays; when `shading_ready`
// is not NULL the gather (which reads the normals, uvs, materials and ids) waits for it.
cudaError_t lbvh_build(const LbvhInput &in, const LbvhOutput &out, void *scratch, cudaStream_t s,
                       cudaEvent_t shading_ready = nullptr);
// Morton codes of the triangle centroids over the scene box, then a stable radix sort;
// codes_out / perm_out receive the sorted codes and triangle indices (device pointers)
cudaError_t lbvh_morton_sort(const LbvhInput &in, uint32_t *codes_out, uint32_t *perm_out, void *scratch,
                             cudaStream_t s);

// per-triangle object index (and, when `ids` is not NULL, the index inside its model) from a
// table of (first, count, object) triples, one per shown model
void launch_tri_objects(const int *ranges, int n_ranges, int n, int *obj, int *ids, cudaStream_t s);

} // namespace rtg
