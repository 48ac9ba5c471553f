// rt_lbvh.cuh — device LBVH build interface (rt_lbvh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtg {

// inputs of one build, all device pointers; triangle i of the scene has points tri_p[9i..],
// normals tri_n[9i..], optional uvs tri_uv[6i..], material tri_mtl[i], reported id tri_id[i]
// and object index tri_obj[i] (whose position obj_pos[3*obj..] is added to the points)
struct LbvhInput {
    const float *tri_p, *tri_n, *tri_uv;
    const int *tri_mtl, *tri_id, *tri_obj;
    const float *obj_pos;
    int n;
};

struct LbvhOutput {
    float4 *nodes;   // 2 * (2n-1)
    float4 *tri;     // 3n
    float4 *trin;    // 3n
    float2 *triuv;   // 3n or NULL
};

// scratch bytes needed for n triangles
size_t lbvh_scratch_bytes(int n);
// build into `out` using `scratch` (lbvh_scratch_bytes(n) bytes, 256-byte aligned)
cudaError_t lbvh_build(const LbvhInput &in, const LbvhOutput &out, void *scratch, cudaStream_t s);
// Morton codes of the triangle centroids over the scene box, then a stable radix sort;
// codes_out / perm_out receive the sorted codes and triangle indices (device pointers)
cudaError_t lbvh_morton_sort(const LbvhInput &in, uint32_t *codes_out, uint32_t *perm_out, void *scratch,
                             cudaStream_t s);

// per-triangle object index (and, when `ids` is not NULL, the index inside its model) from a
// table of (first, count, object) triples, one per shown model
void launch_tri_objects(const int *ranges, int n_ranges, int n, int *obj, int *ids, cudaStream_t s);

} // namespace rtg
