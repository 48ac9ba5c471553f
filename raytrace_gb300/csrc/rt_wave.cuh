// rt_wave.cuh — what the wavefront kernels share (rt_extend.cu, rt_shadow.cu, rt_kernels.cu):
// pixel accumulation, the warp- and block-uniform work loops, the cancel check, the light terms
// of a hit point, and the host-side launch helpers.
#pragma once
#include "rt_fixed.cuh"
#include "rt_kernels.cuh"
#include "rt_trace.cuh"

namespace rtg {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void acc_add(long long *acc, int pix, V3 c)
{
    unsigned long long *a = reinterpret_cast<unsigned long long *>(acc + 3ll * pix);
    if (c.x != 0.0f && c.x == c.x) atomicAdd(a + 0, (unsigned long long)float_to_fix32(c.x));
    if (c.y != 0.0f && c.y == c.y) atomicAdd(a + 1, (unsigned long long)float_to_fix32(c.y));
    if (c.z != 0.0f && c.z == c.z) atomicAdd(a + 2, (unsigned long long)float_to_fix32(c.z));
}

// Warp-uniform loops over the rays [0, n).
//
// for_each_ray: each warp first takes its own 32 rays (no atomics: a launch with at most
// 32 x warps rays touches no counter), then the rest by grid stride (DYN false) or in `tile`-ray
// tiles pulled from a counter (DYN true) — fine-grained, for traversal, whose cost per ray
// varies by orders of magnitude.
template <bool DYN, class F>
__device__ __forceinline__ void for_each_ray(int n, int *work, int tile, F &&body)
{
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int first = min(n, nw * 32);   // the static prefix
    if (w * 32 < first) body(w * 32 + lane, w * 32 + lane < first);
    if (first >= n) return;
    if (!DYN) {
        for (long long base = (long long)first + (long long)w * 32; base < n; base += (long long)nw * 32)
            body((int)(base + lane), base + lane < n);
    } else {
        while (true) {
            int start = 0;
            if (lane == 0) start = atomicAdd(work, tile);
            start = first + __shfl_sync(kFull, start, 0);
            if (start >= n) break;
            const int end = min(start + tile, n);
            for (int base = start; base < end; base += 32)
                body(base + lane, base + lane < end);
        }
    }
}

// Block-uniform loop over [0, n) in steps of blockDim.x items, one per thread: every thread of a
// block runs the body the same number of times, so the body may synchronise the block. Chunks
// come from a counter, a share of what is left (DYN), or by grid stride.
template <bool DYN, class F>
__device__ __forceinline__ void for_each_block_step(int n, int *work, F &&body)
{
    __shared__ int s_start;
    const int B = blockDim.x;
    if (!DYN) {
        for (long long base = (long long)blockIdx.x * B; base < n; base += (long long)gridDim.x * B)
            body((int)base + (int)threadIdx.x, base + threadIdx.x < n);
        return;
    }
    int chunk = max(B, ((n / (2 * (int)gridDim.x)) + B - 1) / B * B);
    while (true) {
        if (threadIdx.x == 0) s_start = atomicAdd(work, chunk);
        __syncthreads();
        const int start = s_start;
        __syncthreads();   // s_start is written again by the next round
        if (start >= n) break;
        const int end = min(start + chunk, n);
        for (int base = start; base < end; base += B) body(base + (int)threadIdx.x, base + (int)threadIdx.x < end);
        chunk = max(B, (((n - end) / (2 * (int)gridDim.x)) + B - 1) / B * B);
    }
}

__device__ __forceinline__ bool cancelled(const volatile int *cancel) { return cancel && *cancel; }

// light terms of one light at P (RayTracer.cpp:482-503)
struct LightTerm {
    V3 p2l;
    float dis, lum;
    bool point;
};
__device__ __forceinline__ LightTerm light_term(const DevLight &L, V3 P)
{
    LightTerm r;
    if (L.type == 2) {   // MY_LIGHT_POINT
        V3 p2l_v = vsub(mk(L.pos[0], L.pos[1], L.pos[2]), P);
        float d2 = dot3(p2l_v, p2l_v);
        float step = __fadd_rn(L.att[0], __fmul_rn(L.att[2], d2));
        r.dis = __fsqrt_rn(d2);
        step = __fadd_rn(step, __fmul_rn(L.att[1], r.dis));
        r.lum = __fdiv_rn(1.0f, step);
        r.p2l = normalise(p2l_v);
        r.point = true;
    } else {
        r.dis = 1e10f;
        r.lum = 1.0f;
        r.p2l = normalise(mk(L.pos[0], L.pos[1], L.pos[2]));
        r.point = false;
    }
    return r;
}

// ---- launch helpers (rt_kernels.cu) --------------------------------------------------------------
// grid of a persistent launch: SM count x resident blocks per SM of `kernel` at the tuning's block
// size with `smem` bytes of dynamic shared memory (queried once per kernel and shape)
int grid_for(const Tuning &t, const void *kernel, size_t smem = 0);
// short-stack bytes of a traversal launch
inline size_t stack_smem(int ss, int block) { return (size_t)ss * (size_t)block * sizeof(int); }
// the one configuration of the untimed counting pass
Tuning count_tuning(const Tuning &t);

} // namespace rtg
