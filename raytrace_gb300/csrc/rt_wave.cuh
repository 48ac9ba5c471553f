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

// Warp time stamps of a profiled render (wf.stamps), taken by each warp's first lane when its
// block starts and when the warp runs out of work; (~start, end) so both combine by max
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned long long *warp_stamp(unsigned long long *stamps, int wslot)
{
    const unsigned w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (!stamps || (threadIdx.x & 31) != 0 || w >= (unsigned)kMaxStampWarps) return nullptr;
    return stamps + 2 * ((size_t)wslot * kMaxStampWarps + w);
}
__device__ __forceinline__ void stamp_start(unsigned long long *stamps, int wslot)
{
    if (unsigned long long *p = warp_stamp(stamps, wslot)) atomicMax(p, ~global_ns());
}
__device__ __forceinline__ void stamp_end(unsigned long long *stamps, int wslot)
{
    if (unsigned long long *p = warp_stamp(stamps, wslot)) atomicMax(p + 1, global_ns());
}

// Warp-uniform loops over the rays [0, n). MODE picks how warps share them:
//
//   kWorkStatic  each warp first takes its own 32 rays (no atomics: a launch with at most
//                32 x warps rays touches no counter), then the rest by grid stride;
//   kWorkDynamic the same first 32 rays, then `tile`-ray tiles pulled from one counter —
//                fine-grained, for traversal, whose cost per ray varies by orders of magnitude;
//   kWorkShares  three quarters of the rays are cut into one contiguous share per SM (SM id
//                from %smid), which that SM's warps drain in tiles from the share's counter, so
//                the rays an SM holds at once are neighbours in the queue (neighbouring pixels,
//                hit points, shadow rays toward one light) and share node lines in its L1; then
//                tiles of the last quarter from one counter; then, 32 shares checked per step,
//                tiles of any share another SM has not finished (an SM that ran no block of the
//                launch, or a slow one). Every ray is traced once whatever the block placement.
constexpr int kWorkStatic = 0, kWorkDynamic = 1, kWorkShares = 2;

template <int MODE, class F>
__device__ __forceinline__ void for_each_ray(int n, int *work, int *shares, int tile, F &&body)
{
    const int lane = threadIdx.x & 31;
    auto run_tile = [&](int start, int end) {
        for (int base = start; base < end; base += 32) body(base + lane, base + lane < end);
    };
    if constexpr (MODE == kWorkShares) {
        unsigned smid, nsmid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
        const unsigned P = min(max(nsmid, 1u), (unsigned)kMaxShares);
        // rays in the shares (a multiple of 32, as every share's start); [m, n) is the common pool
        const long long m = ((long long)n * 3 / 4) & ~31ll;
        auto lo = [&](unsigned p) { return (int)((m * (long long)p / (long long)P) & ~31ll); };
        // 1. this SM's share
        {
            const unsigned me = smid % P;
            const int a = lo(me), b = lo(me + 1);
            while (true) {
                int s = 0;
                if (lane == 0) s = atomicAdd(&shares[me], tile);
                s = a + __shfl_sync(kFull, s, 0);
                if (s >= b) break;
                run_tile(s, min(s + tile, b));
            }
        }
        // 2. the common pool
        while (true) {
            int s = 0;
            if (lane == 0) s = atomicAdd(work, tile);
            s = (int)m + __shfl_sync(kFull, s, 0);
            if (s >= n) break;
            run_tile(s, min(s + tile, n));
        }
        // 3. what is left of other shares. Each round either traces a tile or moves a share's
        // counter past its end, so the loop ends; the bound is a guard only.
        for (unsigned base = 0; base < P; base += 32) {
            for (int guard = 0; guard < (1 << 26); ++guard) {
                const unsigned p = base + (unsigned)lane;
                // the counters are read at L2, where the atomics are made
                const bool left = p < P && __ldcg(&shares[p]) < lo(p + 1) - lo(p);
                const unsigned ball = __ballot_sync(kFull, left);
                if (!ball) break;
                const unsigned q = base + (unsigned)(__ffs(ball) - 1);
                int s = 0;
                if (lane == 0) s = atomicAdd(&shares[q], tile);
                s = lo(q) + __shfl_sync(kFull, s, 0);
                const int b = lo(q + 1);
                if (s < b) run_tile(s, min(s + tile, b));
            }
        }
        return;
    }
    const int nw = gridDim.x * (blockDim.x >> 5);
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int first = min(n, nw * 32);   // the static prefix
    if (w * 32 < first) body(w * 32 + lane, w * 32 + lane < first);
    if (first >= n) return;
    if constexpr (MODE == kWorkStatic) {
        for (long long base = (long long)first + (long long)w * 32; base < n; base += (long long)nw * 32)
            body((int)(base + lane), base + lane < n);
    } else {
        while (true) {
            int start = 0;
            if (lane == 0) start = atomicAdd(work, tile);
            start = first + __shfl_sync(kFull, start, 0);
            if (start >= n) break;
            run_tile(start, min(start + tile, n));
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
