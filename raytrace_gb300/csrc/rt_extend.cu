// rt_extend.cu — the extend kernel of the wavefront: closest hit of every queued ray, one level of
// the reference's RTfrac recursion (RayTracer.cpp:458-465). The first extend of a wave makes its
// primary rays in registers (parallelRT's pinhole rays, RayTracer.cpp:13-27) and appends the rays
// that hit something to the hit queue that shading reads.
#include "rt_wave.cuh"

namespace rtg {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
    const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        unsigned hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        unsigned hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

// ---- ray generation (parallelRT, RayTracer.cpp:13-27) -------------------------------------
// Primary rays are made inside the first extend pass, in registers: a ray queue entry is
// written only for a ray that hits something, which is what shading reads.

// the job that holds global sample gs. Lane 0 searches for the first sample of the warp's 32
// (base), the lanes walk on from there: 32 consecutive samples span few jobs. All lanes call.
__device__ __forceinline__ int job_of(const Wavefront &wf, long long gs, long long base, bool active)
{
    int j = 0;
    if ((threadIdx.x & 31) == 0) {
        int lo = 0, hi = (int)*wf.n_jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (wf.job_sample_end[mid] > base) hi = mid;
            else lo = mid + 1;
        }
        j = lo;
    }
    j = __shfl_sync(kFull, j, 0);
    // ends: the last job's end is the number of samples of all jobs, above any active gs
    if (active)
        while (wf.job_sample_end[j] <= gs) ++j;
    return j;
}

struct PrimaryRay {
    V3 o, d;
    int pixel, row, col;
    int sample;   // sample index within the pixel
};

// The pixel of sequence number p over the xlim x ylim region: row by row (tile 0), or in tiles
// of T x T pixels taken row by row, the pixels of a tile row by row; the last band of rows and
// the last tile of each band may be narrower. A bijection either way: it only sets which rays a
// warp and its neighbours trace together (hit points and shadow rays follow the primary order).
__device__ __forceinline__ void pixel_of(unsigned p, unsigned xlim, unsigned ylim, unsigned T, unsigned &row,
                                         unsigned &col)
{
    if (T == 0) {
        row = p / xlim;
        col = p - row * xlim;
        return;
    }
    const unsigned band_px = xlim * T, band = p / band_px, r = p - band * band_px;
    const unsigned hb = min(T, ylim - band * T);       // rows in this band
    const unsigned t = r / (T * hb), q = r - t * (T * hb);
    const unsigned wt = min(T, xlim - t * T);          // columns in this tile
    const unsigned ri = q / wt;
    row = band * T + ri;
    col = t * T + (q - ri * wt);
}

// camera ray of the job's sample `local` (pixel-major: local = pixel * spp + sample)
__device__ __forceinline__ PrimaryRay primary_ray(const DevJob &J, long long local)
{
    PrimaryRay r;
    long long p;
    int s;
    if (J.spp == 1) {
        p = local;
        s = 0;
    } else if (local < (1ll << 32)) {   // 32-bit division where it suffices
        const unsigned q = (unsigned)local / (unsigned)J.spp;
        p = q;
        s = (int)((unsigned)local - q * (unsigned)J.spp);
    } else {
        p = local / J.spp;
        s = (int)(local - p * J.spp);
    }
    // p < 2^28: frames are at most 16384 x 16384
    unsigned row, col;
    pixel_of((unsigned)p, (unsigned)J.xlim, (unsigned)J.ylim, (unsigned)J.pixel_tile, row, col);
    const int xcur = (int)col - J.width / 2, ycur = (int)row - J.height / 2;
    float a, b;
    DSplit d = split_double_bits((unsigned long long)__double_as_longlong(J.dp));
    if (J.axis) {   // one sample per pixel: the offsets of the frame's table
        a = J.axis[col];
        b = J.axis[J.width + row];
    } else if (J.spp > 1) {   // sub-pixel jitter in [0,1) from a per-pixel Philox stream
        const unsigned pix = row * (unsigned)J.width + col;
        const uint4 x = philox4x32_10(make_uint4(pix, 0u, (unsigned)s, 0u),
                                      make_uint2((unsigned)J.seed, (unsigned)(J.seed >> 32)));
        // (float)(((double)xcur + (x >> 8) * 2^-24) * dp): the sum is exact in 38 bits, so it
        // is the integer xcur * 2^24 + (x >> 8) times dp * 2^-24
        d.e -= 24;
        a = dmul_to_float((long long)xcur * 16777216ll + (long long)(x.x >> 8), d);
        b = dmul_to_float((long long)ycur * 16777216ll + (long long)(x.y >> 8), d);
    } else {   // (float)((double)xcur * dp)
        a = dmul_to_float(xcur, d);
        b = dmul_to_float(ycur, d);
    }
    const V3 n = mk(J.cam_n[0], J.cam_n[1], J.cam_n[2]);
    const V3 u = mk(J.cam_u[0], J.cam_u[1], J.cam_u[2]);
    const V3 v = mk(J.cam_v[0], J.cam_v[1], J.cam_v[2]);
    r.d = normalise(vadd(vadd(n, vscale(u, a)), vscale(v, b)));
    r.o = mk(J.cam_pos[0], J.cam_pos[1], J.cam_pos[2]);
    r.pixel = (int)(row * (unsigned)J.width + col);
    r.row = (int)row, r.col = (int)col;
    r.sample = s;
    return r;
}

// ---- extend: closest hit -------------------------------------------------------------------
// MINB > 0 caps registers so MINB blocks of 128 threads fit on an SM. GEN: the first pass of a
// wave, which makes its primary rays instead of reading a queue. SS: traversal stack entries per
// thread in shared memory (SS * blockDim.x ints of dynamic shared memory). MODE: how warps share
// the rays (kWork*).
template <int SS, int MODE, bool COUNT, int MINB, bool GEN>
__global__ void __launch_bounds__(MINB ? 128 : 256, MINB ? MINB : 1) k_extend(Wavefront wf, int sel, int wslot, int tile)
{
    Counters *C = wf.C;
    const RayQueue q = wf.q[sel];
    const long long total = GEN ? *wf.total_samples : 0, first = GEN ? *wf.sample_offset : 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // the next queue fills in shade
        C->q_count[sel ^ 1] = 0;
        // the rays of this queue are the children the last shading spawned (counted once here,
        // not by an atomic per warp on one address)
        if (!GEN) C->rays_secondary += (unsigned long long)C->q_count[sel];
        if (GEN) {
            C->q_count[sel] = (int)min(total, (long long)q.capacity);
            C->rays_primary = (unsigned long long)total;
            if (total > q.capacity) atomicExch(&C->overflow, 1);
        }
    }
    if (cancelled(wf.cancel)) return;
    stamp_start(wf.stamps, wslot);
    const int n = GEN ? (int)min(total, (long long)q.capacity) : min(C->q_count[sel], q.capacity);
    WorkCount wc{0, 0, 0, 0};
    const int level = wslot / 3;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const HitQueue hq = wf.hq;
    for_each_ray<MODE>(n, &C->work[wslot], wf.shares + wslot * kMaxShares, tile, [&](int i, bool active) {
        Best best;
        best.key = -1;
        int newobj = -1, job = 0, pixel = 0, plane = 0;
        V3 o, d;
        if constexpr (GEN) {
            job = job_of(wf, first + i, first + (i - lane), active);
            if (active) {
                const DevJob &J = wf.jobs[job];
                const PrimaryRay pr = primary_ray(J, first + i - J.sample_base);
                if (J.mode == kModeCheck && ((pr.row >> 6) & 1) == ((pr.col >> 6) & 1))
                    acc_add(J.acc, pr.pixel, mk(1.0f, 1.0f, 1.0f));   // RTcheck: white 64x64 tiles
                plane = pr.sample == 0 && J.plane_obj != nullptr;
                pixel = pr.pixel;
                o = pr.o, d = pr.d;
                closest_hit<SS, COUNT>(wf.scenes[J.scene], o, d, -1, false, best, newobj, wc);
            }
        } else if (active) {
            const float4 o4 = q.o[i], d4 = q.d[i];
            const int4 m4 = q.m[i];
            closest_hit<SS, COUNT>(wf.scenes[wf.jobs[m4.w].scene], mk(o4), mk(d4), m4.x, ray_inside(m4.y) != 0, best,
                                      newobj, wc);
        }
        // the hits go to the hit queue densely (one atomic per warp): shading reads them with
        // coalesced loads, and misses cost it nothing
        const bool is_hit = best.key >= 0;
        const unsigned hb = __ballot_sync(kFull, is_hit);
        if (hb) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&C->h_count[level], __popc(hb));
            base = __shfl_sync(kFull, base, 0);
            if (is_hit) {
                const int h = base + __popc(hb & lt);   // below the queue capacity: one per ray
                hq.h[h] = make_float4(best.t, best.u, best.v, __int_as_float(best.key));
                hq.nob[h] = newobj;
                if constexpr (GEN) {
                    hq.o[h] = make_float4(o.x, o.y, o.z, 1.0f);
                    hq.d[h] = make_float4(d.x, d.y, d.z, 1.0f);
                    hq.w[h] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(pixel));
                    hq.m[h] = make_int4(-1, ray_flags(0, kRayBase, 0, plane), -1, job);
                } else {   // the ray record again (its lines were read at the start of this tile)
                    hq.o[h] = q.o[i];
                    hq.d[h] = q.d[i];
                    hq.w[h] = q.w[i];
                    hq.m[h] = q.m[i];
                }
            }
        }
    });
    stamp_end(wf.stamps, wslot);
    if (wc.err) atomicOr(&C->error, wc.err);
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            wc.nodes += __shfl_down_sync(kFull, wc.nodes, off);
            wc.tris += __shfl_down_sync(kFull, wc.tris, off);
            wc.spheres += __shfl_down_sync(kFull, wc.spheres, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&C->nodes, (unsigned long long)wc.nodes);
            atomicAdd(&C->tris, (unsigned long long)wc.tris);
            atomicAdd(&C->spheres, (unsigned long long)wc.spheres);
        }
    }
}

template <int SS, int MODE, bool CNT, bool GEN>
static void extend_launch(const Wavefront &wf, int sel, int wslot, const Tuning &t, cudaStream_t s)
{
    const size_t smem = stack_smem(SS, t.block);
#define RT_EXT(MB)                                                                                                \
    {                                                                                                             \
        auto k = k_extend<SS, MODE, CNT, MB, GEN>;                                                                \
        k<<<grid_for(t, (const void *)k, smem), t.block, smem, s>>>(wf, sel, wslot, t.tile);                     \
    }
    if constexpr (CNT) RT_EXT(8)
    else if (t.min_blocks == 8) RT_EXT(8) else if (t.min_blocks == 6) RT_EXT(6) else RT_EXT(0)
#undef RT_EXT
}

template <int MODE, bool CNT, bool GEN>
static void extend_stack(const Wavefront &wf, int sel, int wslot, const Tuning &t, cudaStream_t s)
{
    if (!CNT && t.stack == 8) extend_launch<8, MODE, CNT, GEN>(wf, sel, wslot, t, s);
    else extend_launch<0, MODE, CNT, GEN>(wf, sel, wslot, t, s);
}

template <bool GEN>
static void extend_mode(const Wavefront &wf, int sel, int wslot, const Tuning &t, cudaStream_t s)
{
    if (t.count) extend_stack<kWorkDynamic, true, GEN>(wf, sel, wslot, count_tuning(t), s);
    else if (!t.dynamic) extend_stack<kWorkStatic, false, GEN>(wf, sel, wslot, t, s);
    else if (t.shares) extend_stack<kWorkShares, false, GEN>(wf, sel, wslot, t, s);
    else extend_stack<kWorkDynamic, false, GEN>(wf, sel, wslot, t, s);
}

void launch_extend(const Wavefront &wf, int sel, int level, bool gen, const Tuning &t, cudaStream_t s)
{
    const int wslot = 3 * level;
    if (gen) extend_mode<true>(wf, sel, wslot, t, s);
    else extend_mode<false>(wf, sel, wslot, t, s);
}

} // namespace rtg
