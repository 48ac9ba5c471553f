// rt_shadow.cu — the shadow kernel of the wavefront: per hit and light, the shadow ray (any hit
// over the scene) and, when the light is visible, the diffuse and Blinn terms of that light
// (RayTracer.cpp:474-545).
#include "rt_wave.cuh"

namespace rtg {

// ---- shadow: per-light any-hit + direct light ---------------------------------------------------
// Work item w is one (hit, light) pair, light-major within chunks of `chunk` hits (0 = all hits
// in one chunk): neighbouring threads aim at the same light from neighbouring hit points, so
// their traversals stay coherent, and a chunk's lights are traced close together in time, so the
// nodes its rays share stay in L2 between the lights.
template <int SS, int MODE, bool COUNT, int MINB>
__global__ void __launch_bounds__(MINB ? 128 : 256, MINB ? MINB : 1) k_shadow(Wavefront wf, int wslot, int tile, int chunk)
{
    if (cancelled(wf.cancel)) return;
    stamp_start(wf.stamps, wslot);
    Counters *C = wf.C;
    const ShadowQueue sq = wf.sq;
    // slot i holds the shadow record of hit i of this bounce, or is empty (job -1)
    const int n = min(C->h_count[wslot / 3], sq.capacity);
    const int nl = (int)*wf.max_lights;
    WorkCount wc{0, 0, 0, 0};
    unsigned long long rays = 0;
    const int cs = chunk > 0 && chunk < n ? chunk : n;   // hits per chunk
    for_each_ray<MODE>(n * nl, &C->work[wslot], wf.shares + wslot * kMaxShares, tile, [&](int w, bool active) {
        if (!active) return;
        // chunk q holds hits [q*cs, q*cs + m), m = cs except for a shorter last chunk, as m*nl
        // items: light l of hit q*cs + r is item q*cs*nl + l*m + r
        const int q = w / (cs * nl), base = q * cs, m = min(cs, n - base), r = w - base * nl;
        const int l = r / m, i = base + (r - l * m);
        const int job = __float_as_int(sq.wc[i].w);
        if (job < 0) return;
        const DevScene &S = wf.scenes[wf.jobs[job].scene];
        if (l >= S.n_lights) return;
        const DevLight &L = S.lights[l];
        if (!L.on) return;
        ++rays;
        const V3 P = mk(sq.p[i]);
        const LightTerm lt = light_term(L, P);
        if (any_hit<SS, COUNT>(S, P, lt.p2l, lt.dis, __float_as_int(sq.v[i].w), wc)) return;
        // the light is visible: the rest of the hit record comes back from L1/L2 here rather
        // than sitting in registers across the traversal
        const DevJob &J = wf.jobs[job];
        const float4 p4 = sq.p[i], v4 = sq.v[i], n4 = sq.n[i], wc4 = sq.wc[i], ws4 = sq.ws[i];
        const V3 D = mk(v4);
        const DevMaterial &M = S.mtl[__float_as_int(n4.w)];
        const V3 N = mk(n4), Wc = mk(wc4), Ws = mk(ws4);
        V3 ld = mk(L.dif[0], L.dif[1], L.dif[2]), ls = mk(L.spec[0], L.spec[1], L.spec[2]);
        if (lt.point) ld = vscale(ld, lt.lum), ls = vscale(ls, lt.lum);
        V3 sum = mk(0.0f, 0.0f, 0.0f);
        float nn = dot3(N, lt.p2l);
        if (nn > 0) sum = vmul(Wc, vscale(vmul(mk(M.kd[0], M.kd[1], M.kd[2]), ld), nn));
        const V3 h = normalise(vsub(lt.p2l, D));
        nn = dot3(N, h);
        if (nn > 0) sum = vadd(sum, vmul(Ws, vscale(vmul(mk(M.ks[0], M.ks[1], M.ks[2]), ls), powf(nn, M.shininess))));
        acc_add(J.acc, __float_as_int(p4.w), sum);
    });
    stamp_end(wf.stamps, wslot);
    if (wc.err) atomicOr(&C->error, wc.err);
    for (int off = 16; off > 0; off >>= 1) rays += __shfl_down_sync(kFull, rays, off);
    if ((threadIdx.x & 31) == 0 && rays) atomicAdd(&C->rays_shadow, rays);
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            wc.nodes += __shfl_down_sync(kFull, wc.nodes, off);
            wc.tris += __shfl_down_sync(kFull, wc.tris, off);
            wc.spheres += __shfl_down_sync(kFull, wc.spheres, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&C->s_nodes, (unsigned long long)wc.nodes);
            atomicAdd(&C->s_tris, (unsigned long long)wc.tris);
            atomicAdd(&C->s_spheres, (unsigned long long)wc.spheres);
        }
    }
}

template <int SS, int MODE, bool CNT>
static void shadow_launch(const Wavefront &wf, int wslot, const Tuning &t, cudaStream_t s)
{
    const size_t smem = stack_smem(SS, t.block);
#define RT_SHD(MB)                                                                                                \
    {                                                                                                             \
        auto k = k_shadow<SS, MODE, CNT, MB>;                                                                     \
        k<<<grid_for(t, (const void *)k, smem), t.block, smem, s>>>(wf, wslot, t.tile, t.shadow_chunk);          \
    }
    if constexpr (CNT) RT_SHD(8)
    else if (t.min_blocks == 8) RT_SHD(8) else if (t.min_blocks == 6) RT_SHD(6) else RT_SHD(0)
#undef RT_SHD
}

template <int MODE, bool CNT>
static void shadow_stack(const Wavefront &wf, int wslot, const Tuning &t, cudaStream_t s)
{
    if (!CNT && t.stack == 8) shadow_launch<8, MODE, CNT>(wf, wslot, t, s);
    else shadow_launch<0, MODE, CNT>(wf, wslot, t, s);
}

void launch_shadow(const Wavefront &wf, int level, const Tuning &t, cudaStream_t s)
{
    const int wslot = 3 * level + 2;
    if (t.count) shadow_stack<kWorkDynamic, true>(wf, wslot, count_tuning(t), s);
    else if (!t.dynamic) shadow_stack<kWorkStatic, false>(wf, wslot, t, s);
    else if (t.shares) shadow_stack<kWorkShares, false>(wf, wslot, t, s);
    else shadow_stack<kWorkDynamic, false>(wf, wslot, t, s);
}

} // namespace rtg
