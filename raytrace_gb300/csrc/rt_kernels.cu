// rt_kernels.cu — wavefront kernels of the GB300 renderer: shading, frame preparation and
// resolve, and the launch helpers (extend and shadow are in rt_extend.cu and rt_shadow.cu).
//
// One level of the reference's RTfrac recursion (RayTracer.cpp:450-596) is one pass:
//   extend  closest hit of every ray in the queue                 (:458-465)
//   shade   zNear/zFar cut, local ambient term, one shadow work item per hit, reflect and
//           refract children appended to the next queue with warp ballot/popc compaction
//                                                                 (:466-593)
//   shadow  the per-light shadow rays of each hit (any-hit), diffuse and Blinn terms of the
//           unblocked lights                                      (:474-545)
// The recursion tree is flattened into per-ray RGB weights: a child's colour enters its
// parent as r*(1-f)*C_R and f*(C_T (x) Beer), so every node adds weight (x) local colour to its
// pixel. Pixels accumulate in 64-bit fixed point (2^-32) with integer atomics, which makes
// the sum independent of the order in which rays finish: the same frame gives the same bits
// alone or batched with other frames.
#include <cstdio>
#include <cstring>

#include <map>
#include <mutex>

#include "rt_wave.cuh"

namespace rtg {

// texture colour: nearest texel, wrapped, BGR bytes (Color(Texture*,Coord2D), 3DElement.cpp:430-450)
__device__ V3 tex_color(const DevScene &S, int tex, float u, float v)
{
    const DevTexture T = S.tex[tex];
    float ip;
    float nu = modff(u, &ip), nv = modff(v, &ip);
    if (nu < 0) nu = __fadd_rn(nu, 1.0f);
    if (nv < 0) nv = __fadd_rn(nv, 1.0f);
    float fx = __fmul_rn(nu, (float)T.w), fy = __fmul_rn(nv, (float)T.h);
    int x = fx == fx ? (int)(short)(int)fx : 0, y = fy == fy ? (int)(short)(int)fy : 0;
    long long off = ((long long)y * T.w + x) * 3, last = ((long long)T.w * T.h - 1) * 3;
    off = off > last ? last : (off < 0 ? 0 : off);
    const uint8_t *t = S.texels + T.offset + off;
    return mk(__fdiv_rn((float)t[2], 255.0f), __fdiv_rn((float)t[1], 255.0f), __fdiv_rn((float)t[0], 255.0f));
}

// ---- first-hit test modes (RayTracer.cpp:81-220) -----------------------------------------
// RTdepth: Color::set(distance, zNear, zFar) (3DElement.cpp:451-462): red up to zNear, black
// from zFar, else (log zFar - log t) / log zFar
__device__ __forceinline__ V3 mode_depth(float t, float znear, float zfar)
{
    if (t <= znear) return mk(1.0f, 0.0f, 0.0f);
    if (t >= zfar) return mk(0.0f, 0.0f, 0.0f);
    const float after = logf(t), mx = logf(zfar);
    const float g = __fdiv_rn(__fsub_rn(mx, after), mx);
    return mk(g, g, g);
}

// RTmtl: the local Blinn-Phong terms of every switched-on light with no shadow test. A light
// counts as a point light when its position's w is non-zero (point and spot lights,
// 3DElement.cpp:513-525); attenuation x + y*sqrt(d2) + z*d2 in that order; the environment
// ambient comes last.
__device__ V3 mode_material(const DevScene &S, const DevMaterial &M, V3 P, V3 N, V3 D, V3 vc)
{
    const V3 ka = mk(M.ka[0], M.ka[1], M.ka[2]), kd = mk(M.kd[0], M.kd[1], M.kd[2]), ks = mk(M.ks[0], M.ks[1], M.ks[2]);
    V3 mix_vd = mk(0.0f, 0.0f, 0.0f), mix_va = mix_vd, mix_vsc = mix_vd;
    for (int l = 0; l < S.n_lights; ++l) {
        const DevLight &L = S.lights[l];
        if (!L.on) continue;
        float lum = 1.0f;
        V3 p2l;
        if (L.type != 1) {
            const V3 p2l_v = vsub(mk(L.pos[0], L.pos[1], L.pos[2]), P);
            const float d2 = dot3(p2l_v, p2l_v);
            const float step = __fadd_rn(__fadd_rn(L.att[0], __fmul_rn(L.att[1], __fsqrt_rn(d2))), __fmul_rn(L.att[2], d2));
            lum = __fdiv_rn(1.0f, step);
            p2l = normalise(p2l_v);
        } else
            p2l = normalise(mk(L.pos[0], L.pos[1], L.pos[2]));
        const V3 la = vscale(mk(L.amb[0], L.amb[1], L.amb[2]), lum), ld = vscale(mk(L.dif[0], L.dif[1], L.dif[2]), lum),
                 ls = vscale(mk(L.spec[0], L.spec[1], L.spec[2]), lum);
        mix_va = vadd(mix_va, vmul(ka, la));
        float nn = dot3(N, p2l);
        if (nn > 0) mix_vd = vadd(mix_vd, vscale(vmul(kd, ld), nn));
        const V3 h = normalise(vsub(p2l, D));
        nn = dot3(N, h);
        if (nn > 0) mix_vsc = vadd(mix_vsc, vscale(vmul(ks, ls), powf(nn, M.shininess)));
    }
    mix_va = vadd(mix_va, vmul(ka, mk(S.env[0], S.env[1], S.env[2])));
    return vadd(vmul(vc, vadd(mix_vd, mix_va)), mix_vsc);
}

// ---- shade ------------------------------------------------------------------------------------
// 640 resident threads per SM (up to 96 registers, no spills): shading is latency-bound on its
// dependent loads, and 64-register builds spilled the records it writes
template <bool DYN>
__global__ void __launch_bounds__(128, 5) k_shade(Wavefront wf, int sel, int wslot)
{
    if (cancelled(wf.cancel)) return;
    stamp_start(wf.stamps, wslot);
    Counters *C = wf.C;
    const RayQueue q = wf.q[sel], qo = wf.q[sel ^ 1];
    const HitQueue hq = wf.hq;
    const ShadowQueue sq = wf.sq;
    // the hits of this bounce (a miss needs no shading: the hit planes start as misses)
    const int n = min(C->h_count[wslot / 3], q.capacity);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    // children of a block step: per-warp counts (reflected, refracted) and the block's base,
    // double-buffered by step parity
    __shared__ int s_cnt[2][8][2];
    __shared__ int s_base[2];
    int step = 0;
    for_each_block_step<DYN>(n, &C->work[wslot], [&](int j, bool active) {
        // what the hit emits is decided first and written after the block has reserved queue
        // slots, so only the inputs of the records stay live across the reservation
        bool emit = false, c_refl = false, c_refr = false;
        V3 P, N, D, W, Wc;
        float wl = 1.0f;   // the local terms' share of W (Wl = W x wl)
        int pix = 0, mtl_id = 0, nob = 0, job = 0, level = 0, hit_inside = 0;
        float r_bc = 0.0f, r_w = 0.0f, t_bc = 0.0f, t_f = 0.0f, eta = 0.0f, cosIn = 0.0f, cosOut2 = 0.0f, hit_rfr = 1.0f;
        if (active) {
            const float4 h4 = hq.h[j], o4 = hq.o[j], d4 = hq.d[j], w4 = hq.w[j];
            const int4 m4 = hq.m[j];
            nob = hq.nob[j];
            job = m4.w;
            const DevJob &J = wf.jobs[m4.w];
            const DevScene &S = wf.scenes[J.scene];
            const int flags = m4.y, type = ray_type(flags), inside = ray_inside(flags);
            level = ray_level(flags);
            const float t = h4.x;
            const int key = __float_as_int(h4.w);
            pix = __float_as_int(w4.w);
            const bool is_tri = key >= 0 && (key & kTriFlag);
            const DevPrim *pr = (key >= 0 && !is_tri) ? &S.prims[key] : nullptr;
            const int tk = key & ~kTriFlag;
            if (ray_plane(flags)) {
                int obj = -1, prim = 0;
                if (is_tri) {
                    obj = __float_as_int(S.tri[3 * tk + 1].w);
                    prim = __float_as_int(S.tri[3 * tk].w);
                } else if (pr)
                    obj = pr->obj, prim = pr->sub;
                J.plane_obj[pix] = obj;
                J.plane_prim[pix] = prim;
                J.plane_t[pix] = key >= 0 ? t : kMiss;
            }
            const float znear = level == 0 ? J.znear : 0.0f;
            const int mode = J.mode;
            const bool far = t > J.zfar, near = t < znear;
            // the trace modes cut both ends to black; the first-hit test modes (normal, texture,
            // material, shadow) give white before zNear; depth maps the distance itself
            const bool traced = mode == kModeRaytrace || mode == kModeRefract || mode == kModeReflect;
            if (key >= 0 && mode == kModeDepth) {
                acc_add(J.acc, pix, vmul(mk(w4), mode_depth(t, J.znear, J.zfar)));
            } else if (key >= 0 && mode != kModeCheck && !far && near && !traced) {
                acc_add(J.acc, pix, mk(w4));   // Color(true)
            } else if (key >= 0 && mode != kModeCheck && !far && !near) {
                const V3 O = mk(o4);
                D = mk(d4);
                P = vadd(O, vscale(D, t));
                int tex = -1;
                float tu = 0.0f, tv = 0.0f;
                if (is_tri) {
                    const float4 e2 = S.tri[3 * tk + 2];
                    mtl_id = __float_as_int(e2.w);
                    const float u = h4.y, v = h4.z, w = __fsub_rn(__fsub_rn(1.0f, u), v);
                    V3 n0 = mk(S.trin[3 * tk]), n1 = mk(S.trin[3 * tk + 1]), n2 = mk(S.trin[3 * tk + 2]);
                    N = normalise(vadd(vadd(vscale(n0, w), vscale(n1, u)), vscale(n2, v)));
                    const DevMaterial &M = S.mtl[mtl_id];
                    hit_rfr = M.rfr;
                    tex = M.tex;
                    if (tex >= 0 && S.triuv) {
                        float2 a = S.triuv[3 * tk], b = S.triuv[3 * tk + 1], c = S.triuv[3 * tk + 2];
                        tu = __fadd_rn(__fadd_rn(__fmul_rn(a.x, w), __fmul_rn(b.x, u)), __fmul_rn(c.x, v));
                        tv = __fadd_rn(__fadd_rn(__fmul_rn(a.y, w), __fmul_rn(b.y, u)), __fmul_rn(c.y, v));
                    }
                } else {
                    mtl_id = pr->mtl;
                    const DevMaterial &M = S.mtl[mtl_id];
                    if (pr->type == kPrimSphere) {
                        const V3 Cc = mk(pr->a);
                        if (key == m4.x) {   // own sphere from inside (the only way key == excl)
                            N = normalise(vsub(Cc, P));
                            hit_rfr = type == kRayRefract ? 1.0f : M.rfr;
                        } else {
                            N = normalise(vsub(P, Cc));
                            hit_rfr = M.rfr;
                        }
                        hit_inside = inside ? 0 : 0xff;
                    } else if (pr->type == kPrimPlane) {
                        N = mk(pr->b);
                        tex = pr->tex;
                        if (tex >= 0) {
                            const V3 ax = mk(pr->c), ay = mk(pr->d);
                            const V3 p2r = vsub(O, mk(pr->a));
                            const V3 tmp1 = cross3(D, ay);
                            const float f = __fdiv_rn(__fdiv_rn(1.0f, dot3(ax, tmp1)), 5.0f);
                            tu = __fmul_rn(dot3(p2r, tmp1), f);
                            tv = __fmul_rn(dot3(D, cross3(p2r, ax)), f);
                        }
                    } else {   // box face normal (Basic3DObject.cpp:285-293)
                        const V3 b2p = vsub(P, mk(pr->c)), mx = mk(pr->d);
                        V3 pt = mk(0.0f, 0.0f, 0.0f);
                        if (fabsf(__fsub_rn(fabsf(b2p.z), mx.z)) <= kEps6) pt.z = b2p.z > 0 ? 1.0f : -1.0f;
                        if (fabsf(__fsub_rn(fabsf(b2p.y), mx.y)) <= kEps6) pt.y = b2p.y > 0 ? 1.0f : -1.0f;
                        if (fabsf(__fsub_rn(fabsf(b2p.x), mx.x)) <= kEps6) pt.x = b2p.x > 0 ? 1.0f : -1.0f;
                        N = normalise(pt);
                    }
                }
                const DevMaterial &M = S.mtl[mtl_id];
                const V3 vc = tex >= 0 ? tex_color(S, tex, tu, tv) : mk(1.0f, 1.0f, 1.0f);
                W = mk(w4);
                if (mode == kModeNormal || mode == kModeTexture || mode == kModeMaterial) {
                    V3 c;
                    if (mode == kModeNormal)   // Color(Normal): 0.5 * (n + 1), exact in one rounding
                        c = mk(__fadd_rn(__fmul_rn(0.5f, N.x), 0.5f), __fadd_rn(__fmul_rn(0.5f, N.y), 0.5f),
                               __fadd_rn(__fmul_rn(0.5f, N.z), 0.5f));
                    else if (mode == kModeTexture)
                        c = tex >= 0 ? vc : mk(0.588f, 0.588f, 0.588f);
                    else
                        c = mode_material(S, M, P, N, D, vc);
                    acc_add(J.acc, pix, vmul(W, c));
                } else {
                if (m4.z >= 0) {   // Beer factor of a refracted parent that entered a sphere
                    const DevMaterial &B = S.mtl[m4.z];
                    W.x = __fmul_rn(W.x, expf(__fmul_rn(__fmul_rn(B.kd[0], 0.15f), -t)));
                    W.y = __fmul_rn(W.y, expf(__fmul_rn(__fmul_rn(B.kd[1], 0.15f), -t)));
                    W.z = __fmul_rn(W.z, expf(__fmul_rn(__fmul_rn(B.kd[2], 0.15f), -t)));
                }
                // shadow mode (RTshd) is one bounce with unit weights; reflect mode (RTflec) has no
                // refraction
                const bool refl = M.reflect > 0.01f && mode != kModeShadow;
                const bool refr = M.refract > 0.01f && (mode == kModeRaytrace || mode == kModeRefract);
                const float a1 = refl ? __fsub_rn(1.0f, M.reflect) : 1.0f;
                const float a2 = refr ? __fsub_rn(1.0f, M.refract) : 1.0f;
                wl = __fmul_rn(a1, a2);
                const V3 Wl = vscale(W, wl);
                // ambient: environment plus every switched-on light, shadowed or not (RTshd adds
                // the environment last, RTfrac and RTflec first)
                const V3 ka = mk(M.ka[0], M.ka[1], M.ka[2]);
                const V3 env = vmul(ka, mk(S.env[0], S.env[1], S.env[2]));
                V3 mix_va = mode == kModeShadow ? mk(0.0f, 0.0f, 0.0f) : env;
                int lights_on = 0;
                for (int l = 0; l < S.n_lights; ++l) {
                    const DevLight &L = S.lights[l];
                    if (!L.on) continue;
                    ++lights_on;
                    float lum = 1.0f;
                    if (L.type == 2) lum = light_term(L, P).lum;
                    const V3 la = L.type == 2 ? vscale(mk(L.amb[0], L.amb[1], L.amb[2]), lum) : mk(L.amb[0], L.amb[1], L.amb[2]);
                    mix_va = vadd(mix_va, vmul(ka, la));
                }
                if (mode == kModeShadow) mix_va = vadd(mix_va, env);
                Wc = vmul(Wl, vc);
                acc_add(J.acc, pix, vmul(Wc, mix_va));
                emit = lights_on > 0;
                const float bwc = o4.w;
                if (refl && level + 1 <= J.max_level) {
                    r_bc = __fmul_rn(bwc, M.reflect);
                    r_w = __fmul_rn(M.reflect, a2);
                    c_refl = !(r_bc < 1e-5f);
                }
                if (refr && level + 1 <= J.max_level) {
                    t_f = M.refract;
                    eta = __fdiv_rn(d4.w, hit_rfr);
                    cosIn = -dot3(D, N);
                    cosOut2 = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(eta, eta), __fsub_rn(1.0f, __fmul_rn(cosIn, cosIn))));
                    t_bc = __fmul_rn(bwc, t_f);
                    c_refr = !(cosOut2 < 0.0f) && !(t_bc < 1e-5f);
                }
                }
            }
        }
        // the shadow record of hit j goes to slot j, with no atomic: a single counter that every
        // warp reserves from serialises at one L2 slice. A hit without a record marks its slot
        // empty (job -1) and the shadow kernel skips it.
        if (active) {
            if (emit) {
                sq.p[j] = make_float4(P.x, P.y, P.z, __int_as_float(pix));
                sq.n[j] = make_float4(N.x, N.y, N.z, __int_as_float(mtl_id));
                sq.v[j] = make_float4(D.x, D.y, D.z, __int_as_float(nob));
                sq.wc[j] = make_float4(Wc.x, Wc.y, Wc.z, __int_as_float(job));
                const V3 Wl = vscale(W, wl);
                sq.ws[j] = make_float4(Wl.x, Wl.y, Wl.z, 0.0f);
            } else
                sq.wc[j] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        }
        // children: one reservation per block step (an atomic per warp on the one queue counter
        // serialised at its L2 slice): the block's reflected rays in warp order, then its
        // refracted rays
        const unsigned b1 = __ballot_sync(kFull, c_refl), b2 = __ballot_sync(kFull, c_refr);
        const int par = step & 1;
        ++step;
        if (lane == 0) s_cnt[par][warp][0] = __popc(b1), s_cnt[par][warp][1] = __popc(b2);
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int k = 0; k < warps; ++k) tot += s_cnt[par][k][0] + s_cnt[par][k][1];
            s_base[par] = tot ? atomicAdd(&C->q_count[sel ^ 1], tot) : 0;
        }
        __syncthreads();
        int off_r = s_base[par], off_t = s_base[par];
        for (int k = 0; k < warps; ++k) off_t += s_cnt[par][k][0];
        for (int k = 0; k < warp; ++k) off_r += s_cnt[par][k][0], off_t += s_cnt[par][k][1];
        {
            if (c_refl) {
                const int slot = off_r + __popc(b1 & lt);
                if (slot < qo.capacity) {
                    const float nn = __fmul_rn(2.0f, dot3(D, N));
                    const V3 R = normalise(vsub(D, vscale(N, nn)));
                    const V3 Wr = vscale(W, r_w);
                    qo.o[slot] = make_float4(P.x, P.y, P.z, r_bc);
                    qo.d[slot] = make_float4(R.x, R.y, R.z, 1.0f);
                    qo.w[slot] = make_float4(Wr.x, Wr.y, Wr.z, __int_as_float(pix));
                    qo.m[slot] = make_int4(nob, ray_flags(level + 1, kRayReflect, 0, 0), -1, job);
                } else
                    atomicExch(&C->overflow, 1);
            }
            if (c_refr) {
                const int slot = off_t + __popc(b2 & lt);
                if (slot < qo.capacity) {
                    const V3 l2 = vscale(D, eta);
                    const V3 l1 = vscale(N, __fsub_rn(__fmul_rn(eta, cosIn), __fsqrt_rn(cosOut2)));
                    const V3 T = normalise(vadd(l1, l2));
                    const V3 Wt = vscale(W, t_f);
                    qo.o[slot] = make_float4(P.x, P.y, P.z, t_bc);
                    qo.d[slot] = make_float4(T.x, T.y, T.z, hit_rfr);
                    qo.w[slot] = make_float4(Wt.x, Wt.y, Wt.z, __int_as_float(pix));
                    qo.m[slot] = make_int4(nob, ray_flags(level + 1, kRayRefract, hit_inside, 0), hit_inside ? mtl_id : -1,
                                           job);
                } else
                    atomicExch(&C->overflow, 1);
            }
        }
    });
    stamp_end(wf.stamps, wslot);
}

// ---- resolve: fixed point -> float rgb and Color::put bytes ---------------------------------------
__device__ __forceinline__ uint8_t put_channel(float c)
{
    if (c > 1.0f) return 255;
    if (c < 0.0f || c != c) return 0;
    return (uint8_t)(int)(c * 255);
}
// colour = (float)((double)acc * scale), scale = 2^-32 / spp in double (split on the host)
__device__ __forceinline__ float resolve_channel(long long a, DSplit scale) { return a ? dmul_to_float(a, scale) : 0.0f; }

// pixels 4q .. 4q+3 of a frame: 96 B of accumulator in six 16-B loads, 48 B of colour in three
// 16-B stores, 12 B of bytes in three 4-B stores (frame buffers are 256-B aligned); a partial
// last quad goes pixel by pixel
__device__ __forceinline__ void resolve_quad(const FrameBufs &fb, long long q, long long npix, DSplit scale)
{
    if (4 * q + 4 > npix) {
        for (long long p = 4 * q; p < npix; ++p)
            for (int k = 0; k < 3; ++k) {
                const float c = resolve_channel(fb.acc[3 * p + k], scale);
                if (fb.rgb) fb.rgb[3 * p + k] = c;
                if (fb.rgb8) fb.rgb8[3 * p + k] = put_channel(c);
            }
        return;
    }
    const longlong2 *a2 = reinterpret_cast<const longlong2 *>(fb.acc + 12 * q);
    float c[12];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const longlong2 v = a2[k];
        c[2 * k] = resolve_channel(v.x, scale);
        c[2 * k + 1] = resolve_channel(v.y, scale);
    }
    if (fb.rgb) {
        float4 *o = reinterpret_cast<float4 *>(fb.rgb + 12 * q);
        o[0] = make_float4(c[0], c[1], c[2], c[3]);
        o[1] = make_float4(c[4], c[5], c[6], c[7]);
        o[2] = make_float4(c[8], c[9], c[10], c[11]);
    }
    if (fb.rgb8) {
        unsigned *o = reinterpret_cast<unsigned *>(fb.rgb8 + 12 * q);
#pragma unroll
        for (int k = 0; k < 3; ++k)
            o[k] = (unsigned)put_channel(c[4 * k]) | (unsigned)put_channel(c[4 * k + 1]) << 8 |
                   (unsigned)put_channel(c[4 * k + 2]) << 16 | (unsigned)put_channel(c[4 * k + 3]) << 24;
    }
}

__global__ void k_resolve(FrameBufs fb, long long npix, DSplit scale)
{
    const long long nq = (npix + 3) >> 2;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x)
        resolve_quad(fb, q, npix, scale);
}

// A thread's indices in a batch-wide frame launch only grow, so the frame of each is found by
// scanning forward from the frame of the last: at most n steps over the whole loop. The resolve
// goes by quads (six 16-B loads in flight per thread keep enough bytes moving to fill HBM); the
// preparation, which only stores, by 16-B chunks, six per quad (quad_end * 6 is a frame's chunk
// range in the batch), so that consecutive threads write consecutive bytes.
__device__ __forceinline__ int frame_of(const FrameJob *fj, int n, int f, long long g, int per_quad)
{
    while (f < n - 1 && per_quad * fj[f].quad_end <= g) ++f;
    return f;
}

__global__ void k_frames_resolve(const FrameJob *fj, int n, long long quads)
{
    // the current frame's buffers, pixel count, scale and quad range, reloaded only when the
    // thread's quads move on to another frame
    int f = -1;
    FrameBufs fb{};
    long long npix = 0, q0 = 0, q1 = 0;
    DSplit scale{};
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < quads; g += (long long)gridDim.x * blockDim.x) {
        if (g >= q1) {
            f = frame_of(fj, n, f < 0 ? 0 : f, g, 1);
            const FrameJob &F = fj[f];
            fb = F.fb;
            npix = F.npix;
            scale = split_double_bits(F.scale_bits);
            q0 = f ? fj[f - 1].quad_end : 0;
            q1 = F.quad_end;
        }
        resolve_quad(fb, g - q0, npix, scale);
    }
}

// 16-B chunk k of a frame's accumulators (24 B per pixel; 6 chunks per 4-pixel quad, the last
// one 8 B for an odd pixel count) zeroed; the same index k also covers pixel k's hit planes and
// camera axis entry k (a frame has 6 * ceil(npix / 4) >= npix chunks, and >= w + h): consecutive
// threads write consecutive bytes
__device__ __forceinline__ void prepare_chunk(const FrameJob &F, long long k, long long nchunks)
{
    const long long bytes = 24 * F.npix;
    char *a = reinterpret_cast<char *>(F.fb.acc);
    if (16 * k + 16 <= bytes) *reinterpret_cast<longlong2 *>(a + 16 * k) = make_longlong2(0, 0);
    else if (16 * k + 8 <= bytes) *reinterpret_cast<long long *>(a + 16 * k) = 0;
    if (F.planes && k < F.npix) {
        F.fb.plane_obj[k] = -1;
        F.fb.plane_prim[k] = 0;
        F.fb.plane_t[k] = kMiss;
    }
    if (F.dp_bits) {   // (float)((double)xcur * dp), xcur = col - W/2, then the rows (RayTracer.cpp:14-18)
        const DSplit d = split_double_bits(F.dp_bits);
        for (long long j = k; j < F.w + F.h; j += nchunks)
            F.fb.axis[j] = dmul_to_float(j < F.w ? j - F.w / 2 : j - F.w - F.h / 2, d);
    }
}

__global__ void k_frames_prepare(const FrameJob *fj, int n, long long quads)
{
    int f = -1;
    FrameJob F{};
    long long c0 = 0, c1 = 0;   // the current frame's chunk range, reloaded when the chunks leave it
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < 6 * quads;
         c += (long long)gridDim.x * blockDim.x) {
        if (c >= c1) {
            f = frame_of(fj, n, f < 0 ? 0 : f, c, 6);
            F = fj[f];
            c0 = f ? 6 * fj[f - 1].quad_end : 0;
            c1 = 6 * F.quad_end;
        }
        prepare_chunk(F, c - c0, c1 - c0);
    }
}

__global__ void k_frame_prepare(FrameJob F)
{
    const long long nc = 6 * ((F.npix + 3) >> 2);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += (long long)gridDim.x * blockDim.x)
        prepare_chunk(F, k, nc);
}

__global__ void k_selftest_conversions(const long long *x, int n, DSplit d, const float *v, float *out_mul,
                                       long long *out_fix)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out_mul[i] = dmul_to_float(x[i], d);
        out_fix[i] = float_to_fix32(v[i]);
    }
}

void launch_selftest_conversions(const long long *x, int n, unsigned long long d_bits, const float *v, float *out_mul,
                                 long long *out_fix, cudaStream_t s)
{
    k_selftest_conversions<<<std::max(1, std::min((n + 255) / 256, sm_count() * 4)), 256, 0, s>>>(
        x, n, split_double_bits(d_bits), v, out_mul, out_fix);
}

// ---- launchers ------------------------------------------------------------------------------------
int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// resident blocks per SM of a kernel at a block size and dynamic shared memory, queried once (the
// query costs host time on every launch otherwise, which small renders feel as idle gaps between
// kernels)
int grid_for(const Tuning &t, const void *kernel, size_t smem)
{
    if (t.grid > 0) return t.grid;
    static std::mutex mu;
    static std::map<std::pair<const void *, long long>, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(kernel, (long long)t.block << 32 | (long long)smem);
    auto it = cache.find(key);
    if (it == cache.end()) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, t.block, smem);
        it = cache.emplace(key, per_sm > 0 ? per_sm : 1).first;
    }
    return sm_count() * it->second;
}


// The counting pass (an untimed statistics pass) runs in one configuration: what it counts
// does not depend on the launch shape.
Tuning count_tuning(const Tuning &t)
{
    Tuning c = t;
    c.block = 128, c.dynamic = true, c.shares = false, c.min_blocks = 8, c.stack = 0;
    return c;
}

void launch_shade(const Wavefront &wf, int sel, int level, const Tuning &t, cudaStream_t s)
{
    const int wslot = 3 * level + 1;
    Tuning ts = t;   // shading runs in 128-thread blocks whatever the traversal kernels use
    ts.block = 128;
    if (t.dynamic) {
        auto k = k_shade<true>;
        k<<<grid_for(ts, (const void *)k), 128, 0, s>>>(wf, sel, wslot);
    } else {
        auto k = k_shade<false>;
        k<<<grid_for(ts, (const void *)k), 128, 0, s>>>(wf, sel, wslot);
    }
}

// grid of a frame launch over n items: 256 threads a block, at most 8 blocks per SM (grid stride)
static int item_grid(long long n)
{
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)sm_count() * 8));
}

void launch_resolve(const FrameBufs &fb, int width, int height, int spp, cudaStream_t s)
{
    const long long npix = (long long)width * height;
    k_resolve<<<item_grid((npix + 3) / 4), 256, 0, s>>>(fb, npix, split_double_bits(resolve_scale_bits(spp)));
}

unsigned long long resolve_scale_bits(int spp)
{
    const double scale = 1.0 / 4294967296.0 / (double)spp;
    unsigned long long bits;
    std::memcpy(&bits, &scale, sizeof bits);
    return bits;
}

void launch_frames_prepare(const FrameJob *jobs, int n, long long quads, cudaStream_t s)
{
    if (n > 0 && quads > 0) k_frames_prepare<<<item_grid(6 * quads), 256, 0, s>>>(jobs, n, quads);
}

void launch_frame_prepare(const FrameJob &job, cudaStream_t s)
{
    k_frame_prepare<<<item_grid(6 * ((job.npix + 3) / 4)), 256, 0, s>>>(job);
}

void launch_frames_resolve(const FrameJob *jobs, int n, long long quads, cudaStream_t s)
{
    if (n > 0 && quads > 0) k_frames_resolve<<<item_grid(quads), 256, 0, s>>>(jobs, n, quads);
}


} // namespace rtg
