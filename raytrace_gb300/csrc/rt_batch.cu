// rt_batch.cu — batched multi-scene rendering: many (scene, frame) jobs traced as shared
// waves by persistent kernels that pull ray tiles from global work counters, with the
// per-bounce launch sequence captured once as a CUDA graph and replayed per wave; the wave
// runner (also used by the server), the plain loop of per-scene renders it is compared
// against, and the autotuner.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_capi_internal.h"

using namespace rtg;

// ---- wave runner --------------------------------------------------------------------------------------------

WaveRunner::~WaveRunner()
{
    for (WaveStage &st : stages) {
        if (st.done) {
            cudaEventSynchronize(st.done);
            cudaEventDestroy(st.done);
        }
        if (st.start) cudaEventDestroy(st.start);
        if (st.jobs) cudaFreeHost(st.jobs);
    }
    if (ftab_copied) {
        cudaEventSynchronize(ftab_copied);
        cudaEventDestroy(ftab_copied);
    }
    if (ftab_host) cudaFreeHost(ftab_host);
    for (WaveLane &L : lanes) {
        if (L.stream) {
            cudaStreamSynchronize(L.stream);
            cudaStreamDestroy(L.stream);
        }
        if (L.last) cudaEventDestroy(L.last);
    }
    if (go) cudaEventDestroy(go);
}

// A sample's rays at bounce l number at most b^l (b = children per hit, one queue holds one
// bounce), so a wave whose chunks satisfy sum(samples * b^max_level) <= capacity cannot overflow
// its ray queue or its shadow queue (at most one shadow record per hit).
long long wave_weight(int branching, int max_level)
{
    return branching >= 2 ? 1ll << max_level : 1ll;
}

size_t wave_runner_bytes(const WaveRunner &R)
{
    size_t b = R.ftab_dev.bytes;
    for (const WaveLane &L : R.lanes) b += L.ws.mem.bytes;
    return b;
}

void wave_join(WaveRunner &R, cudaStream_t s)
{
    for (WaveLane &L : R.lanes)
        if (L.stream && L.pending) {
            cudaStreamWaitEvent(s, L.last, 0);
            L.pending = false;
        }
}

void wave_join_all_but_last(WaveRunner &R, cudaStream_t s)
{
    const size_t n = R.lanes.size(), last = (R.next_lane + n - 1) % n;
    for (size_t k = 0; k < n; ++k) {
        WaveLane &L = R.lanes[k];
        if (k != last && L.stream && L.pending) {
            cudaStreamWaitEvent(s, L.last, 0);
            L.pending = false;
        }
    }
}

static int stage_harvest(rt_ctx *ctx, WaveRunner &R, WaveStage &st, bool wait)
{
    if (!st.busy) return RT_OK;
    cudaError_t e = cudaEventQuery(st.done);
    if (e == cudaErrorNotReady && wait) {
        const auto t0 = std::chrono::steady_clock::now();
        e = cudaEventSynchronize(st.done);
        R.wait_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (e == cudaErrorNotReady) return RT_OK;
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "wave: %s", cudaGetErrorString(e));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, st.start, st.done) == cudaSuccess) R.wave_ms.push_back(ms);
    const Counters &C = *st.counters;
    R.rays_primary += C.rays_primary;
    R.rays_secondary += C.rays_secondary;
    R.rays_shadow += C.rays_shadow;
    R.overflow |= C.overflow;
    R.error |= C.error;
    st.busy = false;
    return RT_OK;
}

int wave_harvest(rt_ctx *ctx, WaveRunner &R, bool wait)
{
    for (size_t k = 0; k < R.stages.size(); ++k) {   // oldest first
        WaveStage &st = R.stages[(R.next + k) % R.stages.size()];
        int rc = stage_harvest(ctx, R, st, wait);
        if (rc) return rc;
    }
    return RT_OK;
}

int wave_runner_init(rt_ctx *ctx, WaveRunner &R, long long qcap, int jobcap, int n_stages, int n_lanes)
{
    n_lanes = std::max(1, std::min(n_lanes, 2));
    const bool fits = !R.lanes.empty() && (int)R.lanes.size() == n_lanes && R.lanes[0].ws.mem.p &&
                      qcap <= R.lanes[0].ws.qcap && jobcap <= R.jobcap && (int)R.stages.size() >= n_stages;
    if (fits) return RT_OK;
    int rc = wave_harvest(ctx, R, true);
    if (rc) return rc;
    if (!R.lanes.empty()) qcap = std::max(qcap, R.lanes[0].ws.qcap);
    jobcap = std::max(jobcap, R.jobcap);
    n_stages = std::max(n_stages, (int)R.stages.size());
    if ((int)R.lanes.size() != n_lanes) {   // a lane count change starts from new lanes
        for (WaveLane &L : R.lanes) {
            if (L.stream) {
                cudaStreamSynchronize(L.stream);
                cudaStreamDestroy(L.stream);
            }
            if (L.last) cudaEventDestroy(L.last);
        }
        R.lanes.clear();
        R.lanes.resize((size_t)n_lanes);
        R.next_lane = 0;
        if (n_lanes > 1) {
            for (WaveLane &L : R.lanes) {
                CK(ctx, cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
                CK(ctx, cudaEventCreateWithFlags(&L.last, cudaEventDisableTiming));
            }
            if (!R.go) CK(ctx, cudaEventCreateWithFlags(&R.go, cudaEventDisableTiming));
        }
    }
    for (WaveLane &L : R.lanes) {
        rc = ws_ensure(ctx, L.ws, qcap, jobcap);
        if (rc) return rc;
        L.graphs.clear();   // captured graphs point into the old workspace
        L.ws.wf.cancel = nullptr;   // rt_batch_render arms and sets the context's flag
    }
    for (WaveStage &st : R.stages) {
        if (st.jobs) cudaFreeHost(st.jobs);
        if (st.done) cudaEventDestroy(st.done);
        if (st.start) cudaEventDestroy(st.start);
    }
    R.stages.assign((size_t)n_stages, WaveStage());
    R.next = 0;
    R.jobcap = jobcap;
    const size_t o_end = sizeof(DevJob) * jobcap, o_scn = o_end + 8 * (size_t)jobcap,
                 o_sc = o_scn + sizeof(DevScene) * jobcap, o_ctr = o_sc + 64, total = o_ctr + sizeof(Counters);
    for (WaveStage &st : R.stages) {
        void *p = nullptr;
        CK(ctx, cudaHostAlloc(&p, total, cudaHostAllocDefault));
        char *b = (char *)p;
        st.jobs = (DevJob *)b;
        st.end = (long long *)(b + o_end);
        st.scenes = (DevScene *)(b + o_scn);
        st.scalars = (long long *)(b + o_sc);
        st.counters = (Counters *)(b + o_ctr);
        CK(ctx, cudaEventCreate(&st.done));
        CK(ctx, cudaEventCreate(&st.start));
    }
    return RT_OK;
}

static int wave_graph(rt_ctx *ctx, WaveLane &R, int max_level, const Tuning &t, cudaGraphExec_t &exec)
{
    const long long key = tuning_key(max_level, t);
    auto it = R.graphs.find(key);
    if (it != R.graphs.end()) {
        exec = it->second->exec;
        return RT_OK;
    }
    cudaStream_t cap;
    CK(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaMemsetAsync(R.ws.wf.C, 0, kCounterBlockBytes, cap);
    enqueue_levels(ctx, R.ws, max_level, t, cap, nullptr);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    std::unique_ptr<GraphEntry> ge(new GraphEntry());
    e = cudaGraphInstantiate(&ge->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    exec = ge->exec;
    R.graphs[key] = std::move(ge);
    return RT_OK;
}

int wave_enqueue(rt_ctx *ctx, WaveRunner &R, const std::vector<WaveJob *> &jobs, const Tuning &t, bool use_graph,
                 cudaStream_t s, long long *samples_out, KernelProfiler *prof)
{
    *samples_out = 0;
    if (R.stages.empty() || R.lanes.empty() || !R.stages[R.next].jobs)
        return ctx_fail(ctx, RT_ERR_INVALID, "wave runner not initialised");
    WaveStage &st = R.stages[R.next];
    int rc = stage_harvest(ctx, R, st, true);   // the ring is full: wait for its oldest wave
    if (rc) return rc;
    WaveLane &lane = R.lanes[R.next_lane];
    if (!lane.ws.mem.p)   // a failed re-initialisation left the lane without a workspace
        return ctx_fail(ctx, RT_ERR_INVALID, "wave lane %zu has no workspace", R.next_lane);
    const long long Q = lane.ws.qcap;
    long long used = 0, samples = 0;
    int n = 0, n_scenes = 0, max_level = 0, max_lights = 0;
    std::vector<const SceneDev *> seen;
    for (WaveJob *j : jobs) {
        if (j->cursor >= j->total) continue;
        if (n == R.jobcap) break;
        const long long room = (Q - used) / j->weight;
        if (room <= 0) break;   // jobs keep their order: the wave is full
        const long long take = std::min(room, j->total - j->cursor);
        int slot = -1;
        for (int k = 0; k < n_scenes; ++k)
            if (seen[k] == j->scene) slot = k;
        if (slot < 0) {
            slot = n_scenes++;
            seen.push_back(j->scene);
            st.scenes[slot] = j->scene->hdr;
            max_lights = std::max(max_lights, j->scene->hdr.n_lights);
        }
        DevJob J = j->job;
        J.scene = slot;
        J.sample_base = samples - j->cursor;   // wave sample g maps to job sample g - sample_base
        st.jobs[n] = J;
        samples += take;
        st.end[n] = samples;
        used += take * j->weight;
        j->cursor += take;
        max_level = std::max(max_level, J.max_level);
        ++n;
    }
    if (n == 0) return RT_OK;
    st.scalars[0] = samples;
    st.scalars[1] = 0;
    st.scalars[2] = n;
    st.scalars[3] = max_lights;
    st.n_jobs = n;
    st.samples = samples;
    Workspace &ws = lane.ws;
    if (lane.stream) {   // after what the caller enqueued on s (frame preparation, the cancel clear)
        CK(ctx, cudaEventRecord(R.go, s));
        CK(ctx, cudaStreamWaitEvent(lane.stream, R.go, 0));
        s = lane.stream;
    }
    CK(ctx, cudaEventRecord(st.start, s));
    CK(ctx, cudaMemcpyAsync(ws.scenes, st.scenes, sizeof(DevScene) * n_scenes, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(ws.jobs, st.jobs, sizeof(DevJob) * n, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(ws.job_end, st.end, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(ws.scalars, st.scalars, 32, cudaMemcpyHostToDevice, s));
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        rc = wave_graph(ctx, lane, max_level, t, exec);
        if (rc) return rc;
        CK(ctx, cudaGraphLaunch(exec, s));
    } else {
        CK(ctx, cudaMemsetAsync(ws.wf.C, 0, kCounterBlockBytes, s));
        enqueue_levels(ctx, ws, max_level, t, s, prof);
    }
    CK(ctx, cudaMemcpyAsync(st.counters, ws.wf.C, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaEventRecord(st.done, s));
    if (lane.stream) {
        CK(ctx, cudaEventRecord(lane.last, s));
        lane.pending = true;
    }
    st.lane = (int)R.next_lane;
    st.busy = true;
    R.next_lane = (R.next_lane + 1) % R.lanes.size();
    R.next = (R.next + 1) % R.stages.size();
    R.waves++;
    R.wave_jobs += n;
    *samples_out = samples;
    return RT_OK;
}

// ---- batch ---------------------------------------------------------------------------------------------------

namespace {
// ray-queue entries of one batch wave by default: 2^26 entries of kWsBytesPerEntry (292 B),
// 19.6 GB. Fewer, larger waves pay each bounce's tail (the longest
// ray of the pass) fewer times.
constexpr long long kBatchQueue = 1ll << 26;
} // namespace

// RT_FLAG_PROFILE on any job: launches go without the graph, bracketed by events per kernel
static int batch_core(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                      const rt_render_desc *rds, const Tuning &t, bool use_graph, long long wave_rays)
{
    if (n <= 0 || !scene_ids || !frame_ids || !rds) return ctx_fail(ctx, RT_ERR_INVALID, "empty batch");
    std::vector<WaveJob> jobs((size_t)n);
    std::vector<FrameDev *> frames((size_t)n);
    long long weighted = 0, heaviest = 1;
    for (int i = 0; i < n; ++i) {
        auto si = ctx->scenes.find(scene_ids[i]);
        if (si == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", scene_ids[i]);
        auto fi = ctx->frames.find(frame_ids[i]);
        if (fi == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", frame_ids[i]);
        for (int j = 0; j < i; ++j)
            if (frame_ids[j] == frame_ids[i]) return ctx_fail(ctx, RT_ERR_INVALID, "frame %d used twice", frame_ids[i]);
        WaveJob &w = jobs[i];
        int rc = make_job(ctx, *si->second, *fi->second, &rds[i], 0, w.job, w.total);
        if (rc) return rc;
        w.job.pixel_tile = t.pixel_tile;
        w.scene = si->second.get();
        w.weight = wave_weight(w.scene->branching, rds[i].max_level);
        frames[i] = fi->second.get();
        weighted += w.total * w.weight;
        heaviest = std::max(heaviest, w.weight);
    }
    if (!ctx->batch) ctx->batch.reset(new WaveRunner());
    WaveRunner &R = *ctx->batch;
    const long long cap = wave_rays > 0 ? wave_rays : kBatchQueue;
    const long long qcap = std::max(std::min(weighted, cap), std::max<long long>(heaviest, 4096));
    bool profile = false;
    for (int i = 0; i < n; ++i) profile |= (rds[i].flags & RT_FLAG_PROFILE) != 0;
    // a profiled batch runs its waves one after another, so kernel times do not overlap
    const int lanes = profile ? 1 : t.lanes;
    int rc = wave_runner_init(ctx, R, qcap, std::max(n, 64), 2 * lanes, lanes);
    if (rc) return rc;
    ctx->prof.reset(profile);
    if (profile) use_graph = false;
    KernelProfiler *P = profile ? &ctx->prof : nullptr;
    cudaStream_t s = ctx->stream;
    for (WaveLane &L : R.lanes) L.ws.wf.cancel = ctx->cancel_dev;
    rc = cancel_arm(ctx, ctx->cancel_count.load());
    if (rc) return rc;
    R.rays_primary = R.rays_secondary = R.rays_shadow = 0;
    R.overflow = R.error = 0;
    ctx->stamped = false;   // warp stamps belong to profiled plain renders only
    R.wave_ms.clear();
    R.wait_s = 0.0;
    // the frame table; its pinned host copy is rewritten once the previous copy out of it ran
    if (!R.ftab_copied) CK(ctx, cudaEventCreateWithFlags(&R.ftab_copied, cudaEventDisableTiming));
    CK(ctx, cudaEventSynchronize(R.ftab_copied));
    if (R.ftab_cap < n) {
        if (R.ftab_host) cudaFreeHost(R.ftab_host);
        R.ftab_host = nullptr;
        R.ftab_cap = 0;
        CK(ctx, cudaMallocHost((void **)&R.ftab_host, sizeof(FrameJob) * (size_t)n));
        R.ftab_cap = n;
    }
    CK(ctx, R.ftab_dev.ensure(sizeof(FrameJob) * (size_t)n));
    long long quads = 0;
    for (int i = 0; i < n; ++i) {
        FrameJob &F = R.ftab_host[i];
        F = frame_job(frames[i]->fb, frames[i]->w, frames[i]->h, jobs[i].job);
        quads += F.quad_end;
        F.quad_end = quads;
    }
    const FrameJob *ftab = (const FrameJob *)R.ftab_dev.p;
    CK(ctx, cudaEventRecord(ctx->ev_start, s));
    CK(ctx, cudaMemcpyAsync(R.ftab_dev.p, R.ftab_host, sizeof(FrameJob) * (size_t)n, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaEventRecord(R.ftab_copied, s));
    launch_frames_prepare(ftab, n, quads, s);
    std::vector<WaveJob *> order((size_t)n);
    for (int i = 0; i < n; ++i) order[i] = &jobs[i];
    for (;;) {
        long long got = 0;
        rc = wave_enqueue(ctx, R, order, t, use_graph, s, &got, P);
        if (rc) return rc;
        if (!got) break;
    }
    wave_join(R, s);   // the resolve reads what every wave accumulated
    if (P) P->begin(RT_KERNEL_RESOLVE, s);
    launch_frames_resolve(ftab, n, quads, s);
    if (P) P->end(s);
    CK(ctx, cudaGetLastError());
    CK(ctx, cudaEventRecord(ctx->ev_stop, s));
    rc = wave_harvest(ctx, R, true);
    if (rc) return rc;
    CK(ctx, cudaStreamSynchronize(s));
    Counters &C = *ctx->counters_host;
    C.rays_primary = R.rays_primary, C.rays_secondary = R.rays_secondary, C.rays_shadow = R.rays_shadow;
    C.overflow = R.overflow, C.error = R.error;
    ctx->pending.active = false;
    if (cancel_requested(ctx)) return ctx_fail(ctx, RT_ERR_CANCELLED, "batch cancelled");
    if (R.overflow) return ctx_fail(ctx, RT_ERR_OVERFLOW, "batch ray queue overflow");
    if (R.error) return ctx_fail(ctx, RT_ERR_CUDA, "traversal stopped on a corrupt LBVH (flags 0x%x)", R.error);
    return RT_OK;
}

extern "C" int rt_batch_render(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                               const rt_render_desc *rds, const rt_batch_tuning *tuning)
{
    if (!ctx) return RT_ERR_INVALID;
    // defaults: persistent grid, 32-ray tiles, 128-thread blocks capped at 64 registers, two
    // lanes, primary rays in 8x8 pixel tiles (2.8 % faster than row by row on the 256-scene
    // batch, 4 % on the served request mix)
    Tuning t;
    t.pixel_tile = kWavePixelTile;
    bool graph = true;
    long long wave = 0;
    if (tuning) {
        int rc = tuning_from(ctx, tuning, t);
        if (rc) return rc;
        graph = tuning->use_graph != 0;
        wave = tuning->wave_rays;
        if (wave < 0 || wave > (1ll << 27)) return ctx_fail(ctx, RT_ERR_INVALID, "wave_rays %lld outside [0, 2^27]", wave);
    }
    return batch_core(ctx, n, scene_ids, frame_ids, rds, t, graph, wave);
}

extern "C" int rt_batch_render_plain(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                                     const rt_render_desc *rds)
{
    if (!ctx || n <= 0 || !scene_ids || !frame_ids || !rds) return RT_ERR_INVALID;
    unsigned long long prim = 0, sec = 0, shd = 0;
    for (int i = 0; i < n; ++i) {
        int rc = rt_render(ctx, scene_ids[i], frame_ids[i], &rds[i]);
        if (rc) return rc;
        rt_render_stats st;
        rc = rt_render_wait(ctx, &st);
        if (rc) return rc;
        prim += (unsigned long long)st.rays_primary;
        sec += (unsigned long long)st.rays_secondary;
        shd += (unsigned long long)st.rays_shadow;
    }
    Counters &C = *ctx->counters_host;
    C.rays_primary = prim, C.rays_secondary = sec, C.rays_shadow = shd;
    return RT_OK;
}

extern "C" int rt_batch_autotune(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                                 const rt_render_desc *rds, rt_batch_tuning *out)
{
    if (!ctx || !out) return RT_ERR_INVALID;
    // Coordinate search, each candidate timed as the best of five batches after a warm one
    // (which captures its graph): (threads per block, register cap as resident blocks per SM) x
    // rays per tile fetch (0 = the static grid stride), then per-SM shares of the rays, then one
    // wave lane instead of two, then the traversal stack entries kept in shared memory, then the primary rays' pixel tile, then the
    // shadow work chunk, then the wave size. The caller picks the jobs: tuning on a sample of the
    // workload and measuring on the rest keeps the choice honest. The defaults are the incumbent,
    // and a candidate replaces the incumbent only when it is at least 2 % faster: smaller gains
    // are within the spread of repeated batches and did not carry over to other jobs. The lanes
    // trial needs a batch of four waves or more (one lane and two differ only across waves).
    const int shapes[][2] = {{128, 8}, {128, 6}, {64, 8}, {256, 0}};
    const int tiles[] = {0, 32, 64, 128, 256};
    const int stacks[] = {0, 8};
    const int chunks[] = {0, 1024, 4096, 16384};
    const int pixel_tiles[] = {0, 8, 16, 32};
    const long long waves[] = {1ll << 25, 1ll << 27};   // the default is 2^26
    const double kKeep = 0.98;
    double best = 1e30;
    rt_batch_tuning best_t{128, 32, 0, 1, 8, 1, 0, 4096, kWavePixelTile, 0, 0};   // the defaults
    long long batch_waves = 0;   // waves of one batch of the jobs (the defaults' wave size)
    auto trial = [&](const rt_batch_tuning &t) {
        const long long w0 = ctx->batch ? ctx->batch->waves : 0;
        int rc = rt_batch_render(ctx, n, scene_ids, frame_ids, rds, &t);   // warm (captures the graph)
        if (rc) return rc;
        const long long waves = ctx->batch ? ctx->batch->waves - w0 : 0;
        double dt = 1e30;
        for (int rep = 0; rep < 5; ++rep) {
            auto t0 = std::chrono::steady_clock::now();
            rc = rt_batch_render(ctx, n, scene_ids, frame_ids, rds, &t);
            if (rc) return rc;
            cudaStreamSynchronize(ctx->stream);
            dt = std::min(dt, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
        }
        if (best == 1e30) batch_waves = waves;
        if (dt < best * kKeep || best == 1e30) best = dt, best_t = t;
        return RT_OK;
    };
    int rc0 = trial(best_t);
    if (rc0) return rc0;
    for (const auto &sh : shapes)
        for (int tl : tiles) {
            if (sh[0] == 128 && sh[1] == 8 && tl == 32) continue;   // the defaults, timed first
            int rc = trial(rt_batch_tuning{sh[0], tl ? tl : 32, 0, 1, sh[1], tl ? 1 : 2, 0, 4096, kWavePixelTile, 0, 0});
            if (rc) return rc;
        }
    if (best_t.dynamic == 1) {   // the tiles of each SM's own share of the rays first
        rt_batch_tuning t = best_t;
        t.dynamic = 3;
        int rc = trial(t);
        if (rc) return rc;
    }
    if (batch_waves >= 4) {   // waves one after another on one workspace instead of in turn on two
        rt_batch_tuning t = best_t;
        t.lanes = 1;
        int rc = trial(t);
        if (rc) return rc;
    }
    for (int ss : stacks) {
        if (ss == best_t.stack) continue;
        rt_batch_tuning t = best_t;
        t.stack = ss;
        int rc = trial(t);
        if (rc) return rc;
    }
    for (int pt : pixel_tiles) {
        if (pt == best_t.pixel_tile) continue;
        rt_batch_tuning t = best_t;
        t.pixel_tile = pt;
        int rc = trial(t);
        if (rc) return rc;
    }
    for (int ch : chunks) {
        if (ch == best_t.shadow_chunk) continue;
        rt_batch_tuning t = best_t;
        t.shadow_chunk = ch;
        int rc = trial(t);
        if (rc) return rc;
    }
    for (long long w : waves) {
        rt_batch_tuning t = best_t;
        t.wave_rays = w;
        int rc = trial(t);
        if (rc) return rc;
    }
    if (!best_t.lanes) best_t.lanes = 2;   // the batch default, stated
    *out = best_t;
    return RT_OK;
}
