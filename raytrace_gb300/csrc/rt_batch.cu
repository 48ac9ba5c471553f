// rt_batch.cu — batched multi-scene rendering: many (scene, frame) jobs traced as one
// wavefront by persistent kernels that pull ray tiles from global work counters, with the
// per-bounce launch sequence captured once as a CUDA graph and replayed per wave; plus the
// plain loop of per-scene renders it is compared against, and the autotuner.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_capi_internal.h"

using namespace rtg;

namespace {

struct JobPlan {
    std::vector<DevJob> jobs;
    std::vector<long long> samples;
    std::vector<FrameDev *> frames;
    std::vector<int> spp;
    int max_level = 0;
};

int plan_jobs(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids, const rt_render_desc *rds,
              JobPlan &plan, std::vector<DevScene> &hdrs)
{
    if (n <= 0 || !scene_ids || !frame_ids || !rds) return ctx_fail(ctx, RT_ERR_INVALID, "empty batch");
    std::map<int, int> slot_of;
    for (int i = 0; i < n; ++i) {
        auto si = ctx->scenes.find(scene_ids[i]);
        if (si == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", scene_ids[i]);
        auto fi = ctx->frames.find(frame_ids[i]);
        if (fi == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", frame_ids[i]);
        for (int j = 0; j < i; ++j)
            if (frame_ids[j] == frame_ids[i]) return ctx_fail(ctx, RT_ERR_INVALID, "frame %d used twice", frame_ids[i]);
        int slot;
        auto it = slot_of.find(scene_ids[i]);
        if (it == slot_of.end()) {
            slot = (int)hdrs.size();
            slot_of[scene_ids[i]] = slot;
            hdrs.push_back(si->second->hdr);
        } else
            slot = it->second;
        DevJob J;
        long long s = 0;
        int rc = make_job(ctx, *si->second, *fi->second, &rds[i], slot, J, s);
        if (rc) return rc;
        plan.jobs.push_back(J);
        plan.samples.push_back(s);
        plan.frames.push_back(fi->second.get());
        plan.spp.push_back(rds[i].spp);
        plan.max_level = std::max(plan.max_level, rds[i].max_level);
    }
    return RT_OK;
}

// samples per wave: bounds the queue memory of a batch
constexpr long long kWaveSamples = 1ll << 24;

} // namespace

static int batch_core(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                      const rt_render_desc *rds, const Tuning &t, bool use_graph)
{
    JobPlan plan;
    std::vector<DevScene> hdrs;
    int rc = plan_jobs(ctx, n, scene_ids, frame_ids, rds, plan, hdrs);
    if (rc) return rc;
    long long total = 0;
    std::vector<long long> end(plan.jobs.size());
    for (size_t i = 0; i < plan.jobs.size(); ++i) {
        plan.jobs[i].sample_base = total;
        total += plan.samples[i];
        end[i] = total;
    }
    const long long wave = std::min(total, kWaveSamples);
    rc = ws_ensure(ctx, ctx->ws, std::max<long long>(2 * wave, 4096), (int)std::max(plan.jobs.size(), hdrs.size()));
    if (rc) return rc;
    Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    ws.wf.cancel = ctx->cancel_dev;
    *ctx->cancel_host = 0;
    if (cudaEventRecord(ctx->ev_start, s) != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "event record");
    cudaMemcpyAsync(ws.scenes, hdrs.data(), sizeof(DevScene) * hdrs.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.jobs, plan.jobs.data(), sizeof(DevJob) * plan.jobs.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.job_end, end.data(), 8 * end.size(), cudaMemcpyHostToDevice, s);
    for (FrameDev *f : plan.frames) {
        cudaMemsetAsync(f->fb.acc, 0, 24 * (size_t)f->w * f->h, s);
    }
    for (size_t i = 0; i < plan.jobs.size(); ++i)
        if (plan.jobs[i].plane_obj) launch_plane_init(plan.frames[i]->fb, (long long)plan.frames[i]->w * plan.frames[i]->h, s);
    // per-wave sequence; captured once per (max_level, tuning) and replayed
    const long long key = ((long long)plan.max_level << 40) ^ ((long long)t.block << 24) ^ ((long long)t.tile << 8) ^
                          (long long)t.stack ^ ((long long)t.dynamic << 50) ^ ((long long)t.min_blocks << 52);
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        auto it = ctx->graphs.find(key);
        if (it == ctx->graphs.end()) {
            cudaStream_t cap;
            cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
            cudaGraph_t g;
            cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            cudaMemsetAsync(ws.wf.C, 0, sizeof(Counters), cap);
            enqueue_levels(ctx, ws, plan.max_level, t, cap, nullptr);
            cudaError_t e = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
            std::unique_ptr<GraphEntry> ge(new GraphEntry());
            e = cudaGraphInstantiate(&ge->exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
            exec = ge->exec;
            ctx->graphs[key] = std::move(ge);
        } else
            exec = it->second->exec;
    }
    unsigned long long prim = 0, sec = 0, shd = 0;
    int overflow = 0;
    for (long long first = 0; first < total; first += wave) {
        ctx->h_scalars[0] = std::min(wave, total - first);
        ctx->h_scalars[1] = first;
        ctx->h_scalars[2] = (long long)plan.jobs.size();
        long long ml = 0;
        for (const DevScene &hd : hdrs) ml = std::max<long long>(ml, hd.n_lights);
        ctx->h_scalars[3] = ml;
        cudaMemcpyAsync(ws.scalars, ctx->h_scalars, 32, cudaMemcpyHostToDevice, s);
        if (exec)
            cudaGraphLaunch(exec, s);
        else {
            cudaMemsetAsync(ws.wf.C, 0, sizeof(Counters), s);
            enqueue_levels(ctx, ws, plan.max_level, t, s, nullptr);
        }
        cudaMemcpyAsync(ctx->counters_host, ws.wf.C, sizeof(Counters), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "batch wave failed");
        prim += ctx->counters_host->rays_primary;
        sec += ctx->counters_host->rays_secondary;
        shd += ctx->counters_host->rays_shadow;
        overflow |= ctx->counters_host->overflow;
    }
    for (size_t i = 0; i < plan.jobs.size(); ++i)
        launch_resolve(plan.frames[i]->fb, plan.frames[i]->w, plan.frames[i]->h, plan.spp[i], s);
    cudaEventRecord(ctx->ev_stop, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "batch: %s", cudaGetErrorString(e));
    Counters &C = *ctx->counters_host;
    C.rays_primary = prim, C.rays_secondary = sec, C.rays_shadow = shd, C.overflow = overflow;
    ctx->pending.active = false;
    if (overflow) return ctx_fail(ctx, RT_ERR_OVERFLOW, "batch ray queue overflow");
    return RT_OK;
}

extern "C" int rt_batch_render(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                               const rt_render_desc *rds, const rt_batch_tuning *tuning)
{
    if (!ctx) return RT_ERR_INVALID;
    Tuning t;   // defaults: persistent grid, 32-ray tiles, 128-thread blocks capped at 64 registers
    bool graph = true;
    if (tuning) {
        int rc = tuning_from(ctx, tuning, t);
        if (rc) return rc;
        graph = tuning->use_graph != 0;
    }
    return batch_core(ctx, n, scene_ids, frame_ids, rds, t, graph);
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
    // (threads per block, register cap as resident blocks per SM) x rays per tile fetch; the
    // stack stays at 64 entries, the depth bound of a 30-bit Morton LBVH with index tie-breaks
    const int shapes[][2] = {{128, 8}, {128, 6}, {64, 8}, {256, 0}};
    const int tiles[] = {32, 64, 128, 256};
    double best = 1e30;
    rt_batch_tuning best_t{128, 32, 64, 1, 8, 1};
    for (const auto &sh : shapes)
        for (int tl : tiles) {
            rt_batch_tuning t{sh[0], tl, 64, 1, sh[1], 1};
            int rc = rt_batch_render(ctx, n, scene_ids, frame_ids, rds, &t);   // warm (captures the graph)
            if (rc) return rc;
            auto t0 = std::chrono::steady_clock::now();
            rc = rt_batch_render(ctx, n, scene_ids, frame_ids, rds, &t);
            if (rc) return rc;
            cudaStreamSynchronize(ctx->stream);
            double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (dt < best) best = dt, best_t = t;
        }
    *out = best_t;
    return RT_OK;
}
