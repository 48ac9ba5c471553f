// rt_server.cu — continuous-batching render server over device-resident scenes.
//
// Requests (scene, camera, resolution) queue as they arrive. Each step retires finished
// frames, admits queued requests in arrival order while a frame slot, a host result slot and
// the HBM budget allow (evicting idle scenes least-recently-used first and rebuilding an
// evicted scene's LBVH when a request needs it again), and enqueues one wave made of sample
// chunks of every admitted request: requests admitted at different times trace in the same
// kernels. With two lanes (a workspace and a stream each; the tuning's lane count, 1 by
// default) waves go to them in turn, so a wave's kernels can fill the SMs the previous wave's
// kernels leave idle as they drain. The frames admitted in a step are prepared on a stream of
// their own while the previous wave runs; a request whose last chunk is enqueued is resolved on
// another stream once the waves that traced it are done (with two lanes, in the next step, after
// the next wave is enqueued), so neither holds back a wave, and copied to pinned host memory on
// a copy stream. Its frame slot is reused once that copy is done. Colours accumulate as
// exact fixed-point sums, so a frame is bit-identical alone, in any mix and split over any
// waves. The plain mode renders one request at a time through rt_render, for comparison.
//
// No counterpart in the reference: its RayTracer::start (RayTracer.cpp:614) renders one scene
// per call into one output buffer.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_capi_internal.h"

using namespace rtg;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { kQueued, kInflight, kResolving, kDone };

struct SrvScene {
    rt_scene_host *host = nullptr;
    int ctx_id = -1;          // context scene id while resident
    int64_t bytes = 0;        // device bytes when resident
    int64_t scratch = 0;      // LBVH build scratch it needs
    uint64_t last_use = 0;
    int users = 0;            // admitted requests not yet fully enqueued
    rt_camera camera{};
};

struct DevSlot {
    DevBuf mem;
    FrameBufs fb{};
    bool used = false;              // until the image copy out of it is done
};

struct HostSlot {
    void *mem = nullptr;
    float *rgb = nullptr;
    uint8_t *rgb8 = nullptr;
    bool used = false;
};

struct Request {
    int64_t id = 0;
    rt_request req{};
    int scene = 0;
    int state = kQueued;
    int status = RT_OK;
    int dev_slot = -1, host_slot = -1;
    WaveJob wj;
    double arrival_s = 0, admit_s = 0, done_s = 0;
    int rebuilt = 0;
    cudaEvent_t done_ev = nullptr;
    std::vector<float> rgb;       // kept image (keep_images)
    std::vector<uint8_t> rgb8;
};

struct SplitMix {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

const int kServeRes[4][2] = {{256, 256}, {512, 512}, {1024, 768}, {1920, 1080}};

// Frame tables of the per-step prepare or resolve launches (every request admitted in a step
// is prepared by one launch, every request finished in a step is resolved by one): pinned host
// copies in a small ring, each rewritten once the copy out of it has run. Each ring serves one
// stream, so a device table is rewritten only after the kernel that read it.
struct TableRing {
    static constexpr int kSlots = 4;
    FrameJob *host[kSlots] = {};
    DevBuf dev[kSlots];
    cudaEvent_t copied[kSlots] = {};
    int cap = 0, next = 0;
};

} // namespace

struct rt_server {
    rt_ctx *ctx = nullptr;
    rt_server_config cfg{};
    Clock::time_point t0;
    cudaEvent_t base_ev = nullptr;
    double base_s = 0.0;          // server clock at base_ev
    cudaStream_t copy = nullptr;
    cudaStream_t prep = nullptr;      // frame preparation of the admitted requests
    cudaStream_t rsv = nullptr;       // resolves of the finished requests
    cudaEvent_t prep_ev = nullptr;    // the last preparation, before the next wave
    cudaEvent_t wave_ev = nullptr;    // the last wave of a one-lane runner, before its resolves
    cudaEvent_t solo_ev = nullptr;    // the last frame launch of a solo step, before the side streams
    // solo step: nothing else was in flight, so the step's preparation, wave, resolve and copies go
    // on the wave stream itself, without the hops between streams (a lone request's latency)
    bool solo = false;
    // the pixel tile is the default's: requests admitted into an idle server trace row by row (a
    // lone request's render was 3.5 % slower in tiles; waves of many requests are faster in them)
    bool default_tile = true;
    WaveRunner runner;
    // lanes 1 (two concurrent waves served no more rays a second); the waves make primary rays
    // in 8x8 pixel tiles (the served request mix traced 2.7 % faster than row by row), the plain
    // mode row by row (its single-request renders were 3.5 % slower in tiles)
    Tuning tuning;
    std::vector<SrvScene> scenes;
    std::vector<DevSlot> dslots;
    std::deque<int> free_dslots;        // oldest freed first
    std::vector<HostSlot> hslots;
    std::deque<Request *> queue;
    std::vector<Request *> inflight;    // admission order
    std::vector<Request *> deferred;    // last chunk in the last wave: resolved in the next step
    std::deque<Request *> resolving;    // enqueue order
    std::unordered_map<int64_t, std::unique_ptr<Request>> reqs;
    std::vector<cudaEvent_t> ev_pool;
    TableRing tables[2];                // prepare (on prep), resolve (on rsv)
    std::vector<FrameJob> to_prepare, to_resolve;   // this step's frames
    std::vector<Request *> resolved;                // requests of to_resolve
    int64_t next_id = 0;
    uint64_t tick = 0;
    int64_t fixed_bytes = 0, peak_bytes = 0;
    // counters since creation or the last stats reset
    int64_t n_requests = 0, n_completed = 0, n_rejected = 0, evictions = 0, rebuilds = 0, admitted_busy = 0,
            pixels = 0;
    std::vector<double> latencies_ms;
    double first_arrival = -1.0, last_done = 0.0;
    unsigned long long plain_rays = 0;
    long long waves0 = 0, wave_jobs0 = 0;
    double host_step_s = 0.0, host_wait_s = 0.0;   // inside rt_server_step; blocked on frame copies
    int64_t steps = 0;
    std::map<std::pair<int, int>, int> plain_frames;
    int64_t plain_frame_bytes = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

// messages go to the context's last error, which rt_server_last_error reports
static int srv_fail(rt_server *srv, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    srv->ctx->err = buf;
    return code;
}


static int64_t used_bytes(const rt_server *srv)
{
    int64_t b = srv->fixed_bytes + srv->plain_frame_bytes + (int64_t)srv->ctx->lbvh_scratch.bytes +
                (int64_t)spare_bytes(srv->ctx);
    for (const SrvScene &s : srv->scenes)
        if (s.ctx_id >= 0) b += s.bytes;
    return b;
}

static void note_peak(rt_server *srv) { srv->peak_bytes = std::max(srv->peak_bytes, used_bytes(srv)); }

static cudaEvent_t take_event(rt_server *srv)
{
    if (!srv->ev_pool.empty()) {
        cudaEvent_t e = srv->ev_pool.back();
        srv->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

static void evict(rt_server *srv, SrvScene &s)
{
    rt_scene_release(srv->ctx, s.ctx_id);   // waits for the stream: no wave still reads it
    s.ctx_id = -1;
    srv->evictions++;
}

// Make scene `k` resident within the budget. RT_ERR_BUSY: not now (scenes in use hold the
// memory); RT_ERR_BUDGET: never (it does not fit even alone).
static int make_resident(rt_server *srv, int k, int *rebuilt)
{
    SrvScene &s = srv->scenes[(size_t)k];
    s.last_use = ++srv->tick;
    if (s.ctx_id >= 0) return RT_OK;
    const int64_t budget = srv->cfg.hbm_budget_bytes;
    auto need = [&]() {
        return used_bytes(srv) + s.bytes + std::max<int64_t>(0, s.scratch - (int64_t)srv->ctx->lbvh_scratch.bytes);
    };
    while (need() > budget) {
        if (spare_bytes(srv->ctx) > 0) {   // released buffers the context keeps go first
            spare_trim(srv->ctx);
            continue;
        }
        SrvScene *victim = nullptr;
        for (SrvScene &o : srv->scenes)
            if (o.ctx_id >= 0 && o.users == 0 && (!victim || o.last_use < victim->last_use)) victim = &o;
        if (!victim) {
            bool any_resident = false;
            for (SrvScene &o : srv->scenes) any_resident |= o.ctx_id >= 0;
            return any_resident ? RT_ERR_BUSY
                                : srv_fail(srv, RT_ERR_BUDGET, "scene %d needs %lld bytes, over the budget", k, (long long)s.bytes);
        }
        evict(srv, *victim);
    }
    int id = -1;
    int rc = rt_scene_upload(srv->ctx, rt_scene_host_desc(s.host), &id);
    if (rc) return rc;
    s.ctx_id = id;
    srv->rebuilds++;
    if (rebuilt) *rebuilt = 1;
    note_peak(srv);
    return RT_OK;
}

static int find_free(const std::vector<HostSlot> &v)
{
    for (size_t i = 0; i < v.size(); ++i)
        if (!v[i].used) return (int)i;
    return -1;
}

static void reject(rt_server *srv, Request *r, int status)
{
    r->status = status;
    r->state = kDone;
    r->done_s = srv->now();
    srv->n_rejected++;
}

// admit queued requests in arrival order
static int admit(rt_server *srv, bool idle)
{
    rt_ctx *ctx = srv->ctx;
    while (!srv->queue.empty()) {
        Request *r = srv->queue.front();
        const int ds = srv->free_dslots.empty() ? -1 : srv->free_dslots.front(), hs = find_free(srv->hslots);
        if (ds < 0 || hs < 0) break;
        int rebuilt = 0;
        int rc = make_resident(srv, r->scene, &rebuilt);
        if (rc == RT_ERR_BUSY) break;   // wait for scenes in use to retire
        if (rc) {
            srv->queue.pop_front();
            reject(srv, r, rc);
            continue;
        }
        SrvScene &sc = srv->scenes[(size_t)r->scene];
        const SceneDev &sd = *ctx->scenes.at(sc.ctx_id);
        DevSlot &slot = srv->dslots[(size_t)ds];
        FrameDev view;   // the slot seen as a frame of the request's size
        view.w = r->req.width, view.h = r->req.height;
        view.fb = slot.fb;
        rt_camera cam = r->req.camera;
        cam.width = r->req.width, cam.height = r->req.height;
        rt_render_desc rd{r->req.width, r->req.height, srv->cfg.spp, srv->cfg.max_level, RT_MODE_RAYTRACE, 0,
                          r->req.seed, &cam};
        long long samples = 0;
        rc = make_job(ctx, sd, view, &rd, 0, r->wj.job, samples);
        if (rc) {
            srv->queue.pop_front();
            reject(srv, r, rc);
            continue;
        }
        r->wj.job.pixel_tile = idle && srv->default_tile ? 0 : srv->tuning.pixel_tile;
        r->wj.scene = &sd;
        r->wj.total = samples;
        r->wj.cursor = 0;
        r->wj.weight = wave_weight(sd.branching, srv->cfg.max_level);
        srv->to_prepare.push_back(frame_job(slot.fb, r->req.width, r->req.height, r->wj.job));
        slot.used = true;
        srv->free_dslots.pop_front();
        srv->hslots[(size_t)hs].used = true;
        r->dev_slot = ds, r->host_slot = hs;
        r->rebuilt = rebuilt;
        if (!srv->inflight.empty() || !srv->deferred.empty() || !srv->resolving.empty()) srv->admitted_busy++;
        r->admit_s = srv->now();
        r->state = kInflight;
        sc.users++;
        srv->inflight.push_back(r);
        srv->queue.pop_front();
    }
    return RT_OK;
}

// one launch over this step's frames of `jobs` (prepare on prep, or resolve on rsv), its table
// staged through that stream's ring
static int launch_frames(rt_server *srv, std::vector<FrameJob> &jobs, bool resolve)
{
    rt_ctx *ctx = srv->ctx;
    if (jobs.empty()) return RT_OK;
    TableRing &T = srv->tables[resolve ? 1 : 0];
    cudaStream_t s = srv->solo ? ctx->stream : resolve ? srv->rsv : srv->prep;
    const int k = T.next;
    T.next = (k + 1) % TableRing::kSlots;
    if (!T.copied[k]) CK(ctx, cudaEventCreateWithFlags(&T.copied[k], cudaEventDisableTiming));
    CK(ctx, cudaEventSynchronize(T.copied[k]));   // the previous copy out of this host table ran
    if ((int)jobs.size() > T.cap) return srv_fail(srv, RT_ERR_INVALID, "%zu frames in one step", jobs.size());
    long long quads = 0;
    for (size_t i = 0; i < jobs.size(); ++i) {
        quads += jobs[i].quad_end;   // frame_job sets quad_end to the frame's own quads
        jobs[i].quad_end = quads;
        T.host[k][i] = jobs[i];
    }
    CK(ctx, cudaMemcpyAsync(T.dev[k].p, T.host[k], sizeof(FrameJob) * jobs.size(), cudaMemcpyHostToDevice, s));
    CK(ctx, cudaEventRecord(T.copied[k], s));
    const FrameJob *d = (const FrameJob *)T.dev[k].p;
    if (resolve) launch_frames_resolve(d, (int)jobs.size(), quads, s);
    else launch_frames_prepare(d, (int)jobs.size(), quads, s);
    CK(ctx, cudaGetLastError());
    if (srv->solo) {   // the side stream's next use of this ring follows the launch
        CK(ctx, cudaEventRecord(srv->solo_ev, s));
        CK(ctx, cudaStreamWaitEvent(resolve ? srv->rsv : srv->prep, srv->solo_ev, 0));
    }
    jobs.clear();
    return RT_OK;
}

// the last chunk of r is enqueued and every wave that traced it is joined to the resolve stream:
// its resolve and copy-out follow in resolve_finished
static int finish(rt_server *srv, Request *r)
{
    DevSlot &slot = srv->dslots[(size_t)r->dev_slot];
    FrameJob F = frame_job(slot.fb, r->req.width, r->req.height, r->wj.job);
    F.dp_bits = 0;
    if (!srv->cfg.keep_images) F.fb.rgb = nullptr;   // the client gets bytes: no float colour written
    srv->to_resolve.push_back(F);
    srv->resolved.push_back(r);
    return RT_OK;
}

// resolve the frames finished in this step with one launch on rsv, then copy each out on the
// copy stream; a slot is reused only after its copy (complete)
static int resolve_finished(rt_server *srv)
{
    rt_ctx *ctx = srv->ctx;
    if (srv->resolved.empty()) return RT_OK;
    int rc = launch_frames(srv, srv->to_resolve, true);
    if (rc) return rc;
    const cudaStream_t copy = srv->solo ? ctx->stream : srv->copy;
    if (!srv->solo) {
        cudaEvent_t resolved = take_event(srv);
        CK(ctx, cudaEventRecord(resolved, srv->rsv));
        CK(ctx, cudaStreamWaitEvent(copy, resolved, 0));
        srv->ev_pool.push_back(resolved);   // re-recording later does not affect the wait above
    }
    for (Request *r : srv->resolved) {
        DevSlot &slot = srv->dslots[(size_t)r->dev_slot];
        HostSlot &hs = srv->hslots[(size_t)r->host_slot];
        const size_t np = (size_t)r->req.width * r->req.height;
        // the frame a client receives is the uint8 image (Color::put); float colour only when
        // the server keeps images for inspection
        if (srv->cfg.keep_images)
            CK(ctx, cudaMemcpyAsync(hs.rgb, slot.fb.rgb, 12 * np, cudaMemcpyDeviceToHost, copy));
        CK(ctx, cudaMemcpyAsync(hs.rgb8, slot.fb.rgb8, 3 * np, cudaMemcpyDeviceToHost, copy));
        r->done_ev = take_event(srv);
        CK(ctx, cudaEventRecord(r->done_ev, copy));
        r->state = kResolving;
        srv->resolving.push_back(r);
    }
    srv->resolved.clear();
    return RT_OK;
}

// r's image is in host memory: every wave, the resolve and the copy that used its frame slot
// are done, so the slot can be prepared for another request and its scene evicted
static void complete(rt_server *srv, Request *r, double done_s)
{
    if (r->dev_slot >= 0) {
        srv->dslots[(size_t)r->dev_slot].used = false;
        srv->free_dslots.push_back(r->dev_slot);
        r->dev_slot = -1;
        srv->scenes[(size_t)r->scene].users--;
    }
    r->done_s = done_s;
    r->state = kDone;
    srv->n_completed++;
    srv->pixels += (int64_t)r->req.width * r->req.height;
    srv->latencies_ms.push_back(1e3 * (r->done_s - r->arrival_s));
    srv->last_done = std::max(srv->last_done, r->done_s);
    if (r->host_slot >= 0) {
        HostSlot &h = srv->hslots[(size_t)r->host_slot];
        if (srv->cfg.keep_images) {
            const size_t np = (size_t)r->req.width * r->req.height;
            r->rgb.assign(h.rgb, h.rgb + 3 * np);
            r->rgb8.assign(h.rgb8, h.rgb8 + 3 * np);
        }
        h.used = false;
        r->host_slot = -1;
    }
}

// retire resolved requests whose image is in host memory; harvest finished waves
static int retire(rt_server *srv, bool wait_one)
{
    rt_ctx *ctx = srv->ctx;
    while (!srv->resolving.empty()) {
        Request *r = srv->resolving.front();
        cudaError_t e = cudaEventQuery(r->done_ev);
        if (e == cudaErrorNotReady && wait_one) {
            const auto t0 = Clock::now();
            e = cudaEventSynchronize(r->done_ev);
            srv->host_wait_s += std::chrono::duration<double>(Clock::now() - t0).count();
        }
        wait_one = false;
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess) return srv_fail(srv, RT_ERR_CUDA, "frame copy: %s", cudaGetErrorString(e));
        float ms = 0.0f;
        CK(ctx, cudaEventElapsedTime(&ms, srv->base_ev, r->done_ev));
        srv->ev_pool.push_back(r->done_ev);
        r->done_ev = nullptr;
        srv->resolving.pop_front();
        complete(srv, r, srv->base_s + 1e-3 * (double)ms);
    }
    int rc = wave_harvest(ctx, srv->runner, false);
    if (rc) return rc;
    if (srv->runner.overflow || srv->runner.error)
        return srv_fail(srv, RT_ERR_CUDA, "wave failed (overflow %d, traversal flags 0x%x)", srv->runner.overflow,
                        srv->runner.error);
    return RT_OK;
}

static int step_plain(rt_server *srv)
{
    rt_ctx *ctx = srv->ctx;
    if (srv->queue.empty()) return RT_OK;
    Request *r = srv->queue.front();
    srv->queue.pop_front();
    int rebuilt = 0;
    int rc = make_resident(srv, r->scene, &rebuilt);
    if (rc) {
        reject(srv, r, rc == RT_ERR_BUSY ? RT_ERR_BUDGET : rc);
        return RT_OK;
    }
    const int hs = 0;
    const std::pair<int, int> key(r->req.width, r->req.height);
    auto it = srv->plain_frames.find(key);
    if (it == srv->plain_frames.end()) {
        int fid = -1;
        rc = rt_frame_create(ctx, r->req.width, r->req.height, &fid);
        if (rc) return rc;
        srv->plain_frame_bytes += ctx->frames.at(fid)->bytes;
        it = srv->plain_frames.emplace(key, fid).first;
        note_peak(srv);
    }
    SrvScene &sc = srv->scenes[(size_t)r->scene];
    rt_camera cam = r->req.camera;
    cam.width = r->req.width, cam.height = r->req.height;
    rt_render_desc rd{r->req.width, r->req.height, srv->cfg.spp, srv->cfg.max_level, RT_MODE_RAYTRACE, 0, r->req.seed,
                      &cam};
    r->admit_s = srv->now();
    r->rebuilt = rebuilt;
    r->state = kInflight;
    rt_render_stats st{};
    const Tuning keep = ctx->plain_tuning;   // the render takes the server's tuning
    ctx->plain_tuning = srv->tuning;
    rc = rt_render(ctx, sc.ctx_id, it->second, &rd);
    ctx->plain_tuning = keep;
    if (!rc) rc = rt_render_wait(ctx, &st);
    if (rc) {
        reject(srv, r, rc);
        return RT_OK;
    }
    HostSlot &h = srv->hslots[(size_t)hs];
    rc = rt_frame_download(ctx, it->second, srv->cfg.keep_images ? h.rgb : nullptr, h.rgb8, nullptr, nullptr, nullptr);
    if (rc) return rc;
    srv->plain_rays += (unsigned long long)st.rays_primary + st.rays_secondary + st.rays_shadow;
    r->wj.total = (long long)rd.width * rd.height * rd.spp;
    h.used = true;
    r->host_slot = hs;
    complete(srv, r, srv->now());
    return RT_OK;
}

static int pending(const rt_server *srv)
{
    return (int)(srv->queue.size() + srv->inflight.size() + srv->deferred.size() + srv->resolving.size());
}

// nothing is admitted, traced or resolving: the head of a non-empty queue can never be admitted
static bool stuck(const rt_server *srv)
{
    return !srv->cfg.plain && srv->inflight.empty() && srv->deferred.empty() && srv->resolving.empty() &&
           !srv->queue.empty();
}

// resolve the requests the last wave finished; all_waves: no newer wave was enqueued, join every
// lane (else every lane but the newest wave's, which runs on while they resolve). The join is
// made in every step, requests or not, so the resolve stream has always waited for each wave but
// the newest: a request's earlier chunks may have run in any older wave.
static int resolve_deferred(rt_server *srv, bool all_waves)
{
    if (all_waves) wave_join(srv->runner, srv->rsv);
    else wave_join_all_but_last(srv->runner, srv->rsv);
    if (srv->deferred.empty()) return RT_OK;
    for (Request *r : srv->deferred) {
        int rc = finish(srv, r);
        if (rc) return rc;
    }
    srv->deferred.clear();
    return resolve_finished(srv);
}

static void wave_order(const rt_server *srv, std::vector<WaveJob *> &order)
{
    order.clear();
    for (Request *r : srv->inflight)
        if (r->wj.cursor < r->wj.total) order.push_back(&r->wj);
}

// retire, admit, enqueue one wave. With nothing left to enqueue, wait for the oldest frame in
// flight and admit again, so a step that returns with nothing in flight and a non-empty queue
// means the queue head cannot be admitted at all.
static int step_batched(rt_server *srv)
{
    rt_ctx *ctx = srv->ctx;
    srv->solo = false;
    int rc = retire(srv, false);
    if (rc) return rc;
    const bool idle = srv->inflight.empty() && srv->deferred.empty() && srv->resolving.empty();
    rc = admit(srv, idle);
    if (rc) return rc;
    std::vector<WaveJob *> order;
    wave_order(srv, order);
    srv->solo = idle && srv->runner.lanes.size() == 1 && !order.empty();
    if (order.empty()) {   // no wave to enqueue: the last wave's requests resolve now
        rc = resolve_deferred(srv, true);
        if (rc) return rc;
    }
    if (order.empty() && !srv->resolving.empty()) {
        rc = retire(srv, true);
        if (rc) return rc;
        rc = admit(srv, false);
        if (rc) return rc;
        wave_order(srv, order);
    }
    if (!srv->to_prepare.empty()) {   // the admitted frames, before their first wave
        rc = launch_frames(srv, srv->to_prepare, false);
        if (rc) return rc;
        if (!srv->solo) {
            CK(ctx, cudaEventRecord(srv->prep_ev, srv->prep));
            CK(ctx, cudaStreamWaitEvent(ctx->stream, srv->prep_ev, 0));
        }
    }
    if (!order.empty()) {
        long long got = 0;
        rc = wave_enqueue(ctx, srv->runner, order, srv->tuning, true, ctx->stream, &got);
        if (rc) return rc;
        // the previous wave's requests resolve behind the wave just enqueued
        rc = resolve_deferred(srv, false);
        if (rc) return rc;
        const bool one_lane = srv->runner.lanes.size() == 1;   // one stream: resolve right behind the wave
        if (one_lane && !srv->solo) {
            CK(ctx, cudaEventRecord(srv->wave_ev, ctx->stream));
            CK(ctx, cudaStreamWaitEvent(srv->rsv, srv->wave_ev, 0));
        }
        std::vector<Request *> still;
        for (Request *r : srv->inflight) {
            if (r->wj.cursor < r->wj.total) still.push_back(r);
            else if (!one_lane) srv->deferred.push_back(r);
            else {
                rc = finish(srv, r);
                if (rc) return rc;
            }
        }
        srv->inflight.swap(still);
        rc = resolve_finished(srv);
        if (rc) return rc;
        note_peak(srv);
    }
    return RT_OK;
}

static void reset_stats(rt_server *srv)
{
    srv->n_requests = srv->n_completed = srv->n_rejected = srv->evictions = srv->rebuilds = 0;
    srv->admitted_busy = srv->pixels = 0;
    srv->latencies_ms.clear();
    srv->first_arrival = -1.0;
    srv->last_done = 0.0;
    srv->plain_rays = 0;
    srv->runner.rays_primary = srv->runner.rays_secondary = srv->runner.rays_shadow = 0;
    srv->waves0 = srv->runner.waves;
    srv->wave_jobs0 = srv->runner.wave_jobs;
    srv->peak_bytes = used_bytes(srv);
    srv->runner.wave_ms.clear();
    srv->runner.wait_s = 0.0;
    srv->host_step_s = srv->host_wait_s = 0.0;
    srv->steps = 0;
}

static double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    size_t k = (size_t)std::ceil(p * (double)v.size());
    k = std::min(v.size(), std::max<size_t>(k, 1)) - 1;
    return v[k];
}

static void fill_stats(const rt_server *srv, rt_serve_stats *st)
{
    std::memset(st, 0, sizeof *st);
    st->requests = srv->n_requests;
    st->completed = srv->n_completed;
    st->rejected = srv->n_rejected;
    st->evictions = srv->evictions;
    st->rebuilds = srv->rebuilds;
    st->p50_ms = percentile(srv->latencies_ms, 0.50);
    st->p99_ms = percentile(srv->latencies_ms, 0.99);
    double sum = 0.0, mx = 0.0;
    for (double l : srv->latencies_ms) sum += l, mx = std::max(mx, l);
    st->mean_ms = srv->latencies_ms.empty() ? 0.0 : sum / (double)srv->latencies_ms.size();
    st->max_ms = mx;
    const unsigned long long rays = srv->cfg.plain ? srv->plain_rays
                                                   : srv->runner.rays_primary + srv->runner.rays_secondary +
                                                         srv->runner.rays_shadow;
    st->rays = (int64_t)rays;
    st->wall_s = srv->first_arrival >= 0 ? std::max(0.0, srv->last_done - srv->first_arrival) : 0.0;
    st->mrays_per_s = st->wall_s > 0 ? (double)rays / st->wall_s * 1e-6 : 0.0;
    st->peak_bytes = srv->peak_bytes;
    st->waves = srv->runner.waves - srv->waves0;
    st->mean_wave_requests = st->waves ? (double)(srv->runner.wave_jobs - srv->wave_jobs0) / (double)st->waves : 0.0;
    st->admitted_busy = srv->admitted_busy;
    st->pixels = srv->pixels;
    const std::vector<float> &w = srv->runner.wave_ms;
    std::vector<double> wd(w.begin(), w.end());
    double busy = 0.0;
    for (double x : wd) busy += x;
    st->wave_ms_mean = wd.empty() ? 0.0 : busy / (double)wd.size();
    st->wave_ms_p50 = percentile(wd, 0.50);
    st->wave_ms_p99 = percentile(wd, 0.99);
    st->device_busy_s = 1e-3 * busy;
    st->host_step_s = srv->host_step_s;
    st->host_wait_s = srv->host_wait_s + srv->runner.wait_s;
    st->steps = srv->steps;
}

// orbit camera about the world origin (Camera::lookAt with up = +y, 3DElement.cpp:364)
extern "C" int rt_orbit_camera(const rt_camera *base, double azimuth_deg, double elevation_deg, int32_t width,
                               int32_t height, rt_camera *out)
{
    if (!base || !out || width <= 0 || height <= 0) return RT_ERR_INVALID;
    const double pi = 3.14159265358979323846;
    const double r = std::sqrt((double)base->position[0] * base->position[0] +
                               (double)base->position[1] * base->position[1] +
                               (double)base->position[2] * base->position[2]);
    if (!(r > 0)) return RT_ERR_INVALID;
    const double az = azimuth_deg * pi / 180.0, el = elevation_deg * pi / 180.0;
    const double p[3] = {r * std::cos(el) * std::sin(az), r * std::sin(el), -r * std::cos(el) * std::cos(az)};
    auto norm = [](double *v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int k = 0; k < 3; ++k) v[k] /= l;
    };
    double n[3] = {-p[0], -p[1], -p[2]};
    norm(n);
    double u[3] = {-n[2], 0.0, n[0]};   // n x (0,1,0)
    norm(u);
    double v[3] = {u[1] * n[2] - u[2] * n[1], u[2] * n[0] - u[0] * n[2], u[0] * n[1] - u[1] * n[0]};
    norm(v);
    *out = *base;
    for (int k = 0; k < 3; ++k) {
        out->position[k] = (float)p[k];
        out->n[k] = (float)n[k];
        out->u[k] = (float)u[k];
        out->v[k] = (float)v[k];
    }
    out->width = width, out->height = height;
    return RT_OK;
}

extern "C" {

static int server_init(rt_server *srv)
{
    rt_ctx *ctx = srv->ctx;
    rt_server_config &c = srv->cfg;
    const int lanes = srv->tuning.lanes;
    if (c.max_inflight <= 0) c.max_inflight = 64;
    if (c.queue_rays <= 0) {   // 2^27 entries, halved until the wave queues take at most a third of the budget
        c.queue_rays = 1ll << 27;
        while (c.queue_rays > (1ll << 16) && lanes * kWsBytesPerEntry * c.queue_rays > c.hbm_budget_bytes / 3)
            c.queue_rays >>= 1;
    }
    if (c.max_pixels <= 0) c.max_pixels = 1920ll * 1080;
    if (c.stages <= 0) c.stages = 2 * lanes;
    if (c.spp < 1 || c.spp > 1024 || c.max_level < 0 || c.max_level > 4 || c.max_inflight > 4096 ||
        c.queue_rays > (1ll << 27) || c.queue_rays < (1ll << c.max_level) || c.max_pixels > (1ll << 26) ||
        c.stages > 8 || c.hbm_budget_bytes <= 0)
        return ctx_fail(ctx, RT_ERR_INVALID, "server config out of range");
    srv->t0 = Clock::now();
    CK(ctx, cudaSetDevice(ctx->device));
    CK(ctx, cudaStreamCreateWithFlags(&srv->copy, cudaStreamNonBlocking));
    CK(ctx, cudaStreamCreateWithFlags(&srv->prep, cudaStreamNonBlocking));
    CK(ctx, cudaStreamCreateWithFlags(&srv->rsv, cudaStreamNonBlocking));
    CK(ctx, cudaEventCreateWithFlags(&srv->prep_ev, cudaEventDisableTiming));
    CK(ctx, cudaEventCreateWithFlags(&srv->wave_ev, cudaEventDisableTiming));
    CK(ctx, cudaEventCreateWithFlags(&srv->solo_ev, cudaEventDisableTiming));
    const size_t P = (size_t)c.max_pixels;
    const int n_slots = c.plain ? 1 : c.max_inflight;
    srv->dslots.resize(c.plain ? 0 : (size_t)n_slots);
    for (size_t i = 0; i < srv->dslots.size(); ++i) srv->free_dslots.push_back((int)i);
    // a server that keeps no images hands out bytes only: its slots hold no float colour
    const bool keep = c.keep_images != 0;
    for (DevSlot &d : srv->dslots) {
        // accumulators, colour, bytes, and the camera axis table (at most 16384 + 16384 entries)
        size_t o_rgb = (24 * P + 255) & ~(size_t)255, o_rgb8 = o_rgb + (keep ? (12 * P + 255) & ~(size_t)255 : 0);
        size_t o_axis = o_rgb8 + ((3 * P + 255) & ~(size_t)255);
        CK(ctx, d.mem.ensure(o_axis + 4 * 32768));
        char *b = (char *)d.mem.p;
        d.fb.acc = (long long *)b;
        d.fb.rgb = keep ? (float *)(b + o_rgb) : nullptr;
        d.fb.rgb8 = (uint8_t *)(b + o_rgb8);
        d.fb.axis = (float *)(b + o_axis);
        srv->fixed_bytes += (int64_t)d.mem.bytes;
    }
    srv->hslots.resize((size_t)n_slots);
    for (HostSlot &h : srv->hslots) {
        CK(ctx, cudaHostAlloc(&h.mem, (keep ? 15 : 3) * P, cudaHostAllocDefault));
        h.rgb = keep ? (float *)h.mem : nullptr;
        h.rgb8 = (uint8_t *)h.mem + (keep ? 12 * P : 0);
    }
    if (!c.plain) {
        for (TableRing &T : srv->tables) {
            T.cap = c.max_inflight;
            for (int k = 0; k < TableRing::kSlots; ++k) {
                CK(ctx, cudaHostAlloc((void **)&T.host[k], sizeof(FrameJob) * (size_t)T.cap, cudaHostAllocDefault));
                CK(ctx, T.dev[k].ensure(sizeof(FrameJob) * (size_t)T.cap));
                srv->fixed_bytes += (int64_t)T.dev[k].bytes;
            }
        }
        int rc = wave_runner_init(ctx, srv->runner, c.queue_rays, c.max_inflight, c.stages, lanes);
        if (rc) return rc;
        srv->fixed_bytes += (int64_t)wave_runner_bytes(srv->runner);
    }
    if (srv->fixed_bytes > c.hbm_budget_bytes)
        return ctx_fail(ctx, RT_ERR_BUDGET, "frame slots and wave queues need %lld bytes, over the budget of %lld",
                        (long long)srv->fixed_bytes, (long long)c.hbm_budget_bytes);
    CK(ctx, cudaEventCreate(&srv->base_ev));
    CK(ctx, cudaEventRecord(srv->base_ev, ctx->stream));
    CK(ctx, cudaEventSynchronize(srv->base_ev));
    srv->base_s = srv->now();
    srv->peak_bytes = used_bytes(srv);
    return RT_OK;
}

int rt_server_create(rt_ctx *ctx, const rt_server_config *cfg, rt_server **out)
{
    if (!ctx || !cfg || !out) return RT_ERR_INVALID;
    *out = nullptr;
    rt_server *srv = new rt_server();
    srv->ctx = ctx;
    srv->cfg = *cfg;
    srv->tuning.lanes = 1;
    srv->tuning.pixel_tile = cfg->plain ? 0 : kWavePixelTile;
    int rc = server_init(srv);
    if (rc) {
        std::string msg = ctx->err;
        rt_server_destroy(srv);
        ctx->err = msg;
        return rc;
    }
    *out = srv;
    return RT_OK;
}

void rt_server_destroy(rt_server *srv)
{
    if (!srv) return;
    rt_ctx *ctx = srv->ctx;
    cudaStreamSynchronize(ctx->stream);
    for (cudaStream_t s : {srv->prep, srv->rsv, srv->copy})
        if (s) cudaStreamSynchronize(s);
    wave_harvest(ctx, srv->runner, true);
    for (SrvScene &s : srv->scenes) {
        if (s.ctx_id >= 0) rt_scene_release(ctx, s.ctx_id);
        rt_scene_host_free(s.host);
    }
    for (auto &kv : srv->plain_frames) rt_frame_release(ctx, kv.second);
    for (HostSlot &h : srv->hslots)
        if (h.mem) cudaFreeHost(h.mem);
    for (auto &kv : srv->reqs)
        if (kv.second->done_ev) cudaEventDestroy(kv.second->done_ev);
    for (cudaEvent_t e : srv->ev_pool) cudaEventDestroy(e);
    for (TableRing &T : srv->tables)
        for (int k = 0; k < TableRing::kSlots; ++k) {
            if (T.copied[k]) cudaEventDestroy(T.copied[k]);
            if (T.host[k]) cudaFreeHost(T.host[k]);
        }
    if (srv->base_ev) cudaEventDestroy(srv->base_ev);
    for (cudaEvent_t e : {srv->prep_ev, srv->wave_ev, srv->solo_ev})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {srv->prep, srv->rsv, srv->copy})
        if (s) cudaStreamDestroy(s);
    delete srv;
}

const char *rt_server_last_error(const rt_server *srv) { return srv ? srv->ctx->err.c_str() : "no server"; }

int rt_server_set_tuning(rt_server *srv, const rt_batch_tuning *tuning)
{
    if (!srv) return RT_ERR_INVALID;
    Tuning t;
    if (tuning) {
        int rc = tuning_from(srv->ctx, tuning, t);
        if (rc) return rc;
    }
    if (!tuning) t.pixel_tile = srv->cfg.plain ? 0 : kWavePixelTile;   // the server's defaults
    if (!tuning || !tuning->lanes) t.lanes = 1;
    srv->default_tile = !tuning;
    if (srv->cfg.plain) {   // its renders take the tuning one at a time; it has no wave lanes
        srv->tuning = t;
        return RT_OK;
    }
    WaveRunner &R = srv->runner;
    if ((size_t)t.lanes != R.lanes.size()) {   // new lanes of the same queue size, on an idle server
        if (pending(srv) > 0) return srv_fail(srv, RT_ERR_BUSY, "lanes change with requests pending");
        const int64_t lane_bytes = (int64_t)R.lanes[0].ws.mem.bytes;
        const int64_t grow = lane_bytes * ((int64_t)t.lanes - (int64_t)R.lanes.size());
        if (used_bytes(srv) + grow > srv->cfg.hbm_budget_bytes)
            return srv_fail(srv, RT_ERR_BUDGET, "%d lanes need %lld more bytes, over the budget", t.lanes,
                            (long long)grow);
        srv->fixed_bytes -= (int64_t)wave_runner_bytes(R);
        int rc = wave_runner_init(srv->ctx, R, R.lanes[0].ws.qcap, R.jobcap,
                                  std::max<int>(srv->cfg.stages, 2 * t.lanes), t.lanes);
        srv->fixed_bytes += (int64_t)wave_runner_bytes(R);
        if (rc) return rc;
        note_peak(srv);
    }
    srv->tuning = t;
    return RT_OK;
}

int rt_server_add_scene(rt_server *srv, const rt_scene_desc *desc, int32_t *scene)
{
    if (!srv || !desc || !scene) return RT_ERR_INVALID;
    rt_ctx *ctx = srv->ctx;
    int rc = validate_desc(ctx, desc);
    if (rc) return rc;
    SrvScene s;
    rc = rt_scene_host_from_desc(desc, srv->cfg.spp, srv->cfg.max_level, 0, &s.host);
    if (rc) return srv_fail(srv, rc, "scene copy failed");
    rt_scene_host_pin(s.host);   // faster rebuilds; a failure only costs speed
    s.camera = desc->camera;
    // upload once to learn its size, then keep it if the budget allows
    int id = -1;
    rc = rt_scene_upload(ctx, rt_scene_host_desc(s.host), &id);
    if (rc) {
        rt_scene_host_free(s.host);
        return rc;
    }
    const SceneDev &sd = *ctx->scenes.at(id);
    s.bytes = sd.bytes;
    s.scratch = (int64_t)lbvh_scratch_bytes(sd.n_leaves);
    s.ctx_id = id;
    s.last_use = ++srv->tick;
    if (srv->fixed_bytes + s.bytes + s.scratch > srv->cfg.hbm_budget_bytes) {
        rt_scene_release(ctx, id);
        rt_scene_host_free(s.host);
        return srv_fail(srv, RT_ERR_BUDGET, "scene needs %lld bytes, over the budget", (long long)s.bytes);
    }
    srv->scenes.push_back(s);
    // over the budget: evict idle scenes, oldest first (the new one last)
    while (used_bytes(srv) > srv->cfg.hbm_budget_bytes) {
        if (spare_bytes(ctx) > 0) {
            spare_trim(ctx);
            continue;
        }
        SrvScene *victim = nullptr;
        for (SrvScene &o : srv->scenes)
            if (o.ctx_id >= 0 && o.users == 0 && (!victim || o.last_use < victim->last_use)) victim = &o;
        if (!victim) break;
        evict(srv, *victim);
        srv->evictions--;   // registration is not a serving eviction
    }
    note_peak(srv);
    *scene = (int32_t)srv->scenes.size() - 1;
    return RT_OK;
}

int rt_server_submit(rt_server *srv, const rt_request *req, int64_t *request_id)
{
    if (!srv || !req || !request_id) return RT_ERR_INVALID;
    if (req->scene < 0 || req->scene >= (int)srv->scenes.size())
        return srv_fail(srv, RT_ERR_NOT_FOUND, "unknown scene %d", req->scene);
    if (req->width <= 0 || req->height <= 0 || (int64_t)req->width * req->height > srv->cfg.max_pixels ||
        req->width > 16384 || req->height > 16384)
        return srv_fail(srv, RT_ERR_INVALID, "request of %dx%d outside the frame slots (%lld pixels)", req->width,
                        req->height, (long long)srv->cfg.max_pixels);
    std::unique_ptr<Request> r(new Request());
    r->id = srv->next_id++;
    r->req = *req;
    r->scene = req->scene;
    r->arrival_s = req->arrival_s >= 0 ? req->arrival_s : srv->now();
    if (srv->first_arrival < 0 || r->arrival_s < srv->first_arrival) srv->first_arrival = r->arrival_s;
    srv->queue.push_back(r.get());
    *request_id = r->id;
    srv->reqs[r->id] = std::move(r);
    srv->n_requests++;
    return RT_OK;
}

int rt_server_step(rt_server *srv, int32_t *n_pending)
{
    if (!srv) return RT_ERR_INVALID;
    const auto t0 = Clock::now();
    int rc = srv->cfg.plain ? step_plain(srv) : step_batched(srv);
    srv->host_step_s += std::chrono::duration<double>(Clock::now() - t0).count();
    srv->steps++;
    if (n_pending) *n_pending = pending(srv);
    return rc;
}

int rt_server_drain(rt_server *srv)
{
    if (!srv) return RT_ERR_INVALID;
    for (;;) {
        int32_t n = 0;
        int rc = rt_server_step(srv, &n);
        if (rc) return rc;
        if (n == 0) break;
        if (stuck(srv)) {
            // nothing runs and the head request cannot be admitted: it never will be
            return srv_fail(srv, RT_ERR_BUSY, "queued requests cannot be admitted (result slots full?)");
        }
    }
    return srv->cfg.plain ? RT_OK : wave_harvest(srv->ctx, srv->runner, true);
}

int rt_server_result(rt_server *srv, int64_t request_id, rt_request_result *res, float *rgb, uint8_t *rgb8)
{
    if (!srv || !res) return RT_ERR_INVALID;
    auto it = srv->reqs.find(request_id);
    if (it == srv->reqs.end()) return srv_fail(srv, RT_ERR_NOT_FOUND, "unknown request %lld", (long long)request_id);
    Request *r = it->second.get();
    if (r->state != kDone) return RT_ERR_BUSY;
    std::memset(res, 0, sizeof *res);
    res->request = r->id;
    res->status = r->status;
    res->width = r->req.width, res->height = r->req.height;
    res->scene = r->scene;
    res->arrival_s = r->arrival_s, res->admit_s = r->admit_s, res->done_s = r->done_s;
    res->samples = r->status == RT_OK ? r->wj.total : 0;
    res->rebuilt = r->rebuilt;
    if ((rgb || rgb8) && r->status == RT_OK) {
        if (r->rgb.empty()) {
            srv->reqs.erase(it);
            return srv_fail(srv, RT_ERR_NOT_FOUND, "the image was not kept (keep_images = 0)");
        }
        if (rgb) std::memcpy(rgb, r->rgb.data(), sizeof(float) * r->rgb.size());
        if (rgb8) std::memcpy(rgb8, r->rgb8.data(), r->rgb8.size());
    }
    srv->reqs.erase(it);
    return RT_OK;
}

int rt_server_resident(rt_server *srv, int32_t scene, int32_t *resident)
{
    if (!srv || !resident) return RT_ERR_INVALID;
    if (scene < 0 || scene >= (int)srv->scenes.size()) return srv_fail(srv, RT_ERR_NOT_FOUND, "unknown scene %d", scene);
    *resident = srv->scenes[(size_t)scene].ctx_id >= 0;
    return RT_OK;
}

double rt_server_now(rt_server *srv) { return srv ? srv->now() : 0.0; }

int rt_server_stats(rt_server *srv, rt_serve_stats *stats)
{
    if (!srv || !stats) return RT_ERR_INVALID;
    fill_stats(srv, stats);
    return RT_OK;
}

int rt_server_latencies(rt_server *srv, double *ms, int64_t cap, int64_t *n)
{
    if (!srv || !n || cap < 0 || (cap && !ms)) return RT_ERR_INVALID;
    *n = (int64_t)srv->latencies_ms.size();
    const size_t k = std::min(srv->latencies_ms.size(), (size_t)cap);
    if (k) std::memcpy(ms, srv->latencies_ms.data(), k * sizeof(double));
    return RT_OK;
}

int rt_server_wave_ms(rt_server *srv, float *ms, int64_t cap, int64_t *n)
{
    if (!srv || !n || cap < 0 || (cap && !ms)) return RT_ERR_INVALID;
    const std::vector<float> &w = srv->runner.wave_ms;
    *n = (int64_t)w.size();
    const size_t k = std::min(w.size(), (size_t)cap);
    if (k) std::memcpy(ms, w.data(), k * sizeof(float));
    return RT_OK;
}

int rt_server_run_poisson(rt_server *srv, double lambda, double duration, uint64_t seed, rt_serve_stats *stats)
{
    if (!srv || !stats || !(lambda > 0) || !(duration > 0) || srv->scenes.empty()) return RT_ERR_INVALID;
    int rc = rt_server_drain(srv);
    if (rc) return rc;
    // forget earlier requests' records so this run's latencies stand alone
    for (auto it = srv->reqs.begin(); it != srv->reqs.end();) {
        if (it->second->state == kDone && it->second->rgb.empty()) it = srv->reqs.erase(it);
        else ++it;
    }
    reset_stats(srv);
    const int keep = srv->cfg.keep_images;
    srv->cfg.keep_images = 0;   // the run keeps latencies, not images
    struct KeepRestore {
        rt_server *s;
        int k;
        ~KeepRestore() { s->cfg.keep_images = k; }
    } restore{srv, keep};
    struct Arrival {
        double t;
        rt_request req;
    };
    std::vector<Arrival> arr;
    SplitMix rng{seed};
    for (double t = 0.0;;) {
        t += -std::log(1.0 - rng.u01()) / lambda;
        if (t >= duration) break;
        Arrival a;
        a.t = t;
        std::memset(&a.req, 0, sizeof a.req);
        a.req.scene = std::min((int)srv->scenes.size() - 1, (int)(rng.u01() * (double)srv->scenes.size()));
        const double az = 360.0 * rng.u01(), el = 10.0 + 50.0 * rng.u01();
        const int res = std::min(3, (int)(rng.u01() * 4.0));
        a.req.width = kServeRes[res][0], a.req.height = kServeRes[res][1];
        rt_orbit_camera(&srv->scenes[(size_t)a.req.scene].camera, az, el, a.req.width, a.req.height, &a.req.camera);
        a.req.seed = rng.next();
        arr.push_back(a);
    }
    const double start = srv->now();
    srv->first_arrival = start;
    std::vector<int64_t> ids;
    ids.reserve(arr.size());
    size_t k = 0;
    while (k < arr.size() || pending(srv) > 0) {
        const double t = srv->now() - start;
        while (k < arr.size() && arr[k].t <= t) {
            arr[k].req.arrival_s = start + arr[k].t;
            int64_t id = 0;
            rc = rt_server_submit(srv, &arr[k].req, &id);
            if (rc) return rc;
            ids.push_back(id);
            ++k;
        }
        if (pending(srv) > 0) {
            int32_t n = 0;
            rc = rt_server_step(srv, &n);
            if (rc) return rc;
            if (stuck(srv))
                return srv_fail(srv, RT_ERR_BUSY, "queued requests cannot be admitted (result slots full?)");
        } else if (k < arr.size()) {
            const double wait = arr[k].t - (srv->now() - start);
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.002)));
        }
    }
    if (!srv->cfg.plain) {
        rc = wave_harvest(srv->ctx, srv->runner, true);
        if (rc) return rc;
    }
    fill_stats(srv, stats);
    if (!srv->cfg.keep_images)
        for (int64_t id : ids) srv->reqs.erase(id);
    return RT_OK;
}

} // extern "C"
