// rt_capi_internal.h — host-side objects behind the C ABI handles.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_kernels.cuh"
#include "rt_lbvh.cuh"

// one device allocation that only grows
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr, o.bytes = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p, bytes = o.bytes;
            o.p = nullptr, o.bytes = 0;
        }
        return *this;
    }
    ~DevBuf();
    void release();
    cudaError_t ensure(size_t need);
};

struct SceneDev {
    DevBuf mem;                  // tables, triangle inputs, LBVH
    rtg::DevScene hdr{};         // header with device pointers (host copy)
    rtg::DevScene *d_hdr = nullptr;
    rtg::LbvhInput in{};
    rtg::LbvhOutput out{};
    rt_camera camera{};
    int n_tris = 0;
    int n_leaves = 0;   // triangles + spheres in the LBVH
    int branching = 0;  // most child rays one hit can spawn: (reflect > 0.01) + (refract > 0.01)
    int64_t bytes = 0;
    float build_ms = 0.0f;
};

struct FrameDev {
    DevBuf mem;
    rtg::FrameBufs fb{};
    int w = 0, h = 0;
    int64_t bytes = 0;
};

// ray queues, shadow queue, hit buffers, counters and job tables of one wavefront
struct Workspace {
    DevBuf mem;
    rtg::Wavefront wf{};
    rtg::DevJob *jobs = nullptr;
    long long *job_end = nullptr;
    long long *scalars = nullptr;   // [0] samples in the wave, [1] first sample, [2] jobs
    rtg::DevScene *scenes = nullptr;
    long long qcap = 0;
    int jobcap = 0;
    // layout generation: bumped whenever the arrays move. A reallocation can return the old
    // address, so graphs captured against the workspace are keyed on this, not on mem.p.
    unsigned long long gen = 0;
};

struct Pending {
    int scene = -1, frame = -1;
    rt_render_desc rd{};
    bool active = false;
    int retries = 0;
};

// CUDA events around each kernel launch of a render (RT_FLAG_PROFILE)
struct KernelProfiler {
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    size_t used = 0;
    bool on = false;
    int launches[RT_KERNEL_KINDS] = {0};
    void reset(bool enable)
    {
        on = enable;
        used = 0;
        marks.clear();
        for (int &l : launches) l = 0;
    }
    cudaEvent_t next()
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    // bracket one launch of `kind` (call begin before and end after it)
    void begin(int kind, cudaStream_t s)
    {
        launches[kind]++;
        if (!on) return;
        cudaEvent_t a = next();
        cudaEventRecord(a, s);
        marks.push_back({kind, {a, nullptr}});
    }
    void end(cudaStream_t s)
    {
        if (!on || marks.empty()) return;
        cudaEvent_t b = next();
        cudaEventRecord(b, s);
        marks.back().second.second = b;
    }
    void collect(float *ms) const
    {
        for (int k = 0; k < RT_KERNEL_KINDS; ++k) ms[k] = 0.0f;
        for (auto &m : marks) {
            float t = 0.0f;
            if (m.second.second && cudaEventElapsedTime(&t, m.second.first, m.second.second) == cudaSuccess) ms[m.first] += t;
        }
    }
    ~KernelProfiler()
    {
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    ~GraphEntry()
    {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// one job of a wave-run batch (a frame, or a served request): samples [cursor, total) remain
struct WaveJob {
    rtg::DevJob job{};            // job.scene is set per wave (index into that wave's scene table)
    const SceneDev *scene = nullptr;
    long long total = 0;
    long long cursor = 0;
    long long weight = 1;         // queue entries one sample can need at its busiest bounce
};

// pinned host staging of one wave in flight: its tables go up, its counters come back
struct WaveStage {
    rtg::DevJob *jobs = nullptr;
    long long *end = nullptr;
    rtg::DevScene *scenes = nullptr;
    long long *scalars = nullptr;
    rtg::Counters *counters = nullptr;
    cudaEvent_t start = nullptr;         // recorded before the wave's table copies
    cudaEvent_t done = nullptr;
    int lane = 0;
    bool busy = false;
    int n_jobs = 0;
    long long samples = 0;
};

// One wave lane: a workspace, the graphs captured against it and, when the runner has more than
// one lane, a stream of its own. Waves go to the lanes in turn, so a wave's kernels can take the
// SMs the previous wave's kernels leave idle while they drain (every wavefront kernel ends with
// warps out of work waiting for the slowest tile).
struct WaveLane {
    Workspace ws;
    std::map<long long, std::unique_ptr<GraphEntry>> graphs;
    cudaStream_t stream = nullptr;       // own stream of a multi-lane runner (NULL: the caller's)
    cudaEvent_t last = nullptr;          // after the lane's last wave
    bool pending = false;                // a wave was enqueued since the caller's stream joined it
};

// waves of chunks traced through the lanes' workspaces: the per-bounce sequence is a CUDA graph
// replayed per wave, tables are staged through a ring of pinned buffers so the host can run
// ahead of the device by `stages` waves, and the queue never overflows because each wave's
// chunks are sized against the capacity with every sample's branching bound
struct WaveRunner {
    std::vector<WaveLane> lanes;         // at least one after wave_runner_init
    size_t next_lane = 0;
    cudaEvent_t go = nullptr;            // the caller's stream before a wave on a lane's own stream
    std::vector<WaveStage> stages;
    size_t next = 0;
    int jobcap = 0;
    // totals of harvested waves
    unsigned long long rays_primary = 0, rays_secondary = 0, rays_shadow = 0;
    int overflow = 0, error = 0;
    long long waves = 0, wave_jobs = 0;
    std::vector<float> wave_ms;          // device time of each harvested wave (start to done)
    double wait_s = 0.0;                 // host time blocked on waves (a full staging ring, a drain)
    // frame table of a batch (pinned host copy, device copy): prepared and resolved in one
    // launch each
    rtg::FrameJob *ftab_host = nullptr;
    DevBuf ftab_dev;
    int ftab_cap = 0;
    cudaEvent_t ftab_copied = nullptr;   // the last copy out of ftab_host has run
    WaveRunner() = default;
    WaveRunner(const WaveRunner &) = delete;
    WaveRunner &operator=(const WaveRunner &) = delete;
    ~WaveRunner();
};

long long wave_weight(int branching, int max_level);
// lanes: 1, or 2 (each with its own workspace of qcap entries and its own stream)
int wave_runner_init(rt_ctx *ctx, WaveRunner &R, long long qcap, int jobcap, int stages, int lanes = 1);
// plan and enqueue the next wave from `jobs` (taken in order) after the work already on stream s
// (on the next lane's stream, or on s itself with one lane); waits only when the staging ring is
// full. Sets *samples to the samples enqueued (0 = nothing left to trace).
int wave_enqueue(rt_ctx *ctx, WaveRunner &R, const std::vector<WaveJob *> &jobs, const rtg::Tuning &t, bool use_graph,
                 cudaStream_t s, long long *samples, KernelProfiler *prof = nullptr);
// make stream s wait for every wave enqueued so far (work on s that reads the waves' frames)
void wave_join(WaveRunner &R, cudaStream_t s);
// make stream s wait for every wave enqueued so far but the last one: the frames finished by the
// previous wave can be resolved on s while the last wave runs on its own lane
void wave_join_all_but_last(WaveRunner &R, cudaStream_t s);
// harvest every finished wave (wait = block until all enqueued waves are done)
int wave_harvest(rt_ctx *ctx, WaveRunner &R, bool wait);
size_t wave_runner_bytes(const WaveRunner &R);

constexpr size_t kPlainStageBytes = 4096;
// primary-ray pixel tile of the wave paths (batch, batched server) when no tuning says otherwise
constexpr int kWavePixelTile = 8;
// workspace bytes per ray-queue entry: two ray queues (64 B each), the shadow queue (80 B) and
// the hit queue (84 B)
constexpr long long kWsBytesPerEntry = 292;

struct rt_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::string err;
    std::map<int, std::unique_ptr<SceneDev>> scenes;
    std::map<int, std::unique_ptr<FrameDev>> frames;
    int next_scene = 0, next_frame = 0;
    Workspace ws;
    DevBuf lbvh_scratch;
    DevBuf stamps;                       // warp time stamps of a profiled render (kStampBytes)
    bool stamped = false;                // the last render wrote them
    // Cancel: rt_cancel counts its calls; a render (or rt_render_host_since call) is cancelled
    // once the count passes the mark it began from. The mutex orders rt_cancel's write of the
    // device flag against the clear a new render makes, so no cancel made after a render's mark
    // is wiped out by that render's clear.
    std::mutex cancel_mu;
    std::atomic<unsigned long long> cancel_count{0};   // rt_cancel calls so far
    unsigned long long cancel_base = 0;  // mark of the current render
    int *cancel_dev = nullptr;           // device copy the kernels read (written on `side`)
    int *cancel_vals = nullptr;          // page-locked {0, 1}: sources of those writes
    cudaStream_t side = nullptr;         // cancel writes, ordered apart from the render stream
    cudaEvent_t ev_armed = nullptr;      // the last clear of the device flag
    rtg::Counters *counters_host = nullptr;
    long long h_scalars[4] = {0, 0, 0, 0};
    long long h_job_end[1] = {0};
    Pending pending;
    rtg::Tuning plain_tuning;
    KernelProfiler prof;
    std::unique_ptr<WaveRunner> batch;   // workspace + graphs of rt_batch_render
    std::map<long long, std::unique_ptr<GraphEntry>> plain_graphs;   // level loops of rt_render
    unsigned long long plain_graph_gen = 0;   // workspace layout the plain graphs point into (0 = none)
    void *plain_stage = nullptr;         // page-locked staging of the plain job tables
    cudaEvent_t ev_staged = nullptr;     // the last staging copy
    std::vector<DevBuf> spare;           // released scene / frame buffers kept for reuse
    void *upload_stage = nullptr;        // page-locked staging of a scene upload's small tables
    size_t upload_stage_bytes = 0;
    cudaEvent_t ev_upload = nullptr;     // the last upload's staging copy
    cudaStream_t upload_side = nullptr;  // copies of the triangle shading data, beside the build
    int build_mode = RT_BUILD_RADIX;     // hierarchy of the next builds (rt_ctx_set_build)
    long long test_queue = 0;            // rt_ctx_test_queue_entries: first-attempt queue size (0 = default)
    cudaEvent_t ev_upload_go = nullptr;  // the render stream's work before an upload
    cudaEvent_t ev_shading = nullptr;    // the shading data of the last upload has arrived
    int *build_flag = nullptr;           // page-locked: the LBVH build's material check
};

int ctx_fail(rt_ctx *ctx, int code, const char *fmt, ...);
// begin a render cancelled by any rt_cancel counted after `mark`: clear the device flag for the
// kernels about to be enqueued on the context stream, or return RT_ERR_CANCELLED (flag left set)
// when such a cancel has already come
int cancel_arm(rt_ctx *ctx, unsigned long long mark);
// a cancel has come since the current render's mark
inline bool cancel_requested(const rt_ctx *ctx) { return ctx->cancel_count.load() != ctx->cancel_base; }
// released scene / frame buffers the context keeps for reuse: their bytes, and freeing them
size_t spare_bytes(const rt_ctx *ctx);
void spare_trim(rt_ctx *ctx);
#define CK(ctx, call)                                                                                             \
    do {                                                                                                          \
        cudaError_t e_ = (call);                                                                                  \
        if (e_ != cudaSuccess)                                                                                    \
            return ctx_fail(ctx, e_ == cudaErrorMemoryAllocation ? RT_ERR_OOM : RT_ERR_CUDA, "%s: %s (%s:%d)",       \
                            #call, cudaGetErrorString(e_), __FILE__, __LINE__);                                  \
    } while (0)

int validate_desc(rt_ctx *ctx, const rt_scene_desc *d);
int frame_alloc(rt_ctx *ctx, int32_t w, int32_t h, FrameDev &f);
int ws_ensure(rt_ctx *ctx, Workspace &ws, long long qcap, int njobs);
int make_job(rt_ctx *ctx, const SceneDev &sc, FrameDev &f, const rt_render_desc *rd, int scene_slot, rtg::DevJob &J,
             long long &samples);
// the preparation / resolve record of a frame rendered by job J (w x h pixels)
rtg::FrameJob frame_job(const rtg::FrameBufs &fb, int w, int h, const rtg::DevJob &J);
int tuning_from(rt_ctx *ctx, const rt_batch_tuning *in, rtg::Tuning &t);
// key of a captured level loop (max_level and every tuning value its launches depend on)
long long tuning_key(int max_level, const rtg::Tuning &t);
// (extend, shade, shadow) per level, the first extend making the primary rays; `prof` (may be
// NULL) brackets every launch
void enqueue_levels(rt_ctx *ctx, Workspace &ws, int max_level, const rtg::Tuning &t, cudaStream_t s,
                    KernelProfiler *prof);
