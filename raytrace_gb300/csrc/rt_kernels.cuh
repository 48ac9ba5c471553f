// rt_kernels.cuh — launch interface of the wavefront kernels (rt_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "rt_device.cuh"

namespace rtg {

// per-frame device buffers
struct FrameBufs {
    long long *acc;     // 3 x int64 fixed point (2^-32) per pixel
    float *rgb;         // 3 floats per pixel
    uint8_t *rgb8;      // 3 bytes per pixel
    int *plane_obj;     // primary hit object, sample 0
    int *plane_prim;
    float *plane_t;
    float *axis;        // camera offsets of a 1-sample render: (float)((double)xcur * dp) for the
                        // W columns, then (float)((double)ycur * dp) for the H rows
};

// one frame of a batch, for the batch-wide prepare and resolve launches. Pixels are counted in
// groups of four (quads); the frame's quads are [quad_end of the previous frame, quad_end). The
// resolve gives each quad a thread, the preparation six, one per 16 B of its 96 B of accumulators.
struct FrameJob {
    FrameBufs fb;
    long long npix;
    long long quad_end;             // inclusive prefix of quads over the batch's frames
    unsigned long long scale_bits;  // resolve scale 2^-32 / spp as double bits
    unsigned long long dp_bits;     // camera dp as double bits: fill fb.axis (0 = no table)
    int w, h;
    int planes;                     // reset the hit planes
    int pad;
};

// everything one wavefront pass needs
struct Wavefront {
    const DevScene *scenes;
    const DevJob *jobs;
    const long long *job_sample_end;  // inclusive prefix of samples per job (device)
    const long long *total_samples;   // device scalar: samples in this wave
    const long long *sample_offset;   // device scalar: global index of the wave's first sample
    const long long *n_jobs;          // device scalar: jobs in the job table
    const long long *max_lights;      // device scalar: most lights of any scene in the wave
    RayQueue q[2];
    ShadowQueue sq;
    HitQueue hq;                      // the rays that hit, densely, per bounce (C->h_count)
    Counters *C;
    int *shares;                      // per work slot, kMaxShares counters of the SM-share mode
    unsigned long long *stamps;       // RT_FLAG_PROFILE: per work slot and warp, (~start, end) in
                                      // globaltimer ns, combined with atomicMax (NULL = not kept)
    const volatile int *cancel;       // device cancel flag (NULL = not cancellable)
};

// warp time stamps of a profiled render: 16 work slots x kMaxStampWarps warps x 2
constexpr int kMaxStampWarps = 16384;
constexpr size_t kStampBytes = 16ull * kMaxStampWarps * 2 * sizeof(unsigned long long);

// SM-share work counters: 16 work slots (as Counters::work) x kMaxShares shares, right after the
// Counters in the workspace and zeroed with them
constexpr int kMaxShares = 512;
constexpr size_t kCounterBlockBytes = ((sizeof(Counters) + 255) / 256) * 256 + 16 * kMaxShares * sizeof(int);

struct Tuning {
    int block = 128;     // threads per block of the traversal kernels
    int tile = 32;       // rays per dynamic work fetch (multiple of 32)
    int stack = 0;       // traversal stack entries kept in shared memory per thread: 0 or 8
                         // (the rest of the kStack entries in local memory)
    bool dynamic = true; // persistent grid pulling tiles from a global counter
    bool shares = false; // with dynamic: each SM first drains its own share of the rays
    bool count = false;  // count BVH nodes / triangles / spheres
    int grid = 0;        // blocks (0 = derived from the SM count)
    int min_blocks = 8;  // 0, 6 or 8: register cap of the traversal kernels (128-thread blocks)
    int shadow_chunk = 4096;   // shadow work in light-major chunks of this many hits (0 = one chunk)
    int pixel_tile = 0;     // primary rays in square pixel tiles of this edge (0 = row by row)
    int lanes = 2;          // batch: waves in turn on this many workspaces and streams (1 or 2)
};

int sm_count();
// kernels of one level; `sel` picks the input ray queue
// gen: the first extend of a wave, which makes the wave's primary rays itself
void launch_extend(const Wavefront &wf, int sel, int level, bool gen, const Tuning &t, cudaStream_t s);
void launch_shade(const Wavefront &wf, int sel, int level, const Tuning &t, cudaStream_t s);
void launch_shadow(const Wavefront &wf, int level, const Tuning &t, cudaStream_t s);
void launch_resolve(const FrameBufs &fb, int width, int height, int spp, cudaStream_t s);
// zero the accumulators, reset the hit planes and fill the camera axis table (as each FrameJob
// asks) / resolve the colours: n frames in one launch each
void launch_frames_prepare(const FrameJob *jobs, int n, long long quads, cudaStream_t s);
// the same preparation for one frame
void launch_frame_prepare(const FrameJob &job, cudaStream_t s);
void launch_frames_resolve(const FrameJob *jobs, int n, long long quads, cudaStream_t s);
// the resolve scale of spp samples per pixel, as double bits
unsigned long long resolve_scale_bits(int spp);
// the integer-exact conversions of the kernels, on n inputs (a test hook)
void launch_selftest_conversions(const long long *x, int n, unsigned long long d_bits, const float *v, float *out_mul,
                                 long long *out_fix, cudaStream_t s);

} // namespace rtg
