/*
 * rt_gb300.h — C ABI of the GB300 renderer for the RayTracer per-pixel loop.
 *
 * This is the drop-in boundary. The C++ classes Scene / RayTracer / Sphere / Plane /
 * Box / BallPlane / Model (raytrace_gb300/cpp/) flatten a scene into an rt_scene_desc and
 * call these functions; so can any C, ctypes or FFI caller. All calls return RT_OK (0) or a
 * negative RT_ERR_* code and never throw. rt_last_error() gives a message for the last
 * failing call on a context.
 *
 * Reference interfaces replaced (paths within the XZiar/RayTrace project):
 *   - RayTracer::start / stop / isFinish / useTime / output   RayTracer.h:44-56, RayTracer.cpp:614-701
 *   - DrawObject::RTPrepare (Model octant lists)              3DElement.h:200, Model.cpp:402-480
 *   - the per-pixel loop parallelRT + RTfrac recursion        RayTracer.cpp:5-45, 450-596
 *   - Sphere / Plane / Box / BallPlane / Model ::intersect    Basic3DObject.cpp:135-551, Model.cpp:748-811
 * Units and conventions follow the reference: the camera looks along n with u to the right
 * and v up, pixel (col,row) maps to xcur = col - W/2, ycur = row - H/2, and output row 0 is
 * the bottom row (RayTracer.cpp:20-27).
 */
#ifndef RT_GB300_H
#define RT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RT_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------------------- */
#define RT_OK               0
#define RT_ERR_INVALID     -1   /* bad argument, size or id                        */
#define RT_ERR_CUDA        -2   /* CUDA runtime error or no usable GPU             */
#define RT_ERR_OOM         -3   /* device allocation failed                        */
#define RT_ERR_CANCELLED   -4   /* rt_cancel() ended the render                    */
#define RT_ERR_OVERFLOW    -5   /* a ray queue overflowed (render is retried)      */
#define RT_ERR_TIMEOUT     -6   /* a bounded device wait gave up                   */
#define RT_ERR_BUDGET      -7   /* the serving HBM budget cannot admit the request */
#define RT_ERR_NOT_FOUND   -8   /* unknown scene / frame / request id              */
#define RT_ERR_BUSY        -9   /* the object is in use by an unfinished render    */
#define RT_ERR_TOO_LARGE  -10   /* the request exceeds a fixed capacity            */

/* ---- scene vocabulary (values match the reference's macros) --------------------- */
#define RT_OBJECT_SPHERE     0x1   /* MY_OBJECT_SPHERE     3DElement.h:4  */
#define RT_OBJECT_CUBE       0x2   /* MY_OBJECT_CUBE       3DElement.h:5  */
#define RT_OBJECT_MODEL      0x3   /* MY_OBJECT_MODEL      3DElement.h:6  */
#define RT_OBJECT_PLANE      0x4   /* MY_OBJECT_PLANE      3DElement.h:7  */
#define RT_OBJECT_BALLPLANE  0x5   /* MY_OBJECT_BALLPLANE  3DElement.h:8  */

#define RT_LIGHT_PARALLEL    0x1   /* MY_LIGHT_PARALLEL    3DElement.h:13 */
#define RT_LIGHT_POINT       0x2   /* MY_LIGHT_POINT       3DElement.h:14 */
#define RT_LIGHT_SPOT        0x3   /* MY_LIGHT_SPOT (shaded as parallel, RayTracer.cpp:482-503) */

/* render modes = the reference's start() types (RayTracer.h:5-13) */
#define RT_MODE_CHECK        0x1
#define RT_MODE_DEPTH        0x2
#define RT_MODE_NORMAL       0x3
#define RT_MODE_TEXTURE      0x4
#define RT_MODE_MATERIAL     0x5
#define RT_MODE_SHADOW       0x6
#define RT_MODE_REFLECT      0x7
#define RT_MODE_REFRACT      0x8
#define RT_MODE_RAYTRACE     0x80

/* render flags */
#define RT_FLAG_REF_TILES    0x1   /* render only the 64x64-tile region the reference covers
                                      (W and H floored to multiples of 64, RayTracer.cpp:13) */
#define RT_FLAG_HIT_PLANES   0x2   /* also write per-pixel primary hit id / distance planes   */
#define RT_FLAG_COUNT_WORK   0x4   /* count BVH nodes visited and primitives tested (slower)  */
#define RT_FLAG_PROFILE      0x8   /* time every kernel with CUDA events (rt_render_stats.kernel_ms) */

/* kernel kinds of rt_render_stats.kernel_ms / kernel_launches */
#define RT_KERNEL_RAYGEN     0
#define RT_KERNEL_EXTEND     1
#define RT_KERNEL_SHADE      2
#define RT_KERNEL_SHADOW     3
#define RT_KERNEL_RESOLVE    4
#define RT_KERNEL_OTHER      5
#define RT_KERNEL_KINDS      6

typedef struct rt_camera {
    float position[3];
    float u[3], v[3], n[3];      /* right, up, toward (Camera, 3DElement.h:225-237) */
    int32_t width, height;
    float fovy;                  /* degrees */
    float znear, zfar;
} rt_camera;

typedef struct rt_light {
    int32_t type;                /* RT_LIGHT_* */
    int32_t on;                  /* Light::bLight */
    float position[3];
    float ambient[3], diffuse[3], specular[3];
    float attenuation[3];        /* constant, linear, quadratic */
} rt_light;

typedef struct rt_material {
    float ambient[3], diffuse[3], specular[3];
    float shininess, reflect, refract, rfr;
    int32_t texture;             /* index into rt_scene_desc.textures, -1 = none */
} rt_material;

typedef struct rt_texture {
    int32_t w, h;
    const uint8_t *bgr;          /* w*h*3 bytes, B,G,R per texel, row y at offset (y*w+x)*3 */
} rt_texture;

typedef struct rt_object {
    int32_t type;                /* RT_OBJECT_* */
    int32_t show;                /* DrawObject::bShow; hidden objects are skipped */
    int32_t material;            /* sphere/cube/plane/ballplane material index */
    int32_t texture;             /* plane texture index, -1 = none */
    float position[3];
    float radius;                /* sphere, ballplane */
    float normal[3];             /* plane, ballplane frame (Plane::rotate, Basic3DObject.cpp:312-330) */
    float axisx[3], axisy[3];
    float bmin[3], bmax[3];      /* cube: min/max relative to position; model: VerMin/VerMax */
    int64_t tri_first;           /* model: first triangle in the scene triangle arrays */
    int64_t tri_count;           /* model: number of triangles */
} rt_object;

/*
 * A scene in flat form. Triangles of every Model are concatenated; triangle i has its three
 * points at tri_p[9i..9i+8] (model space, before the object's position is added), vertex
 * normals at tri_n[9i..], texture coordinates at tri_uv[6i..] (NULL = all zero) and material
 * tri_mtl[i] (the part material). tri_id[i] is the primitive id reported for that triangle
 * (NULL = its index within its model).
 */
typedef struct rt_scene_desc {
    rt_camera camera;
    float env_light[3];                  /* Scene::EnvLight */
    int32_t n_lights;   const rt_light    *lights;
    int32_t n_materials; const rt_material *materials;
    int32_t n_textures; const rt_texture  *textures;
    int32_t n_objects;  const rt_object   *objects;
    int64_t n_tris;
    const float   *tri_p;
    const float   *tri_n;
    const float   *tri_uv;
    const int32_t *tri_mtl;
    const int32_t *tri_id;
} rt_scene_desc;

typedef struct rt_render_desc {
    int32_t width, height;       /* 0 = the scene camera's */
    int32_t spp;                 /* samples per pixel (>1 = Philox-jittered sub-pixel offsets) */
    int32_t max_level;           /* RayTracer::maxLevel: levels 0..max_level are traced */
    int32_t mode;                /* RT_MODE_* */
    int32_t flags;               /* RT_FLAG_* */
    uint64_t seed;               /* jitter seed */
    const rt_camera *camera;     /* NULL = the scene camera */
} rt_render_desc;

typedef struct rt_render_stats {
    int64_t rays_primary;        /* W*H*spp rays generated */
    int64_t rays_secondary;      /* reflect + refract rays traced */
    int64_t rays_shadow;         /* shadow rays traced */
    int64_t nodes_visited;       /* with RT_FLAG_COUNT_WORK: BVH node boxes tested by extend */
    int64_t tris_tested;         /* with RT_FLAG_COUNT_WORK: by extend */
    int64_t spheres_tested;      /* with RT_FLAG_COUNT_WORK */
    int64_t shadow_nodes_visited;   /* the same three counts for the shadow (any-hit) kernels */
    int64_t shadow_tris_tested;
    int64_t shadow_spheres_tested;
    float   ms;                  /* device time of the last render (CUDA events) */
    int32_t overflow_retries;
    float   kernel_ms[RT_KERNEL_KINDS];       /* with RT_FLAG_PROFILE: device time per kernel kind */
    int32_t kernel_launches[RT_KERNEL_KINDS]; /* kernels launched per kind (always filled) */
    float   kernel_idle[RT_KERNEL_KINDS];     /* with RT_FLAG_PROFILE, for extend, shade and shadow:
                                                 the share of the launches' warp time (warps x span
                                                 from the first warp's start to the last warp's end)
                                                 spent before a warp's block started or after the
                                                 warp ran out of work: the SM time a kernel that
                                                 never drains between bounces could use */
} rt_render_stats;

typedef struct rt_ctx rt_ctx;

/* ---- context ------------------------------------------------------------------------ */
int         rt_version(void);
int         rt_ctx_create(int device, rt_ctx **out);
void        rt_ctx_destroy(rt_ctx *ctx);
const char *rt_last_error(const rt_ctx *ctx);
int         rt_ctx_synchronize(rt_ctx *ctx);
/* stream used by every call of this context (NULL = the context's own stream) */
int         rt_ctx_set_stream(rt_ctx *ctx, void *cuda_stream);
/* Hierarchy of the scenes this context builds from now on:
 *   RT_BUILD_RADIX    Karras radix tree over 30-bit Morton codes (default; fastest build, 0.7 ms
 *                     for 2.1M triangles; best for flat, regular meshes such as terrains)
 *   RT_BUILD_CLUSTER  locally-ordered agglomerative clustering over the Morton order (a few ms;
 *                     10-14 % lower SAH cost and ~11 % fewer shadow-ray node visits on irregular
 *                     scenes — meant for scenes that stay resident and are rendered many times)
 * Both give the same images: only the traversal cost differs. A clustered tree deeper than 63
 * levels is replaced by the radix tree. */
#define RT_BUILD_RADIX   0
#define RT_BUILD_CLUSTER 1
int rt_ctx_set_build(rt_ctx *ctx, int32_t mode);
/* Released scene and frame buffers stay with the context (at most 4, 8 GB) and are reused by
 * the next upload or frame that fits, saving a cudaMalloc / cudaFree per scene and frame;
 * this frees them now, together with the batch path's wave workspace (up to 31 GB). */
int rt_ctx_release_cached(rt_ctx *ctx);

/* ---- scenes: upload + device LBVH build (replaces RTPrepare, Model.cpp:402-480) ------ */
int rt_scene_upload(rt_ctx *ctx, const rt_scene_desc *desc, int32_t *scene_id);
int rt_scene_update_camera(rt_ctx *ctx, int32_t scene_id, const rt_camera *cam);
int rt_scene_rebuild(rt_ctx *ctx, int32_t scene_id);      /* re-run the hierarchy build (the context's build mode) */
int rt_scene_release(rt_ctx *ctx, int32_t scene_id);
int rt_scene_device_bytes(rt_ctx *ctx, int32_t scene_id, int64_t *bytes);
/* last LBVH build time in ms (device time, CUDA events) */
int rt_scene_build_ms(rt_ctx *ctx, int32_t scene_id, float *ms);

/* ---- frames (device framebuffers) ------------------------------------------------------ */
int rt_frame_create(rt_ctx *ctx, int32_t width, int32_t height, int32_t *frame_id);
int rt_frame_release(rt_ctx *ctx, int32_t frame_id);
/*
 * Copy a finished frame to host buffers (any may be NULL):
 *   rgb      float[H*W*3]  colour before clamping (Color before put, 3DElement.cpp:463-468)
 *   rgb8     uint8[H*W*3]  Color::put of rgb
 *   hit_obj  int32[H*W]    primary hit object index (-1 = miss), sample 0
 *   hit_prim int32[H*W]    primary hit primitive id (triangle id, ballplane sphere 1..16, else 0)
 *   hit_t    float[H*W]    primary hit distance (1e20 = miss)
 * Rows are bottom-up, row stride W. The call waits for the frame's render.
 */
int rt_frame_download(rt_ctx *ctx, int32_t frame_id, float *rgb, uint8_t *rgb8,
                      int32_t *hit_obj, int32_t *hit_prim, float *hit_t);
/* device pointers of a frame (rgb float, rgb8) for zero-copy consumers */
int rt_frame_device_ptrs(rt_ctx *ctx, int32_t frame_id, void **rgb, void **rgb8);

/* ---- one render (the plain per-scene path) ----------------------------------------------- */
/* enqueue on the context stream; returns immediately */
int rt_render(rt_ctx *ctx, int32_t scene_id, int32_t frame_id, const rt_render_desc *rd);
/* wait for the last render of the context; fills stats if not NULL */
int rt_render_wait(rt_ctx *ctx, rt_render_stats *stats);
/* cooperative cancel of the running render (RayTracer::stop, RayTracer.cpp:698-701). Callable
 * from any thread. A render is cancelled by every rt_cancel made after it began (rt_render,
 * rt_batch_render, rt_render_host) or after the mark it was given (rt_render_host_since);
 * earlier calls do not affect it. */
int rt_cancel(rt_ctx *ctx);
/* the context's cancel mark: the number of rt_cancel calls made so far (thread-safe) */
uint64_t rt_cancel_mark(rt_ctx *ctx);
/* 1 if the last render finished, 0 if still running (RayTracer::isFinish) */
int rt_poll(rt_ctx *ctx);

/*
 * End-to-end drop-in for RayTracer::start + wait: upload the host scene, build the LBVH,
 * render, and write the reference's uint8 output (bottom-up rows of stride 3*W over the
 * 64x64 tiles when RT_FLAG_REF_TILES is set) plus optional float rgb, all from host memory.
 */
int rt_render_host(rt_ctx *ctx, const rt_scene_desc *desc, const rt_render_desc *rd,
                   uint8_t *out_rgb8, float *out_rgb, rt_render_stats *stats);
/*
 * rt_render_host for a render started on another thread: it is cancelled (RT_ERR_CANCELLED) by
 * any rt_cancel made after `cancel_mark` was taken with rt_cancel_mark, including one made
 * before this call began. The reference's start() sets isRun before its threads run, so a stop()
 * right after start() ends that render (RayTracer.cpp:614-617, 698-701); a caller taking the mark
 * in its start() gets the same. rt_render_host(...) is this call with the mark taken at entry.
 */
int rt_render_host_since(rt_ctx *ctx, uint64_t cancel_mark, const rt_scene_desc *desc,
                         const rt_render_desc *rd, uint8_t *out_rgb8, float *out_rgb,
                         rt_render_stats *stats);

/* ---- batched multi-scene rendering (persistent wavefront kernel + CUDA graph) ------------ */
typedef struct rt_batch_tuning {
    int32_t block;               /* threads per block of the traversal kernels (0 = default) */
    int32_t tile;                /* rays taken per work-counter fetch (0 = default; at most 4096) */
    int32_t stack;               /* traversal stack entries per thread kept in shared memory: 0 or 8;
                                    the rest of the 96 entries that bound any path stay in local
                                    memory (0 = all of them) */
    int32_t use_graph;           /* capture the per-bounce launch sequence as a CUDA graph */
    int32_t min_blocks;          /* 0, 6 or 8: resident 128-thread blocks per SM the register budget
                                    of the traversal kernels must allow (0 = compiler's) */
    int32_t dynamic;             /* 0 or 1: pull ray tiles from a counter; 2: static grid stride;
                                    3: each SM first drains its own contiguous share of the rays */
    int64_t wave_rays;           /* batch: ray-queue entries of one wave (0 = 2^26) */
    int32_t shadow_chunk;        /* shadow rays light-major within chunks of this many hits, a
                                    multiple of 32 (0 = all of a bounce's hits in one chunk; the
                                    default tuning uses 4096) */
    int32_t pixel_tile;          /* primary rays traced in square pixel tiles of this edge, 0 (row by
                                    row) or 2..64; the image does not depend on it (with no tuning
                                    given, batches and batched servers use 8, plain renders 0) */
    int32_t lanes;               /* batch and server: consecutive waves go in turn to this many workspaces, each
                                    with its own stream, so one wave's kernels can use the SMs the
                                    other's leave idle while they drain: 1 or 2 (0 = 2 for a batch,
                                    1 for a server; a profiled batch uses 1). Each lane holds a wave workspace (wave_rays
                                    entries x 292 B) */
    int32_t reserved;            /* 0 */
} rt_batch_tuning;

/* kernel tuning of the plain per-scene path (rt_render); NULL restores the defaults */
int rt_ctx_set_tuning(rt_ctx *ctx, const rt_batch_tuning *tuning);
/* the plain path's current tuning (the defaults unless rt_ctx_set_tuning changed them) */
int rt_ctx_get_tuning(const rt_ctx *ctx, rt_batch_tuning *out);

/* render n (scene, frame, desc) jobs as one wavefront; returns after enqueueing */
int rt_batch_render(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                    const rt_render_desc *rds, const rt_batch_tuning *tuning);
/* the same jobs through a loop of plain per-scene renders (the comparison path) */
int rt_batch_render_plain(rt_ctx *ctx, int32_t n, const int32_t *scene_ids,
                          const int32_t *frame_ids, const rt_render_desc *rds);
/* pick block size, register cap and ray tile (or the static stride) for these jobs by timing
 * candidates, then per-SM shares of the rays, the wave lanes, the short-stack depth in shared
 * memory, the pixel tile, the shadow chunk and the wave size.
 * Writes the choice. */
int rt_batch_autotune(rt_ctx *ctx, int32_t n, const int32_t *scene_ids, const int32_t *frame_ids,
                      const rt_render_desc *rds, rt_batch_tuning *out);

/* ---- serving: continuous batching over resident scenes ----------------------------------
 * No counterpart in the reference (its RayTracer renders one scene per start() call).
 * Requests (scene, camera, resolution) are queued as they arrive; each step admits queued
 * requests while frame slots and the HBM budget allow (LRU-evicting idle scenes, rebuilding
 * an evicted scene's LBVH on a miss), then traces one wave made of sample chunks of every
 * admitted request, so frames admitted at different times share the same kernels. A finished
 * frame is resolved and its uint8 image (and, with keep_images, its float colour) copied to
 * pinned host memory on a copy stream. Each frame is the same
 * alone or in any mix: colours accumulate as exact fixed-point sums. */
typedef struct rt_server rt_server;

typedef struct rt_server_config {
    int64_t hbm_budget_bytes;    /* device bytes for resident scenes + frame slots + wave queues */
    int32_t max_inflight;        /* frame slots: requests admitted at once (0 = 64) */
    int32_t max_level;           /* recursion depth of every request */
    int32_t spp;                 /* samples per pixel of every request (>= 1) */
    int32_t plain;               /* 1: one request at a time through rt_render (comparison path) */
    int64_t queue_rays;          /* ray-queue entries of one wave, 292 B each, per lane (0 = 2^27,
                                    halved until the queues take at most a third of the
                                    budget) */
    int64_t max_pixels;          /* largest width*height of a request (0 = 1920*1080) */
    int32_t keep_images;         /* 1: keep finished images in host memory until rt_server_result */
    int32_t stages;              /* waves the host may enqueue ahead of the device (0 = 2 per lane) */
} rt_server_config;

typedef struct rt_request {
    int32_t scene;               /* server scene id */
    int32_t width, height;
    rt_camera camera;            /* the camera's own width/height are ignored */
    uint64_t seed;               /* sub-pixel jitter seed (spp > 1) */
    double arrival_s;            /* arrival on the server clock; < 0 = now */
} rt_request;

typedef struct rt_request_result {
    int64_t request;
    int32_t status;              /* RT_OK or RT_ERR_* */
    int32_t width, height;
    int32_t scene;
    double arrival_s, admit_s, done_s;   /* server clock; done = image in host memory */
    int64_t samples;             /* primary rays of the frame */
    int32_t rebuilt;             /* 1 when the scene was rebuilt on a miss for this request */
    int32_t pad;
} rt_request_result;

typedef struct rt_serve_stats {
    int64_t requests, completed, rejected, evictions, rebuilds;
    double p50_ms, p99_ms, mean_ms, max_ms;   /* frame latency: arrival to image in host memory */
    double mrays_per_s;          /* ray segments traced / wall time */
    double wall_s;
    int64_t rays;
    int64_t peak_bytes;          /* most device bytes held against the budget */
    int64_t waves;
    double mean_wave_requests;   /* requests sharing a wave, averaged over waves */
    int64_t admitted_busy;       /* requests admitted while other requests were in flight */
    int64_t pixels;              /* pixels of the completed frames */
    double wave_ms_mean, wave_ms_p50, wave_ms_p99;   /* device time of one wave, table copies to
                                                        counters back (CUDA events) */
    double device_busy_s;        /* sum of the waves' device times: the compute stream's busy time */
    double host_step_s;          /* host time inside rt_server_step: admission, staging, enqueue,
                                    retirement (for the plain mode: the renders themselves) */
    double host_wait_s;          /* of it, blocked on the device (a full staging ring, a frame copy) */
    int64_t steps;
} rt_serve_stats;

int    rt_server_create(rt_ctx *ctx, const rt_server_config *cfg, rt_server **out);
void   rt_server_destroy(rt_server *srv);
const char *rt_server_last_error(const rt_server *srv);
/* kernel tuning of the server's waves, or of the plain mode's renders (NULL = the server's
 * defaults: one lane; primary rays in 8x8 pixel tiles, but row by row in the plain mode and for
 * requests admitted into an idle server); requests admitted from now on use it.
 * Images do not depend on it.
 * A new lane count takes an idle server (RT_ERR_BUSY while requests are pending) and keeps the
 * queue size of a lane (RT_ERR_BUDGET when the new lanes do not fit the budget). */
int    rt_server_set_tuning(rt_server *srv, const rt_batch_tuning *tuning);
/* register a scene (deep copy kept for rebuilds); it is uploaded now if the budget allows */
int    rt_server_add_scene(rt_server *srv, const rt_scene_desc *desc, int32_t *scene);
int    rt_server_submit(rt_server *srv, const rt_request *req, int64_t *request_id);
/* one continuous-batching step: retire finished frames, admit, enqueue one wave.
 * *n_pending = requests queued or in flight afterwards. */
int    rt_server_step(rt_server *srv, int32_t *n_pending);
/* step until nothing is queued or in flight */
int    rt_server_drain(rt_server *srv);
/* result (and image, if kept) of a finished request; the request is forgotten afterwards.
 * RT_ERR_BUSY while it is queued or in flight, RT_ERR_NOT_FOUND if unknown. */
int    rt_server_result(rt_server *srv, int64_t request_id, rt_request_result *res, float *rgb, uint8_t *rgb8);
int    rt_server_resident(rt_server *srv, int32_t scene, int32_t *resident);
double rt_server_now(rt_server *srv);
/* counters since creation or the last rt_server_run_poisson; latency over finished requests */
int    rt_server_stats(rt_server *srv, rt_serve_stats *stats);
/* frame latencies (ms, completion order) behind the current stats; *n = their count, at most
 * `cap` are copied (replicas merge these to exact percentiles across GPUs) */
int    rt_server_latencies(rt_server *srv, double *ms, int64_t cap, int64_t *n);
/* device time (ms, CUDA events) of each wave harvested since the current stats began, in the
 * order the waves ran; *n = their count, at most `cap` are copied */
int    rt_server_wave_ms(rt_server *srv, float *ms, int64_t cap, int64_t *n);
/* a Poisson stream of requests in real time over the registered scenes: scene uniform, camera
 * orbiting the world origin at the distance of the scene's own camera (azimuth U[0,360),
 * elevation U[10,60] degrees), resolution uniform over 256^2, 512^2, 1024x768, 1920x1080.
 * Arrivals stop at duration_s; the server then drains. Stats cover this run only. */
int    rt_server_run_poisson(rt_server *srv, double lambda_per_s, double duration_s, uint64_t seed,
                             rt_serve_stats *stats);
/* the orbit camera of those requests: `base` moved to the given azimuth/elevation about the
 * world origin at its own distance, looking at the origin with up = +y (host only) */
int    rt_orbit_camera(const rt_camera *base, double azimuth_deg, double elevation_deg, int32_t width,
                       int32_t height, rt_camera *out);

/* ---- test hook: the kernels' integer-exact replacements of FP64 expressions --------------
 * out_mul[i] = (float)((double)x[i] * d) and out_fix[i] = llrint(v[i] * 2^32) (finite v,
 * |v| < 2^31), computed on the device the way ray generation, frame resolve and colour
 * accumulation compute them. d must be a positive normal double. Synchronous. */
int rt_selftest_conversions(rt_ctx *ctx, const int64_t *x, int32_t n, double d, const float *v,
                            float *out_mul, int64_t *out_fix);

/* ---- LBVH pieces exposed for tests ------------------------------------------------------ */
/* 30-bit Morton codes of triangle centroids over the AABB of the centroids, radix-sorted
   (stable): codes[i] and perm[i] are the i-th smallest code and its triangle index */
int rt_morton_sort(rt_ctx *ctx, const float *tri_p, int64_t n_tris, uint32_t *codes, uint32_t *perm);
/*
 * rt_morton_sort on device buffers with no device allocation, for callers that cannot
 * allocate (a plugin whose host application owns the device memory, a latency-bound path
 * where cudaMalloc would block). d_tri_p, d_codes and d_perm are device pointers the caller
 * owns; the working memory is one fixed static device array sized for RT_NOALLOC_MAX_TRIS
 * triangles (about 7.5 MB, held by every GPU that loads the library). Larger inputs return
 * RT_ERR_TOO_LARGE. Runs on cuda_stream (NULL = default stream) and returns after enqueueing.
 * The first call on a device loads the array there; make it before any stream capture. An
 * error already pending from the caller's own CUDA work is left pending and the call returns
 * RT_ERR_CUDA without enqueueing anything. Calls that overlap on the GPU share the array and
 * race. No counterpart in the reference.
 */
#define RT_NOALLOC_MAX_TRIS (1 << 18)
int rt_morton_sort_noalloc(const float *d_tri_p, int64_t n_tris, uint32_t *d_codes, uint32_t *d_perm,
                           void *cuda_stream);
/* Test hooks for the device-side limits (a corrupt tree, an overflowing queue), no counterpart
 * in the reference. rt_scene_test_set_node_refs overwrites the four child references of 4-wide
 * node `node` (0..L-2) of a scene's hierarchy: >= 0 an internal node 0..L-2, < 0 leaf ~k with
 * k < L. Only references inside the tree are accepted, so a traversal of the changed tree reads
 * no memory outside it; a cycle among valid nodes makes the traversal's visit limit (2^22 node
 * visits per ray) and stack bound fire, and the render reports RT_ERR_CUDA ("corrupt LBVH")
 * instead of looping. rt_ctx_test_queue_entries makes the first attempt of each later rt_render
 * size its ray queues for `entries` rays (0 = twice the frame's samples, the default); a
 * context whose workspace is already larger keeps the larger queues. A render that overflows
 * its queues is retried with queues twice as large (rt_render_stats.overflow_retries). */
int rt_scene_test_set_node_refs(rt_ctx *ctx, int32_t scene_id, int32_t node, const int32_t *refs);
int rt_ctx_test_queue_entries(rt_ctx *ctx, int64_t entries);
/* download the LBVH of a scene with L leaves (triangles and spheres): nodes float[(2L-1)*8]
   (min xyz, left | max xyz, right; leaf k is node L-1+k) and perm[L], the leaf order: the
   reported id of a triangle leaf, 0x80000000 | primitive index of a sphere leaf */
int rt_scene_bvh_download(rt_ctx *ctx, int32_t scene_id, float *nodes, uint32_t *perm,
                          int64_t *n_nodes);

/* ---- seeded synthetic scenes (the benchmark workloads) ---------------------------------- */
typedef struct rt_scene_host rt_scene_host;
/* config 0..4 as in the benchmark definition, index = scene number inside configs 3/4 */
int  rt_scenegen(int32_t config, int32_t index, rt_scene_host **out);
/* a small scene for tests: plane + n spheres (+ an icosphere of the given frequency, 0 = none) */
int  rt_scenegen_small(uint64_t seed, int32_t n_spheres, int32_t ico_freq, int32_t width,
                       int32_t height, int32_t refractive_every, rt_scene_host **out);
/* every object kind in one scene: plane, ballplane, cubes, spheres, a mesh, parallel + point light */
int  rt_scenegen_extras(uint64_t seed, int32_t width, int32_t height, rt_scene_host **out);
/* textured meshes: checker-textured plane, an icosphere with planar texture coordinates and a
 * procedural texture, spheres, a cube, two point lights */
int  rt_scenegen_textured(uint64_t seed, int32_t width, int32_t height, rt_scene_host **out);
/* a model read from OBJ/MTL files through the drop-in Scene::AddModel (Model::loadOBJ,
 * Model.cpp:341 of the reference: texture files are read as <name>.bmp relative to the working
 * directory), two point lights, a camera facing it. RT_ERR_NOT_FOUND when nothing was read. */
int  rt_scenegen_obj(const char *obj_path, const char *mtl_path, int32_t width, int32_t height,
                     rt_scene_host **out);
/* deep copy of a caller-built description (render parameters attached) */
int  rt_scene_host_from_desc(const rt_scene_desc *desc, int32_t spp, int32_t max_level, uint64_t seed,
                             rt_scene_host **out);
const rt_scene_desc *rt_scene_host_desc(const rt_scene_host *s);
int  rt_scene_host_render_params(const rt_scene_host *s, int32_t *spp, int32_t *max_level,
                                 uint64_t *seed);
int  rt_scene_host_save(const rt_scene_host *s, const char *path);
/* page-lock the scene's host arrays so uploads run at full link speed (0 = pinned) */
int  rt_scene_host_pin(rt_scene_host *s);
/* bytes of the scene's host arrays that an upload copies to the device */
int64_t rt_scene_host_bytes(const rt_scene_host *s);
int  rt_scene_host_load(const char *path, rt_scene_host **out);
void rt_scene_host_free(rt_scene_host *s);

#ifdef __cplusplus
}
#endif
#endif
