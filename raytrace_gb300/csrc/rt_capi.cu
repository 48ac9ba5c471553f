// rt_capi.cu — the C ABI (include/rt_gb300.h): contexts, scene upload + LBVH build, frames,
// the plain per-scene render path, the batched multi-scene path and the test hooks.
//
// Scene flattening into device tables replaces the per-pixel virtual calls over
// Scene::Objects (RayTracer.cpp:458-465); the LBVH replaces Model::RTPrepare
// (Model.cpp:402-480); one render = the parallelRT tile loop (RayTracer.cpp:5-45) over every
// pixel, as a wavefront of prepare -> (extend -> shade -> shadow) x (maxLevel+1) -> resolve, the
// first extend making the primary rays.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_capi_internal.h"
#include "rt_kernels.cuh"
#include "rt_lbvh.cuh"

using namespace rtg;

// ---- helpers -------------------------------------------------------------------------------------
int ctx_fail(rt_ctx *ctx, int code, const char *fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

DevBuf::~DevBuf() { release(); }
void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}
cudaError_t DevBuf::ensure(size_t need)
{
    if (need <= bytes && p) return cudaSuccess;
    release();
    size_t b = std::max<size_t>(need, 256);
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        return e;
    }
    bytes = b;
    return cudaSuccess;
}

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---- buffer reuse ----------------------------------------------------------------------------------
// Released scene and frame buffers stay with the context (a few, up to kSpareBytes) and are
// handed to the next upload or frame that fits, saving a cudaMalloc and a cudaFree (which
// synchronises the device) per scene and frame. Reuse is ordered by the context stream: work
// still reading a released buffer runs before anything the next owner enqueues.
constexpr size_t kSpareBytes = 8ull << 30;
constexpr size_t kSpareCount = 4;

void spare_put(rt_ctx *ctx, DevBuf &&b)
{
    if (!b.p) return;
    ctx->spare.push_back(std::move(b));
    size_t total = 0;
    for (const DevBuf &x : ctx->spare) total += x.bytes;
    if (total > kSpareBytes || ctx->spare.size() > kSpareCount) {
        cudaStreamSynchronize(ctx->stream);   // a freed buffer must not be in use
        while (!ctx->spare.empty() && (total > kSpareBytes || ctx->spare.size() > kSpareCount)) {
            total -= ctx->spare.front().bytes;
            ctx->spare.erase(ctx->spare.begin());
        }
    }
}

size_t spare_bytes(const rt_ctx *ctx)
{
    size_t total = 0;
    for (const DevBuf &x : ctx->spare) total += x.bytes;
    return total;
}

void spare_trim(rt_ctx *ctx)
{
    if (ctx->spare.empty()) return;
    cudaStreamSynchronize(ctx->stream);
    ctx->spare.clear();
}

// the smallest spare buffer holding `need` bytes without wasting more than half of it
void spare_take(rt_ctx *ctx, DevBuf &dst, size_t need)
{
    int best = -1;
    for (size_t i = 0; i < ctx->spare.size(); ++i) {
        const size_t b = ctx->spare[i].bytes;
        if (b >= need && b <= 2 * need + (64u << 20) && (best < 0 || b < ctx->spare[(size_t)best].bytes)) best = (int)i;
    }
    if (best < 0) return;
    dst = std::move(ctx->spare[(size_t)best]);
    ctx->spare.erase(ctx->spare.begin() + best);
}

// ---- version / context -------------------------------------------------------------------------------
// Cancel: rt_cancel writes 1 into a device word from page-locked memory on a side stream, which
// runs beside the render; each render clears it on the same stream first and its kernels wait
// for the clear. Kernels then read device memory, not host memory over the bus. Both writes are
// made under the context's cancel mutex, and a render whose mark a cancel has already passed
// does not clear the flag: the side stream then holds every cancel's write after the clear
// that could hide it.
int cancel_arm(rt_ctx *ctx, unsigned long long mark)
{
    std::lock_guard<std::mutex> lock(ctx->cancel_mu);
    ctx->cancel_base = mark;
    if (ctx->cancel_count.load() != mark) return ctx_fail(ctx, RT_ERR_CANCELLED, "render cancelled");
    CK(ctx, cudaMemcpyAsync(ctx->cancel_dev, ctx->cancel_vals, sizeof(int), cudaMemcpyHostToDevice, ctx->side));
    CK(ctx, cudaEventRecord(ctx->ev_armed, ctx->side));
    CK(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_armed, 0));
    return RT_OK;
}

extern "C" int rt_version(void) { return RT_ABI_VERSION; }

extern "C" int rt_ctx_create(int device, rt_ctx **out)
{
    if (!out) return RT_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return RT_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return RT_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return RT_ERR_CUDA;
    std::unique_ptr<rt_ctx> c(new rt_ctx());
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return RT_ERR_CUDA;
    c->stream = c->own_stream;
    if (cudaEventCreate(&c->ev_start) != cudaSuccess || cudaEventCreate(&c->ev_stop) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMalloc((void **)&c->cancel_dev, sizeof(int)) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMallocHost((void **)&c->cancel_vals, 2 * sizeof(int)) != cudaSuccess) return RT_ERR_CUDA;
    c->cancel_vals[0] = 0, c->cancel_vals[1] = 1;
    if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_armed, cudaEventDisableTiming) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMemset(c->cancel_dev, 0, sizeof(int)) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMallocHost((void **)&c->counters_host, sizeof(Counters)) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMallocHost(&c->plain_stage, kPlainStageBytes) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_staged, cudaEventDisableTiming) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventRecord(c->ev_staged, c->stream) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_upload, cudaEventDisableTiming) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&c->upload_side, cudaStreamNonBlocking) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_upload_go, cudaEventDisableTiming) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_shading, cudaEventDisableTiming) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventRecord(c->ev_shading, c->stream) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaMallocHost((void **)&c->build_flag, sizeof(int)) != cudaSuccess) return RT_ERR_CUDA;
    if (cudaEventRecord(c->ev_upload, c->stream) != cudaSuccess) return RT_ERR_CUDA;
    *out = c.release();
    return RT_OK;
}

extern "C" void rt_ctx_destroy(rt_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->scenes.clear();
    ctx->frames.clear();
    ctx->batch.reset();
    ctx->plain_graphs.clear();
    ctx->spare.clear();
    ctx->ws = Workspace();
    if (ctx->upload_stage) cudaFreeHost(ctx->upload_stage);
    if (ctx->build_flag) cudaFreeHost(ctx->build_flag);
    if (ctx->ev_upload) cudaEventDestroy(ctx->ev_upload);
    if (ctx->upload_side) {
        cudaStreamSynchronize(ctx->upload_side);
        cudaStreamDestroy(ctx->upload_side);
    }
    if (ctx->ev_upload_go) cudaEventDestroy(ctx->ev_upload_go);
    if (ctx->ev_shading) cudaEventDestroy(ctx->ev_shading);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->cancel_dev) cudaFree(ctx->cancel_dev);
    if (ctx->cancel_vals) cudaFreeHost(ctx->cancel_vals);
    if (ctx->ev_armed) cudaEventDestroy(ctx->ev_armed);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->counters_host) cudaFreeHost(ctx->counters_host);
    if (ctx->plain_stage) cudaFreeHost(ctx->plain_stage);
    if (ctx->ev_staged) cudaEventDestroy(ctx->ev_staged);
    cudaEventDestroy(ctx->ev_start);
    cudaEventDestroy(ctx->ev_stop);
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

extern "C" const char *rt_last_error(const rt_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

extern "C" int rt_ctx_synchronize(rt_ctx *ctx)
{
    if (!ctx) return RT_ERR_INVALID;
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return RT_OK;
}

extern "C" int rt_ctx_set_build(rt_ctx *ctx, int32_t mode)
{
    if (!ctx) return RT_ERR_INVALID;
    if (mode != RT_BUILD_RADIX && mode != RT_BUILD_CLUSTER) return ctx_fail(ctx, RT_ERR_INVALID, "build mode %d", mode);
    ctx->build_mode = mode;
    return RT_OK;
}

extern "C" int rt_ctx_release_cached(rt_ctx *ctx)
{
    if (!ctx) return RT_ERR_INVALID;
    spare_trim(ctx);
    if (ctx->batch) {
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->batch.reset();
    }
    return RT_OK;
}

extern "C" int rt_ctx_set_stream(rt_ctx *ctx, void *stream)
{
    if (!ctx) return RT_ERR_INVALID;
    // released buffers are reused in the order of the context stream: finish the old stream
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return RT_OK;
}

// ---- scenes ------------------------------------------------------------------------------------------
static bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

int validate_desc(rt_ctx *ctx, const rt_scene_desc *d)
{
    if (!d) return ctx_fail(ctx, RT_ERR_INVALID, "scene desc is NULL");
    if (d->n_lights < 0 || d->n_lights > 8) return ctx_fail(ctx, RT_ERR_INVALID, "n_lights %d outside [0,8]", d->n_lights);
    if (d->n_materials < 0 || d->n_objects < 0 || d->n_textures < 0 || d->n_tris < 0)
        return ctx_fail(ctx, RT_ERR_INVALID, "negative count in scene desc");
    if ((d->n_lights && !d->lights) || (d->n_materials && !d->materials) || (d->n_objects && !d->objects) ||
        (d->n_textures && !d->textures))
        return ctx_fail(ctx, RT_ERR_INVALID, "NULL table with a non-zero count");
    if (d->n_tris > 0 && (!d->tri_p || !d->tri_n || !d->tri_mtl))
        return ctx_fail(ctx, RT_ERR_INVALID, "triangles need tri_p, tri_n and tri_mtl");
    if (d->n_tris >= (int64_t)1 << 30) return ctx_fail(ctx, RT_ERR_INVALID, "too many triangles (%lld)", (long long)d->n_tris);
    for (int i = 0; i < d->n_textures; ++i)
        if (d->textures[i].w <= 0 || d->textures[i].h <= 0 || !d->textures[i].bgr)
            return ctx_fail(ctx, RT_ERR_INVALID, "texture %d is empty", i);
    for (int i = 0; i < d->n_objects; ++i) {
        const rt_object &o = d->objects[i];
        if (o.type < RT_OBJECT_SPHERE || o.type > RT_OBJECT_BALLPLANE)
            return ctx_fail(ctx, RT_ERR_INVALID, "object %d has unknown type %d", i, o.type);
        if (o.type != RT_OBJECT_MODEL && (o.material < 0 || o.material >= d->n_materials))
            return ctx_fail(ctx, RT_ERR_INVALID, "object %d material %d out of range", i, o.material);
        if (o.type == RT_OBJECT_PLANE && o.texture >= d->n_textures)
            return ctx_fail(ctx, RT_ERR_INVALID, "object %d texture out of range", i);
        if (o.type == RT_OBJECT_MODEL &&
            (o.tri_first < 0 || o.tri_count < 0 || o.tri_first + o.tri_count > d->n_tris))
            return ctx_fail(ctx, RT_ERR_INVALID, "object %d triangle range out of bounds", i);
        if (!finite3(o.position)) return ctx_fail(ctx, RT_ERR_INVALID, "object %d position not finite", i);
    }
    for (int i = 0; i < d->n_materials; ++i)
        if (d->materials[i].texture >= d->n_textures)
            return ctx_fail(ctx, RT_ERR_INVALID, "material %d texture out of range", i);
    // per-triangle material indices are checked on the device by the LBVH build
    return RT_OK;
}

static void f4(float4 &d, const float *v, float w = 0.0f) { d = make_float4(v[0], v[1], v[2], w); }

// host side of the device tables
struct HostTables {
    std::vector<DevPrim> prims;
    std::vector<DevMaterial> mtl;
    std::vector<DevLight> lights;
    std::vector<DevTexture> tex;
    std::vector<uint8_t> texels;
    std::vector<float> obj_pos;
    // shown models' triangles, compacted
    std::vector<std::pair<int64_t, int64_t>> tri_ranges;   // (first, count) per shown model
    std::vector<int> tri_range_obj;
    int64_t n_tris = 0;
    int n_linear = 0;   // prims before this index are planes / boxes, the rest spheres
};

static void build_tables(const rt_scene_desc *d, HostTables &h)
{
    for (int i = 0; i < d->n_materials; ++i) {
        const rt_material &m = d->materials[i];
        DevMaterial dm{};
        for (int k = 0; k < 3; ++k) dm.ka[k] = m.ambient[k], dm.kd[k] = m.diffuse[k], dm.ks[k] = m.specular[k];
        dm.shininess = m.shininess, dm.reflect = m.reflect, dm.refract = m.refract, dm.rfr = m.rfr;
        dm.tex = m.texture;
        h.mtl.push_back(dm);
    }
    if (h.mtl.empty()) h.mtl.push_back(DevMaterial{});
    for (int i = 0; i < d->n_lights; ++i) {
        const rt_light &l = d->lights[i];
        DevLight dl{};
        dl.type = l.type, dl.on = l.on;
        for (int k = 0; k < 3; ++k) {
            dl.pos[k] = l.position[k], dl.amb[k] = l.ambient[k], dl.dif[k] = l.diffuse[k];
            dl.spec[k] = l.specular[k], dl.att[k] = l.attenuation[k];
        }
        h.lights.push_back(dl);
    }
    for (int i = 0; i < d->n_textures; ++i) {
        const rt_texture &t = d->textures[i];
        DevTexture dt{t.w, t.h, (long long)h.texels.size()};
        h.texels.insert(h.texels.end(), t.bgr, t.bgr + (size_t)t.w * t.h * 3);
        h.tex.push_back(dt);
    }
    if (h.texels.empty()) h.texels.push_back(0xff);
    h.obj_pos.assign((size_t)std::max(1, d->n_objects) * 3, 0.0f);
    for (int k = 0; k < d->n_objects; ++k) {
        const rt_object &o = d->objects[k];
        for (int j = 0; j < 3; ++j) h.obj_pos[3 * k + j] = o.position[j];
        if (!o.show) continue;
        DevPrim p{};
        p.obj = k;
        p.mtl = o.material;
        p.tex = -1;
        switch (o.type) {
        case RT_OBJECT_SPHERE:
            p.type = kPrimSphere;
            f4(p.a, o.position, o.radius * o.radius);
            p.b = make_float4(o.radius, 0, 0, 0);
            h.prims.push_back(p);
            break;
        case RT_OBJECT_PLANE:
            p.type = kPrimPlane;
            f4(p.a, o.position);
            f4(p.b, o.normal);
            f4(p.c, o.axisx);
            f4(p.d, o.axisy);
            p.tex = o.texture;
            h.prims.push_back(p);
            break;
        case RT_OBJECT_CUBE: {   // BorderTest(ray, min + position, max + position)
            p.type = kPrimBox;
            float mn[3], mx[3];
            for (int j = 0; j < 3; ++j) mn[j] = o.bmin[j] + o.position[j], mx[j] = o.bmax[j] + o.position[j];
            f4(p.a, mn);
            f4(p.b, mx);
            f4(p.c, o.position);
            f4(p.d, o.bmax);
            h.prims.push_back(p);
            break;
        }
        case RT_OBJECT_BALLPLANE: {   // 4x4 spheres visited cx-major (Basic3DObject.cpp:492-497)
            const float r = o.radius;
            int cnt = 0;
            for (float cx = r * -6; cx < r * 8; cx += r * 4)
                for (float cy = r * -6; cy < r * 8; cy += r * 4) {
                    ++cnt;
                    float c[3];
                    for (int j = 0; j < 3; ++j) {
                        float t = o.axisx[j] * cx + o.axisy[j] * cy;
                        c[j] = t + o.position[j];
                    }
                    DevPrim s = p;
                    s.type = kPrimSphere;
                    s.sub = cnt;
                    f4(s.a, c, r * r);
                    s.b = make_float4(r, 0, 0, 0);
                    h.prims.push_back(s);
                }
            break;
        }
        case RT_OBJECT_MODEL:
            if (o.tri_count > 0) {
                h.tri_ranges.push_back({o.tri_first, o.tri_count});
                h.tri_range_obj.push_back(k);
                h.n_tris += o.tri_count;
            }
            break;
        }
    }
    // planes and boxes first (tested linearly per ray), spheres after them (LBVH leaves);
    // the order among primitives does not matter: ties resolve by object index
    std::stable_partition(h.prims.begin(), h.prims.end(), [](const DevPrim &p) { return p.type != kPrimSphere; });
    h.n_linear = 0;
    for (const DevPrim &p : h.prims)
        if (p.type != kPrimSphere) ++h.n_linear;
}

extern "C" int rt_scene_upload(rt_ctx *ctx, const rt_scene_desc *d, int32_t *scene_id)
{
    if (!ctx || !scene_id) return RT_ERR_INVALID;
    int rc = validate_desc(ctx, d);
    if (rc) return rc;
    CK(ctx, cudaSetDevice(ctx->device));
    HostTables h;
    build_tables(d, h);
    std::unique_ptr<SceneDev> sc(new SceneDev());
    sc->camera = d->camera;
    for (const DevMaterial &m : h.mtl)   // the spawn tests of the shade kernel
        sc->branching = std::max(sc->branching, (int)(m.reflect > 0.01f) + (int)(m.refract > 0.01f));
    const int64_t n = h.n_tris;
    sc->n_tris = (int)n;
    sc->n_leaves = (int)(n + (int64_t)h.prims.size() - h.n_linear);
    // one allocation for tables, triangle inputs and the LBVH
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += a256(bytes);
        return o;
    };
    // the small tables first (one staging copy covers [0, o_small)), then the triangle inputs
    // (copied straight from the caller's arrays), then what the LBVH build writes
    const size_t o_prims = take(sizeof(DevPrim) * std::max<size_t>(1, h.prims.size()));
    const size_t o_mtl = take(sizeof(DevMaterial) * h.mtl.size());
    const size_t o_lights = take(sizeof(DevLight) * std::max<size_t>(1, h.lights.size()));
    const size_t o_tex = take(sizeof(DevTexture) * std::max<size_t>(1, h.tex.size()));
    const size_t o_texels = take(h.texels.size());
    const size_t o_objpos = take(sizeof(float) * h.obj_pos.size());
    const size_t o_rng = take(sizeof(int) * 3 * std::max<size_t>(1, h.tri_ranges.size()));
    const int n_sph = (int)h.prims.size() - h.n_linear;
    const int64_t L = n + n_sph;   // LBVH leaves
    const size_t o_sph = take(sizeof(float4) * (size_t)std::max(1, n_sph)), o_sphr = take(sizeof(float) * (size_t)std::max(1, n_sph));
    const size_t o_sphp = take(sizeof(int) * (size_t)std::max(1, n_sph)), o_spho = take(sizeof(int) * (size_t)std::max(1, n_sph));
    const size_t o_hdr = take(sizeof(DevScene));
    const size_t o_bad = take(sizeof(int));   // material check flag of the build (staged as 0)
    const size_t o_small = off;
    const bool has_uv = d->tri_uv != nullptr;
    const size_t o_tp = take(sizeof(float) * 9 * (size_t)n), o_tn = take(sizeof(float) * 9 * (size_t)n);
    const size_t o_tuv = has_uv ? take(sizeof(float) * 6 * (size_t)n) : 0;
    const size_t o_tm = take(sizeof(int) * (size_t)n), o_ti = take(sizeof(int) * (size_t)n), o_to = take(sizeof(int) * (size_t)n);
    const size_t o_nodes = take(sizeof(float4) * 2 * (size_t)std::max<int64_t>(1, 2 * L - 1));
    const size_t o_quads = take(sizeof(float4) * 8 * (size_t)std::max<int64_t>(1, L - 1));
    const size_t o_tri = take(sizeof(float4) * 3 * (size_t)L), o_trin = take(sizeof(float4) * 3 * (size_t)L);
    const size_t o_triuv = has_uv ? take(sizeof(float2) * 3 * (size_t)L) : 0;
    spare_take(ctx, sc->mem, off);
    CK(ctx, sc->mem.ensure(off));
    char *base = (char *)sc->mem.p;
    cudaStream_t s = ctx->stream;
    // triangle inputs: straight from the caller's arrays when the shown models cover them in
    // order (the usual case, and the fast path for page-locked host memory); otherwise
    // compacted through staging copies
    bool direct = true;
    {
        int64_t expect = 0;
        for (auto &r : h.tri_ranges) {
            if (r.first != expect) direct = false;
            expect = r.first + r.second;
        }
        if (expect != d->n_tris) direct = false;
    }
    std::vector<int> range_tab;   // (first, count, obj) per shown model, in the compacted numbering
    {
        int64_t w = 0;
        for (size_t r = 0; r < h.tri_ranges.size(); ++r) {
            range_tab.insert(range_tab.end(), {(int)w, (int)h.tri_ranges[r].second, h.tri_range_obj[r]});
            w += h.tri_ranges[r].second;
        }
    }
    if (n > 0) {
        if (direct) {
            // the points go first on the render stream: the LBVH build starts from them. The
            // shading data (normals, uvs, materials, ids) follows on a second stream and arrives
            // while the build sorts; only its gather step waits for it. That stream first waits
            // for the render stream's earlier work, which may still use this (reused) memory.
            CK(ctx, cudaMemcpyAsync(base + o_tp, d->tri_p, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, s));
            cudaStream_t s2 = ctx->upload_side;
            CK(ctx, cudaEventRecord(ctx->ev_upload_go, s));
            CK(ctx, cudaStreamWaitEvent(s2, ctx->ev_upload_go, 0));
            CK(ctx, cudaMemcpyAsync(base + o_tn, d->tri_n, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, s2));
            if (has_uv) CK(ctx, cudaMemcpyAsync(base + o_tuv, d->tri_uv, sizeof(float) * 6 * (size_t)n, cudaMemcpyHostToDevice, s2));
            CK(ctx, cudaMemcpyAsync(base + o_tm, d->tri_mtl, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s2));
            if (d->tri_id) CK(ctx, cudaMemcpyAsync(base + o_ti, d->tri_id, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s2));
            CK(ctx, cudaEventRecord(ctx->ev_shading, s2));
        } else {
            std::vector<float> tp((size_t)n * 9), tn((size_t)n * 9), tuv(has_uv ? (size_t)n * 6 : 0);
            std::vector<int> tm((size_t)n), ti((size_t)n);
            size_t w = 0;
            for (size_t r = 0; r < h.tri_ranges.size(); ++r) {
                const int64_t first = h.tri_ranges[r].first, cnt = h.tri_ranges[r].second;
                std::memcpy(&tp[w * 9], d->tri_p + first * 9, sizeof(float) * 9 * (size_t)cnt);
                std::memcpy(&tn[w * 9], d->tri_n + first * 9, sizeof(float) * 9 * (size_t)cnt);
                if (has_uv) std::memcpy(&tuv[w * 6], d->tri_uv + first * 6, sizeof(float) * 6 * (size_t)cnt);
                for (int64_t i = 0; i < cnt; ++i) {
                    tm[w + i] = d->tri_mtl[first + i];
                    ti[w + i] = d->tri_id ? d->tri_id[first + i] : (int)i;
                }
                w += (size_t)cnt;
            }
            CK(ctx, cudaMemcpyAsync(base + o_tp, tp.data(), sizeof(float) * tp.size(), cudaMemcpyHostToDevice, s));
            CK(ctx, cudaMemcpyAsync(base + o_tn, tn.data(), sizeof(float) * tn.size(), cudaMemcpyHostToDevice, s));
            if (has_uv) CK(ctx, cudaMemcpyAsync(base + o_tuv, tuv.data(), sizeof(float) * tuv.size(), cudaMemcpyHostToDevice, s));
            CK(ctx, cudaMemcpyAsync(base + o_tm, tm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s));
            CK(ctx, cudaMemcpyAsync(base + o_ti, ti.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s));
            CK(ctx, cudaStreamSynchronize(s));   // the staging vectors go out of scope
        }
    }
    DevScene &H = sc->hdr;
    H.prims = (const DevPrim *)(base + o_prims);
    H.n_prims = (int)h.prims.size();
    H.n_linear = h.n_linear;
    H.n_tris = (int)n;
    H.n_leaves = (int)L;
    H.nodes = (const float4 *)(base + o_nodes);
    H.quads = (const float4 *)(base + o_quads);
    H.tri = (const float4 *)(base + o_tri);
    H.trin = (const float4 *)(base + o_trin);
    H.triuv = has_uv ? (const float2 *)(base + o_triuv) : nullptr;
    H.mtl = (const DevMaterial *)(base + o_mtl);
    H.lights = (const DevLight *)(base + o_lights);
    H.tex = (const DevTexture *)(base + o_tex);
    H.texels = (const uint8_t *)(base + o_texels);
    H.n_lights = (int)h.lights.size();
    H.n_mtl = (int)h.mtl.size();
    for (int k = 0; k < 3; ++k) H.env[k] = d->env_light[k];
    sc->d_hdr = (DevScene *)(base + o_hdr);
    {   // the small tables, sphere leaves, model range table and header: one page-locked copy
        CK(ctx, cudaEventSynchronize(ctx->ev_upload));   // the previous upload's copy has left the staging
        if (ctx->upload_stage_bytes < o_small) {
            if (ctx->upload_stage) CK(ctx, cudaFreeHost(ctx->upload_stage));
            ctx->upload_stage = nullptr;
            ctx->upload_stage_bytes = 0;
            CK(ctx, cudaMallocHost(&ctx->upload_stage, o_small));
            ctx->upload_stage_bytes = o_small;
        }
        char *st = (char *)ctx->upload_stage;
        auto put = [&](size_t o, const void *src, size_t bytes) {
            if (bytes) std::memcpy(st + o, src, bytes);
        };
        put(o_prims, h.prims.data(), sizeof(DevPrim) * h.prims.size());
        put(o_mtl, h.mtl.data(), sizeof(DevMaterial) * h.mtl.size());
        put(o_lights, h.lights.data(), sizeof(DevLight) * h.lights.size());
        put(o_tex, h.tex.data(), sizeof(DevTexture) * h.tex.size());
        put(o_texels, h.texels.data(), h.texels.size());
        put(o_objpos, h.obj_pos.data(), sizeof(float) * h.obj_pos.size());
        put(o_rng, range_tab.data(), sizeof(int) * range_tab.size());
        for (int j = 0; j < n_sph; ++j) {
            const DevPrim &p = h.prims[(size_t)(h.n_linear + j)];
            const int prim = h.n_linear + j;
            put(o_sph + sizeof(float4) * (size_t)j, &p.a, sizeof(float4));
            put(o_sphr + sizeof(float) * (size_t)j, &p.b.x, sizeof(float));
            put(o_sphp + sizeof(int) * (size_t)j, &prim, sizeof(int));
            put(o_spho + sizeof(int) * (size_t)j, &p.obj, sizeof(int));
        }
        put(o_hdr, &H, sizeof(DevScene));
        const int zero = 0;
        put(o_bad, &zero, sizeof zero);
        CK(ctx, cudaMemcpyAsync(base, st, o_small, cudaMemcpyHostToDevice, s));
        CK(ctx, cudaEventRecord(ctx->ev_upload, s));
    }
    if (n > 0)   // per-triangle object (and model-local id) from the range table just copied
        launch_tri_objects((const int *)(base + o_rng), (int)h.tri_ranges.size(), (int)n, (int *)(base + o_to),
                           (direct && !d->tri_id) ? (int *)(base + o_ti) : nullptr, s);
    CK(ctx, cudaGetLastError());
    sc->in.tri_p = (const float *)(base + o_tp);
    sc->in.tri_n = (const float *)(base + o_tn);
    sc->in.tri_uv = has_uv ? (const float *)(base + o_tuv) : nullptr;
    sc->in.tri_mtl = (const int *)(base + o_tm);
    sc->in.tri_id = (const int *)(base + o_ti);
    sc->in.tri_obj = (const int *)(base + o_to);
    sc->in.obj_pos = (const float *)(base + o_objpos);
    sc->in.n = (int)n;
    sc->in.sph = (const float4 *)(base + o_sph);
    sc->in.sph_r = (const float *)(base + o_sphr);
    sc->in.sph_prim = (const int *)(base + o_sphp);
    sc->in.sph_obj = (const int *)(base + o_spho);
    sc->in.n_sph = n_sph;
    sc->in.n_mtl = (int)h.mtl.size();
    sc->in.bad = (int *)(base + o_bad);
    sc->out.nodes = (float4 *)(base + o_nodes);
    sc->out.quads = (float4 *)(base + o_quads);
    sc->out.tri = (float4 *)(base + o_tri);
    sc->out.trin = (float4 *)(base + o_trin);
    sc->out.triuv = has_uv ? (float2 *)(base + o_triuv) : nullptr;
    sc->bytes = (int64_t)off;
    const int id = ctx->next_scene++;
    ctx->scenes[id] = std::move(sc);
    rc = rt_scene_rebuild(ctx, id);
    if (rc) {
        ctx->scenes.erase(id);
        return rc;
    }
    *scene_id = id;
    return RT_OK;
}

extern "C" int rt_scene_rebuild(rt_ctx *ctx, int32_t id)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    SceneDev &sc = *it->second;
    if (sc.n_leaves <= 0) {
        sc.build_ms = 0.0f;
        return RT_OK;
    }
    CK(ctx, ctx->lbvh_scratch.ensure(lbvh_scratch_bytes(sc.n_leaves)));
    cudaEvent_t a, b;
    CK(ctx, cudaEventCreate(&a));
    CK(ctx, cudaEventCreate(&b));
    {   // an error left by an earlier unchecked call would be mistaken for a build failure
        const cudaError_t stale = cudaGetLastError();
        if (stale != cudaSuccess)
            return ctx_fail(ctx, RT_ERR_CUDA, "CUDA error pending before the LBVH build: %s", cudaGetErrorString(stale));
    }
    if (sc.in.bad) CK(ctx, cudaMemsetAsync(sc.in.bad, 0, sizeof(int), ctx->stream));
    g_build_step = "";
    cudaEventRecord(a, ctx->stream);
    // the clustering build reads each round's survivor count through the page-locked flag buffer
    sc.in.cluster_count =
        ctx->build_mode == RT_BUILD_CLUSTER ? reinterpret_cast<int *>(reinterpret_cast<char *>(ctx->build_flag) + 48) : nullptr;
    cudaError_t e = lbvh_build(sc.in, sc.out, ctx->lbvh_scratch.p, ctx->stream, ctx->ev_shading);
    cudaEventRecord(b, ctx->stream);
    int bad = 0;
    if (e == cudaSuccess && sc.in.bad)
        e = cudaMemcpyAsync(ctx->build_flag, sc.in.bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && sc.in.bad) bad = *ctx->build_flag;
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "LBVH build (%s): %s", g_build_step, cudaGetErrorString(e));
    if (bad) return ctx_fail(ctx, RT_ERR_INVALID, "a triangle's material is outside the material table");
    sc.build_ms = ms;
    return RT_OK;
}

extern "C" int rt_scene_update_camera(rt_ctx *ctx, int32_t id, const rt_camera *cam)
{
    if (!ctx || !cam) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    it->second->camera = *cam;
    return RT_OK;
}

extern "C" int rt_scene_release(rt_ctx *ctx, int32_t id)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    spare_put(ctx, std::move(it->second->mem));   // reused in stream order, freed only when spares overflow
    ctx->scenes.erase(it);
    return RT_OK;
}

extern "C" int rt_scene_device_bytes(rt_ctx *ctx, int32_t id, int64_t *bytes)
{
    if (!ctx || !bytes) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    *bytes = it->second->bytes;
    return RT_OK;
}

extern "C" int rt_scene_build_ms(rt_ctx *ctx, int32_t id, float *ms)
{
    if (!ctx || !ms) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    *ms = it->second->build_ms;
    return RT_OK;
}

// ---- frames --------------------------------------------------------------------------------------------
int frame_alloc(rt_ctx *ctx, int32_t w, int32_t h, FrameDev &f)
{
    if (w <= 0 || h <= 0 || w > 16384 || h > 16384)
        return ctx_fail(ctx, RT_ERR_INVALID, "frame size %dx%d outside [1,16384]", w, h);
    const size_t np = (size_t)w * h;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += a256(bytes);
        return o;
    };
    const size_t o_acc = take(24 * np), o_rgb = take(12 * np), o_rgb8 = take(3 * np), o_po = take(4 * np),
                 o_pp = take(4 * np), o_pt = take(4 * np), o_ax = take(4 * ((size_t)w + h));
    spare_take(ctx, f.mem, off);
    CK(ctx, f.mem.ensure(off));
    char *b = (char *)f.mem.p;
    f.w = w, f.h = h;
    f.fb.acc = (long long *)(b + o_acc);
    f.fb.rgb = (float *)(b + o_rgb);
    f.fb.rgb8 = (uint8_t *)(b + o_rgb8);
    f.fb.plane_obj = (int *)(b + o_po);
    f.fb.plane_prim = (int *)(b + o_pp);
    f.fb.plane_t = (float *)(b + o_pt);
    f.fb.axis = (float *)(b + o_ax);
    f.bytes = (int64_t)off;
    return RT_OK;
}

extern "C" int rt_frame_create(rt_ctx *ctx, int32_t w, int32_t h, int32_t *frame_id)
{
    if (!ctx || !frame_id) return RT_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    std::unique_ptr<FrameDev> f(new FrameDev());
    int rc = frame_alloc(ctx, w, h, *f);
    if (rc) return rc;
    CK(ctx, cudaMemsetAsync(f->mem.p, 0, f->bytes, ctx->stream));
    const int id = ctx->next_frame++;
    ctx->frames[id] = std::move(f);
    *frame_id = id;
    return RT_OK;
}

extern "C" int rt_frame_release(rt_ctx *ctx, int32_t id)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->frames.find(id);
    if (it == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", id);
    spare_put(ctx, std::move(it->second->mem));
    ctx->frames.erase(it);
    return RT_OK;
}

extern "C" int rt_frame_device_ptrs(rt_ctx *ctx, int32_t id, void **rgb, void **rgb8)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->frames.find(id);
    if (it == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", id);
    if (rgb) *rgb = it->second->fb.rgb;
    if (rgb8) *rgb8 = it->second->fb.rgb8;
    return RT_OK;
}

extern "C" int rt_frame_download(rt_ctx *ctx, int32_t id, float *rgb, uint8_t *rgb8, int32_t *hit_obj,
                                 int32_t *hit_prim, float *hit_t)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->frames.find(id);
    if (it == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", id);
    FrameDev &f = *it->second;
    const size_t np = (size_t)f.w * f.h;
    cudaStream_t s = ctx->stream;
    if (rgb) CK(ctx, cudaMemcpyAsync(rgb, f.fb.rgb, 12 * np, cudaMemcpyDeviceToHost, s));
    if (rgb8) CK(ctx, cudaMemcpyAsync(rgb8, f.fb.rgb8, 3 * np, cudaMemcpyDeviceToHost, s));
    if (hit_obj) CK(ctx, cudaMemcpyAsync(hit_obj, f.fb.plane_obj, 4 * np, cudaMemcpyDeviceToHost, s));
    if (hit_prim) CK(ctx, cudaMemcpyAsync(hit_prim, f.fb.plane_prim, 4 * np, cudaMemcpyDeviceToHost, s));
    if (hit_t) CK(ctx, cudaMemcpyAsync(hit_t, f.fb.plane_t, 4 * np, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaStreamSynchronize(s));
    return RT_OK;
}

// ---- workspace --------------------------------------------------------------------------------------------
int ws_ensure(rt_ctx *ctx, Workspace &ws, long long qcap, int njobs)
{
    // queue capacity x 8 lights must fit the shadow kernel's int work index
    if (qcap > (1ll << 27)) return ctx_fail(ctx, RT_ERR_OOM, "ray queue of %lld rays is too large", qcap);
    if (qcap <= ws.qcap && njobs <= ws.jobcap && ws.mem.p) return RT_OK;
    qcap = std::max(qcap, ws.qcap);
    njobs = std::max(njobs, ws.jobcap);
    cudaStreamSynchronize(ctx->stream);
    static std::atomic<unsigned long long> layouts{0};   // process-wide: no two layouts share a number
    ws.gen = ++layouts;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += a256(bytes);
        return o;
    };
    const size_t q = (size_t)qcap;
    size_t oq[2][4];
    for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 4; ++j) oq[k][j] = take(16 * q);
    size_t os[5];
    for (int j = 0; j < 5; ++j) os[j] = take(16 * q);
    size_t oh[5];
    for (int j = 0; j < 5; ++j) oh[j] = take(16 * q);
    const size_t o_nob = take(4 * q), o_ctr = take(kCounterBlockBytes),
                 o_jobs = take(sizeof(DevJob) * (size_t)njobs), o_end = take(8 * (size_t)njobs), o_tot = take(32),
                 o_scn = take(sizeof(DevScene) * (size_t)njobs);
    CK(ctx, ws.mem.ensure(off));
    char *b = (char *)ws.mem.p;
    for (int k = 0; k < 2; ++k) {
        ws.wf.q[k].o = (float4 *)(b + oq[k][0]);
        ws.wf.q[k].d = (float4 *)(b + oq[k][1]);
        ws.wf.q[k].w = (float4 *)(b + oq[k][2]);
        ws.wf.q[k].m = (int4 *)(b + oq[k][3]);
        ws.wf.q[k].capacity = (int)q;
    }
    ws.wf.sq.p = (float4 *)(b + os[0]);
    ws.wf.sq.n = (float4 *)(b + os[1]);
    ws.wf.sq.v = (float4 *)(b + os[2]);
    ws.wf.sq.wc = (float4 *)(b + os[3]);
    ws.wf.sq.ws = (float4 *)(b + os[4]);
    ws.wf.sq.capacity = (int)q;
    ws.wf.hq.o = (float4 *)(b + oh[0]);
    ws.wf.hq.d = (float4 *)(b + oh[1]);
    ws.wf.hq.w = (float4 *)(b + oh[2]);
    ws.wf.hq.m = (int4 *)(b + oh[3]);
    ws.wf.hq.h = (float4 *)(b + oh[4]);
    ws.wf.hq.nob = (int *)(b + o_nob);
    ws.wf.C = (Counters *)(b + o_ctr);
    ws.wf.shares = (int *)(b + o_ctr + ((sizeof(Counters) + 255) / 256) * 256);
    ws.jobs = (DevJob *)(b + o_jobs);
    ws.job_end = (long long *)(b + o_end);
    ws.scalars = (long long *)(b + o_tot);
    ws.scenes = (DevScene *)(b + o_scn);
    ws.wf.jobs = ws.jobs;
    ws.wf.job_sample_end = ws.job_end;
    ws.wf.total_samples = ws.scalars;
    ws.wf.sample_offset = ws.scalars + 1;
    ws.wf.n_jobs = ws.scalars + 2;
    ws.wf.max_lights = ws.scalars + 3;
    ws.wf.scenes = ws.scenes;
    ws.qcap = qcap;
    ws.jobcap = njobs;
    return RT_OK;
}

// ---- jobs ---------------------------------------------------------------------------------------------------
int make_job(rt_ctx *ctx, const SceneDev &sc, FrameDev &f, const rt_render_desc *rd, int scene_slot, DevJob &J,
             long long &samples)
{
    if (!rd) return ctx_fail(ctx, RT_ERR_INVALID, "render desc is NULL");
    const rt_camera &cam = rd->camera ? *rd->camera : sc.camera;
    const int W = rd->width > 0 ? rd->width : cam.width, H = rd->height > 0 ? rd->height : cam.height;
    if (W != f.w || H != f.h) return ctx_fail(ctx, RT_ERR_INVALID, "frame is %dx%d but the render is %dx%d", f.w, f.h, W, H);
    if (rd->spp < 1 || rd->spp > 1024) return ctx_fail(ctx, RT_ERR_INVALID, "spp %d outside [1,1024]", rd->spp);
    if (rd->max_level < 0 || rd->max_level > 4) return ctx_fail(ctx, RT_ERR_INVALID, "max_level %d outside [0,4]", rd->max_level);
    const int mode = rd->mode;
    if (!(mode >= RT_MODE_CHECK && mode <= RT_MODE_REFRACT) && mode != RT_MODE_RAYTRACE)
        return ctx_fail(ctx, RT_ERR_INVALID, "render mode 0x%x is not supported", rd->mode);
    if (!(cam.fovy > 0 && cam.fovy < 180) || !finite3(cam.position) || !finite3(cam.n))
        return ctx_fail(ctx, RT_ERR_INVALID, "camera is not valid");
    J = DevJob{};
    J.scene = scene_slot;
    J.width = W, J.height = H, J.spp = rd->spp;
    // the test modes but reflect and refract look at the first hit only (RayTracer.cpp:81-320)
    const bool recursive = mode == RT_MODE_RAYTRACE || mode == RT_MODE_REFRACT || mode == RT_MODE_REFLECT;
    J.max_level = recursive ? rd->max_level : 0, J.flags = rd->flags, J.mode = mode;
    J.xlim = (rd->flags & RT_FLAG_REF_TILES) ? (W / 64) * 64 : W;
    J.ylim = (rd->flags & RT_FLAG_REF_TILES) ? (H / 64) * 64 : H;
    J.acc = f.fb.acc;
    J.axis = rd->spp == 1 ? f.fb.axis : nullptr;
    if (rd->flags & RT_FLAG_HIT_PLANES) {
        J.plane_obj = f.fb.plane_obj, J.plane_prim = f.fb.plane_prim, J.plane_t = f.fb.plane_t;
    }
    for (int k = 0; k < 3; ++k) {
        J.cam_pos[k] = cam.position[k], J.cam_u[k] = cam.u[k], J.cam_v[k] = cam.v[k], J.cam_n[k] = cam.n[k];
    }
    const double PIr = 3.1415926535897932384;
    J.dp = std::tan(cam.fovy * PIr / 360) / (H / 2);
    J.znear = cam.znear;
    J.zfar = (float)(std::sqrt(2.0) * (double)cam.zfar);
    J.seed = rd->seed;
    J.slot = -1;
    samples = (long long)J.xlim * J.ylim * J.spp;
    return RT_OK;
}

FrameJob frame_job(const FrameBufs &fb, int w, int h, const DevJob &J)
{
    FrameJob F{};
    F.fb = fb;
    F.npix = (long long)w * h;
    F.quad_end = (F.npix + 3) / 4;
    F.scale_bits = resolve_scale_bits(J.spp);
    if (J.axis) std::memcpy(&F.dp_bits, &J.dp, sizeof F.dp_bits);
    F.w = w, F.h = h;
    F.planes = J.plane_obj != nullptr;
    return F;
}

// enqueue the level loop of one wave whose jobs are already in the workspace
void enqueue_levels(rt_ctx *ctx, Workspace &ws, int max_level, const Tuning &t, cudaStream_t s, KernelProfiler *prof)
{
    (void)ctx;
    auto B = [&](int kind) {
        if (prof) prof->begin(kind, s);
    };
    auto E = [&]() {
        if (prof) prof->end(s);
    };
    for (int level = 0; level <= max_level; ++level) {
        const int sel = level & 1;
        B(RT_KERNEL_EXTEND);
        launch_extend(ws.wf, sel, level, level == 0, t, s);
        E();
        B(RT_KERNEL_SHADE);
        launch_shade(ws.wf, sel, level, t, s);
        E();
        B(RT_KERNEL_SHADOW);
        launch_shadow(ws.wf, level, t, s);
        E();
    }
}

// the level loop of a plain render as a CUDA graph, captured once per (depth, tuning) and
// recaptured when the workspace moves
static int plain_graph(rt_ctx *ctx, int max_level, const Tuning &t, cudaGraphExec_t &exec)
{
    Workspace &ws = ctx->ws;
    if (ctx->plain_graph_gen != ws.gen) {
        ctx->plain_graphs.clear();
        ctx->plain_graph_gen = ws.gen;
    }
    const long long key = tuning_key(max_level, t);
    auto it = ctx->plain_graphs.find(key);
    if (it != ctx->plain_graphs.end()) {
        exec = it->second->exec;
        return RT_OK;
    }
    cudaStream_t cap;
    CK(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaMemsetAsync(ws.wf.C, 0, kCounterBlockBytes, cap);
    enqueue_levels(ctx, ws, max_level, t, cap, nullptr);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    std::unique_ptr<GraphEntry> ge(new GraphEntry());
    e = cudaGraphInstantiate(&ge->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    exec = ge->exec;
    ctx->plain_graphs[key] = std::move(ge);
    return RT_OK;
}

static int render_once(rt_ctx *ctx, SceneDev &sc, FrameDev &f, const rt_render_desc *rd, long long qcap,
                       unsigned long long cancel_mark)
{
    DevJob J;
    long long samples = 0;
    int rc = make_job(ctx, sc, f, rd, 0, J, samples);
    if (rc) return rc;
    J.pixel_tile = ctx->plain_tuning.pixel_tile;
    if (qcap <= 0) qcap = ctx->test_queue > 0 ? ctx->test_queue : std::max<long long>(2 * samples, 4096);
    rc = ws_ensure(ctx, ctx->ws, qcap, 1);
    if (rc) return rc;
    Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    ws.wf.cancel = ctx->cancel_dev;
    rc = cancel_arm(ctx, cancel_mark);
    if (rc) return rc;
    // the job tables (job, its sample end, the wave scalars, the scene header) go up in one copy
    // from page-locked memory laid out as in the workspace
    char *dst = (char *)ws.jobs;
    const size_t span = (size_t)((char *)ws.scenes + sizeof(DevScene) - dst);
    if (span > kPlainStageBytes) return ctx_fail(ctx, RT_ERR_INVALID, "job tables of %zu bytes exceed the staging", span);
    CK(ctx, cudaEventSynchronize(ctx->ev_staged));   // the previous render's copy has left the staging
    char *st = (char *)ctx->plain_stage;
    const long long end = samples, scal[4] = {samples, 0, 1, sc.hdr.n_lights};
    std::memcpy(st + ((char *)ws.jobs - dst), &J, sizeof J);
    std::memcpy(st + ((char *)ws.job_end - dst), &end, sizeof end);
    std::memcpy(st + ((char *)ws.scalars - dst), scal, sizeof scal);
    std::memcpy(st + ((char *)ws.scenes - dst), &sc.hdr, sizeof(DevScene));
    CK(ctx, cudaEventRecord(ctx->ev_start, s));
    CK(ctx, cudaMemcpyAsync(dst, st, span, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaEventRecord(ctx->ev_staged, s));
    KernelProfiler &P = ctx->prof;
    const bool profile = (rd->flags & RT_FLAG_PROFILE) != 0;
    P.reset(profile);
    P.begin(RT_KERNEL_OTHER, s);
    launch_frame_prepare(frame_job(f.fb, f.w, f.h, J), s);
    P.end(s);
    Tuning t = ctx->plain_tuning;
    t.count = (rd->flags & RT_FLAG_COUNT_WORK) != 0;
    ctx->stamped = false;
    if (profile) {   // kernels one by one between events, warps stamping their start and end
        CK(ctx, cudaMemsetAsync(ws.wf.C, 0, kCounterBlockBytes, s));
        CK(ctx, ctx->stamps.ensure(kStampBytes));
        CK(ctx, cudaMemsetAsync(ctx->stamps.p, 0, kStampBytes, s));
        ws.wf.stamps = (unsigned long long *)ctx->stamps.p;
        enqueue_levels(ctx, ws, rd->max_level, t, s, &P);
        ws.wf.stamps = nullptr;   // launches copied their parameters; captured graphs never stamp
        ctx->stamped = true;
    } else {
        cudaGraphExec_t exec = nullptr;
        rc = plain_graph(ctx, rd->max_level, t, exec);
        if (rc) return rc;
        CK(ctx, cudaGraphLaunch(exec, s));
        // launches of the captured sequence, as the profiler would count them
        P.launches[RT_KERNEL_EXTEND] = P.launches[RT_KERNEL_SHADE] = P.launches[RT_KERNEL_SHADOW] = rd->max_level + 1;
    }
    P.begin(RT_KERNEL_RESOLVE, s);
    launch_resolve(f.fb, f.w, f.h, rd->spp, s);
    P.end(s);
    CK(ctx, cudaGetLastError());
    CK(ctx, cudaMemcpyAsync(ctx->counters_host, ws.wf.C, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaEventRecord(ctx->ev_stop, s));
    return RT_OK;
}

// rt_render, cancelled by any rt_cancel counted after `cancel_mark`
static int render_since(rt_ctx *ctx, unsigned long long cancel_mark, int32_t scene_id, int32_t frame_id,
                        const rt_render_desc *rd)
{
    if (!ctx) return RT_ERR_INVALID;
    auto si = ctx->scenes.find(scene_id);
    if (si == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", scene_id);
    auto fi = ctx->frames.find(frame_id);
    if (fi == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown frame %d", frame_id);
    CK(ctx, cudaSetDevice(ctx->device));
    ctx->pending = Pending{scene_id, frame_id, rd ? *rd : rt_render_desc{}, true, 0};
    int rc = render_once(ctx, *si->second, *fi->second, rd, 0, cancel_mark);
    if (rc) ctx->pending.active = false;
    return rc;
}

extern "C" int rt_render(rt_ctx *ctx, int32_t scene_id, int32_t frame_id, const rt_render_desc *rd)
{
    if (!ctx) return RT_ERR_INVALID;
    return render_since(ctx, ctx->cancel_count.load(), scene_id, frame_id, rd);
}

// From the warp stamps of a profiled render: per kernel kind, the share of its launches' warp
// time (warps x launch span) spent before a warp's block started or after the warp ran out of
// work. A warp that never ran has no stamps and does not count.
static int idle_shares(rt_ctx *ctx, float *idle)
{
    std::vector<unsigned long long> st(kStampBytes / sizeof(unsigned long long));
    CK(ctx, cudaMemcpy(st.data(), ctx->stamps.p, kStampBytes, cudaMemcpyDeviceToHost));
    double wasted[3] = {0, 0, 0}, total[3] = {0, 0, 0};
    for (int slot = 0; slot < 15; ++slot) {
        const unsigned long long *p = st.data() + 2ull * slot * kMaxStampWarps;
        unsigned long long t0 = ~0ull, t1 = 0;
        long long warps = 0;
        for (int w = 0; w < kMaxStampWarps; ++w) {
            if (!p[2 * w + 1]) continue;
            t0 = std::min(t0, ~p[2 * w]);
            t1 = std::max(t1, p[2 * w + 1]);
            ++warps;
        }
        if (!warps || t1 <= t0) continue;
        double w_idle = 0;
        for (int w = 0; w < kMaxStampWarps; ++w)
            if (p[2 * w + 1]) w_idle += (double)((~p[2 * w]) - t0) + (double)(t1 - p[2 * w + 1]);
        wasted[slot % 3] += w_idle;
        total[slot % 3] += (double)warps * (double)(t1 - t0);
    }
    const int kind[3] = {RT_KERNEL_EXTEND, RT_KERNEL_SHADE, RT_KERNEL_SHADOW};
    for (int k = 0; k < 3; ++k) idle[kind[k]] = total[k] > 0 ? (float)(wasted[k] / total[k]) : 0.0f;
    return RT_OK;
}

extern "C" int rt_render_wait(rt_ctx *ctx, rt_render_stats *stats)
{
    if (!ctx) return RT_ERR_INVALID;
    CK(ctx, cudaEventSynchronize(ctx->ev_stop));
    int retries = 0;
    while (ctx->pending.active && ctx->counters_host->overflow) {
        if (++retries > 4) return ctx_fail(ctx, RT_ERR_OVERFLOW, "ray queues overflowed after %d retries", retries - 1);
        auto si = ctx->scenes.find(ctx->pending.scene);
        auto fi = ctx->frames.find(ctx->pending.frame);
        if (si == ctx->scenes.end() || fi == ctx->frames.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "render target released");
        int rc = render_once(ctx, *si->second, *fi->second, &ctx->pending.rd, ctx->ws.qcap * 2, ctx->cancel_base);
        if (rc) {
            ctx->pending.active = false;
            return rc;
        }
        CK(ctx, cudaEventSynchronize(ctx->ev_stop));
    }
    ctx->pending.retries = retries;
    const bool was_cancelled = cancel_requested(ctx);
    if (stats) {
        const Counters &C = *ctx->counters_host;
        stats->rays_primary = (int64_t)C.rays_primary;
        stats->rays_secondary = (int64_t)C.rays_secondary;
        stats->rays_shadow = (int64_t)C.rays_shadow;
        stats->nodes_visited = (int64_t)C.nodes;
        stats->tris_tested = (int64_t)C.tris;
        stats->spheres_tested = (int64_t)C.spheres;
        stats->shadow_nodes_visited = (int64_t)C.s_nodes;
        stats->shadow_tris_tested = (int64_t)C.s_tris;
        stats->shadow_spheres_tested = (int64_t)C.s_spheres;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
        stats->ms = ms;
        stats->overflow_retries = retries;
        ctx->prof.collect(stats->kernel_ms);
        for (int k = 0; k < RT_KERNEL_KINDS; ++k) stats->kernel_launches[k] = ctx->prof.launches[k], stats->kernel_idle[k] = 0;
        if (ctx->stamped) {
            int rc = idle_shares(ctx, stats->kernel_idle);
            if (rc) return rc;
        }
    }
    ctx->pending.active = false;
    if (was_cancelled) return ctx_fail(ctx, RT_ERR_CANCELLED, "render cancelled");
    if (ctx->counters_host->error)
        return ctx_fail(ctx, RT_ERR_CUDA, "traversal stopped on a corrupt LBVH (flags 0x%x)", ctx->counters_host->error);
    return RT_OK;
}

// shared by the plain path and the batch path: tuning values a kernel launch accepts
int tuning_from(rt_ctx *ctx, const rt_batch_tuning *in, Tuning &t)
{
    if (!in) return RT_OK;
    if (in->block) t.block = in->block;
    if (in->tile) t.tile = in->tile;
    t.stack = in->stack;
    t.min_blocks = in->min_blocks;
    t.shadow_chunk = in->shadow_chunk;
    t.pixel_tile = in->pixel_tile;
    if (in->lanes) t.lanes = in->lanes;
    if (t.lanes != 1 && t.lanes != 2) return ctx_fail(ctx, RT_ERR_INVALID, "lanes %d: use 0 (default), 1 or 2", t.lanes);
    if (in->dynamic < 0 || in->dynamic > 3) return ctx_fail(ctx, RT_ERR_INVALID, "dynamic %d: use 0..3", in->dynamic);
    t.dynamic = in->dynamic != 2;
    t.shares = in->dynamic == 3;
    if (t.block % 32 || t.block < 32 || t.block > 256 || t.tile % 32 || t.tile <= 0 || t.tile > 4096)
        return ctx_fail(ctx, RT_ERR_INVALID, "tuning block %d / tile %d not supported", t.block, t.tile);
    if (t.min_blocks != 0 && t.min_blocks != 6 && t.min_blocks != 8)
        return ctx_fail(ctx, RT_ERR_INVALID, "min_blocks %d: use 0, 6 or 8", t.min_blocks);
    if (t.min_blocks && t.block > 128) return ctx_fail(ctx, RT_ERR_INVALID, "min_blocks needs blocks of at most 128 threads");
    if (t.stack != 0 && t.stack != 8)
        return ctx_fail(ctx, RT_ERR_INVALID, "stack %d: use 0 or 8 shared-memory entries", t.stack);
    if (t.shadow_chunk < 0 || t.shadow_chunk % 32 || t.shadow_chunk > (1 << 27))
        return ctx_fail(ctx, RT_ERR_INVALID, "shadow_chunk %d: a multiple of 32 in [0, 2^27]", t.shadow_chunk);
    if (t.pixel_tile < 0 || t.pixel_tile == 1 || t.pixel_tile > 64)
        return ctx_fail(ctx, RT_ERR_INVALID, "pixel_tile %d: 0 or 2..64", t.pixel_tile);
    return RT_OK;
}

// key of a captured level loop: every tuning value a launch in it depends on
long long tuning_key(int max_level, const Tuning &t)
{
    return (long long)max_level | (long long)(t.block / 32) << 3 | (long long)(t.tile / 32) << 7 |
           (long long)t.stack << 15 | (long long)t.dynamic << 20 | (long long)t.min_blocks << 21 |
           (long long)t.count << 25 | (long long)(t.shadow_chunk / 32) << 26 | (long long)t.pixel_tile << 48 |
           (long long)t.shares << 56;
}

extern "C" int rt_ctx_get_tuning(const rt_ctx *ctx, rt_batch_tuning *out)
{
    if (!ctx || !out) return RT_ERR_INVALID;
    const Tuning &t = ctx->plain_tuning;
    *out = rt_batch_tuning{t.block, t.tile, t.stack, 1, t.min_blocks, t.dynamic ? (t.shares ? 3 : 1) : 2, 0,
                           t.shadow_chunk, t.pixel_tile, t.lanes, 0};
    return RT_OK;
}

extern "C" int rt_ctx_set_tuning(rt_ctx *ctx, const rt_batch_tuning *tuning)
{
    if (!ctx) return RT_ERR_INVALID;
    Tuning t;
    if (tuning) {
        int rc = tuning_from(ctx, tuning, t);
        if (rc) return rc;
    }
    ctx->plain_tuning = t;
    return RT_OK;
}

extern "C" int rt_cancel(rt_ctx *ctx)
{
    if (!ctx) return RT_ERR_INVALID;
    // callable from any thread: the write goes on the context's device, the caller's current
    // device is left as it was
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    std::lock_guard<std::mutex> lock(ctx->cancel_mu);
    ctx->cancel_count.fetch_add(1);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->cancel_dev, ctx->cancel_vals + 1, sizeof(int), cudaMemcpyHostToDevice, ctx->side);
    if (prev >= 0 && prev != ctx->device) cudaSetDevice(prev);
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "rt_cancel: %s", cudaGetErrorString(e));
    return RT_OK;
}

extern "C" uint64_t rt_cancel_mark(rt_ctx *ctx) { return ctx ? (uint64_t)ctx->cancel_count.load() : 0; }

extern "C" int rt_poll(rt_ctx *ctx)
{
    if (!ctx) return RT_ERR_INVALID;
    cudaError_t e = cudaEventQuery(ctx->ev_stop);
    if (e == cudaErrorNotReady) return 0;
    if (e != cudaSuccess) return ctx_fail(ctx, RT_ERR_CUDA, "%s", cudaGetErrorString(e));
    return 1;
}

extern "C" int rt_render_host_since(rt_ctx *ctx, uint64_t cancel_mark, const rt_scene_desc *desc,
                                    const rt_render_desc *rd, uint8_t *out_rgb8, float *out_rgb, rt_render_stats *stats)
{
    if (!ctx || !desc || !rd) return RT_ERR_INVALID;
    // a cancel that came before or between the stages ends the call there; one that comes
    // while the kernels run stops them through the device flag
    auto cancelled = [&] {
        if (ctx->cancel_count.load() == cancel_mark) return false;
        ctx_fail(ctx, RT_ERR_CANCELLED, "render cancelled");
        return true;
    };
    if (cancelled()) return RT_ERR_CANCELLED;
    int32_t sid = -1, fid = -1;
    int rc = rt_scene_upload(ctx, desc, &sid);
    if (rc) return rc;
    const rt_camera &cam = rd->camera ? *rd->camera : desc->camera;
    const int W = rd->width > 0 ? rd->width : cam.width, H = rd->height > 0 ? rd->height : cam.height;
    rc = cancelled() ? RT_ERR_CANCELLED : rt_frame_create(ctx, W, H, &fid);
    if (!rc) rc = render_since(ctx, cancel_mark, sid, fid, rd);
    if (!rc) rc = rt_render_wait(ctx, stats);
    if (!rc) rc = rt_frame_download(ctx, fid, out_rgb, out_rgb8, nullptr, nullptr, nullptr);
    if (fid >= 0) rt_frame_release(ctx, fid);
    rt_scene_release(ctx, sid);
    return rc;
}

extern "C" int rt_render_host(rt_ctx *ctx, const rt_scene_desc *desc, const rt_render_desc *rd, uint8_t *out_rgb8,
                              float *out_rgb, rt_render_stats *stats)
{
    return rt_render_host_since(ctx, rt_cancel_mark(ctx), desc, rd, out_rgb8, out_rgb, stats);
}

// ---- LBVH test hooks ------------------------------------------------------------------------------------------
extern "C" int rt_morton_sort(rt_ctx *ctx, const float *tri_p, int64_t n, uint32_t *codes, uint32_t *perm)
{
    if (!ctx || (n > 0 && (!tri_p || !codes || !perm)) || n < 0 || n >= (1ll << 30)) return RT_ERR_INVALID;
    if (n == 0) return RT_OK;
    CK(ctx, cudaSetDevice(ctx->device));
    DevBuf buf;
    const size_t o_p = 0, o_o = a256(36 * (size_t)n), o_pos = o_o + a256(4 * (size_t)n), o_c = o_pos + 256,
                 o_pm = o_c + a256(4 * (size_t)n), end = o_pm + a256(4 * (size_t)n);
    CK(ctx, buf.ensure(end));
    CK(ctx, ctx->lbvh_scratch.ensure(lbvh_scratch_bytes((int)n)));
    char *b = (char *)buf.p;
    cudaStream_t s = ctx->stream;
    CK(ctx, cudaMemcpyAsync(b + o_p, tri_p, 36 * (size_t)n, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemsetAsync(b + o_o, 0, 4 * (size_t)n, s));
    CK(ctx, cudaMemsetAsync(b + o_pos, 0, 256, s));
    LbvhInput in{};
    in.tri_p = (const float *)(b + o_p);
    in.tri_obj = (const int *)(b + o_o);
    in.obj_pos = (const float *)(b + o_pos);
    in.n = (int)n;
    CK(ctx, lbvh_morton_sort(in, (uint32_t *)(b + o_c), (uint32_t *)(b + o_pm), ctx->lbvh_scratch.p, s));
    CK(ctx, cudaMemcpyAsync(codes, b + o_c, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaMemcpyAsync(perm, b + o_pm, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaStreamSynchronize(s));
    return RT_OK;
}

extern "C" int rt_scene_bvh_download(rt_ctx *ctx, int32_t id, float *nodes, uint32_t *perm, int64_t *n_nodes)
{
    if (!ctx) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", id);
    SceneDev &sc = *it->second;
    const int64_t n = sc.n_leaves, nn = n > 0 ? 2 * n - 1 : 0;
    if (n_nodes) *n_nodes = nn;
    cudaStream_t s = ctx->stream;
    if (nodes && nn) CK(ctx, cudaMemcpyAsync(nodes, sc.out.nodes, 32 * (size_t)nn, cudaMemcpyDeviceToHost, s));
    if (perm && n) {   // original triangle order = reported id is not unique, so read p0.w of each slot
        std::vector<float4> tri((size_t)n * 3);
        CK(ctx, cudaMemcpyAsync(tri.data(), sc.out.tri, 48 * (size_t)n, cudaMemcpyDeviceToHost, s));
        CK(ctx, cudaStreamSynchronize(s));
        for (int64_t k = 0; k < n; ++k) {   // triangle: its reported id; sphere: 0x80000000 | primitive
            int32_t id32, tag;
            std::memcpy(&id32, &tri[(size_t)k * 3].w, 4);
            std::memcpy(&tag, &tri[(size_t)k * 3 + 2].w, 4);
            perm[k] = tag >= 0 ? (uint32_t)id32 : (0x80000000u | (uint32_t)(-1 - tag));
        }
    }
    CK(ctx, cudaStreamSynchronize(s));
    return RT_OK;
}

// ---- test hooks: a corrupt hierarchy, a queue too small for the frame -------------------------------------
extern "C" int rt_scene_test_set_node_refs(rt_ctx *ctx, int32_t scene_id, int32_t node, const int32_t *refs)
{
    if (!ctx || !refs) return RT_ERR_INVALID;
    auto it = ctx->scenes.find(scene_id);
    if (it == ctx->scenes.end()) return ctx_fail(ctx, RT_ERR_NOT_FOUND, "unknown scene %d", scene_id);
    SceneDev &sc = *it->second;
    const int L = sc.n_leaves;
    if (L < 2 || node < 0 || node > L - 2) return ctx_fail(ctx, RT_ERR_INVALID, "node %d outside 0..%d", node, L - 2);
    for (int k = 0; k < 4; ++k) {   // only existing nodes and leaves: the changed tree reads nothing outside itself
        const int c = refs[k];
        if (c >= 0 ? c > L - 2 : ~c >= L) return ctx_fail(ctx, RT_ERR_INVALID, "reference %d outside the tree", c);
    }
    CK(ctx, cudaSetDevice(ctx->device));
    float4 *slot = const_cast<float4 *>(sc.hdr.quads) + 8ll * node + 6;   // the record's child references
    CK(ctx, cudaMemcpyAsync(slot, refs, 4 * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return RT_OK;
}

extern "C" int rt_ctx_test_queue_entries(rt_ctx *ctx, int64_t entries)
{
    if (!ctx || entries < 0 || entries > (1ll << 27)) return RT_ERR_INVALID;
    ctx->test_queue = entries;
    return RT_OK;
}

// ---- test hook: the kernels' integer-exact conversions ------------------------------------------------------
extern "C" int rt_selftest_conversions(rt_ctx *ctx, const int64_t *x, int32_t n, double d, const float *v,
                                       float *out_mul, int64_t *out_fix)
{
    if (!ctx || n < 0 || (n && (!x || !v || !out_mul || !out_fix)) || !(d > 0) || !std::isfinite(d))
        return RT_ERR_INVALID;
    if (n == 0) return RT_OK;
    CK(ctx, cudaSetDevice(ctx->device));
    DevBuf buf;
    const size_t nn = (size_t)n;
    CK(ctx, buf.ensure(nn * (8 + 4 + 4 + 8)));
    char *b = (char *)buf.p;
    long long *dx = (long long *)b;
    long long *dfix = (long long *)(b + 8 * nn);
    float *dv = (float *)(b + 16 * nn), *dmul = (float *)(b + 20 * nn);
    unsigned long long bits;
    std::memcpy(&bits, &d, sizeof bits);
    cudaStream_t s = ctx->stream;
    CK(ctx, cudaMemcpyAsync(dx, x, 8 * nn, cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(dv, v, 4 * nn, cudaMemcpyHostToDevice, s));
    launch_selftest_conversions(dx, n, bits, dv, dmul, dfix, s);
    CK(ctx, cudaGetLastError());
    CK(ctx, cudaMemcpyAsync(out_mul, dmul, 4 * nn, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaMemcpyAsync(out_fix, dfix, 8 * nn, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaStreamSynchronize(s));
    return RT_OK;
}
