// RayTracer.cpp — the drop-in RayTracer on top of rt_render_host.
#include "RayTracer.h"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

static constexpr size_t kOutputBytes = 2048u * 2048u * 3u;   // the reference's fixed buffer

RayTracer::RayTracer(Scene &s, int device) : scene(&s), device_(device)
{
    output = new uint8_t[kOutputBytes];
    std::memset(output, 127, kOutputBytes);
    int rc = rt_ctx_create(device, &ctx);
    if (rc != RT_OK) {
        ctx = nullptr;
        status_ = rc;
        error_ = "no usable CUDA device for the renderer";
        std::fprintf(stderr, "RayTracer: %s (rt_ctx_create returned %d)\n", error_.c_str(), rc);
    }
}

RayTracer::~RayTracer()
{
    if (worker.joinable()) {
        if (ctx) rt_cancel(ctx);
        worker.join();
    }
    if (ctx) rt_ctx_destroy(ctx);
    delete[] output;
}

void RayTracer::start(const uint8_t type, const int8_t)
{
    if (worker.joinable()) worker.join();
    isFinish = false;
    width = scene->cam.width;
    height = scene->cam.height;
    std::memset(output, 127, kOutputBytes);
    // every mode of the reference's start() (RayTracer.cpp:629-662): the MY_MODEL_* values are
    // the RT_MODE_* values of the C ABI
    const int mode = ((type >= MY_MODEL_CHECK && type <= MY_MODEL_REFRACTTEST) || type == MY_MODEL_RAYTRACE) ? type : -1;
    if (!ctx || mode < 0 || width <= 0 || height <= 0 || width > 2048 || height > 2048) {
        status_ = !ctx ? RT_ERR_CUDA : RT_ERR_INVALID;
        error_ = !ctx ? "no usable CUDA device for the renderer"
                      : (mode < 0 ? "render mode not supported by the GPU renderer" : "camera size outside 1..2048");
        std::fprintf(stderr, "RayTracer::start: %s\n", error_.c_str());
        useTime = 0.0;
        isFinish = true;
        return;
    }
    // the scene is read now, so the caller may edit it once start() has returned
    flatten_scene(*scene, flat);
    const uint8_t level = maxLevel;
    // the cancel mark is taken here, before the render thread runs: a stop() from now on ends
    // this render even while the thread is still uploading the scene (the reference sets isRun
    // in start(), RayTracer.cpp:617)
    const uint64_t mark = rt_cancel_mark(ctx);
    worker = std::thread([this, mode, level, mark] {
        const int W = width, H = height;
        std::vector<uint8_t> img((size_t)W * H * 3);
        rt_render_desc rd{};
        rd.width = W, rd.height = H, rd.spp = 1, rd.max_level = level, rd.mode = mode;
        rd.flags = RT_FLAG_REF_TILES;
        const auto t0 = std::chrono::steady_clock::now();
        int rc = rt_render_host_since(ctx, mark, &flat.desc, &rd, img.data(), nullptr, nullptr);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rc == RT_OK) {
            const int bw = W / 64, bh = H / 64;
            for (int row = 0; row < bh * 64; ++row)
                std::memcpy(output + (size_t)row * 3 * W, img.data() + (size_t)row * 3 * W, (size_t)bw * 64 * 3);
        } else {
            error_ = rt_last_error(ctx);
        }
        status_ = rc;
        useTime = secs;
        isFinish = true;
    });
}

void RayTracer::stop()
{
    if (ctx) rt_cancel(ctx);
}
