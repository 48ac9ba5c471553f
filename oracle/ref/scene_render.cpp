// scene_render.cpp — builds the scene of tests/cpp/scene_render_sequence.inc with the
// reference's own classes and renders it with the reference's RayTracer::start
// (RayTracer.cpp:614-696), writing the uint8 output region to argv[1] (rows in the output's
// bottom-up order). TEST INFRASTRUCTURE ONLY: compiled from the reference sources by
// oracle/ref/Makefile into oracle/_ref/rt_ref_scene_render; its image is the golden
// tests/golden/scene_api/render_ref.npz (tests/golden/make_scene_api_golden.py).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "RayTracer.h"
#include "Scene.h"

#include "../../tests/cpp/scene_render_sequence.inc"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    const int mode = argc > 2 ? (int)std::strtol(argv[2], nullptr, 0) : MY_MODEL_RAYTRACE;
    const int variant = argc > 3 ? std::atoi(argv[3]) : 0;
    if (variant < 0 || variant >= kRenderVariants) return 2;
    Scene scene;
    build_render_scene(scene, variant);
    RayTracer rt(scene);
    rt.maxLevel = kRenderLevel;
    const unsigned hc = std::thread::hardware_concurrency();
    rt.start((uint8_t)mode, (int8_t)(hc == 0 ? 1 : hc > 32 ? 32 : hc));
    while (!rt.isFinish) std::this_thread::sleep_for(std::chrono::milliseconds(1));
    const int W = rt.width, H = rt.height;
    std::vector<uint8_t> img((size_t)W * H * 3);
    for (int row = 0; row < H; ++row)
        std::memcpy(&img[(size_t)row * W * 3], rt.output + (size_t)row * 3 * W, (size_t)W * 3);
    FILE *f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    std::fwrite(img.data(), 1, img.size(), f);
    std::fclose(f);
    std::printf("{\"width\": %d, \"height\": %d, \"mode\": %d, \"variant\": %d, \"objects\": %d, \"lights\": %d}\n", W, H, mode, variant,
                (int)scene.Objects.size(), (int)scene.Lights.size());
    return 0;
}
