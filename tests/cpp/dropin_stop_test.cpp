// RayTracer::stop() through the drop-in API: a stop() made right after start() ends that render
// (the reference sets isRun in start() before its threads run, RayTracer.cpp:614-617, and each
// pixel checks it, :29-33), a stop() made before start() does not affect the next render, and a
// cancelled render leaves `output` as start() set it (all 127). Prints one JSON line.
// Usage: dropin_stop_test
#include <chrono>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../raytrace_gb300/cpp/RayTracer.h"

static double wait_finish(RayTracer &rt, double limit_s)
{
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rt.isFinish || s > limit_s) return s;
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

static bool output_untouched(const RayTracer &rt)
{
    const size_t n = (size_t)rt.width * rt.height * 3;
    for (size_t i = 0; i < n; ++i)
        if (rt.output[i] != 127) return false;
    return true;
}

int main()
{
    // a 700x700-cell height grid (980,000 triangles) under two spheres: upload and hierarchy
    // build alone take milliseconds, so a stop() lands long before the kernels would start
    Scene scene;
    scene.AddPlane();
    uint8_t a = scene.AddSphere(1.0f);
    scene.MovePos(MY_MODEL_OBJECT, a, Vertex(-1.5f, 1.5f, 0.5f));
    uint8_t b = scene.AddSphere(0.7f);
    scene.MovePos(MY_MODEL_OBJECT, b, Vertex(1.2f, 1.3f, -0.5f));
    scene.ChgMtl(b, scene.MtlLiby[4]);
    const int G = 700;
    std::vector<Vertex> P((size_t)(G + 1) * (G + 1));
    for (int z = 0; z <= G; ++z)
        for (int x = 0; x <= G; ++x) {
            const float fx = -6.0f + 12.0f * x / G, fz = -6.0f + 12.0f * z / G;
            P[(size_t)z * (G + 1) + x] = Vertex(fx, 0.3f + 0.2f * (float)((x * 7 + z * 13) % 17) / 17.0f, fz);
        }
    std::vector<Triangle> tris;
    tris.reserve((size_t)2 * G * G);
    const Normal up(Vertex(0, 1, 0));
    for (int z = 0; z < G; ++z)
        for (int x = 0; x < G; ++x) {
            const Vertex &p00 = P[(size_t)z * (G + 1) + x], &p10 = P[(size_t)z * (G + 1) + x + 1];
            const Vertex &p01 = P[(size_t)(z + 1) * (G + 1) + x], &p11 = P[(size_t)(z + 1) * (G + 1) + x + 1];
            tris.push_back(Triangle(p00, up, p01, up, p10, up));
            tris.push_back(Triangle(p10, up, p01, up, p11, up));
        }
    Model *m = new Model();
    m->setMesh(tris, scene.MtlLiby[0]);
    scene.AddObject(m);
    scene.AddLight(MY_LIGHT_POINT, Vertex(0.15f, 0.55f, 0.3f), Vertex(1.0f, 0.0f, 0.0f, 1.0f));
    scene.MovePos(MY_MODEL_LIGHT, 0, Vertex(-40, 30, -4));
    scene.cam.resize(1920, 1024);
    scene.cam.fovy = 60.0f;
    scene.cam.lookAt(Vertex(0, 5, -12), Vertex(0, 0.5f, 0));

    RayTracer rt(scene);
    rt.maxLevel = 4;

    // 1. a whole render, for its time
    rt.start(MY_MODEL_RAYTRACE, 8);
    const double full_s = wait_finish(rt, 60.0);
    const int full_status = rt.status();

    // 2. stop() at once after start(): cancelled, output untouched
    rt.start(MY_MODEL_RAYTRACE, 8);
    rt.stop();
    const double stop_s = wait_finish(rt, 60.0);
    const int stop_status = rt.status();
    const bool untouched = rt.isFinish && output_untouched(rt);

    // 3. stop() with nothing running, then start(): the earlier stop() does not end it
    rt.stop();
    rt.start(MY_MODEL_RAYTRACE, 8);
    const double after_s = wait_finish(rt, 60.0);
    const int after_status = rt.status();
    const bool written = rt.isFinish && !output_untouched(rt);

    std::printf("{\"full_s\": %.6f, \"full_status\": %d, \"stop_s\": %.6f, \"stop_status\": %d, \"untouched\": %d, "
                "\"after_s\": %.6f, \"after_status\": %d, \"written\": %d}\n",
                full_s, full_status, stop_s, stop_status, (int)untouched, after_s, after_status, (int)written);
    return 0;
}
