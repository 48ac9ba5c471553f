// Builds a scene through the drop-in C++ API (Scene / objects / lights / RayTracer), renders it
// with RayTracer::start on the GPU, and writes (1) the uint8 `output` region and (2) the
// flattened scene, so the Python test can compare with the C ABI and the CPU oracle.
// Usage: dropin_test out.rgb8 scene.rtsc
#include <chrono>
#include <cstdio>
#include <thread>
#include <vector>

#include "../../raytrace_gb300/cpp/RayTracer.h"

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    Scene scene;
    scene.AddPlane();
    uint8_t a = scene.AddSphere(1.0f);
    scene.MovePos(MY_MODEL_OBJECT, a, Vertex(-1.5f, 0.0f, 0.5f));
    uint8_t b = scene.AddSphere(0.7f);
    scene.MovePos(MY_MODEL_OBJECT, b, Vertex(1.2f, 0.3f, -0.5f));
    scene.ChgMtl(b, scene.MtlLiby[4]);   // refractive preset
    uint8_t c = scene.AddSphere(0.4f);
    scene.MovePos(MY_MODEL_OBJECT, c, Vertex(0.0f, 2.0f, 1.0f));
    scene.ChgMtl(c, scene.MtlLiby[2]);   // mirror
    uint8_t d = scene.AddSphere(0.5f);
    scene.Switch(MY_MODEL_OBJECT, d, false);   // hidden object keeps its index
    uint8_t e = scene.AddCube(0.8f);
    scene.MovePos(MY_MODEL_OBJECT, e, Vertex(2.5f, 0.2f, 1.5f));
    // a small procedural mesh: an octahedron
    std::vector<Triangle> tris;
    Vertex P[6] = {Vertex(0, 1.6f, 2), Vertex(0, 0.4f, 2), Vertex(0.6f, 1, 2), Vertex(-0.6f, 1, 2), Vertex(0, 1, 2.6f), Vertex(0, 1, 1.4f)};
    int F[8][3] = {{0, 2, 4}, {0, 4, 3}, {0, 3, 5}, {0, 5, 2}, {1, 4, 2}, {1, 3, 4}, {1, 5, 3}, {1, 2, 5}};
    for (auto &f : F) {
        Normal n = Normal((P[f[1]] - P[f[0]]) * (P[f[2]] - P[f[0]]));
        tris.push_back(Triangle(P[f[0]], n, P[f[1]], n, P[f[2]], n));
    }
    Model *m = new Model();
    m->setMesh(tris, scene.MtlLiby[0]);
    scene.AddObject(m);
    scene.AddLight(MY_LIGHT_POINT, Vertex(0.15f, 0.55f, 0.3f), Vertex(1.0f, 0.0f, 0.0f, 1.0f));
    scene.MovePos(MY_MODEL_LIGHT, 0, Vertex(-40, 30, -4));
    uint8_t pl = scene.AddLight(MY_LIGHT_PARALLEL, Vertex(0.1f, 0.45f, 0.45f));
    scene.MovePos(MY_MODEL_LIGHT, pl, Vertex(-45, 45, 0));
    scene.cam.resize(192, 128);
    scene.cam.fovy = 60.0f;
    scene.cam.lookAt(Vertex(0, 3, -9), Vertex(0, 0.8f, 0));

    RayTracer rt(scene);
    rt.maxLevel = 3;
    rt.start(MY_MODEL_RAYTRACE, 4);
    while (!rt.isFinish) std::this_thread::sleep_for(std::chrono::milliseconds(1));
    if (rt.status() != RT_OK) {
        std::fprintf(stderr, "render failed: %d %s\n", rt.status(), rt.lastError().c_str());
        return 1;
    }
    FILE *f = std::fopen(argv[1], "wb");
    std::fwrite(rt.output, 1, (size_t)rt.width * rt.height * 3, f);
    std::fclose(f);
    FlatScene flat;
    flatten_scene(scene, flat);
    rt_scene_host *h = nullptr;
    if (rt_scene_host_from_desc(&flat.desc, 1, 3, 0, &h) != RT_OK || rt_scene_host_save(h, argv[2]) != RT_OK) return 1;
    rt_scene_host_free(h);
    std::printf("{\"width\": %d, \"height\": %d, \"use_time\": %.6f}\n", rt.width, rt.height, (double)rt.useTime);
    return 0;
}
