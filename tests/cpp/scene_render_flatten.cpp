// scene_render_flatten.cpp — builds the scene of scene_render_sequence.inc with the drop-in
// classes, flattens it the way RayTracer::start does (flatten_scene) and saves the flattened
// description as a scene file (argv[1]) for the CPU oracle; argv[2] picks the scene variant.
// No GPU is involved: the scene-host functions of the library are host code. Run from the directory holding the OBJ asset.
#include <cstdio>
#include <cstdlib>

#include "../../raytrace_gb300/cpp/Flatten.h"
#include "../../raytrace_gb300/cpp/Scene.h"

#include "scene_render_sequence.inc"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    const int variant = argc > 2 ? std::atoi(argv[2]) : 0;
    if (variant < 0 || variant >= kRenderVariants) return 2;
    Scene scene;
    build_render_scene(scene, variant);
    FlatScene flat;
    flatten_scene(scene, flat);
    rt_scene_host *h = nullptr;
    if (rt_scene_host_from_desc(&flat.desc, 1, kRenderLevel, 0, &h) != RT_OK) return 1;
    const int rc = rt_scene_host_save(h, argv[1]);
    rt_scene_host_free(h);
    if (rc != RT_OK) return 1;
    std::printf("{\"width\": %d, \"height\": %d, \"objects\": %d, \"lights\": %d}\n", scene.cam.width, scene.cam.height,
                (int)scene.Objects.size(), (int)scene.Lights.size());
    return 0;
}
