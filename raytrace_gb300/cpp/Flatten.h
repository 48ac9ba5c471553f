// Flatten.h — turn a drop-in Scene into the flat rt_scene_desc consumed by the C ABI.
// This replaces the per-pixel virtual dispatch over Scene::Objects (RayTracer.cpp:458-465 of
// the reference) with device tables built once per start().
#pragma once
#include <memory>
#include <vector>

#include "../../include/rt_gb300.h"
#include "Scene.h"

struct FlatScene {
    rt_scene_desc desc{};
    std::vector<rt_light> lights;
    std::vector<rt_material> materials;
    std::vector<rt_texture> textures;
    std::vector<std::vector<uint8_t>> texels;
    std::vector<rt_object> objects;
    std::vector<float> tri_p, tri_n, tri_uv;
    std::vector<int32_t> tri_mtl, tri_id;
    // point desc at the vectors (call after any vector changes)
    void finalize();
};

// cam -> rt_camera (dimensions from the camera)
rt_camera flatten_camera(const Camera &cam);
// flatten every object (hidden ones keep their index with show = 0)
void flatten_scene(const Scene &scene, FlatScene &out);
