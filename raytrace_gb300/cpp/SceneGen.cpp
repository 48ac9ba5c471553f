// SceneGen.cpp — seeded synthetic scenes of the benchmark (configs 0-4) built through the
// drop-in Scene API and flattened for the C ABI.
//
// Everything here is deterministic across x86 and Arm: integer PRNG (SplitMix64), value noise
// from an integer lattice hash, float arithmetic without contraction (-ffp-contract=off) and
// only sqrt / floor among the math functions (trigonometry appears only through the
// reference's own Plane / Light frame code, which uses double sin/cos).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>

#include "../../include/rt_gb300.h"
#include "Flatten.h"
#include "Scene.h"

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 40) * (1.0 / 16777216.0); }
    float uni(double a, double b) { return (float)(a + (b - a) * u01()); }
};

uint32_t hash3(int32_t x, int32_t y, int32_t z, uint32_t seed)
{
    uint32_t h = seed * 0x9E3779B1u;
    h ^= (uint32_t)x * 0x85EBCA77u;
    h = (h << 13) | (h >> 19);
    h ^= (uint32_t)y * 0xC2B2AE3Du;
    h = (h << 13) | (h >> 19);
    h ^= (uint32_t)z * 0x27D4EB2Fu;
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

inline float lattice(int32_t x, int32_t y, int32_t z, uint32_t seed)
{
    return (float)(hash3(x, y, z, seed) >> 8) * (1.0f / 8388608.0f) - 1.0f;
}
inline float smooth(float t) { return t * t * (3.0f - 2.0f * t); }
inline float lerp(float a, float b, float t) { return a + (b - a) * t; }

float noise3(float x, float y, float z, uint32_t seed)
{
    float fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
    int32_t ix = (int32_t)fx0, iy = (int32_t)fy0, iz = (int32_t)fz0;
    float sx = smooth(x - fx0), sy = smooth(y - fy0), sz = smooth(z - fz0);
    float c000 = lattice(ix, iy, iz, seed), c100 = lattice(ix + 1, iy, iz, seed);
    float c010 = lattice(ix, iy + 1, iz, seed), c110 = lattice(ix + 1, iy + 1, iz, seed);
    float c001 = lattice(ix, iy, iz + 1, seed), c101 = lattice(ix + 1, iy, iz + 1, seed);
    float c011 = lattice(ix, iy + 1, iz + 1, seed), c111 = lattice(ix + 1, iy + 1, iz + 1, seed);
    float x00 = lerp(c000, c100, sx), x10 = lerp(c010, c110, sx);
    float x01 = lerp(c001, c101, sx), x11 = lerp(c011, c111, sx);
    float y0 = lerp(x00, x10, sy), y1 = lerp(x01, x11, sy);
    return lerp(y0, y1, sz);
}

float fbm3(float x, float y, float z, int octaves, uint32_t seed)
{
    float sum = 0.0f, amp = 1.0f, freq = 1.0f, norm = 0.0f;
    for (int o = 0; o < octaves; ++o) {
        sum = sum + amp * noise3(x * freq, y * freq, z * freq, seed + (uint32_t)o);
        norm = norm + amp;
        amp = amp * 0.5f;
        freq = freq * 2.0f;
    }
    return sum / norm;
}

// 2D fBm = a slice of the 3D noise at z = 0
float fbm2(float x, float z, int octaves, uint32_t seed) { return fbm3(x, 0.0f, z, octaves, seed); }

float terrain_height(float x, float z, uint32_t seed, float amp) { return amp * fbm2(x * 0.1f, z * 0.1f, 6, seed); }

struct MeshBuild {
    std::vector<Vertex> pos;
    std::vector<uint32_t> idx;   // 3 per triangle
};

// vertex normals = normalised sum of the (area-weighted) face normals around each vertex
std::vector<Triangle> to_triangles(const MeshBuild &m)
{
    std::vector<Vertex> acc(m.pos.size());
    size_t nt = m.idx.size() / 3;
    for (size_t t = 0; t < nt; ++t) {
        const Vertex &a = m.pos[m.idx[3 * t]], &b = m.pos[m.idx[3 * t + 1]], &c = m.pos[m.idx[3 * t + 2]];
        Vertex fn = (b - a) * (c - a);
        for (int k = 0; k < 3; ++k)
            acc[m.idx[3 * t + k]] += fn;
    }
    std::vector<Normal> nrm(acc.size());
    for (size_t i = 0; i < acc.size(); ++i)
        nrm[i] = Normal(acc[i]);
    std::vector<Triangle> tris;
    tris.reserve(nt);
    for (size_t t = 0; t < nt; ++t) {
        uint32_t i0 = m.idx[3 * t], i1 = m.idx[3 * t + 1], i2 = m.idx[3 * t + 2];
        tris.push_back(Triangle(m.pos[i0], nrm[i0], m.pos[i1], nrm[i1], m.pos[i2], nrm[i2]));
    }
    return tris;
}

// geodesic icosphere of frequency f (20 f^2 triangles, 10 f^2 + 2 vertices), each vertex
// pushed radially to R * (1 + amp * fbm3(2 * unit, 3 octaves))
std::vector<Triangle> make_icosphere(int f, Vertex centre, float R, float amp, uint32_t seed)
{
    const float t = (float)1.6180339887498949;
    const float base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                               {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    int faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                        {11, 10, 2}, {10, 7, 6}, {7, 1, 8},   {3, 9, 4},  {3, 4, 2},   {3, 2, 6}, {3, 6, 8},
                        {3, 8, 9},  {4, 9, 5},  {2, 4, 11},  {6, 2, 10}, {8, 6, 7},   {9, 8, 1}};
    Vertex V[12];
    for (int i = 0; i < 12; ++i)
        V[i] = Normal(Vertex(base[i][0], base[i][1], base[i][2]));
    for (auto &fc : faces) {   // make every face wind outward
        Vertex n = (V[fc[1]] - V[fc[0]]) * (V[fc[2]] - V[fc[0]]);
        Vertex cen = V[fc[0]] + V[fc[1]] + V[fc[2]];
        if ((n & cen) < 0)
            std::swap(fc[1], fc[2]);
    }
    MeshBuild mb;
    std::map<uint64_t, uint32_t> key2idx;
    std::map<std::pair<int, int>, int> edge_id;
    auto vertex_at = [&](int face, int i, int j) -> uint32_t {
        int a = faces[face][0], b = faces[face][1], c = faces[face][2];
        int wa = f - i - j, wb = i, wc = j;
        uint64_t key;
        if (wa == f) key = (uint64_t)a;
        else if (wb == f) key = (uint64_t)b;
        else if (wc == f) key = (uint64_t)c;
        else if (wa == 0 || wb == 0 || wc == 0) {
            int p, q, wq;   // edge (p,q) with weight of q
            if (wc == 0) p = a, q = b, wq = wb;
            else if (wb == 0) p = a, q = c, wq = wc;
            else p = b, q = c, wq = wc;
            if (p > q) std::swap(p, q), wq = f - wq;
            auto it = edge_id.find({p, q});
            int e = it == edge_id.end() ? (edge_id[{p, q}] = (int)edge_id.size()) : it->second;
            key = (1ULL << 60) | ((uint64_t)e << 20) | (uint64_t)wq;
        } else
            key = (2ULL << 60) | ((uint64_t)face << 40) | ((uint64_t)i << 20) | (uint64_t)j;
        auto it = key2idx.find(key);
        if (it != key2idx.end()) return it->second;
        float inv = 1.0f / (float)f;
        Vertex p = (V[a] * (float)wa + V[b] * (float)wb + V[c] * (float)wc) * inv;
        Vertex unit = Normal(p);
        float n = fbm3(unit.x * 2.0f, unit.y * 2.0f, unit.z * 2.0f, 3, seed);
        float s = R * (1.0f + amp * n);
        mb.pos.push_back(centre + unit * s);
        uint32_t id = (uint32_t)mb.pos.size() - 1;
        key2idx[key] = id;
        return id;
    };
    for (int fc = 0; fc < 20; ++fc)
        for (int i = 0; i < f; ++i)
            for (int j = 0; j + i < f; ++j) {
                uint32_t v0 = vertex_at(fc, i, j), v1 = vertex_at(fc, i + 1, j), v2 = vertex_at(fc, i, j + 1);
                mb.idx.insert(mb.idx.end(), {v0, v1, v2});
                if (i + j < f - 1) {
                    uint32_t v3 = vertex_at(fc, i + 1, j + 1);
                    mb.idx.insert(mb.idx.end(), {v1, v3, v2});
                }
            }
    return to_triangles(mb);
}

// N x N heightfield over [-half, half]^2 in x/z
std::vector<Triangle> make_terrain(int N, float half, float amp, uint32_t seed)
{
    MeshBuild mb;
    mb.pos.resize((size_t)N * N);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            float x = (float)(-(double)half + 2.0 * half * i / (N - 1));
            float z = (float)(-(double)half + 2.0 * half * j / (N - 1));
            mb.pos[(size_t)j * N + i] = Vertex(x, terrain_height(x, z, seed, amp), z);
        }
    mb.idx.reserve((size_t)(N - 1) * (N - 1) * 6);
    for (int j = 0; j + 1 < N; ++j)
        for (int i = 0; i + 1 < N; ++i) {
            uint32_t v00 = (uint32_t)(j * N + i), v10 = v00 + 1, v01 = v00 + (uint32_t)N, v11 = v01 + 1;
            mb.idx.insert(mb.idx.end(), {v00, v01, v11, v00, v11, v10});
        }
    return to_triangles(mb);
}

Material law_material(Rng &r)
{
    Material m;
    float kd0 = r.uni(0.2, 0.9), kd1 = r.uni(0.2, 0.9), kd2 = r.uni(0.2, 0.9);
    float ks = r.uni(0.0, 0.5), n = r.uni(8.0, 128.0), refl = r.uni(0.0, 0.5);
    m.SetMtl(MY_MODEL_DIFFUSE, kd0, kd1, kd2);
    m.SetMtl(MY_MODEL_SPECULAR, ks, ks, ks);
    m.SetMtl(MY_MODEL_SHINESS, n);
    m.reflect = refl;
    return m;
}

struct SphereBox {
    double x0, x1, y0, y1, z0, z1;
};

void add_spheres(Scene &sc, Rng &r, int count, SphereBox box, int refractive_every, const std::function<float(float, float)> *ground)
{
    for (int i = 0; i < count; ++i) {
        float cx = r.uni(box.x0, box.x1), cy = r.uni(box.y0, box.y1), cz = r.uni(box.z0, box.z1);
        float rad = r.uni(0.3, 1.0);
        Material m = law_material(r);
        if (refractive_every > 0 && i % refractive_every == 0)
            m = sc.MtlLiby[4];   // "grass": reflect 0.15, refract 0.75, rfr 1.5
        if (ground)
            cy = (*ground)(cx, cz) + cy;
        uint8_t id = sc.AddSphere(rad);
        sc.Objects[id]->position = Vertex(cx, cy, cz);
        sc.Objects[id]->SetMtl(m);
    }
}

void add_point_lights(Scene &sc, Rng &r, int count, SphereBox box)
{
    for (int i = 0; i < count; ++i) {
        float x = r.uni(box.x0, box.x1), y = r.uni(box.y0, box.y1), z = r.uni(box.z0, box.z1);
        Light l(MY_LIGHT_POINT);
        l.position = Vertex(x, y, z, 1.0f);
        sc.Lights.push_back(l);
    }
}

void set_camera(Scene &sc, Vertex pos, Vertex target, int w, int h, float fovy)
{
    sc.cam.resize(w, h);
    sc.cam.fovy = fovy;
    sc.cam.lookAt(pos, target);
}

uint8_t add_mesh(Scene &sc, const std::vector<Triangle> &tris, const Material &m)
{
    Model *model = new Model();
    model->setMesh(tris, m);
    return sc.AddObject(model);
}

const int kRes[4][2] = {{256, 256}, {512, 512}, {1024, 768}, {1920, 1080}};
const SphereBox kSphereBox0 = {-4, 4, 0.5, 3, -4, 4};
const SphereBox kLightBox0 = {-6, 6, 4, 8, -6, 6};

} // namespace

struct rt_scene_host {
    FlatScene flat;
    int32_t spp = 1, max_level = 3;
    uint64_t seed = 0;
    std::vector<void *> pinned;
    ~rt_scene_host()
    {
        for (void *p : pinned) cudaHostUnregister(p);
    }
};

static rt_scene_host *finish(Scene &sc, int spp, int max_level, uint64_t seed)
{
    auto *h = new rt_scene_host();
    flatten_scene(sc, h->flat);
    h->spp = spp;
    h->max_level = max_level;
    h->seed = seed;
    return h;
}

// benchmark workloads
extern "C" int rt_scenegen(int32_t config, int32_t index, rt_scene_host **out)
{
    if (!out) return RT_ERR_INVALID;
    *out = nullptr;
    Scene sc;
    switch (config) {
    case 0: {   // plane + 8 spheres, 2 point lights, 512^2, depth 3
        Rng r(0);
        sc.AddPlane();
        add_spheres(sc, r, 8, kSphereBox0, 0, nullptr);
        add_point_lights(sc, r, 2, kLightBox0);
        set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0, 0), 512, 512, 60.0f);
        *out = finish(sc, 1, 3, 0);
        return RT_OK;
    }
    case 1: {   // plane + 81,920-triangle displaced icosphere, 1024x768, depth 3
        Rng r(1);
        Material m = law_material(r);
        sc.AddPlane();
        add_mesh(sc, make_icosphere(64, Vertex(0, 1.5f, 0), 1.5f, 0.15f, 1u), m);
        add_point_lights(sc, r, 2, kLightBox0);
        set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0, 0), 1024, 768, 60.0f);
        *out = finish(sc, 1, 3, 1);
        return RT_OK;
    }
    case 2: {   // 1024^2-vertex terrain + 64 spheres (25% refractive), 4 lights, 1080p, 4 spp, depth 4
        Rng r(2);
        Material m = law_material(r);
        add_mesh(sc, make_terrain(1024, 20.0f, 2.0f, 2u), m);
        std::function<float(float, float)> ground = [](float x, float z) { return terrain_height(x, z, 2u, 2.0f); };
        add_spheres(sc, r, 64, SphereBox{-20, 20, 0.5, 3, -20, 20}, 4, &ground);
        add_point_lights(sc, r, 4, SphereBox{-20, 20, 8, 16, -20, 20});
        set_camera(sc, Vertex(0, 12, -30), Vertex(0, 0, 0), 1920, 1080, 60.0f);
        *out = finish(sc, 4, 4, 2);
        return RT_OK;
    }
    case 3:
    case 4: {   // one scene of the batched / served population
        if (index < 0) return RT_ERR_INVALID;
        Rng r(((uint64_t)config << 32) | (uint64_t)index);
        double lnN = std::log(1000.0) + (std::log(500000.0) - std::log(1000.0)) * r.u01();
        int f = (int)std::lround(std::sqrt(std::exp(lnN) / 20.0));
        f = std::min(158, std::max(8, f));
        int res = std::min(3, (int)(r.u01() * 4.0));
        Material m = law_material(r);
        add_mesh(sc, make_icosphere(f, Vertex(0, 1.5f, 0), 1.5f, 0.15f, (uint32_t)(config * 100000 + index)), m);
        add_spheres(sc, r, 16, kSphereBox0, 0, nullptr);
        add_point_lights(sc, r, 2, kLightBox0);
        if (config == 3)
            set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0, 0), kRes[res][0], kRes[res][1], 60.0f);
        else {   // served scenes get a random orbit camera per request; this is the default one
            set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0, 0), kRes[res][0], kRes[res][1], 60.0f);
        }
        *out = finish(sc, 1, 3, (uint64_t)index);
        return RT_OK;
    }
    default:
        return RT_ERR_INVALID;
    }
}

extern "C" int rt_scenegen_small(uint64_t seed, int32_t n_spheres, int32_t ico_freq, int32_t width, int32_t height,
                                 int32_t refractive_every, rt_scene_host **out)
{
    if (!out || n_spheres < 0 || ico_freq < 0 || width <= 0 || height <= 0) return RT_ERR_INVALID;
    Scene sc;
    Rng r(seed);
    sc.AddPlane();
    if (ico_freq > 0) {
        Material m = law_material(r);
        add_mesh(sc, make_icosphere(ico_freq, Vertex(0, 1.5f, 0), 1.5f, 0.15f, (uint32_t)seed), m);
    }
    add_spheres(sc, r, n_spheres, kSphereBox0, refractive_every, nullptr);
    add_point_lights(sc, r, 2, kLightBox0);
    set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0, 0), width, height, 60.0f);
    *out = finish(sc, 1, 3, seed);
    return RT_OK;
}

// every object kind of the drop-in API in one scene: plane, ballplane, two cubes, spheres
// (some refractive), a small mesh, one parallel and one attenuated point light
extern "C" int rt_scenegen_extras(uint64_t seed, int32_t width, int32_t height, rt_scene_host **out)
{
    if (!out || width <= 0 || height <= 0) return RT_ERR_INVALID;
    Scene sc;
    Rng r(seed);
    sc.AddPlane();
    uint8_t bp = sc.AddBallPlane(0.3f);
    (void)bp;
    uint8_t c1 = sc.AddCube(1.0f);
    sc.MovePos(MY_MODEL_OBJECT, c1, Vertex(-2.5f, 0.25f, -1.0f));
    uint8_t c2 = sc.AddCube(0.6f);
    sc.MovePos(MY_MODEL_OBJECT, c2, Vertex(2.0f, 1.2f, -2.0f));
    sc.ChgMtl(c2, sc.MtlLiby[2]);
    add_spheres(sc, r, 6, kSphereBox0, 3, nullptr);
    Material m = law_material(r);
    add_mesh(sc, make_icosphere(4, Vertex(1.5f, 1.0f, 2.0f), 0.9f, 0.15f, (uint32_t)seed), m);
    uint8_t pl = sc.AddLight(MY_LIGHT_PARALLEL, Vertex(0.1f, 0.45f, 0.45f));
    sc.MovePos(MY_MODEL_LIGHT, pl, Vertex(-45, 45, 0));
    uint8_t pt = sc.AddLight(MY_LIGHT_POINT, Vertex(0.15f, 0.55f, 0.3f), Vertex(0.0f, 0.0f, 1.0f, 256));
    sc.MovePos(MY_MODEL_LIGHT, pt, Vertex(-30, 20, 0));   // off the ground plane
    sc.EnvLight = Vertex(0.05f, 0.05f, 0.05f, 1.0f);
    set_camera(sc, Vertex(0, 2, -10), Vertex(0, 0.5f, 0), width, height, 60.0f);
    *out = finish(sc, 1, 3, seed);
    return RT_OK;
}

// textured meshes: the plane with its default checker texture, a displaced icosphere with
// planar texture coordinates and a 64x32 procedural texture (map_Kd of its material), 6
// spheres (some refractive), a cube, two point lights
extern "C" int rt_scenegen_textured(uint64_t seed, int32_t width, int32_t height, rt_scene_host **out)
{
    if (!out || width <= 0 || height <= 0) return RT_ERR_INVALID;
    Scene sc;
    Rng r(seed);
    sc.AddPlane();
    const Vertex centre(0.0f, 1.4f, 0.5f);
    std::vector<Triangle> tris = make_icosphere(12, centre, 1.3f, 0.15f, (uint32_t)seed);
    for (Triangle &t : tris)   // planar projection along z (arithmetic only: the same on every host)
        for (int k = 0; k < 3; ++k) {
            const Vertex d = t.points[k] - centre;
            t.tcoords[k] = Coord2D(0.5f + d.x / 2.6f, 0.5f + d.y / 2.6f);
        }
    Material m = law_material(r);
    Model *model = new Model();
    model->setMesh(tris, m);
    std::vector<uint8_t> img(64 * 32 * 3);
    for (int y = 0; y < 32; ++y)
        for (int x = 0; x < 64; ++x) {
            uint8_t *px = &img[(size_t)(y * 64 + x) * 3];   // B, G, R
            px[0] = (uint8_t)(x * 4);
            px[1] = (uint8_t)(y * 8);
            px[2] = ((x / 8 + y / 8) & 1) ? 230 : 40;
        }
    model->texs.push_back(Texture("procedural", 64, 32, img.data()));
    model->mtl_tex[0] = 0;
    sc.AddObject(model);
    add_spheres(sc, r, 6, kSphereBox0, 3, nullptr);
    uint8_t c = sc.AddCube(0.8f);
    sc.MovePos(MY_MODEL_OBJECT, c, Vertex(-2.5f, 0.4f, 1.5f));
    add_point_lights(sc, r, 2, kLightBox0);
    sc.EnvLight = Vertex(0.1f, 0.1f, 0.1f, 1.0f);
    set_camera(sc, Vertex(0, 2.5f, -8), Vertex(0, 1.0f, 0), width, height, 60.0f);
    *out = finish(sc, 1, 3, seed);
    return RT_OK;
}

// a model read from OBJ/MTL files through the drop-in Scene::AddModel (the reference's loader:
// quads split, materials inherited, map_Kd read as <name>.bmp from the working directory,
// rescaled to extent 8; Model.cpp:14-349), two point lights and a camera facing the model
extern "C" int rt_scenegen_obj(const char *obj_path, const char *mtl_path, int32_t width, int32_t height,
                               rt_scene_host **out)
{
    if (!out || !obj_path || !mtl_path || width <= 0 || height <= 0) return RT_ERR_INVALID;
    *out = nullptr;
    Scene sc;
    const std::string so(obj_path), sm(mtl_path);
    const uint8_t id = sc.AddModel(std::wstring(so.begin(), so.end()), std::wstring(sm.begin(), sm.end()));
    const Model *m = static_cast<const Model *>(sc.Objects[id]);
    size_t n = 0;
    for (const auto &part : m->parts) n += part.size();
    if (n == 0) return RT_ERR_NOT_FOUND;   // no such file or no faces
    Light l1(MY_LIGHT_POINT), l2(MY_LIGHT_POINT);
    l1.position = Vertex(6.0f, 10.0f, -8.0f, 1.0f);
    l2.position = Vertex(-8.0f, 6.0f, -4.0f, 1.0f);
    sc.Lights.push_back(l1);
    sc.Lights.push_back(l2);
    sc.EnvLight = Vertex(0.1f, 0.1f, 0.1f, 1.0f);
    set_camera(sc, Vertex(0, 3, -14), Vertex(0, 0, 0), width, height, 60.0f);
    *out = finish(sc, 1, 3, 0);
    return RT_OK;
}

// deep copy of a caller's scene description
extern "C" int rt_scene_host_from_desc(const rt_scene_desc *d, int32_t spp, int32_t max_level, uint64_t seed,
                                       rt_scene_host **out)
{
    if (!d || !out) return RT_ERR_INVALID;
    auto *h = new rt_scene_host();
    FlatScene &f = h->flat;
    f.desc.camera = d->camera;
    std::memcpy(f.desc.env_light, d->env_light, sizeof f.desc.env_light);
    f.lights.assign(d->lights, d->lights + d->n_lights);
    f.materials.assign(d->materials, d->materials + d->n_materials);
    f.objects.assign(d->objects, d->objects + d->n_objects);
    for (int i = 0; i < d->n_textures; ++i) {
        f.textures.push_back(d->textures[i]);
        f.texels.emplace_back(d->textures[i].bgr, d->textures[i].bgr + (size_t)d->textures[i].w * d->textures[i].h * 3);
    }
    const size_t n = (size_t)d->n_tris;
    if (n) {
        f.tri_p.assign(d->tri_p, d->tri_p + 9 * n);
        f.tri_n.assign(d->tri_n, d->tri_n + 9 * n);
        if (d->tri_uv) f.tri_uv.assign(d->tri_uv, d->tri_uv + 6 * n);
        f.tri_mtl.assign(d->tri_mtl, d->tri_mtl + n);
        if (d->tri_id) f.tri_id.assign(d->tri_id, d->tri_id + n);
        else {
            f.tri_id.resize(n);
            for (const rt_object &o : f.objects)
                if (o.type == RT_OBJECT_MODEL)
                    for (int64_t i = 0; i < o.tri_count; ++i) f.tri_id[(size_t)(o.tri_first + i)] = (int32_t)i;
        }
    }
    f.finalize();
    h->spp = spp, h->max_level = max_level, h->seed = seed;
    *out = h;
    return RT_OK;
}

extern "C" const rt_scene_desc *rt_scene_host_desc(const rt_scene_host *s) { return s ? &s->flat.desc : nullptr; }

extern "C" int rt_scene_host_render_params(const rt_scene_host *s, int32_t *spp, int32_t *max_level, uint64_t *seed)
{
    if (!s) return RT_ERR_INVALID;
    if (spp) *spp = s->spp;
    if (max_level) *max_level = s->max_level;
    if (seed) *seed = s->seed;
    return RT_OK;
}

extern "C" void rt_scene_host_free(rt_scene_host *s) { delete s; }

extern "C" int64_t rt_scene_host_bytes(const rt_scene_host *s)
{
    if (!s) return 0;
    const FlatScene &f = s->flat;
    int64_t b = (int64_t)(f.tri_p.size() + f.tri_n.size() + f.tri_uv.size()) * 4 +
                (int64_t)(f.tri_mtl.size() + f.tri_id.size()) * 4 + (int64_t)f.objects.size() * (int64_t)sizeof(rt_object) +
                (int64_t)f.materials.size() * (int64_t)sizeof(rt_material) + (int64_t)f.lights.size() * (int64_t)sizeof(rt_light);
    for (auto &t : f.texels) b += (int64_t)t.size();
    return b;
}

extern "C" int rt_scene_host_pin(rt_scene_host *s)
{
    if (!s) return RT_ERR_INVALID;
    if (!s->pinned.empty()) return RT_OK;
    FlatScene &f = s->flat;
    auto pin = [&](void *p, size_t bytes) -> bool {
        if (!p || !bytes) return true;
        if (cudaHostRegister(p, bytes, cudaHostRegisterDefault) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        s->pinned.push_back(p);
        return true;
    };
    bool ok = pin(f.tri_p.data(), f.tri_p.size() * 4) && pin(f.tri_n.data(), f.tri_n.size() * 4) &&
              pin(f.tri_uv.data(), f.tri_uv.size() * 4) && pin(f.tri_mtl.data(), f.tri_mtl.size() * 4) &&
              pin(f.tri_id.data(), f.tri_id.size() * 4);
    return ok ? RT_OK : RT_ERR_CUDA;
}

// ---- binary scene file: "RTSC", version, fixed-size records, then arrays ------------------
namespace {
template <class T> bool wr(FILE *f, const T *p, size_t n) { return n == 0 || std::fwrite(p, sizeof(T), n, f) == n; }
template <class T> bool rd(FILE *f, T *p, size_t n) { return n == 0 || std::fread(p, sizeof(T), n, f) == n; }
} // namespace

extern "C" int rt_scene_host_save(const rt_scene_host *s, const char *path)
{
    if (!s || !path) return RT_ERR_INVALID;
    FILE *f = std::fopen(path, "wb");
    if (!f) return RT_ERR_INVALID;
    const FlatScene &fs = s->flat;
    const char magic[4] = {'R', 'T', 'S', 'C'};
    int32_t ver = 1;
    int64_t counts[8] = {(int64_t)fs.lights.size(), (int64_t)fs.materials.size(), (int64_t)fs.textures.size(),
                         (int64_t)fs.objects.size(), (int64_t)fs.tri_mtl.size(), (int64_t)fs.tri_uv.size(), 0, 0};
    int32_t params[2] = {s->spp, s->max_level};
    bool ok = wr(f, magic, 4) && wr(f, &ver, 1) && wr(f, counts, 8) && wr(f, params, 2) && wr(f, &s->seed, 1) &&
              wr(f, &fs.desc.camera, 1) && wr(f, fs.desc.env_light, 3) && wr(f, fs.lights.data(), fs.lights.size()) &&
              wr(f, fs.materials.data(), fs.materials.size()) && wr(f, fs.objects.data(), fs.objects.size());
    for (size_t i = 0; ok && i < fs.textures.size(); ++i)
        ok = wr(f, &fs.textures[i].w, 1) && wr(f, &fs.textures[i].h, 1) && wr(f, fs.texels[i].data(), fs.texels[i].size());
    ok = ok && wr(f, fs.tri_p.data(), fs.tri_p.size()) && wr(f, fs.tri_n.data(), fs.tri_n.size()) &&
         wr(f, fs.tri_uv.data(), fs.tri_uv.size()) && wr(f, fs.tri_mtl.data(), fs.tri_mtl.size()) &&
         wr(f, fs.tri_id.data(), fs.tri_id.size());
    std::fclose(f);
    return ok ? RT_OK : RT_ERR_INVALID;
}

extern "C" int rt_scene_host_load(const char *path, rt_scene_host **out)
{
    if (!path || !out) return RT_ERR_INVALID;
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return RT_ERR_NOT_FOUND;
    std::unique_ptr<rt_scene_host> s(new rt_scene_host());
    FlatScene &fs = s->flat;
    char magic[4];
    int32_t ver = 0;
    int64_t c[8];
    int32_t params[2];
    bool ok = rd(f, magic, 4) && std::memcmp(magic, "RTSC", 4) == 0 && rd(f, &ver, 1) && ver == 1 && rd(f, c, 8) &&
              rd(f, params, 2) && rd(f, &s->seed, 1) && rd(f, &fs.desc.camera, 1) && rd(f, fs.desc.env_light, 3);
    for (int i = 0; ok && i < 6; ++i)
        ok = c[i] >= 0 && c[i] < ((int64_t)1 << 34);
    if (ok) {
        s->spp = params[0];
        s->max_level = params[1];
        fs.lights.resize((size_t)c[0]);
        fs.materials.resize((size_t)c[1]);
        fs.textures.resize((size_t)c[2]);
        fs.texels.resize((size_t)c[2]);
        fs.objects.resize((size_t)c[3]);
        ok = rd(f, fs.lights.data(), fs.lights.size()) && rd(f, fs.materials.data(), fs.materials.size()) &&
             rd(f, fs.objects.data(), fs.objects.size());
        for (size_t i = 0; ok && i < fs.textures.size(); ++i) {
            ok = rd(f, &fs.textures[i].w, 1) && rd(f, &fs.textures[i].h, 1) && fs.textures[i].w >= 0 &&
                 fs.textures[i].h >= 0 && fs.textures[i].w <= 65535 && fs.textures[i].h <= 65535;
            if (ok) {
                fs.texels[i].resize((size_t)fs.textures[i].w * fs.textures[i].h * 3);
                ok = rd(f, fs.texels[i].data(), fs.texels[i].size());
            }
        }
        size_t nt = (size_t)c[4];
        fs.tri_p.resize(nt * 9);
        fs.tri_n.resize(nt * 9);
        fs.tri_uv.resize((size_t)c[5]);
        fs.tri_mtl.resize(nt);
        fs.tri_id.resize(nt);
        ok = ok && rd(f, fs.tri_p.data(), fs.tri_p.size()) && rd(f, fs.tri_n.data(), fs.tri_n.size()) &&
             rd(f, fs.tri_uv.data(), fs.tri_uv.size()) && rd(f, fs.tri_mtl.data(), nt) && rd(f, fs.tri_id.data(), nt);
    }
    std::fclose(f);
    if (!ok) return RT_ERR_INVALID;
    fs.finalize();
    *out = s.release();
    return RT_OK;
}
