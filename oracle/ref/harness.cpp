// harness.cpp — drives the reference's own classes (compiled from its sources by
// oracle/ref/Makefile) on a scene file written by rt_scene_host_save. TEST INFRASTRUCTURE ONLY.
//
// For every pixel of the 64x64-tile region the reference renders (RayTracer.cpp:13) it
// writes: the float colour of proxyRTfrac before Color::put (RayTracer.cpp:28, 327-330), the
// primary hit object / primitive / distance found by the same closest-hit loop as RTfrac
// (RayTracer.cpp:458-465), and, for one sample per pixel, the uint8 image of
// RayTracer::start(MY_MODEL_RAYTRACE, threads) itself (RayTracer.cpp:614-696).
// Usage: rt_ref_harness scene.rtsc out_prefix [threads] [tile_list_file]
#define private public
#define protected public
#include "RayTracer.h"
#include "Scene.h"
#undef private
#undef protected

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rt_gb300.h"

namespace {

struct FileScene {
    rt_camera cam;
    float env[3];
    int32_t spp = 1, max_level = 3;
    uint64_t seed = 0;
    std::vector<rt_light> lights;
    std::vector<rt_material> mtls;
    std::vector<rt_object> objs;
    std::vector<int> tw, th;
    std::vector<std::vector<uint8_t>> texels;
    std::vector<float> tri_p, tri_n, tri_uv;
    std::vector<int32_t> tri_mtl, tri_id;
};

template <class T> bool rd(FILE *f, T *p, size_t n) { return n == 0 || std::fread(p, sizeof(T), n, f) == n; }

bool load(const char *path, FileScene &s)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[4];
    int32_t ver;
    int64_t c[8];
    int32_t params[2];
    bool ok = rd(f, magic, 4) && !std::memcmp(magic, "RTSC", 4) && rd(f, &ver, 1) && ver == 1 && rd(f, c, 8) &&
              rd(f, params, 2) && rd(f, &s.seed, 1) && rd(f, &s.cam, 1) && rd(f, s.env, 3);
    if (ok) {
        s.spp = params[0], s.max_level = params[1];
        s.lights.resize((size_t)c[0]);
        s.mtls.resize((size_t)c[1]);
        s.objs.resize((size_t)c[3]);
        ok = rd(f, s.lights.data(), s.lights.size()) && rd(f, s.mtls.data(), s.mtls.size()) && rd(f, s.objs.data(), s.objs.size());
        for (int64_t i = 0; ok && i < c[2]; ++i) {
            int32_t w, h;
            ok = rd(f, &w, 1) && rd(f, &h, 1);
            s.tw.push_back(w), s.th.push_back(h);
            s.texels.emplace_back((size_t)w * h * 3);
            ok = ok && rd(f, s.texels.back().data(), s.texels.back().size());
        }
        const size_t n = (size_t)c[4];
        s.tri_p.resize(9 * n), s.tri_n.resize(9 * n), s.tri_uv.resize((size_t)c[5]), s.tri_mtl.resize(n), s.tri_id.resize(n);
        ok = ok && rd(f, s.tri_p.data(), 9 * n) && rd(f, s.tri_n.data(), 9 * n) && rd(f, s.tri_uv.data(), s.tri_uv.size()) &&
             rd(f, s.tri_mtl.data(), n) && rd(f, s.tri_id.data(), n);
    }
    std::fclose(f);
    return ok;
}

Vertex vx(const float *p, float w = 0.0f) { return Vertex(p[0], p[1], p[2], w); }

Material material(const rt_material &m)
{
    Material r;
    r.SetMtl(MY_MODEL_AMBIENT, m.ambient[0], m.ambient[1], m.ambient[2]);
    r.SetMtl(MY_MODEL_DIFFUSE, m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    r.SetMtl(MY_MODEL_SPECULAR, m.specular[0], m.specular[1], m.specular[2]);
    r.SetMtl(MY_MODEL_SHINESS, m.shininess);
    r.reflect = m.reflect, r.refract = m.refract, r.rfr = m.rfr;
    return r;
}

Texture texture(const FileScene &s, int i) { return Texture("t" + std::to_string(i), (int16_t)s.tw[i], (int16_t)s.th[i], s.texels[i].data()); }

bool same3(const Vertex &a, const float *b) { return a.x == b[0] && a.y == b[1] && a.z == b[2]; }

// the reference objects for the file's object list, in order
void build(const FileScene &s, Scene &scene, std::vector<int> &model_base)
{
    scene.EnvLight = Vertex(s.env[0], s.env[1], s.env[2], 1.0f);
    for (const rt_light &l : s.lights) {
        Light L((uint8_t)l.type);
        L.position = vx(l.position, L.position.alpha);
        L.ambient = vx(l.ambient, 1.0f);
        L.diffuse = vx(l.diffuse, 1.0f);
        L.specular = vx(l.specular, 1.0f);
        L.attenuation = vx(l.attenuation, L.attenuation.alpha);
        L.bLight = l.on != 0;
        scene.Lights.push_back(L);
    }
    model_base.assign(s.objs.size(), 0);
    for (size_t k = 0; k < s.objs.size(); ++k) {
        const rt_object &o = s.objs[k];
        switch (o.type) {
        case RT_OBJECT_PLANE: {
            scene.AddPlane();
            Plane *p = dynamic_cast<Plane *>(scene.Objects.back());
            if (!same3(p->normal, o.normal) || !same3(p->axisx, o.axisx) || !same3(p->axisy, o.axisy))
                std::fprintf(stderr, "warning: plane frame of object %zu differs from the scene file\n", k);
            p->SetMtl(material(s.mtls[(size_t)o.material]));
            if (o.texture >= 0) p->setTex(texture(s, o.texture));
            break;
        }
        case RT_OBJECT_SPHERE:
            scene.AddSphere(o.radius);
            scene.Objects.back()->position = vx(o.position);
            scene.Objects.back()->SetMtl(material(s.mtls[(size_t)o.material]));
            break;
        case RT_OBJECT_BALLPLANE:
            scene.AddBallPlane(o.radius);
            scene.Objects.back()->SetMtl(material(s.mtls[(size_t)o.material]));
            break;
        case RT_OBJECT_CUBE: {
            scene.AddCube(1.0f);
            Box *b = dynamic_cast<Box *>(scene.Objects.back());
            b->position = vx(o.position);
            b->min = vx(o.bmin);
            b->max = vx(o.bmax);
            b->SetMtl(material(s.mtls[(size_t)o.material]));
            break;
        }
        case RT_OBJECT_MODEL: {
            Model *m = new Model(0);
            m->position = vx(o.position);
            for (size_t i = 0; i < s.mtls.size(); ++i) {
                m->mtls.push_back(material(s.mtls[i]));
                m->mtl_tex.push_back((int8_t)s.mtls[i].texture);
            }
            for (size_t i = 0; i < s.tw.size(); ++i) m->texs.push_back(texture(s, (int)i));
            // parts = runs of triangles with one material, as the OBJ loader groups them, and
            // at most 32767 per part: clTri numbers triangles with int16_t (3DElement.h:125)
            for (int64_t i = 0; i < o.tri_count; ++i) {
                const int64_t g = o.tri_first + i;
                if (m->parts.empty() || s.tri_mtl[(size_t)g] != m->part_mtl.back() || m->parts.back().size() >= 32767) {
                    m->parts.emplace_back();
                    m->part_mtl.push_back((int8_t)s.tri_mtl[(size_t)g]);
                }
                const float *P = &s.tri_p[(size_t)g * 9], *N = &s.tri_n[(size_t)g * 9];
                const float *U = s.tri_uv.empty() ? nullptr : &s.tri_uv[(size_t)g * 6];
                Coord2D t0, t1, t2;
                if (U) t0 = Coord2D(U[0], U[1]), t1 = Coord2D(U[2], U[3]), t2 = Coord2D(U[4], U[5]);
                m->parts.back().push_back(Triangle(vx(P), Normal(N[0], N[1], N[2]), t0, vx(P + 3), Normal(N[3], N[4], N[5]), t1,
                                                   vx(P + 6), Normal(N[6], N[7], N[8]), t2));
            }
            for (auto &part : m->parts) {   // part borders (SSE lane min / max of the points)
                Vertex mn = part[0].points[0], mx = mn;
                for (auto &t : part)
                    for (auto &p : t.points) {
                        mn.dat = _mm_min_ps(mn.dat, p.dat);
                        mx.dat = _mm_max_ps(mx.dat, p.dat);
                    }
                m->borders.push_back(mn);
                m->borders.push_back(mx);
            }
            m->VerMin = vx(o.bmin);
            m->VerMax = vx(o.bmax);
            model_base[k] = (int)o.tri_first;
            scene.Objects.push_back(m);
            break;
        }
        }
        scene.Objects.back()->bShow = o.show != 0;
    }
    Camera &c = scene.cam;
    c.position = vx(s.cam.position);
    c.u = Normal(s.cam.u[0], s.cam.u[1], s.cam.u[2]);
    c.v = Normal(s.cam.v[0], s.cam.v[1], s.cam.v[2]);
    c.n = Normal(s.cam.n[0], s.cam.n[1], s.cam.n[2]);
    c.width = s.cam.width, c.height = s.cam.height;
    c.fovy = s.cam.fovy, c.zNear = s.cam.znear, c.zFar = s.cam.zfar;
}

// Philox4x32-10 jitter stream (same definition as the renderer and the CPU oracle)
void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0, c[1] = (uint32_t)p1, c[2] = n2, c[3] = (uint32_t)p0;
        k0 += 0x9E3779B9u, k1 += 0xBB67AE85u;
    }
}

template <class T> void dump(const std::string &path, const std::vector<T> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

} // namespace

// --obj model.obj model.mtl out_prefix: load a model through the reference's own
// Model::loadOBJ (Model.cpp:14-349, textures relative to the working directory as there) and
// write what it built: per triangle its part, points, normals and texture coordinates; per part
// its material; per material Ka, Kd, Ks (xyzw), Ns, reflect, refract, rfr and texture; the
// textures' texels; VerMin / VerMax.
int dump_obj(const char *obj, const char *mtl, const std::string &out)
{
    std::string so(obj), sm(mtl);
    Model m(0);
    m.loadOBJ(std::wstring(so.begin(), so.end()), std::wstring(sm.begin(), sm.end()));
    std::vector<float> tris, mtls, bounds;
    std::vector<int32_t> tri_part, part_mtl, mtl_tex, tex_dims;
    std::vector<uint8_t> texels;
    for (size_t pa = 0; pa < m.parts.size(); ++pa)
        for (const Triangle &t : m.parts[pa]) {
            tri_part.push_back((int32_t)pa);
            for (int k = 0; k < 3; ++k) tris.insert(tris.end(), {t.points[k].x, t.points[k].y, t.points[k].z});
            for (int k = 0; k < 3; ++k) tris.insert(tris.end(), {t.norms[k].x, t.norms[k].y, t.norms[k].z});
            for (int k = 0; k < 3; ++k) tris.insert(tris.end(), {t.tcoords[k].u, t.tcoords[k].v});
        }
    for (int8_t pm : m.part_mtl) part_mtl.push_back(pm);
    for (size_t i = 0; i < m.mtls.size(); ++i) {
        const Material &M = m.mtls[i];
        for (const Vertex *v : {&M.ambient, &M.diffuse, &M.specular}) mtls.insert(mtls.end(), {v->x, v->y, v->z, v->alpha});
        mtls.insert(mtls.end(), {M.shiness, M.reflect, M.refract, M.rfr});
        mtl_tex.push_back(i < m.mtl_tex.size() ? m.mtl_tex[i] : -1);
    }
    for (const Texture &t : m.texs) {
        tex_dims.push_back(t.w), tex_dims.push_back(t.h);
        texels.insert(texels.end(), t.data, t.data + (size_t)t.w * t.h * 3);
    }
    bounds = {m.VerMin.x, m.VerMin.y, m.VerMin.z, m.VerMax.x, m.VerMax.y, m.VerMax.z};
    dump(out + ".tris.f32", tris);
    dump(out + ".tripart.i32", tri_part);
    dump(out + ".partmtl.i32", part_mtl);
    dump(out + ".mtls.f32", mtls);
    dump(out + ".mtltex.i32", mtl_tex);
    dump(out + ".texdims.i32", tex_dims);
    dump(out + ".texels.u8", texels);
    dump(out + ".bounds.f32", bounds);
    std::printf("{\"parts\": %zu, \"triangles\": %zu, \"materials\": %zu, \"textures\": %zu}\n", m.parts.size(),
                tri_part.size(), m.mtls.size(), m.texs.size());
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 5 && std::strcmp(argv[1], "--obj") == 0) return dump_obj(argv[2], argv[3], argv[4]);
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s scene.rtsc out_prefix [threads] [tiles_file|-] [mode]\n", argv[0]);
        return 2;
    }
    FileScene fs;
    if (!load(argv[1], fs)) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 1;
    }
    const std::string out = argv[2];
    const int threads = argc > 3 ? std::max(1, std::atoi(argv[3])) : 1;
    std::vector<int> tiles;
    // render mode: MY_MODEL_* (RayTracer.cpp:629-662), MY_MODEL_RAYTRACE by default
    const int mode = argc > 5 ? std::atoi(argv[5]) : MY_MODEL_RAYTRACE;
    if (argc > 4 && std::strcmp(argv[4], "-") != 0) {
        FILE *f = std::fopen(argv[4], "r");
        int t;
        while (f && std::fscanf(f, "%d", &t) == 1) tiles.push_back(t);
        if (f) std::fclose(f);
    }
    Scene scene;
    std::vector<int> model_base;
    build(fs, scene, model_base);
    RayTracer rt(scene);
    rt.maxLevel = (uint8_t)fs.max_level;
    rt.width = scene.cam.width, rt.height = scene.cam.height;
    const int W = rt.width, H = rt.height, bw = W / 64, bh = H / 64;
    if (tiles.empty())
        for (int i = 0; i < bw * bh; ++i) tiles.push_back(i);
    for (auto *o : scene.Objects)
        if (o->bShow) o->RTPrepare();

    // per-pixel pass through proxyRTfrac (the worker parallelRT calls for MY_MODEL_RAYTRACE)
    const Camera &cam = scene.cam;
    const double dp = tan(cam.fovy * PI / 360) / (H / 2);
    const float zNear = cam.zNear, zFar = sqrt(2) * cam.zFar;
    std::vector<float> rgb((size_t)W * H * 3, 0.0f), tt((size_t)W * H, 1e20f);
    std::vector<int32_t> obj((size_t)W * H, -1), prim((size_t)W * H, 0);
    std::vector<uint8_t> rgb8((size_t)W * H * 3, 0);
    // work units: 8x8 pieces of each 64x64 tile (pixels are independent of each other)
    std::atomic<size_t> next(0);
    auto worker = [&]() {
        while (true) {
            const size_t k = next.fetch_add(1);
            if (k >= tiles.size() * 64) break;
            const int tile = tiles[k / 64], sub = (int)(k % 64);
            const int bx = tile % bw, by = tile / bw;
            const int r0 = by * 64 + (sub / 8) * 8, c0 = bx * 64 + (sub % 8) * 8;
            for (int row = r0; row < r0 + 8; ++row)
                for (int col = c0; col < c0 + 8; ++col) {
                    const int xcur = col - W / 2, ycur = row - H / 2;
                    const size_t pix = (size_t)row * W + col;
                    float acc[3] = {0, 0, 0};
                    for (int s = 0; s < fs.spp; ++s) {
                        Vertex dir;
                        if (fs.spp > 1) {
                            uint32_t c[4] = {(uint32_t)pix, 0u, (uint32_t)s, 0u};
                            philox(c, (uint32_t)fs.seed, (uint32_t)(fs.seed >> 32));
                            double jx = (c[0] >> 8) * (1.0 / 16777216.0), jy = (c[1] >> 8) * (1.0 / 16777216.0);
                            dir = cam.n + cam.u * ((xcur + jx) * dp) + cam.v * ((ycur + jy) * dp);
                        } else
                            dir = cam.n + cam.u * (xcur * dp) + cam.v * (ycur * dp);
                        Ray ray(cam.position, dir, MY_RAY_BASERAY);
                        Color c(false);
                        switch (mode) {   // the worker start() would use for this mode
                        case MY_MODEL_CHECK: c = Color(((row / 64) & 1) == ((col / 64) & 1)); break;   // RTcheck
                        case MY_MODEL_DEPTHTEST: c = rt.RTdepth(zNear, zFar, ray); break;
                        case MY_MODEL_NORMALTEST: c = rt.RTnorm(zNear, zFar, ray); break;
                        case MY_MODEL_TEXTURETEST: c = rt.RTtex(zNear, zFar, ray); break;
                        case MY_MODEL_MATERIALTEST: c = rt.RTmtl(zNear, zFar, ray); break;
                        case MY_MODEL_SHADOWTEST: c = rt.RTshd(zNear, zFar, ray); break;
                        case MY_MODEL_REFLECTTEST: c = rt.proxyRTflec(zNear, zFar, ray); break;
                        default: c = rt.proxyRTfrac(zNear, zFar, ray); break;
                        }
                        acc[0] += c.r, acc[1] += c.g, acc[2] += c.b;
                        if (s == 0) {   // primary closest hit, RTfrac's object loop
                            HitRes hr = rt.tmphr;
                            const intptr_t base = rt.tmphr.obj;
                            int win = -1;
                            intptr_t winkey = base;
                            for (size_t oi = 0; oi < scene.Objects.size(); ++oi) {
                                DrawObject *o = scene.Objects[oi];
                                if (!o->bShow) continue;
                                hr.obj = base;
                                hr = o->intersect(ray, hr);
                                if (hr.obj != base) win = (int)oi, winkey = hr.obj;
                            }
                            hr.obj = winkey;
                            if (win >= 0 && hr.distance < 1e20f) {
                                obj[pix] = win;
                                tt[pix] = hr.distance;
                                DrawObject *o = scene.Objects[(size_t)win];
                                if (o->type == MY_OBJECT_BALLPLANE) prim[pix] = (int)(hr.obj - (intptr_t)o);
                                else if (o->type == MY_OBJECT_MODEL) {
                                    const clTri *t = (const clTri *)hr.obj;
                                    const Model *m = dynamic_cast<const Model *>(o);
                                    int offs = 0;
                                    for (int a = 0; a < t->numa; ++a) offs += (int)m->parts[(size_t)a].size();
                                    prim[pix] = offs + t->numb;
                                }
                            }
                        }
                    }
                    Color avg(fs.spp > 1 ? acc[0] * (1.0f / fs.spp) : acc[0], fs.spp > 1 ? acc[1] * (1.0f / fs.spp) : acc[1],
                              fs.spp > 1 ? acc[2] * (1.0f / fs.spp) : acc[2]);
                    for (int k2 = 0; k2 < 3; ++k2) rgb[3 * pix + k2] = (&avg.r)[k2];
                    avg.put(&rgb8[3 * pix]);
                }
        }
    };
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int i = 1; i < threads; ++i) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    dump(out + ".rgb.f32", rgb);
    dump(out + ".obj.i32", obj);
    dump(out + ".prim.i32", prim);
    dump(out + ".t.f32", tt);
    dump(out + ".rgb8", rgb8);

    // the reference's own start(): its uint8 output over the full tile region (1 spp only)
    double start_wall = 0.0, use_time = 0.0;
    if (fs.spp == 1 && (argc <= 4 || std::strcmp(argv[4], "-") == 0)) {
        const auto s0 = std::chrono::steady_clock::now();
        rt.start((uint8_t)mode, (int8_t)std::min(threads, 32));
        while (!rt.isFinish) std::this_thread::sleep_for(std::chrono::milliseconds(1));
        start_wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
        use_time = rt.useTime;
        std::vector<uint8_t> so((size_t)W * H * 3, 0);
        for (int row = 0; row < bh * 64; ++row)
            std::memcpy(&so[(size_t)row * W * 3], rt.output + (size_t)row * 3 * W, (size_t)bw * 64 * 3);
        dump(out + ".start.rgb8", so);
    }
    std::printf("{\"width\": %d, \"height\": %d, \"tiles\": %zu, \"threads\": %d, \"pixel_pass_s\": %.6f, "
                "\"start_wall_s\": %.6f, \"start_use_time_s\": %.6f}\n",
                W, H, tiles.size(), threads, secs, start_wall, use_time);
    return 0;
}
