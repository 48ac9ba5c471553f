// Flatten.cpp — Scene -> rt_scene_desc.
#include "Flatten.h"

#include <cstring>

static void put3(float *d, const Vertex &v)
{
    d[0] = v.x, d[1] = v.y, d[2] = v.z;
}

void FlatScene::finalize()
{
    desc.n_lights = (int32_t)lights.size();
    desc.lights = lights.data();
    desc.n_materials = (int32_t)materials.size();
    desc.materials = materials.data();
    for (size_t i = 0; i < textures.size(); ++i)
        textures[i].bgr = texels[i].data();
    desc.n_textures = (int32_t)textures.size();
    desc.textures = textures.data();
    desc.n_objects = (int32_t)objects.size();
    desc.objects = objects.data();
    desc.n_tris = (int64_t)tri_mtl.size();
    desc.tri_p = tri_p.data();
    desc.tri_n = tri_n.data();
    desc.tri_uv = tri_uv.empty() ? nullptr : tri_uv.data();
    desc.tri_mtl = tri_mtl.data();
    desc.tri_id = tri_id.data();
}

rt_camera flatten_camera(const Camera &cam)
{
    rt_camera c{};
    put3(c.position, cam.position);
    put3(c.u, cam.u);
    put3(c.v, cam.v);
    put3(c.n, cam.n);
    c.width = cam.width;
    c.height = cam.height;
    c.fovy = cam.fovy;
    c.znear = cam.zNear;
    c.zfar = cam.zFar;
    return c;
}

static rt_material flat_material(const Material &m, int32_t tex)
{
    rt_material r{};
    put3(r.ambient, m.ambient);
    put3(r.diffuse, m.diffuse);
    put3(r.specular, m.specular);
    r.shininess = m.shiness;
    r.reflect = m.reflect;
    r.refract = m.refract;
    r.rfr = m.rfr;
    r.texture = tex;
    return r;
}

static int32_t add_texture(FlatScene &out, const Texture &t)
{
    rt_texture r{};
    r.w = t.w;
    r.h = t.h;
    size_t n = (size_t)(t.w > 0 ? t.w : 0) * (size_t)(t.h > 0 ? t.h : 0) * 3;
    out.texels.emplace_back(t.data ? std::vector<uint8_t>(t.data, t.data + n) : std::vector<uint8_t>(n, 0xff));
    out.textures.push_back(r);
    return (int32_t)out.textures.size() - 1;
}

void flatten_scene(const Scene &scene, FlatScene &out)
{
    out = FlatScene();
    out.desc.camera = flatten_camera(scene.cam);
    put3(out.desc.env_light, scene.EnvLight);
    for (const Light &l : scene.Lights) {
        rt_light r{};
        r.type = l.type;
        r.on = l.bLight ? 1 : 0;
        put3(r.position, l.position);
        put3(r.ambient, l.ambient);
        put3(r.diffuse, l.diffuse);
        put3(r.specular, l.specular);
        put3(r.attenuation, l.attenuation);
        out.lights.push_back(r);
    }
    for (const DrawObject *o : scene.Objects) {
        rt_object r{};
        r.type = o->type;
        r.show = o->bShow ? 1 : 0;
        r.material = -1;
        r.texture = -1;
        put3(r.position, o->position);
        switch (o->type) {
        case MY_OBJECT_SPHERE: {
            auto *s = static_cast<const Sphere *>(o);
            r.radius = s->getRadius();
            out.materials.push_back(flat_material(o->mtl, -1));
            r.material = (int32_t)out.materials.size() - 1;
            break;
        }
        case MY_OBJECT_CUBE: {
            auto *b = static_cast<const Box *>(o);
            put3(r.bmin, b->getMin());
            put3(r.bmax, b->getMax());
            out.materials.push_back(flat_material(o->mtl, -1));
            r.material = (int32_t)out.materials.size() - 1;
            break;
        }
        case MY_OBJECT_PLANE: {
            auto *p = static_cast<const Plane *>(o);
            put3(r.normal, p->normal);
            put3(r.axisx, p->getAxisX());
            put3(r.axisy, p->getAxisY());
            r.texture = add_texture(out, p->getTex());
            out.materials.push_back(flat_material(o->mtl, -1));
            r.material = (int32_t)out.materials.size() - 1;
            break;
        }
        case MY_OBJECT_BALLPLANE: {
            auto *bp = static_cast<const BallPlane *>(o);
            r.radius = bp->getRadius();
            put3(r.normal, bp->normal);
            put3(r.axisx, bp->getAxisX());
            put3(r.axisy, bp->getAxisY());
            out.materials.push_back(flat_material(o->mtl, -1));
            r.material = (int32_t)out.materials.size() - 1;
            break;
        }
        case MY_OBJECT_MODEL: {
            auto *m = static_cast<const Model *>(o);
            put3(r.bmin, m->getVerMin());
            put3(r.bmax, m->getVerMax());
            int32_t tex_base = (int32_t)out.textures.size();
            for (const Texture &t : m->texs)
                add_texture(out, t);
            int32_t mtl_base = (int32_t)out.materials.size();
            for (size_t k = 0; k < m->mtls.size(); ++k) {
                int tex = k < m->mtl_tex.size() ? m->mtl_tex[k] : -1;
                out.materials.push_back(flat_material(m->mtls[k], tex >= 0 ? tex_base + tex : -1));
            }
            r.material = mtl_base;
            r.tri_first = (int64_t)out.tri_mtl.size();
            int32_t local = 0;
            for (size_t pa = 0; pa < m->parts.size(); ++pa) {
                int pm = pa < m->part_mtl.size() ? m->part_mtl[pa] : 0;
                for (const Triangle &t : m->parts[pa]) {
                    for (int k = 0; k < 3; ++k) {
                        out.tri_p.insert(out.tri_p.end(), {t.points[k].x, t.points[k].y, t.points[k].z});
                        out.tri_n.insert(out.tri_n.end(), {t.norms[k].x, t.norms[k].y, t.norms[k].z});
                        out.tri_uv.insert(out.tri_uv.end(), {t.tcoords[k].u, t.tcoords[k].v});
                    }
                    out.tri_mtl.push_back(mtl_base + pm);
                    out.tri_id.push_back(local++);
                }
            }
            r.tri_count = (int64_t)out.tri_mtl.size() - r.tri_first;
            break;
        }
        default:
            break;
        }
        out.objects.push_back(r);
    }
    // drop the uv array when every coordinate is zero (saves device memory)
    bool any_uv = false;
    for (float f : out.tri_uv)
        if (f != 0.0f) {
            any_uv = true;
            break;
        }
    if (!any_uv)
        out.tri_uv.clear();
    out.finalize();
}
