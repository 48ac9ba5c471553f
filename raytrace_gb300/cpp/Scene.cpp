// Scene.cpp — the drop-in scene container. Adders, movers and switches follow the
// reference's Scene.cpp:83-301 (return 0xff / false on failure, no exceptions).
#include "Scene.h"

Scene::Scene()
{
    EnvLight = Vertex(0.2f, 0.2f, 0.2f, 1.0f);
    // material presets of the reference's library (Scene.cpp:12-66): the values are data the
    // scenes depend on, so they are kept as they are
    struct Preset {
        const char *name;
        float ka[3], kd[3], ks[3], shininess, reflect, refract, rfr;
    };
    static const Preset presets[] = {
        {"brass", {0.329412f, 0.223529f, 0.027451f}, {0.780392f, 0.568627f, 0.113725f},
         {0.992157f, 0.941176f, 0.807843f}, 27.8974f, 0.0f, 0.0f, 1.0f},
        {"bas-sphere", {0.1f, 0.1f, 0.1f}, {0.1f, 0.5f, 0.8f}, {1.0f, 1.0f, 1.0f}, 100.0f, 0.35f, 0.0f, 1.0f},
        {"mirror", {0.1f, 0.1f, 0.1f}, {0.1f, 0.1f, 0.1f}, {1.0f, 1.0f, 1.0f}, 127.0f, 0.95f, 0.0f, 1.0f},
        {"green grass", {0.1f, 0.4f, 0.1f}, {0.1f, 0.5f, 0.1f}, {1.0f, 1.0f, 1.0f}, 127.0f, 0.55f, 0.0f, 1.0f},
        {"grass", {0.1f, 0.1f, 0.1f}, {0.9f, 0.9f, 0.9f}, {1.0f, 1.0f, 1.0f}, 127.0f, 0.15f, 0.75f, 1.5f},
        {"wall", {0.2f, 0.2f, 0.2f}, {0.7f, 0.7f, 0.7f}, {0.5f, 0.5f, 0.5f}, 5.0f, 0.15f, 0.0f, 1.0f},
    };
    for (const Preset &p : presets) {
        Material m;
        m.name = p.name;
        m.SetMtl(MY_MODEL_AMBIENT, p.ka[0], p.ka[1], p.ka[2]);
        m.SetMtl(MY_MODEL_DIFFUSE, p.kd[0], p.kd[1], p.kd[2]);
        m.SetMtl(MY_MODEL_SPECULAR, p.ks[0], p.ks[1], p.ks[2]);
        m.SetMtl(MY_MODEL_SHINESS, p.shininess);
        m.reflect = p.reflect;
        m.refract = p.refract;
        m.rfr = p.rfr;
        MtlLiby.push_back(m);
    }
}

Scene::~Scene()
{
    for (auto *o : Objects)
        delete o;
}

uint8_t Scene::AddLight(const uint8_t type, const Vertex &comp, const Vertex &atte)
{
    if (Lights.size() == 8)
        return 0xff;
    Light light(type);
    float sum = comp.x + comp.y + comp.z;
    Vertex nc = comp / sum;
    light.SetProperty(MY_MODEL_AMBIENT, nc.x, nc.x, nc.x);
    light.SetProperty(MY_MODEL_DIFFUSE, nc.y, nc.y, nc.y);
    light.SetProperty(MY_MODEL_SPECULAR, nc.z, nc.z, nc.z);
    light.SetProperty(MY_MODEL_ATTENUATION, atte.x, atte.y, atte.z);
    light.SetLumi(atte.alpha);
    Lights.push_back(light);
    return (uint8_t)(Lights.size() - 1);
}

uint8_t Scene::AddSphere(const float radius)
{
    Sphere *s = new Sphere(radius);
    s->position = Vertex(0.0f, radius, 0.0f);
    s->SetMtl(MtlLiby[1]);
    Objects.push_back(s);
    return (uint8_t)(Objects.size() - 1);
}

uint8_t Scene::AddCube(const float len)
{
    Box *b = new Box(len);
    b->position = Vertex(0.0f, len / 2, 0.0f);
    b->SetMtl(MtlLiby[0]);
    Objects.push_back(b);
    return (uint8_t)(Objects.size() - 1);
}

uint8_t Scene::AddModel(const std::wstring &objname, const std::wstring &mtlname, uint8_t code)
{
    Model *m = new Model();
    m->loadOBJ(objname, mtlname, code);
    Objects.push_back(m);
    return (uint8_t)(Objects.size() - 1);
}

uint8_t Scene::AddPlane()
{
    Plane *p = new Plane();
    Material m;
    m.reflect = 0.6f;
    p->SetMtl(m);
    Objects.push_back(p);
    return (uint8_t)(Objects.size() - 1);
}

uint8_t Scene::AddBallPlane(const float radius)
{
    BallPlane *bp = new BallPlane(radius);
    bp->SetMtl(MtlLiby[1]);
    Objects.push_back(bp);
    return (uint8_t)(Objects.size() - 1);
}

uint8_t Scene::AddObject(DrawObject *obj)
{
    Objects.push_back(obj);
    return (uint8_t)(Objects.size() - 1);
}

bool Scene::ChgLightComp(const uint8_t type, const uint8_t num, const Vertex &v)
{
    if (num >= Lights.size())
        return false;
    Light &light = Lights[num];
    Vertex ta, td, ts;
    float tmp;
    switch (type) {
    case MY_LIGHT_COMPENT:
        ta = light.ambient * v.x;
        td = light.diffuse * v.y;
        ts = light.specular * v.z;
        tmp = (ta.x + td.x + ts.x) / light.attenuation.alpha;
        ta.x /= tmp, ts.x /= tmp, td.x /= tmp;
        tmp = (ta.y + td.y + ts.y) / light.attenuation.alpha;
        ta.y /= tmp, ts.y /= tmp, td.y /= tmp;
        tmp = (ta.z + td.z + ts.z) / light.attenuation.alpha;
        ta.z /= tmp, ts.z /= tmp, td.z /= tmp;
        light.SetProperty(MY_MODEL_AMBIENT, ta.x, ta.y, ta.z);
        light.SetProperty(MY_MODEL_DIFFUSE, td.x, td.y, td.z);
        light.SetProperty(MY_MODEL_SPECULAR, ts.x, ts.y, ts.z);
        break;
    case MY_LIGHT_LUMI:
        tmp = light.attenuation.alpha * v.alpha;
        light.SetLumi(tmp);
        break;
    default:
        return false;
    }
    return true;
}

bool Scene::ChgMtl(const uint8_t num, const Material &m)
{
    if (num >= Objects.size())
        return false;
    Objects[num]->SetMtl(m);
    Plane *p = dynamic_cast<Plane *>(Objects[num]);
    if (m.name == "wall" && p != nullptr)
        p->setTex(Texture(false));
    return true;
}

bool Scene::ChgMtl(const uint8_t num, const Normal &clr)
{
    if (num >= Objects.size())
        return false;
    auto chg = [&clr](Vertex &c) {
        if (clr.w < 0.5f) {
            float sum = c.r + c.g + c.b;
            c = clr * sum;
        } else
            c = clr;
    };
    if (Objects[num]->type == MY_OBJECT_MODEL) {
        Model &m = dynamic_cast<Model &>(*Objects[num]);
        for (Material &mt : m.mtls)
            chg(mt.diffuse);
    } else
        chg(Objects[num]->mtl.diffuse);
    return true;
}

bool Scene::Delete(uint8_t type, const uint8_t num)
{
    switch (type) {
    case MY_MODEL_OBJECT:
        if (num >= Objects.size())
            return false;
        delete Objects[num];
        Objects.erase(Objects.begin() + num);
        break;
    case MY_MODEL_LIGHT:
        if (num >= Lights.size())
            return false;
        Lights.erase(Lights.begin() + num);
        break;
    }
    return true;
}

bool Scene::MovePos(const uint8_t type, const uint8_t num, const Vertex &v)
{
    switch (type) {
    case MY_MODEL_OBJECT:
        if (num >= Objects.size())
            return false;
        if (Objects[num]->type == MY_OBJECT_PLANE)
            dynamic_cast<Plane &>(*Objects[num]).rotate(v);
        else if (Objects[num]->type == MY_OBJECT_BALLPLANE)
            dynamic_cast<BallPlane &>(*Objects[num]).rotate(v);
        else
            Objects[num]->position += v;
        break;
    case MY_MODEL_LIGHT:
        if (num >= Lights.size())
            return false;
        Lights[num].move(v.x, v.y, v.z);
        break;
    default:
        return false;
    }
    return true;
}

bool Scene::Switch(uint8_t type, const uint8_t num, const bool isShow)
{
    bool old, isSwitch = type & MY_MODEL_SWITCH;
    switch (type & 0x7f) {
    case MY_MODEL_LIGHT:
        if (num >= Lights.size())
            return false;
        Lights[num].bLight = isSwitch ? !Lights[num].bLight : isShow;
        return true;
    case MY_MODEL_OBJECT:
        if (num >= Objects.size())
            return false;
        old = Objects[num]->bShow;
        Objects[num]->bShow = isSwitch ? !old : isShow;
        return old;
    }
    return false;
}
