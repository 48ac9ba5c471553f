// Model.cpp — mesh container, procedural-mesh injection and the OBJ/MTL/BMP loader of the
// drop-in API. The loader keeps the reference's observable behaviour (Model.cpp:14-312 of the
// reference): 1-based index lists with a dummy entry 0, quads split as (0,1,2),(0,2,3),
// `usemtl` starts a new part, materials inherit the previous material's values, map_Kd is
// rewritten to "<stem>.bmp", and the whole mesh is rescaled so its largest extent is 8.
#include "Model.h"

#include "Basic3DObject.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

static inline float lane_min(float a, float b) { return a < b ? a : b; }   // MINPS lane rule
static inline float lane_max(float a, float b) { return a > b ? a : b; }   // MAXPS lane rule

static void border(Vertex &mn, Vertex &mx, const Vertex &v)
{
    mn = Vertex(lane_min(mn.x, v.x), lane_min(mn.y, v.y), lane_min(mn.z, v.z), lane_min(mn.w, v.w));
    mx = Vertex(lane_max(mx.x, v.x), lane_max(mx.y, v.y), lane_max(mx.z, v.z), lane_max(mx.w, v.w));
}

void Model::reset()
{
    VerMin = VerMax = Vertex();
    mtl_tex.clear();
    part_mtl.clear();
    texs.clear();
    mtls.clear();
    parts.clear();
    borders.clear();
    bboxs.clear();
    vers.clear();
    nors.clear();
    txcs.clear();
}

size_t Model::triangleCount() const
{
    size_t n = 0;
    for (auto &p : parts)
        n += p.size();
    return n;
}

void Model::SetMtl(const Material &m)
{
    for (auto &old : mtls)
        old = m;
}

void Model::RTPrepare()
{
    BorderMin = VerMin + position, BorderMax = VerMax + position;
    bboxs.clear();
    for (size_t i = 0; i + 1 < borders.size(); i += 2) {
        bboxs.push_back(borders[i] + position);
        bboxs.push_back(borders[i + 1] + position);
    }
}

// Moller-Trumbore as the reference's TriangleTest (Model.cpp:720-744): edges e1 = p1 - p0,
// e2 = p2 - p0 and the corner p0 + position (RTPrepare's clTri, Model.cpp:425), no determinant
// check; the distance when t > 1e-5 with the barycentrics in `coord` = (1-u-v, u, v), else 1e20
static float triangle_test(const Ray &ray, const Triangle &tri, const Vertex &pos, Vertex &coord)
{
    const Vertex e1 = tri.points[1] - tri.points[0], e2 = tri.points[2] - tri.points[0];
    const Vertex p0 = tri.points[0] + pos;
    const Vertex pv = ray.direction * e2;
    const Vertex t2r = ray.origin - p0;
    const float f = 1.0f / (e1 & pv);
    const float u = (t2r & pv) * f;
    if (u < 0.0f || u > 1.0f) return 1e20f;
    const Vertex qv = t2r * e1;
    const float v = (ray.direction & qv) * f, w = 1 - u - v;
    if (v < 0.0f || w < 0.0f) return 1e20f;
    const float t = (e2 & qv) * f;
    if (!(t > 1e-5f)) return 1e20f;
    coord = Vertex(w, u, v);
    return t;
}

HitRes Model::intersect(const Ray &ray, const HitRes &hr, const float min)
{
    // The reference bins each part's triangles into octant lists around the part centre and
    // tests the lists of the octants the ray enters (Model.cpp:748-811); here every triangle of
    // a part whose box the ray enters is tested, in part order. Both find the nearest triangle
    // (strict <, the first found wins a tie) and stop at the first one closer than `min`.
    float exit;
    if (!(BorderTest(ray, BorderMin, BorderMax, &exit) < hr.distance)) return hr;
    float best = hr.distance;
    const Triangle *hit = nullptr;
    size_t hit_part = 0;
    Vertex coord;
    for (size_t a = 0; a < parts.size() && 2 * a + 1 < bboxs.size() && !(hit && best < min); ++a) {
        if (!(BorderTest(ray, bboxs[2 * a], bboxs[2 * a + 1], &exit) < hr.distance)) continue;
        for (const Triangle &t : parts[a]) {
            if (hr.obj == (intptr_t)&t) continue;   // the triangle the ray starts on
            Vertex c;
            const float d = triangle_test(ray, t, position, c);
            if (d < best) {
                best = d, hit = &t, hit_part = a, coord = c;
                if (d < min) break;
            }
        }
    }
    if (!hit) return hr;
    HitRes h(best);
    h.position = ray.origin + ray.direction * best;
    h.normal = hit->norms[0] * coord.x + hit->norms[1] * coord.y + hit->norms[2] * coord.z;
    h.tcoord = hit->tcoords[0] * coord.x + hit->tcoords[1] * coord.y + hit->tcoords[2] * coord.z;
    const int m = part_mtl[hit_part];
    h.mtl = &mtls[(size_t)m];
    h.rfr = h.mtl->rfr;
    const int tx = mtl_tex[(size_t)m];
    if (tx >= 0) h.tex = &texs[(size_t)tx];
    h.obj = (intptr_t)hit;
    return h;
}

void Model::setMesh(const std::vector<Triangle> &tris, const Material &m)
{
    // parts of at most 32767 triangles: the reference numbers a part's triangles with
    // int16_t (clTri::numb, 3DElement.h:125), so larger parts cannot be represented there
    reset();
    mtls.push_back(m);
    mtl_tex.push_back(-1);
    Vertex all_mn(1000, 1000, 1000), all_mx(-1000, -1000, -1000);
    for (size_t first = 0; first < tris.size(); first += kMaxPartTris) {
        const size_t last = std::min(tris.size(), first + kMaxPartTris);
        parts.emplace_back(tris.begin() + (std::ptrdiff_t)first, tris.begin() + (std::ptrdiff_t)last);
        part_mtl.push_back(0);
        Vertex mn = tris[first].points[0], mx = mn;
        for (size_t i = first; i < last; ++i)
            for (auto &p : tris[i].points)
                border(mn, mx, p);
        borders.push_back(mn);
        borders.push_back(mx);
        if (first == 0) all_mn = mn, all_mx = mx;
        border(all_mn, all_mx, mn);
        border(all_mn, all_mx, mx);
    }
    VerMin = all_mn, VerMax = all_mx;
}

void Model::zRotate()
{
    for (Vertex &v : vers) {
        std::swap(v.y, v.z);
        v.z *= -1;
    }
    for (Normal &n : nors) {
        std::swap(n.y, n.z);
        n.z *= -1;
    }
    for (auto &part : parts)
        for (Triangle &t : part)
            for (int a = 0; a < 3; ++a) {
                std::swap(t.points[a].y, t.points[a].z);
                std::swap(t.norms[a].y, t.norms[a].z);
                t.points[a].z *= -1;
                t.norms[a].z *= -1;
            }
    for (size_t a = 0; a + 1 < borders.size(); a += 2) {
        Vertex &va = borders[a], &vb = borders[a + 1];
        std::swap(va.y, va.z);
        std::swap(vb.y, vb.z);
        va.z *= -1;
        vb.z *= -1;
        std::swap(va.z, vb.z);
    }
    std::swap(VerMin.y, VerMin.z);
    VerMin.z *= -1;
    std::swap(VerMax.y, VerMax.z);
    VerMax.z *= -1;
}

// ---- loader -------------------------------------------------------------------------------------
namespace {

// one text line split into at most 5 whitespace tokens; the first token gets "****" appended
// so that short keywords compare on three characters (Model.cpp:5-12, 876-890 of the reference)
struct LineReader {
    FILE *fp = nullptr;
    explicit LineReader(const std::wstring &name)
    {
        std::string n(name.begin(), name.end());
        fp = std::fopen(n.c_str(), "r");
    }
    ~LineReader()
    {
        if (fp) std::fclose(fp);
    }
    // returns token count, -1 for an empty line, -128 at end of file
    int read(std::string tok[5])
    {
        if (!fp) return -128;
        char line[256], t[5][256];
        if (!std::fgets(line, sizeof line, fp)) return -128;
        int a = std::sscanf(line, "%255s%255s%255s%255s%255s", t[0], t[1], t[2], t[3], t[4]);
        if (a <= 0) return -1;
        for (int b = 0; b < a; ++b)
            tok[b] = t[b];
        tok[0] += "****";
        return a;
    }
};

int key3(const std::string &s)
{
    std::string t = s;
    if (t.length() < 3) t += "****";
    return t[2] + 256 * t[1] + 65536 * t[0];
}
constexpr int K3(char a, char b, char c) { return a * 65536 + b * 256 + c; }

// "%d/%d/%d" groups: v, v/t, v/t/n or v//n (out[0]=v, out[1]=t, out[2]=n); returns fields read
int parse_group(const std::string &in, int out[4])
{
    int a = std::sscanf(in.c_str(), "%d/%d/%d/%d", &out[0], &out[1], &out[2], &out[3]);
    if (a < 2) a = std::sscanf(in.c_str(), "%d//%d/%d", &out[0], &out[2], &out[3]);
    return a;
}

template <class T> const T &at(const std::vector<T> &v, int i)
{
    static const T zero{};
    return (i >= 0 && (size_t)i < v.size()) ? v[(size_t)i] : zero;
}

} // namespace

int32_t Model::loadobj(const std::wstring &name, const uint8_t)
{
    LineReader ldr(name);
    std::string ele[5];
    int ti[16] = {0};
    bool firstO = true;
    std::vector<Triangle> tris;
    vers.push_back(Vertex());
    nors.push_back(Normal());
    txcs.push_back(Coord2D());
    VerMin = Vertex(1000, 1000, 1000);
    VerMax = Vertex(-1000, -1000, -1000);
    while (true) {
        int num = ldr.read(ele);
        if (num == -128) break;
        if (num == -1) continue;
        switch (key3(ele[0])) {
        case K3('v', '*', '*'):
            vers.push_back(Vertex((float)std::atof(ele[1].c_str()), (float)std::atof(ele[2].c_str()),
                                  (float)std::atof(ele[3].c_str())));
            break;
        case K3('v', 'n', '*'):
            nors.push_back(Normal((float)std::atof(ele[1].c_str()), (float)std::atof(ele[2].c_str()),
                                  (float)std::atof(ele[3].c_str())));
            break;
        case K3('v', 't', '*'):
            txcs.push_back(Coord2D((float)std::atof(ele[1].c_str()), (float)std::atof(ele[2].c_str())));
            break;
        case K3('f', '*', '*'):
            if (num > 4) {
                int pn = parse_group(ele[1], &ti[0]) + parse_group(ele[2], &ti[3]) + parse_group(ele[3], &ti[6]) +
                         parse_group(ele[4], &ti[9]);
                if (pn < 12) {
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(vers, ti[3]), at(nors, ti[5]),
                                            at(vers, ti[6]), at(nors, ti[8])));
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(vers, ti[6]), at(nors, ti[8]),
                                            at(vers, ti[9]), at(nors, ti[11])));
                } else {
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(txcs, ti[1]), at(vers, ti[3]),
                                            at(nors, ti[5]), at(txcs, ti[4]), at(vers, ti[6]), at(nors, ti[8]),
                                            at(txcs, ti[7])));
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(txcs, ti[1]), at(vers, ti[6]),
                                            at(nors, ti[8]), at(txcs, ti[7]), at(vers, ti[9]), at(nors, ti[11]),
                                            at(txcs, ti[10])));
                }
                border(VerMin, VerMax, at(vers, ti[0]));
                border(VerMin, VerMax, at(vers, ti[3]));
                border(VerMin, VerMax, at(vers, ti[6]));
                border(VerMin, VerMax, at(vers, ti[9]));
            } else {
                int pn = parse_group(ele[1], &ti[0]) + parse_group(ele[2], &ti[3]) + parse_group(ele[3], &ti[6]);
                if (pn < 9)
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(vers, ti[3]), at(nors, ti[5]),
                                            at(vers, ti[6]), at(nors, ti[8])));
                else
                    tris.push_back(Triangle(at(vers, ti[0]), at(nors, ti[2]), at(txcs, ti[1]), at(vers, ti[3]),
                                            at(nors, ti[5]), at(txcs, ti[4]), at(vers, ti[6]), at(nors, ti[8]),
                                            at(txcs, ti[7])));
                border(VerMin, VerMax, at(vers, ti[0]));
                border(VerMin, VerMax, at(vers, ti[3]));
                border(VerMin, VerMax, at(vers, ti[6]));
            }
            break;
        case K3('u', 's', 'e'): {
            if (!firstO) {
                parts.push_back(std::move(tris));
                tris.clear();
                borders.push_back(VerMin);
                borders.push_back(VerMax);
            }
            VerMin = Vertex(1000, 1000, 1000);
            VerMax = Vertex(-1000, -1000, -1000);
            firstO = false;
            int a = (int)mtls.size();
            while (--a > 0)
                if (num > 1 && mtls[(size_t)a].name == ele[1]) break;
            if (a < 0) a = 0;
            part_mtl.push_back((int8_t)a);
            break;
        }
        default:
            break;
        }
    }
    if (firstO) part_mtl.push_back(0);
    parts.push_back(std::move(tris));
    borders.push_back(VerMin);
    borders.push_back(VerMax);

    // rescale so the largest extent of the union of part borders is 8
    VerMin = Vertex(1000, 1000, 1000);
    VerMax = Vertex(-1000, -1000, -1000);
    for (size_t a = 0; a + 1 < borders.size(); a += 2) {
        border(VerMin, VerMax, borders[a]);
        border(VerMin, VerMax, borders[a + 1]);
    }
    Vertex dif = VerMax - VerMin;
    float mdif = dif.x > dif.y ? dif.x : dif.y;
    mdif = (float)(dif.z > mdif ? dif.z / 8.0 : mdif / 8.0);
    VerMax /= mdif, VerMin /= mdif;
    for (Vertex &v : borders)
        v /= mdif;
    for (auto &part : parts)
        for (Triangle &t : part)
            for (Vertex &v : t.points)
                v /= mdif;
    return (int32_t)parts.size();
}

int32_t Model::loadmtl(const std::wstring &name, const uint8_t code)
{
    LineReader ldr(name);
    std::string ele[5];
    int8_t cur_tex = -1;
    bool firstM = true;
    Material mtl;
    mtls.push_back(mtl);
    mtl_tex.push_back(cur_tex);
    while (true) {
        int num = ldr.read(ele);
        if (num == -128) break;
        if (num == -1) continue;
        auto f = [&](int i) { return (float)(num > i ? std::atof(ele[i].c_str()) : 0.0); };
        switch (key3(ele[0])) {
        case K3('n', 'e', 'w'):
            if (!firstM) {
                mtls.push_back(mtl);
                mtl_tex.push_back(cur_tex);
            }
            mtl.name = num > 1 ? ele[1] : std::string();
            cur_tex = -1;
            firstM = false;
            break;
        case K3('K', 'a', '*'): mtl.SetMtl(MY_MODEL_AMBIENT, f(1), f(2), f(3)); break;
        case K3('K', 'd', '*'): mtl.SetMtl(MY_MODEL_DIFFUSE, f(1), f(2), f(3)); break;
        case K3('K', 's', '*'): mtl.SetMtl(MY_MODEL_SPECULAR, f(1), f(2), f(3)); break;
        case K3('K', 'e', '*'): mtl.SetMtl(MY_MODEL_EMISSION, f(1), f(2), f(3)); break;
        case K3('N', 's', '*'): mtl.SetMtl(MY_MODEL_SHINESS, 0, 0, 0, f(1)); break;
        case K3('m', 'a', 'p'):
            if (ele[0] == "map_Kd****" && num > 1) {
                size_t loff = ele[1].find_last_of('\\'), roff = ele[1].find_last_of('.');
                std::string tn = ele[1].substr(loff + 1, roff - loff) + "bmp";
                int a = (int)texs.size();
                while (--a >= 0)
                    if (texs[(size_t)a].name == tn) {
                        cur_tex = (int8_t)a;
                        break;
                    }
                if (a < 0) {
                    loadtex(tn, code);
                    cur_tex = (int8_t)((int)texs.size() - 1);
                }
            }
            break;
        default:
            break;
        }
    }
    mtls.push_back(mtl);
    mtl_tex.push_back(cur_tex);
    return 0;
}

int32_t Model::loadtex(const std::string &texname, const uint8_t)
{
    FILE *fp = std::fopen(texname.c_str(), "rb");
    if (!fp) return -1;
    unsigned char fh[14], ih[40];
    if (std::fread(fh, 1, 14, fp) != 14 || fh[0] != 'B' || fh[1] != 'M' || std::fread(ih, 1, 40, fp) != 40) {
        std::fclose(fp);
        return -1;
    }
    auto u32 = [](const unsigned char *p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; };
    uint32_t off = u32(fh + 10);
    int32_t width = (int32_t)u32(ih + 4), height = (int32_t)u32(ih + 8), size = (int32_t)u32(ih + 20);
    if (size == 0) size = width * height * 3;
    int16_t w16 = (int16_t)width, h16 = (int16_t)height;
    size_t need = (size_t)(w16 > 0 ? w16 : 0) * (size_t)(h16 > 0 ? h16 : 0) * 3;
    std::vector<uint8_t> image(std::max<size_t>((size_t)(size > 0 ? size : 0), need), 0);
    std::fseek(fp, (long)off, SEEK_SET);
    size_t got = std::fread(image.data(), 1, (size_t)(size > 0 ? size : 0), fp);
    (void)got;
    std::fclose(fp);
    texs.push_back(Texture(texname, w16, h16, image.data()));
    return 0;
}

int32_t Model::loadOBJ(const std::wstring &obj, const std::wstring &mtl, const uint8_t code)
{
    objname = obj, mtlname = mtl;
    reset();
    loadmtl(mtl, code);
    loadobj(obj, code);
    return 1;
}
