// 3DElement.cpp — portable implementation of the drop-in value types.
// Floating-point order follows the reference's live SSE4/AVX/AVX2 branches
// (3DElement.cpp:56-238 of the reference): DPPS-style dot, AVX cross, AVX2 normalise.
#include "3DElement.h"

#include <cmath>
#include <cstdlib>
#include <utility>

// ---- angle helpers (double trigonometry, results stored as float) ---------------------
float mod(const float &l, const float &r)
{
    float t;
    std::modf(l / r, &t);
    float e = t * r;
    return l - e;
}

void Coord_sph2car(float &angy, float &angz, const float dis, Vertex &v)
{
    v.z = (float)((double)dis * std::sin(angy * PI / 180) * std::cos(angz * PI / 180.0));
    v.x = (float)((double)dis * std::sin(angy * PI / 180) * std::sin(angz * PI / 180));
    v.y = (float)((double)dis * std::cos(angy * PI / 180));
}

void Coord_sph2car2(float &angy, float &angz, const float dis, Vertex &v)
{
    bool fix = false;
    if (angz >= 180)
        angz = mod(angz, 180.0f), angy = mod(360 - angy, 360.0f), fix = true;
    if (angy < 1e-6)
        angy = 360;
    v.z = (float)((double)dis * std::sin(angy * PI / 180) * std::cos(angz * PI / 180.0));
    v.x = (float)((double)dis * std::sin(angy * PI / 180) * std::sin(angz * PI / 180));
    if (fix && mod(angy, 180.0f) < 1e-6)
        v.z *= -1, v.x *= -1;
    v.y = (float)((double)dis * std::cos(angy * PI / 180));
}

void Coord_car2sph(const Vertex &v, float &angy, float &angz, float &dis)
{
    dis = v.length();
    angy = (float)(std::acos(v.y / dis) * 180 / PI);
    angz = (float)(std::atan2(v.x, v.z) * 180 / PI);
}

// ---- Vertex ----------------------------------------------------------------------------
static inline float dot3(const Vertex &a, const Vertex &b)
{
    // DPPS with mask 0x71: (a0*b0 + a1*b1) + (a2*b2 + (+0.0))
    float p0 = a.x * b.x, p1 = a.y * b.y, p2 = a.z * b.z;
    float s01 = p0 + p1;
    float s23 = p2 + 0.0f;
    return s01 + s23;
}

float Vertex::length() const { return std::sqrt(dot3(*this, *this)); }
float Vertex::length_sqr() const { return dot3(*this, *this); }
Vertex Vertex::muladd(const float &n, const Vertex &v) const
{
    return Vertex(std::fma(x, n, v.x), std::fma(y, n, v.y), std::fma(z, n, v.z), std::fma(w, n, v.w));
}
Vertex Vertex::mixmul(const Vertex &v) const { return Vertex(x * v.x, y * v.y, z * v.z, w * v.w); }
Vertex Vertex::operator+(const Vertex &v) const { return Vertex(x + v.x, y + v.y, z + v.z, w + v.w); }
Vertex &Vertex::operator+=(const Vertex &r) { return *this = *this + r; }
Vertex Vertex::operator-(const Vertex &v) const { return Vertex(x - v.x, y - v.y, z - v.z, w - v.w); }
Vertex &Vertex::operator-=(const Vertex &r) { return *this = *this - r; }
Vertex Vertex::operator/(const float &n) const
{
    float rec = 1 / n;
    return Vertex(x * rec, y * rec, z * rec, w * rec);
}
Vertex &Vertex::operator/=(const float &r) { return *this = *this / r; }
Vertex Vertex::operator*(const float &n) const { return Vertex(x * n, y * n, z * n, w * n); }
Vertex &Vertex::operator*=(const float &r) { return *this = *this * r; }
Vertex Vertex::operator*(const Vertex &v) const
{
    // l = (y*z', z*x', x*y', w*w'), r = (z*y', x*z', y*x', w*w'), result l - r
    float lx = y * v.z, ly = z * v.x, lz = x * v.y, lw = w * v.w;
    float rx = z * v.y, ry = x * v.z, rz = y * v.x, rw = w * v.w;
    return Vertex(lx - rx, ly - ry, lz - rz, lw - rw);
}
float Vertex::operator&(const Vertex &v) const { return dot3(*this, v); }

Normal::Normal(const Vertex &v)
{
    float len = std::sqrt(dot3(v, v));
    x = v.x / len;
    y = v.y / len;
    z = v.z / len;
    w = v.w / len;
}

// ---- Texture -----------------------------------------------------------------------------
Texture::Texture(bool check)
{
    w = 4, h = 4;
    data = new uint8_t[48];
    if (check) {
        name = "check";
        for (int row = 0; row < 4; ++row)
            for (int col = 0; col < 4; ++col) {
                uint8_t c = ((row & 2) == (col & 2)) ? 0xff : 0x7f;
                uint8_t *t = data + (4 * row + col) * 3;
                t[0] = t[1] = t[2] = c;
            }
    } else {
        name = "empty";
        std::memset(data, 0xff, 48);
    }
}

Texture::Texture(const std::string &iname, const int16_t iw, const int16_t ih, const uint8_t *img)
    : name(iname), w(iw), h(ih)
{
    size_t size = (size_t)w * h * 3;
    data = new uint8_t[size];
    std::memcpy(data, img, size);
}

Texture::~Texture() { delete[] data; }

Texture::Texture(const Texture &t) : name(t.name), w(t.w), h(t.h)
{
    if (t.data) {
        size_t size = (size_t)w * h * 3;
        data = new uint8_t[size];
        std::memcpy(data, t.data, size);
    }
}

Texture::Texture(Texture &&t) : name(std::move(t.name)), w(t.w), h(t.h)
{
    data = t.data;
    t.data = nullptr;
}

Texture &Texture::operator=(const Texture &t)
{
    if (this == &t)
        return *this;
    name = t.name;
    w = t.w, h = t.h;
    delete[] data;
    data = nullptr;
    if (t.data) {
        size_t size = (size_t)w * h * 3;
        data = new uint8_t[size];
        std::memcpy(data, t.data, size);
    }
    return *this;
}

// ---- Material ------------------------------------------------------------------------------
Material::Material()
{
    name = "simple";
    SetMtl(MY_MODEL_AMBIENT | MY_MODEL_DIFFUSE, 0.588f, 0.588f, 0.588f);
    SetMtl(MY_MODEL_EMISSION | MY_MODEL_SPECULAR, 0.0f, 0.0f, 0.0f);
    SetMtl(MY_MODEL_SHINESS, 10.0f);
    reflect = refract = 0.0f;
    rfr = 1.0f;
}

void Material::SetMtl(const uint8_t prop, const float r, const float g, const float b, const float a)
{
    SetMtl(prop, Vertex(r, g, b, a));
    SetMtl(prop, a);
}

void Material::SetMtl(const uint8_t prop, const Vertex &v)
{
    if (prop & MY_MODEL_AMBIENT) ambient = v;
    if (prop & MY_MODEL_DIFFUSE) diffuse = v;
    if (prop & MY_MODEL_EMISSION) emission = v;
    if (prop & MY_MODEL_SPECULAR) specular = v;
}

void Material::SetMtl(const uint8_t prop, const float val)
{
    if (prop & MY_MODEL_SHINESS) shiness = val;
}

// ---- Triangle -------------------------------------------------------------------------------
Triangle::Triangle(const Vertex &va, const Vertex &vb, const Vertex &vc)
{
    points[0] = va, points[1] = vb, points[2] = vc;
}
Triangle::Triangle(const Vertex &va, const Normal &na, const Vertex &vb, const Normal &nb, const Vertex &vc,
                   const Normal &nc)
{
    points[0] = va, points[1] = vb, points[2] = vc;
    norms[0] = na, norms[1] = nb, norms[2] = nc;
}
Triangle::Triangle(const Vertex &va, const Normal &na, const Coord2D &ta, const Vertex &vb, const Normal &nb,
                   const Coord2D &tb, const Vertex &vc, const Normal &nc, const Coord2D &tc)
{
    points[0] = va, points[1] = vb, points[2] = vc;
    norms[0] = na, norms[1] = nb, norms[2] = nc;
    tcoords[0] = ta, tcoords[1] = tb, tcoords[2] = tc;
}

// ---- Color -----------------------------------------------------------------------------------
Color::Color(const bool white)
{
    r = g = b = white ? 1.0f : 0.0f;
    alpha = 1e20f;
}
Color::Color(const Vertex &v)
{
    r = v.x, g = v.y, b = v.z;
    alpha = 1e20f;
}
Color::Color(const Normal &n)
{
    r = (float)(0.5 * (n.x + 1));
    g = (float)(0.5 * (n.y + 1));
    b = (float)(0.5 * (n.z + 1));
}
Color::Color(const Texture *tex, const Coord2D &coord)
{
    if (tex == nullptr) {
        r = g = b = 1.0f;
        return;
    }
    float empty;
    float nu = std::modf(coord.u, &empty), nv = std::modf(coord.v, &empty);
    if (nu < 0) nu += 1;
    if (nv < 0) nv += 1;
    int16_t tx = (int16_t)(nu * tex->w), ty = (int16_t)(nv * tex->h);
    int32_t offset = (ty * tex->w + tx) * 3;
    int32_t last = (tex->w * tex->h - 1) * 3;   // the reference reads past the end here
    if (offset > last) offset = last;
    if (offset < 0) offset = 0;
    b = tex->data[offset] / 255.0f;
    g = tex->data[offset + 1] / 255.0f;
    r = tex->data[offset + 2] / 255.0f;
}
void Color::set(const float depth, const float mindepth, const float maxdepth)
{
    if (depth <= mindepth)
        r = 1.0f, g = b = 0.0f;
    else if (depth >= maxdepth)
        r = g = b = 0.0f;
    else {
        float after = std::log(depth), mx = std::log(maxdepth);
        r = g = b = (mx - after) / mx;
    }
}
static inline uint8_t put_channel(float c)
{
    if (c > 1.0f) return 255;
    if (c < 0.0f) return 0;
    if (c != c) return 0;
    return (uint8_t)(c * 255);
}
void Color::put(uint8_t *addr)
{
    addr[0] = put_channel(r);
    addr[1] = put_channel(g);
    addr[2] = put_channel(b);
}
void Color::get(uint8_t *addr)
{
    r = addr[0] / 255.0f, g = addr[1] / 255.0f, b = addr[2] / 255.0f;
}

// ---- Light --------------------------------------------------------------------------------------
Light::Light(const uint8_t t)
{
    type = t;
    bLight = true;
    rangy = 90, rangz = 0, rdis = 16;
    coang = 0, exponent = 0;
    move(0, 0, 0);
    SetProperty(MY_MODEL_AMBIENT, 0.05f, 0.05f, 0.05f);
    SetProperty(MY_MODEL_DIFFUSE | MY_MODEL_SPECULAR, 1.0f, 1.0f, 1.0f);
    SetProperty(MY_MODEL_ATTENUATION, 1.0f, 0.0f, 0.0f);
    position.alpha = (type == MY_LIGHT_PARALLEL) ? 0.0f : 1.0f;
}

bool Light::turn() { return bLight = !bLight; }

void Light::move(const float dangy, const float dangz, const float ddis)
{
    rdis += ddis;
    if (rdis < 2)
        rdis = 2;
    else if (rdis > 64)
        rdis = 64;
    angy = rangy = mod(360 + rangy + dangy, 360.0f);
    angz = rangz = mod(360 + rangz + dangz, 360.0f);
    dis = rdis;
    Coord_sph2car2(angy, angz, dis, position);
}

void Light::SetProperty(const int16_t prop, const float r, const float g, const float b, const float a)
{
    Vertex s(r, g, b, a);
    if (prop & MY_MODEL_AMBIENT) ambient = s;
    if (prop & MY_MODEL_DIFFUSE) diffuse = s;
    if (prop & MY_MODEL_SPECULAR) specular = s;
    if (prop & MY_MODEL_ATTENUATION) attenuation = s;
    if (prop & MY_MODEL_POSITION) position = s;
}

void Light::SetLumi(const float lum)
{
    float ext = lum / attenuation.alpha;
    attenuation.alpha = lum;
    ambient *= ext;
    diffuse *= ext;
    specular *= ext;
}

// ---- Camera --------------------------------------------------------------------------------------
Camera::Camera(int w, int h)
{
    width = w, height = h;
    aspect = (float)w / h;
    fovy = 45.0f, zNear = 1.0f, zFar = 100.0f;
    position = Vertex(0, 4, 15);
    u = Normal(1, 0, 0);
    v = Normal(0, 1, 0);
    n = Normal(0, 0, -1);
}

void Camera::move(const float &x, const float &y, const float &z)
{
    position += u * x;
    position += v * y;
    position += n * z;
}

void Camera::yaw(const float angz)
{
    float oangy = (float)(std::acos(n.y / 1) * 180 / PI), oangz = (float)(std::atan2(n.x, n.z) * 180 / PI);
    oangz -= angz;
    Coord_sph2car(oangy, oangz, 1, n);
    oangy = (float)(std::acos(u.y / 1) * 180 / PI);
    oangz = (float)(std::atan2(u.x, u.z) * 180 / PI);
    oangz -= angz;
    Coord_sph2car(oangy, oangz, 1, u);
}

void Camera::pitch(float angy)
{
    float oangy = (float)(std::acos(n.y / 1) * 180 / PI), oangz = (float)(std::atan2(n.x, n.z) * 180 / PI);
    if (oangy - angy < 1.0)
        angy = (float)(oangy - 1.0);
    if (oangy - angy > 179.0)
        angy = (float)(oangy - 179.0);
    oangy -= angy;
    Coord_sph2car(oangy, oangz, 1, n);
    v = u * n;
}

void Camera::resize(int w, int h)
{
    width = w, height = h;
    aspect = (float)w / h;
}

void Camera::lookAt(const Vertex &pos, const Vertex &target, const Vertex &up)
{
    position = pos;
    n = Normal(target - pos);
    u = Normal(n * up);
    v = Normal(u * n);
}
