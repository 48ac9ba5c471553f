// 3DElement.h — value types of the drop-in scene API (Vertex, Normal, Color, Ray, HitRes,
// Material, Light, Camera, Texture, Triangle, DrawObject).
//
// Same class names, members and macro values as the reference's 3DElement.h:1-246 so code
// written against the reference compiles against this header. The arithmetic is portable C++
// (no SSE): every operation that the renderer reproduces bit-exactly keeps the reference's
// floating-point order (dot = (x*x'+y*y')+(z*z'+0), normalise = v / sqrt(dot) per lane,
// cross = l - r with separate products; 3DElement.cpp:137-238). Build with -ffp-contract=off.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#define MY_OBJECT_SPHERE    0x1
#define MY_OBJECT_CUBE      0x2
#define MY_OBJECT_MODEL     0x3
#define MY_OBJECT_PLANE     0x4
#define MY_OBJECT_BALLPLANE 0x5

#define MY_LIGHT_PARALLEL 0x1
#define MY_LIGHT_POINT    0x2
#define MY_LIGHT_SPOT     0x3

#define MY_MODEL_AMBIENT     0x1
#define MY_MODEL_DIFFUSE     0x2
#define MY_MODEL_SPECULAR    0x4
#define MY_MODEL_SHINESS     0x8
#define MY_MODEL_EMISSION    0x10
#define MY_MODEL_POSITION    0x100
#define MY_MODEL_ATTENUATION 0x200

#define MY_RAY_BASERAY    0x1
#define MY_RAY_SHADOWRAY  0x2
#define MY_RAY_REFLECTRAY 0x3
#define MY_RAY_REFRACTRAY 0x4

#ifndef PI
#define PI 3.1415926535897932384
#endif

class Coord2D
{
public:
    float u, v;
    Coord2D() : u(0.0f), v(0.0f) {}
    Coord2D(const float &iu, const float &iv) : u(iu), v(iv) {}
    Coord2D operator+(const Coord2D &c) const { return Coord2D(u + c.u, v + c.v); }
    Coord2D operator*(const float &n) const { return Coord2D(u * n, v * n); }
    operator float *() { return &u; }
};

class alignas(16) Vertex
{
public:
    union {
        float dat[4];
        struct { float x, y, z, w; };
        struct { float r, g, b, alpha; };
    };
    Vertex() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    Vertex(const float ix, const float iy, const float iz, const float ia = 0) : x(ix), y(iy), z(iz), w(ia) {}
    operator float *() { return &x; }
    operator const float *() const { return &x; }

    float length() const;
    float length_sqr() const;
    Vertex muladd(const float &n, const Vertex &v) const;   // fused per lane
    Vertex mixmul(const Vertex &v) const;                   // per-lane product

    Vertex operator+(const Vertex &v) const;
    Vertex &operator+=(const Vertex &right);
    Vertex operator-(const Vertex &v) const;
    Vertex &operator-=(const Vertex &right);
    Vertex operator/(const float &n) const;                 // multiply by 1/n
    Vertex &operator/=(const float &right);
    Vertex operator*(const float &n) const;
    Vertex &operator*=(const float &right);
    Vertex operator*(const Vertex &v) const;                // cross product
    float operator&(const Vertex &v) const;                 // dot product of x,y,z
};

class Normal : public Vertex
{
public:
    Normal() : Vertex() {}
    Normal(const float &ix, const float &iy, const float &iz, const float &iw = 0.0f) : Vertex(ix, iy, iz, iw) {}
    Normal(const Vertex &v);                                // normalises
};

class Texture
{
public:
    std::string name;
    int16_t w, h;
    uint8_t *data = nullptr;
    Texture(bool check = false);                            // 4x4 checker (0xff/0x7f) or white
    Texture(const std::string &iname, const int16_t iw, const int16_t ih, const uint8_t *img);
    ~Texture();
    Texture(const Texture &t);
    Texture(Texture &&t);
    Texture &operator=(const Texture &t);
};

class Material
{
public:
    Vertex ambient, diffuse, specular, emission;
    float shiness, reflect, refract, rfr;
    std::string name;
    Material();
    void SetMtl(const uint8_t prop, const float r, const float g, const float b, const float a = 1.0f);
    void SetMtl(const uint8_t prop, const Vertex &v);
    void SetMtl(const uint8_t prop, const float val);
};

class Triangle
{
public:
    Vertex points[3];
    Normal norms[3];
    Coord2D tcoords[3];
    Triangle() {}
    Triangle(const Vertex &va, const Vertex &vb, const Vertex &vc);
    Triangle(const Vertex &va, const Normal &na, const Vertex &vb, const Normal &nb, const Vertex &vc, const Normal &nc);
    Triangle(const Vertex &va, const Normal &na, const Coord2D &ta, const Vertex &vb, const Normal &nb,
             const Coord2D &tb, const Vertex &vc, const Normal &nc, const Coord2D &tc);
};

class Color : public Vertex
{
public:
    Color(const bool white = false);
    Color(const float &ix, const float &iy, const float &iz) : Vertex(ix, iy, iz, 1e20f) {}
    Color(const Vertex &v);
    Color(const Normal &n);
    Color(const Texture *tex, const Coord2D &coord);        // nearest texel, wrapped, BGR
    void set(const float depth, const float mindepth, const float maxdepth);
    void put(uint8_t *addr);                                // clamp to [0,1], *255, truncate
    void get(uint8_t *addr);
};

class Ray
{
public:
    Vertex origin;
    Normal direction;
    float mtlrfr = 1.0f;
    uint8_t type, isInside = 0x0;
    Ray(const Vertex &o, const Normal &dir, const uint8_t type = 0x0) : origin(o), direction(dir), type(type) {}
};

class HitRes
{
public:
    Vertex position;
    Normal normal;
    Coord2D tcoord;
    const Material *mtl = nullptr;
    const Texture *tex = nullptr;
    intptr_t obj = (intptr_t)this;
    float distance, rfr = 1.0f;
    uint8_t isInside = 0x0;
    HitRes(bool b = false) : distance(b ? 1e8f : 1e20f) {}
    HitRes(float dis) : distance(dis) {}
    bool operator<(const HitRes &right) const { return distance < right.distance; }
    operator bool() const { return distance < 1e8; }
};

// Base of every scene object. The renderer never calls a virtual per pixel: RayTracer::start
// flattens Scene::Objects into device tables (raytrace_gb300/cpp/Flatten.cpp). intersect() is
// the reference's per-ray test (3DElement.h:201) for host-side tools such as picking or a
// visibility query: it returns `hr` unchanged, or a closer hit with the reference's distance,
// position, normal, texture coordinate, material and identity token (`obj`: the object, a
// ball-plane sphere as this + 1..16, a model triangle as the address of its Triangle); a ray
// whose `hr.obj` is an object's token skips it (a sphere then takes its inside branch when the
// ray is inside), and a hit below `min` ends a model's search at once (the shadow rays' any-hit).
// Call RTPrepare() after moving or editing an object and before intersect(). There is no
// OpenGL on the target machines, so GLPrepare/GLDraw are no-ops kept for source compatibility.
class DrawObject
{
protected:
    unsigned int GLListNum;
public:
    Vertex position;
    Material mtl;
    uint8_t type;
    bool bShow = true;
    DrawObject(unsigned int n) : GLListNum(n) {}
    virtual ~DrawObject() {}
    virtual void SetMtl(const Material &m) { this->mtl = m; }
    void GLDraw() {}
    virtual void GLPrepare() {}
    virtual void RTPrepare() {}
    virtual HitRes intersect(const Ray &ray, const HitRes &hr, const float min = 0) = 0;
};

class Light
{
public:
    Vertex position, ambient, diffuse, specular, attenuation;
    float rangy, rangz, rdis, angy, angz, dis;
    float coang, exponent;
    uint8_t type;
    bool bLight;
    Light(const uint8_t type);
    bool turn();
    void move(const float dangy, const float dangz, const float ddis);
    void SetProperty(const int16_t prop, const float r, const float g, const float b, const float a = 1.0f);
    void SetLumi(const float lum);
};

class Camera
{
public:
    Normal u, v, n;      // right, up, toward
    Vertex position;
    int width, height;
    float fovy, aspect, zNear, zFar;
    Camera(int w = 1120, int h = 630);
    void move(const float &x, const float &y, const float &z);
    void yaw(const float angz);
    void pitch(float angy);
    void resize(int w, int h);
    // set position and basis looking at a target (n = normalise(target-pos),
    // u = normalise(n x up), v = normalise(u x n))
    void lookAt(const Vertex &pos, const Vertex &target, const Vertex &up = Vertex(0, 1, 0));
};

void Coord_sph2car(float &angy, float &angz, const float dis, Vertex &v);
void Coord_sph2car2(float &angy, float &angz, const float dis, Vertex &v);
void Coord_car2sph(const Vertex &v, float &angy, float &angz, float &dis);
float mod(const float &l, const float &r);
