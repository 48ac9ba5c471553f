// Model.h — triangle-mesh object of the drop-in API (the reference's Model.h:6-50).
// Parts, per-part materials and textures are kept as in the reference. RTPrepare's octant
// lists (Model.cpp:402-480 of the reference) are replaced by the device LBVH built in
// rt_scene_upload; on the host, RTPrepare places the part boxes and intersect() tests a ray
// against the triangles of every part whose box it enters.
#pragma once
#include "3DElement.h"

class Model : public DrawObject
{
public:
    static constexpr size_t kMaxPartTris = 32767;   // clTri::numb is int16_t in the reference
private:
    Vertex VerMin, VerMax, BorderMin, BorderMax;
    int32_t loadobj(const std::wstring &objname, const uint8_t code);
    int32_t loadmtl(const std::wstring &mtlname, const uint8_t code);
    int32_t loadtex(const std::string &texname, const uint8_t code);
public:
    std::vector<Vertex> vers;
    std::vector<Normal> nors;
    std::vector<Coord2D> txcs;
    std::vector<std::vector<Triangle>> parts;
    std::vector<Vertex> borders;      // per part: min, max
    std::vector<Vertex> bboxs;        // borders + position (filled by RTPrepare)
    std::vector<Material> mtls;
    std::vector<Texture> texs;
    std::vector<int8_t> part_mtl, mtl_tex;
    std::wstring objname, mtlname;

    Model(unsigned int num = 0) : DrawObject(num) { type = MY_OBJECT_MODEL; }
    ~Model() override {}
    void reset();
    // OBJ/MTL/BMP loading with the reference's rescale of the largest extent to 8
    int32_t loadOBJ(const std::wstring &objname, const std::wstring &mtlname, const uint8_t code = 0x0);
    void zRotate();
    void SetMtl(const Material &mtl) override;
    void RTPrepare() override;
    HitRes intersect(const Ray &ray, const HitRes &hr, const float min = 0) override;
    // inject a procedural mesh as a single part with one material (no rescale)
    void setMesh(const std::vector<Triangle> &tris, const Material &mtl);
    const Vertex &getVerMin() const { return VerMin; }
    const Vertex &getVerMax() const { return VerMax; }
    size_t triangleCount() const;
};
