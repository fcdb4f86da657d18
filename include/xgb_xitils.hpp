// xgb_xitils.hpp -- C++ host-side adapter with the shape of Xitils' render API,
// implemented over the C ABI of include/xgb.h (header-only; link libxgb.so).
//
// It mirrors the reference's construction and render calls so that a sandbox
// switches by changing namespaces:
//   xitils::TriangleMesh::setGeometry  (Include/Xitils/TriangleMesh.h:151-161) -> xgb::TriangleMesh::setGeometry
//   xitils::TriangleMesh::setGeometryWithShellMapping (TriangleMesh.h:163-177) -> the same name
//   xitils::Object(shape, material, T) (Include/Xitils/Object.h:32-34)         -> xgb::Object
//   xitils::Scene::addObject / buildAccelerationStructure (Scene.h:17-28)     -> xgb::Scene
//   xitils::PinholeCamera(T, fov, aspect) (Camera.h:32-36)                     -> xgb::PinholeCamera
//   xitils::Diffuse / Metal / Glossy / ... (Material.h)                        -> xgb::Diffuse / Metal / ...
//   RenderTarget<Vector3f>::render(scene, spp, lambda) + StandardPathTracer::eval
//     (RenderTarget.h:109-127, PathTracer.h:117-251)                           -> xgb::RenderTarget::render(scene, spp, tracer)
// Positions, normals, tangents and bitangents may be passed as xitils::Vector3f
// arrays (16-byte stride) or packed float3 (12-byte stride); matrices are
// row-major float[16] (xitils::Matrix4x4::m). Errors throw xgb::Error.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "xgb.h"

namespace xgb {

struct Error : std::runtime_error {
    xgb_status status;
    Error(xgb_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(xgb_status s, const xgb_ctx* ctx, const char* what) {
    if (s != XGB_OK) throw Error(s, std::string(what) + ": " + (ctx ? xgb_get_last_error(ctx) : "no context"));
}

class Context {
public:
    explicit Context(int device = 0) {
        xgb_status s = xgb_ctx_create(device, &h_);
        if (s != XGB_OK) throw Error(s, "xgb_ctx_create failed (no CUDA device?)");
    }
    ~Context() { if (h_) xgb_ctx_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    xgb_ctx* get() const { return h_; }

private:
    xgb_ctx* h_ = nullptr;
};

// Row-major object-to-world matrix and its inverse (xitils::Transform::mat / matInv).
struct Transform {
    float mat[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float matInv[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    Transform() = default;
    Transform(const float* m, const float* mi) {
        for (int i = 0; i < 16; ++i) { mat[i] = m[i]; matInv[i] = mi[i]; }
    }
    // Any type laid out like xitils::Transform (two Matrix4x4 with float m[4][4]).
    template <class XT> static Transform from(const XT& t) { return Transform(&t.mat.m[0][0], &t.matInv.m[0][0]); }
};

class Texture {
public:
    Texture(Context& ctx, int w, int h, const float* rgb, int channels = 3, bool warpClamp = true, bool filter = true)
        : ctx_(ctx.get()) {
        check(xgb_texture_create(ctx_, w, h, channels, rgb, warpClamp, filter, &h_), ctx_, "Texture");
    }
    // takes ownership of a texture the library made (the SVNDF's low-resolution map)
    Texture(Context& ctx, xgb_texture* made) : ctx_(ctx.get()), h_(made) {}
    ~Texture() { if (h_) xgb_texture_destroy(h_); }
    const xgb_texture* get() const { return h_; }

private:
    xgb_ctx* ctx_;
    xgb_texture* h_ = nullptr;
};

// SVNDF + downsampleDisplacementTexture of the displacement sandbox
// (Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/Main.cpp:361-470),
// fitted on the GPU; low() is the downsampled height texture.
class SVNDF {
public:
    SVNDF(Context& ctx, const Texture& displacement, float displacementScale, int rate = 8, uint32_t seed = 0)
        : ctx_(ctx.get()) {
        xgb_texture* low = nullptr;
        check(xgb_svndf_create(ctx_, displacement.get(), displacementScale, rate, seed, &h_, &low), ctx_, "SVNDF");
        low_ = std::make_shared<Texture>(ctx, low);
    }
    ~SVNDF() { if (h_) xgb_svndf_destroy(h_); }
    const xgb_svndf* get() const { return h_; }
    std::shared_ptr<Texture> low() const { return low_; }

private:
    xgb_ctx* ctx_;
    xgb_svndf* h_ = nullptr;
    std::shared_ptr<Texture> low_;
};

class TriangleMesh {
public:
    explicit TriangleMesh(Context& ctx) : ctx_(ctx.get()) {}
    ~TriangleMesh() { if (h_) xgb_mesh_destroy(h_); }
    // Same argument order as xitils::TriangleMesh::setGeometry. vec3Stride = 16 and
    // uvStride = 16 match xitils::Vector3f / Vector2f arrays.
    void setGeometry(int vertexNum, const float* positions, const float* texCoords, const float* normals,
                     const float* tangents, const float* bitangents, int indexNum, const int* indexData,
                     int vec3Stride = 16, int uvStride = 16) {
        if (h_) { xgb_mesh_destroy(h_); h_ = nullptr; }
        check(xgb_mesh_create(ctx_, vertexNum, positions, texCoords, normals, tangents, bitangents, vec3Stride,
                              uvStride, indexNum, indexData, &h_),
              ctx_, "TriangleMesh::setGeometry");
    }
    // xitils::TriangleMesh::setGeometryWithShellMapping (TriangleMesh.h:163-177): the mesh
    // keeps the displacement texture alive.
    void setGeometryWithShellMapping(int vertexNum, const float* positions, const float* texCoords,
                                     const float* normals, const float* tangents, const float* bitangents,
                                     int indexNum, const int* indexData, std::shared_ptr<const Texture> displacement,
                                     float displacementScale, int layerNum, int vec3Stride = 16, int uvStride = 16) {
        if (h_) { xgb_mesh_destroy(h_); h_ = nullptr; }
        displacement_ = displacement;
        check(xgb_mesh_create_shell(ctx_, vertexNum, positions, texCoords, normals, tangents, bitangents, vec3Stride,
                                    uvStride, indexNum, indexData, displacement ? displacement->get() : nullptr,
                                    displacementScale, layerNum, &h_),
              ctx_, "TriangleMesh::setGeometryWithShellMapping");
    }
    int triangleNum() const { int n = 0; if (h_) xgb_mesh_triangle_count(h_, &n); return n; }
    const xgb_mesh* get() const { return h_; }

private:
    xgb_ctx* ctx_;
    xgb_mesh* h_ = nullptr;
    std::shared_ptr<const Texture> displacement_;
};

class Material {
public:
    virtual ~Material() { if (h_) xgb_material_destroy(h_); }
    const xgb_material* get() const { return h_; }
    // Material::normalmap (Material.h:13)
    void setNormalmap(std::shared_ptr<Texture> tex) {
        normalmap_ = tex;
        check(xgb_material_set_normalmap(h_, tex ? tex->get() : nullptr), ctx_, "normalmap");
    }

protected:
    explicit Material(Context& ctx) : ctx_(ctx.get()) {}
    xgb_ctx* ctx_;
    xgb_material* h_ = nullptr;
    std::shared_ptr<Texture> normalmap_;
};

struct Diffuse : Material {
    Diffuse(Context& c, const float albedo[3], std::shared_ptr<Texture> tex = nullptr) : Material(c), tex_(tex) {
        check(xgb_material_diffuse(ctx_, albedo, tex ? tex->get() : nullptr, &h_), ctx_, "Diffuse");
    }
    std::shared_ptr<Texture> tex_;
};
struct Metal : Material {
    Metal(Context& c, float roughness, const float f0[3], std::shared_ptr<Texture> roughnessTex = nullptr)
        : Material(c), tex_(roughnessTex) {
        check(xgb_material_metal(ctx_, roughness, f0, roughnessTex ? roughnessTex->get() : nullptr, &h_), ctx_, "Metal");
    }
    std::shared_ptr<Texture> tex_;
};
struct Glossy : Material {
    Glossy(Context& c, const float albedo[3], float sharpness) : Material(c) {
        check(xgb_material_glossy(ctx_, albedo, sharpness, &h_), ctx_, "Glossy");
    }
};
struct GlossyWithHighLight : Material {
    GlossyWithHighLight(Context& c, const float albedo[3], const float highlight[3], float sharpness,
                        float sharpnessHighLight, float highlightRate) : Material(c) {
        check(xgb_material_glossy_highlight(ctx_, albedo, highlight, sharpness, sharpnessHighLight, highlightRate, &h_),
              ctx_, "GlossyWithHighLight");
    }
};
struct GlossyClamped : Material {
    GlossyClamped(Context& c, const float albedo[3], float sharpness) : Material(c) {
        check(xgb_material_glossy_clamped(ctx_, albedo, sharpness, &h_), ctx_, "GlossyClamped");
    }
};
struct Emission : Material {
    Emission(Context& c, const float power[3]) : Material(c) {
        check(xgb_material_emission(ctx_, power, &h_), ctx_, "Emission");
    }
};
struct SpecularReflection : Material {
    explicit SpecularReflection(Context& c) : Material(c) {
        check(xgb_material_specular_reflection(ctx_, &h_), ctx_, "SpecularReflection");
    }
};
struct SpecularRefraction : Material {
    SpecularRefraction(Context& c, float index) : Material(c) {
        check(xgb_material_specular_refraction(ctx_, index, &h_), ctx_, "SpecularRefraction");
    }
};
struct SpecularFresnel : Material {
    SpecularFresnel(Context& c, float index) : Material(c) {
        check(xgb_material_specular_fresnel(ctx_, index, &h_), ctx_, "SpecularFresnel");
    }
};
struct MicrofacetNormalMapping : Material {
    MicrofacetNormalMapping(Context& c, std::shared_ptr<Material> base) : Material(c), base_(base) {
        check(xgb_material_mf_normalmap(ctx_, base->get(), &h_), ctx_, "MicrofacetNormalMapping");
    }
    std::shared_ptr<Material> base_;
};
// MultiLobeSVBRDF(baseMaterial, displacementTexLow, displacementScale, svndf) (Main.cpp:472-517).
struct MultiLobeSVBRDF : Material {
    MultiLobeSVBRDF(Context& c, std::shared_ptr<Material> base, std::shared_ptr<SVNDF> svndf)
        : Material(c), base_(base), svndf_(svndf) {
        check(xgb_material_multilobe_svbrdf(ctx_, base->get(), svndf->get(), &h_), ctx_, "MultiLobeSVBRDF");
    }
    std::shared_ptr<Material> base_;
    std::shared_ptr<SVNDF> svndf_;
};

struct Object {
    Object(std::shared_ptr<TriangleMesh> shape, std::shared_ptr<Material> material, const Transform& objectToWorld)
        : shape(shape), material(material), objectToWorld(objectToWorld) {}
    std::shared_ptr<TriangleMesh> shape;
    std::shared_ptr<Material> material;
    Transform objectToWorld;
};

struct PinholeCamera {
    PinholeCamera(const Transform& cameraToWorld, float fov, float aspectRatio)
        : cameraToWorld(cameraToWorld), fov(fov), aspectRatio(aspectRatio) {}
    Transform cameraToWorld;
    float fov, aspectRatio;
};

struct StandardPathTracer {
    xgb_integrator_params params;
    StandardPathTracer() { xgb_integrator_params_default(&params); }
};
struct NaivePathTracer {
    xgb_integrator_params params;
    NaivePathTracer() { xgb_integrator_params_default(&params); params.integrator = XGB_INTEGRATOR_NAIVE; }
};

class Scene {
public:
    explicit Scene(Context& ctx) : ctx_(ctx.get()) { check(xgb_scene_create(ctx_, &h_), ctx_, "Scene"); }
    ~Scene() { if (h_) xgb_scene_destroy(h_); }
    void addObject(std::shared_ptr<Object> o) {
        check(xgb_scene_add_object(h_, o->shape->get(), o->material->get(), o->objectToWorld.mat,
                                   o->objectToWorld.matInv),
              ctx_, "Scene::addObject");
        objects_.push_back(o);
    }
    void setCamera(const PinholeCamera& c) {
        check(xgb_scene_set_camera_pinhole(h_, c.cameraToWorld.mat, c.cameraToWorld.matInv, c.fov, c.aspectRatio),
              ctx_, "Scene::camera");
    }
    void setSkyUniform(const float rgb[3]) { check(xgb_scene_set_sky_uniform(h_, rgb), ctx_, "SkySphereUniform"); }
    void setSkyProbe(std::shared_ptr<Texture> t) { sky_ = t; check(xgb_scene_set_sky_probe(h_, t->get()), ctx_, "SkySphereFromImage"); }
    void setSkyLatLong(std::shared_ptr<Texture> t) { sky_ = t; check(xgb_scene_set_sky_latlong(h_, t->get()), ctx_, "sky"); }
    void buildAccelerationStructure(void* stream = nullptr) {
        check(xgb_scene_build(h_, stream), ctx_, "Scene::buildAccelerationStructure");
    }
    xgb_scene* get() const { return h_; }
    xgb_ctx* ctx() const { return ctx_; }

private:
    xgb_ctx* ctx_;
    xgb_scene* h_ = nullptr;
    std::vector<std::shared_ptr<Object>> objects_;
    std::shared_ptr<Texture> sky_;
};

// Device film of radiance sums (RenderTarget<Vector3f>).
class RenderTarget {
public:
    RenderTarget(Context& ctx, int width, int height, bool fp64 = false) : ctx_(ctx.get()), width(width), height(height) {
        check(xgb_film_create(ctx_, width, height, fp64 ? 1 : 0, &h_), ctx_, "RenderTarget");
    }
    ~RenderTarget() { if (h_) xgb_film_destroy(h_); }
    void clear(void* stream = nullptr) { check(xgb_film_clear(h_, stream), ctx_, "RenderTarget::clear"); }
    // Adds samples [sampleBegin, sampleBegin + sampleNum) of every pixel.
    template <class Tracer>
    void render(Scene& scene, int sampleNum, const Tracer& tracer, unsigned sampleBegin = 0, void* stream = nullptr) {
        check(xgb_render(scene.get(), &tracer.params, h_, sampleBegin, (uint32_t)sampleNum, stream), ctx_,
              "RenderTarget::render");
    }
    // Copies the sums into host memory: strideBytes 16 for xitils::Vector3f, 12 for packed float3.
    void download(float* host, int strideBytes = 16, void* stream = nullptr) {
        check(xgb_film_download(h_, host, strideBytes, stream), ctx_, "RenderTarget::download");
    }
    const int width, height;

protected:
    xgb_film* handle() const { return h_; }
    xgb_ctx* ctx_;

private:
    xgb_film* h_ = nullptr;
};

// DenoisableRenderTarget (RenderTarget.h:131-145): radiance plus the first-hit
// albedo and normal sums that a denoiser takes as auxiliary images.
class DenoisableRenderTarget : public RenderTarget {
public:
    DenoisableRenderTarget(Context& ctx, int width, int height, bool fp64 = false) : RenderTarget(ctx, width, height, fp64) {
        check(xgb_film_enable_aovs(handle()), ctx_, "DenoisableRenderTarget");
    }
    void downloadAlbedo(float* host, int strideBytes = 16, void* stream = nullptr) {
        check(xgb_film_download_aov(handle(), XGB_AOV_ALBEDO, host, strideBytes, stream), ctx_, "downloadAlbedo");
    }
    void downloadNormal(float* host, int strideBytes = 16, void* stream = nullptr) {
        check(xgb_film_download_aov(handle(), XGB_AOV_NORMAL, host, strideBytes, stream), ctx_, "downloadNormal");
    }
};

}  // namespace xgb
