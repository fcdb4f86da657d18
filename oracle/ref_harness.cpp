// ref_harness — runs the reference's own path tracer (Xitils headers) behind
// the checker API of oracle/scene_api.h.
//
// TEST INFRASTRUCTURE ONLY. Built by oracle/build_ref.py into
// oracle/_ref/libxref.so from a patched copy of the reference headers in
// oracle/_ref/src (two mechanical g++ fixes; see build_ref.py) plus the shims
// in oracle/shim. Nothing here is part of the product.
//
// Everything on the rendering path is the reference's code:
//   TriangleMesh::setGeometry (TriangleMesh.h:151-161), Object (Object.h:32-34),
//   Scene::addObject / buildAccelerationStructure (Scene.h:17-28),
//   PinholeCamera (Camera.h:32-55), the materials (Material.h), SkySphereFromImage
//   and SkySphereUniform (SkySphere.h), StandardPathTracer / NaivePathTracer
//   (PathTracer.h), RenderTarget / RenderTargetTile (RenderTarget.h), and the
//   sandbox materials GlossyClamped / MicrofacetNormalMapping extracted verbatim
//   from Sandbox/MicrofacetBasedNormalMapping/Main.cpp:13-340, and SVNDF /
//   MultiLobeSVBRDF extracted verbatim from
//   Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/Main.cpp:361-389, 472-517.
// The harness adds, through the reference's own virtual interfaces (the way
// the sandboxes extend it):
//   - PcgSampler: a Sampler whose protected virtual rand() (Sampler.h:74) draws
//     from the per-(pixel, sample) PCG32 stream shared with the GPU path;
//   - MetalRoughnessTexture: Metal (Material.h:275-384) whose roughness is read
//     per hit from a texture (nearest lookup, red channel); every call builds a
//     reference Metal with that roughness and delegates to it;
//   - SkySphereLatLong: a lat-long environment map looked up with the
//     reference's Texture::rgb (SkySphere.h:9-12 is a virtual interface).
#include "cinder_prelude.h"

#include <Xitils/AccelerationStructure.h>
#include <Xitils/Camera.h>
#include <Xitils/Geometry.h>
#include <Xitils/Material.h>
#include <Xitils/PathTracer.h>
#include <Xitils/RenderTarget.h>
#include <Xitils/Scene.h>
#include <Xitils/SkySphere.h>
#include <Xitils/TriangleMesh.h>
#include <Xitils/VonMisesFisherDistribution.h>

#include "mfnm_extract.h"
#include "svndf_extract.h"

#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "scene_api.h"

using namespace xitils;

namespace {

uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

class PcgSampler : public _SamplerMersenneTwister {
public:
    PcgSampler() : _SamplerMersenneTwister(0) {}
    void seedPath(uint32_t pixel, uint32_t sample, uint32_t seed) {
        uint64_t initstate = splitmix64(((uint64_t)seed << 32) ^ (uint64_t)sample);
        state = 0;
        inc = ((uint64_t)pixel << 1) | 1u;
        step();
        state += initstate;
        step();
    }

protected:
    unsigned int rand() override { return step(); }

private:
    uint64_t state = 0, inc = 1;
    uint32_t step() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((-rot) & 31));
    }
};

class MetalRoughnessTexture : public Material {
public:
    MetalRoughnessTexture(std::shared_ptr<Texture> rough, const Vector3f& f0) : rough(rough), f0(f0) {}
    Vector3f bsdfCos(const SurfaceIntersection& isect, Sampler& sampler, const Vector3f& wi) const override {
        return at(isect).bsdfCos(isect, sampler, wi);
    }
    Vector3f evalAndSample(const SurfaceIntersection& isect, Sampler& sampler, Vector3f* wi, float* pdf) const override {
        return at(isect).evalAndSample(isect, sampler, wi, pdf);
    }
    float getPDF(const SurfaceIntersection& isect, const Vector3f& wi) const override { return at(isect).getPDF(isect, wi); }
    Vector3f getAlbedo(const SurfaceIntersection& isect) const override { return f0; }

private:
    Metal at(const SurfaceIntersection& isect) const { return Metal(rough->rgb(isect.texCoord).x, f0); }
    std::shared_ptr<Texture> rough;
    Vector3f f0;
};

class SkySphereLatLong : public SkySphere {
public:
    explicit SkySphereLatLong(std::shared_ptr<Texture> tex) : tex(tex) {}
    Vector3f getRadiance(const Vector3f& wi) override {
        float u = atan2f(wi.x, -wi.z) * (0.5f / Pi) + 0.5f;
        float cy = wi.y < -1.0f ? -1.0f : (wi.y > 1.0f ? 1.0f : wi.y);
        float v = acosf(cy) * (1.0f / Pi);
        return tex->rgb(Vector2f(u, v));
    }

private:
    std::shared_ptr<Texture> tex;
};

struct RefScene {
    Scene scene;
    std::vector<std::shared_ptr<Texture>> textures;
    std::vector<std::string> textureNames;
    std::vector<std::shared_ptr<TriangleMesh>> meshes;
    std::vector<std::shared_ptr<Material>> materials;
    std::vector<std::shared_ptr<SVNDF>> svndfs;
    std::vector<std::shared_ptr<Texture>> svndfLow;
    std::vector<float> svndfScale;
    std::vector<const Object*> objects;  // in add_object order, for the queries' object index
    bool built = false;
    int serial = 0;
};

// downsampleDisplacementTexture (Prefiltering sandbox Main.cpp:391-470) restated with
// the reference's own Texture and VonMisesFisherDistribution<VMFLobeNum>::approximateBySEM:
// the reference seeds one sampler per OpenMP thread (scheduling decides which texel
// draws from which stream); here low texel t draws from the PCG stream (t, 0, seed).
std::shared_ptr<Texture> svndfBuild(const Texture& orig, float scale, int rate, uint32_t seed, SVNDF& sv) {
    auto low = std::make_shared<Texture>((orig.getWidth() + rate - 1) / rate, (orig.getHeight() + rate - 1) / rate);
    low->warpClamp = orig.warpClamp;
    sv.resolutionU = low->getWidth();
    sv.resolutionV = low->getHeight();
    sv.vmfs.clear();
    sv.vmfs.resize(low->getWidth() * low->getHeight());
    for (int py = 0; py < low->getHeight(); ++py) {
        for (int px = 0; px < low->getWidth(); ++px) {
            const int t = py * low->getWidth() + px;
            PcgSampler sampler;
            sampler.seedPath((uint32_t)t, 0, seed);
            int count = 0;
            std::vector<Vector3f> normals;
            for (int ly = 0; ly < rate; ++ly) {
                int y = py * rate + ly;
                if (y >= orig.getHeight()) continue;
                for (int lx = 0; lx < rate; ++lx) {
                    int x = px * rate + lx;
                    if (x >= orig.getWidth()) continue;
                    Vector2f slope = Vector2f(orig.rgbDifferentialU(x, y).x, orig.rgbDifferentialV(x, y).x);
                    Vector3f n = Vector3f(-slope.u * scale, -slope.v * scale, 1).normalize();
                    low->r(px, py) += orig.r(x, y);
                    normals.push_back(n);
                    ++count;
                }
            }
            low->r(px, py) /= count;
            sv.vmfs[t] = VonMisesFisherDistribution<VMFLobeNum>::approximateBySEM(normals, sampler);
        }
    }
    return low;
}

int g_serial = 0;

std::vector<Vector3f> toV3(const float* a, int n) {
    std::vector<Vector3f> v(n);
    for (int i = 0; i < n; ++i) v[i] = Vector3f(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return v;
}

Transform toTransform(const float* m, const float* mi) { return Transform(Matrix4x4(m), Matrix4x4(mi)); }

}  // namespace

extern "C" {
ORC_DECLARE_SCENE_API(xref_)

void* xref_scene_new(void) {
    RefScene* s = new RefScene();
    s->serial = ++g_serial;
    return s;
}
void xref_scene_free(void* p) {
    RefScene* s = (RefScene*)p;
    for (auto& n : s->textureNames) stbi_mem_registry().erase(n);
    delete s;
}

int xref_add_texture(void* p, int w, int h, const float* rgb, int wrap_clamp, int filter) {
    RefScene* s = (RefScene*)p;
    std::string name = "mem:" + std::to_string(s->serial) + ":" + std::to_string(s->textures.size());
    stbi_mem_image img;
    img.width = w; img.height = h;
    img.rgb.assign(rgb, rgb + (size_t)w * h * 3);
    stbi_mem_registry()[name] = std::move(img);
    auto tex = std::make_shared<Texture>(name);  // Texture.h:17-23
    tex->warpClamp = wrap_clamp != 0;
    tex->filter = filter != 0;
    s->textures.push_back(tex);
    s->textureNames.push_back(name);
    return (int)s->textures.size() - 1;
}

int xref_add_mesh(void* p, int nV, const float* pos, const float* uv, const float* nrm, const float* tan,
                  const float* bit, int nIdx, const int32_t* idx) {
    RefScene* s = (RefScene*)p;
    std::vector<Vector3f> P = toV3(pos, nV), N, T, B;
    std::vector<Vector2f> UV;
    if (nrm) N = toV3(nrm, nV);
    if (tan) T = toV3(tan, nV);
    if (bit) B = toV3(bit, nV);
    if (uv) { UV.resize(nV); for (int i = 0; i < nV; ++i) UV[i] = Vector2f(uv[2 * i], uv[2 * i + 1]); }
    std::vector<int> I(idx, idx + nIdx);
    auto mesh = std::make_shared<TriangleMesh>();
    mesh->setGeometry(nV, P.data(), uv ? UV.data() : nullptr, nrm ? N.data() : nullptr, tan ? T.data() : nullptr,
                      bit ? B.data() : nullptr, nIdx, I.data());
    s->meshes.push_back(mesh);
    return (int)s->meshes.size() - 1;
}

// The reference's own TriangleMesh::setGeometryWithShellMapping (TriangleMesh.h:163-177).
// Every attribute is required: the reference replicates each array per layer.
int xref_add_mesh_shell(void* p, int nV, const float* pos, const float* uv, const float* nrm, const float* tan,
                        const float* bit, int nIdx, const int32_t* idx, int tex, float scale, int layers) {
    RefScene* s = (RefScene*)p;
    if (!uv || !nrm || !tan || !bit || layers < 1 || tex < 0 || tex >= (int)s->textures.size()) return -1;
    std::vector<Vector3f> P = toV3(pos, nV), N = toV3(nrm, nV), T = toV3(tan, nV), B = toV3(bit, nV);
    std::vector<Vector2f> UV(nV);
    for (int i = 0; i < nV; ++i) UV[i] = Vector2f(uv[2 * i], uv[2 * i + 1]);
    std::vector<int> I(idx, idx + nIdx);
    auto mesh = std::make_shared<TriangleMesh>();
    mesh->setGeometryWithShellMapping(nV, P.data(), UV.data(), N.data(), T.data(), B.data(), nIdx, I.data(),
                                      s->textures[tex], scale, layers);
    s->meshes.push_back(mesh);
    return (int)s->meshes.size() - 1;
}

int xref_add_svndf(void* p, int tex, float scale, int rate, uint32_t seed, int* low_tex) {
    RefScene* s = (RefScene*)p;
    if (tex < 0 || tex >= (int)s->textures.size() || rate < 1 || !low_tex) return -1;
    auto sv = std::make_shared<SVNDF>();
    auto low = svndfBuild(*s->textures[tex], scale, rate, seed, *sv);
    s->textures.push_back(low);
    *low_tex = (int)s->textures.size() - 1;
    s->svndfs.push_back(sv);
    s->svndfLow.push_back(low);
    s->svndfScale.push_back(scale);
    return (int)s->svndfs.size() - 1;
}

int xref_svndf_fit(const float* rgb, int w, int h, int wrap_clamp, float scale, int rate, uint32_t seed,
                   float* low_r, float* lobes) {
    if (!rgb || w <= 0 || h <= 0 || rate < 1) return -1;
    Texture t(w, h);
    for (int i = 0; i < w * h * 3; ++i) t[i] = rgb[i];
    t.warpClamp = wrap_clamp != 0;
    SVNDF sv;
    auto low = svndfBuild(t, scale, rate, seed, sv);
    for (size_t i = 0; i < sv.vmfs.size(); ++i) {
        low_r[i] = low->r((int)(i % low->getWidth()), (int)(i / low->getWidth()));
        for (int j = 0; j < VMFLobeNum; ++j) {
            float* o = lobes + (i * VMFLobeNum + j) * 5;
            o[0] = sv.vmfs[i].mu[j].x; o[1] = sv.vmfs[i].mu[j].y; o[2] = sv.vmfs[i].mu[j].z;
            o[3] = sv.vmfs[i].kappa[j]; o[4] = sv.vmfs[i].alpha[j];
        }
    }
    return 0;
}

int xref_vmf4_sample_pcg(const float* lobes, int n, uint32_t seed, float* dirs) {
    VonMisesFisherDistribution<4> v;
    for (int j = 0; j < 4; ++j) {
        v.mu[j] = Vector3f(lobes[5 * j], lobes[5 * j + 1], lobes[5 * j + 2]);
        v.kappa[j] = lobes[5 * j + 3];
        v.alpha[j] = lobes[5 * j + 4];
    }
    PcgSampler sampler;
    for (int i = 0; i < n; ++i) {
        sampler.seedPath((uint32_t)i, 0, seed);
        Vector3f d = v.sample(sampler);
        dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    }
    return 0;
}

// Flat shading point of the per-material queries (scene_api.h), as a
// SurfaceIntersection (Interaction.h:16-32).
static SurfaceIntersection flatIsect(const float* wo) {
    SurfaceIntersection is;
    is.p = Vector3f(0, 0, 0);
    is.wo = Vector3f(wo[0], wo[1], wo[2]);
    is.n = is.shading.n = Vector3f(0, 0, 1);
    is.tangent = is.shading.tangent = Vector3f(1, 0, 0);
    is.bitangent = is.shading.bitangent = Vector3f(0, 1, 0);
    is.texCoord = Vector2f(0.5f, 0.5f);
    return is;
}

int xref_bsdf_sample_pcg(void* p, int material, const float* wo, int n, uint32_t seed, float* out) {
    RefScene* s = (RefScene*)p;
    if (!s || !wo || !out || n < 0 || material < 0 || material >= (int)s->materials.size()) return -1;
    const SurfaceIntersection is = flatIsect(wo);
    PcgSampler sampler;
    try {
        for (int k = 0; k < n; ++k) {
            sampler.seedPath((uint32_t)k, 0, seed);
            Vector3f wi(0, 0, 0);
            float pdf = 0.0f;
            Vector3f f = s->materials[material]->evalAndSample(is, sampler, &wi, &pdf);
            float* o = out + 7 * (size_t)k;
            o[0] = wi.x; o[1] = wi.y; o[2] = wi.z; o[3] = f.x; o[4] = f.y; o[5] = f.z; o[6] = pdf;
        }
    } catch (...) {
        return -2;
    }
    return 0;
}

int xref_bsdf_eval_pcg(void* p, int material, const float* wo, int n, const float* wi, uint32_t seed, float* out) {
    RefScene* s = (RefScene*)p;
    if (!s || !wo || !wi || !out || n < 0 || material < 0 || material >= (int)s->materials.size()) return -1;
    const SurfaceIntersection is = flatIsect(wo);
    PcgSampler sampler;
    try {
        for (int k = 0; k < n; ++k) {
            sampler.seedPath((uint32_t)k, 1, seed);
            const Vector3f w(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
            float pdf = s->materials[material]->getPDF(is, w);
            Vector3f f = s->materials[material]->bsdfCos(is, sampler, w);
            float* o = out + 4 * (size_t)k;
            o[0] = pdf; o[1] = f.x; o[2] = f.y; o[3] = f.z;
        }
    } catch (...) {  // specular materials and Emission throw NOT_IMPLEMENTED (Utils.h:27)
        return -2;
    }
    return 0;
}

int xref_light_sample_pcg(void* p, int n, uint32_t seed, float* out) {
    RefScene* s = (RefScene*)p;
    if (!s || !out || n < 0) return -1;
    if (!s->built) return -3;
    if (!s->scene.canSampleLight()) return -2;
    PcgSampler sampler;
    for (int k = 0; k < n; ++k) {
        sampler.seedPath((uint32_t)k, 2, seed);
        float pdf = 0.0f;
        auto ls = s->scene.sampleSurface(sampler, &pdf);
        float* o = out + 7 * (size_t)k;
        o[0] = ls.p.x; o[1] = ls.p.y; o[2] = ls.p.z; o[3] = ls.n.x; o[4] = ls.n.y; o[5] = ls.n.z; o[6] = pdf;
    }
    return 0;
}

int xref_intersect(void* p, int n, const float* rays, float* out) {
    RefScene* s = (RefScene*)p;
    if (!s || !rays || !out || n < 0) return -1;
    if (!s->built) return -3;
    for (int i = 0; i < n; ++i) {
        Ray r(Vector3f(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]),
              Vector3f(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]), rays[7 * i + 6]);
        SurfaceIntersection is;
        float* o = out + 8 * (size_t)i;
        const bool hit = s->scene.intersect(r, &is);
        int obj = -1;
        if (hit)
            for (size_t k = 0; k < s->objects.size(); ++k)
                if (s->objects[k] == is.object) obj = (int)k;
        o[0] = r.tMax;
        o[1] = (float)obj;
        o[2] = hit ? is.p.x : 0.0f; o[3] = hit ? is.p.y : 0.0f; o[4] = hit ? is.p.z : 0.0f;
        o[5] = hit ? is.shading.n.x : 0.0f; o[6] = hit ? is.shading.n.y : 0.0f; o[7] = hit ? is.shading.n.z : 0.0f;
    }
    return 0;
}

int xref_intersect_any(void* p, int n, const float* rays, int32_t* out) {
    RefScene* s = (RefScene*)p;
    if (!s || !rays || !out || n < 0) return -1;
    if (!s->built) return -3;
    for (int i = 0; i < n; ++i) {
        Ray r(Vector3f(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]),
              Vector3f(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]), rays[7 * i + 6]);
        out[i] = s->scene.intersectAny(r) ? 1 : 0;
    }
    return 0;
}

int xref_add_material(void* p, int type, const float* f, int base, int tex, int normalmap) {
    RefScene* s = (RefScene*)p;
    std::shared_ptr<Material> m;
    switch (type) {
    case ORC_MAT_DIFFUSE: {
        auto d = std::make_shared<Diffuse>(Vector3f(f[0], f[1], f[2]));
        if (tex >= 0) d->texture = s->textures[tex];
        m = d;
        break;
    }
    case ORC_MAT_METAL:
        if (f[4] != 0.0f) return -1;  // the below-horizon fix is not a reference behaviour
        if (tex >= 0) m = std::make_shared<MetalRoughnessTexture>(s->textures[tex], Vector3f(f[1], f[2], f[3]));
        else m = std::make_shared<Metal>(f[0], Vector3f(f[1], f[2], f[3]));
        break;
    case ORC_MAT_GLOSSY: m = std::make_shared<Glossy>(Vector3f(f[0], f[1], f[2]), f[3]); break;
    case ORC_MAT_GLOSSY_CLAMPED: m = std::make_shared<GlossyClamped>(Vector3f(f[0], f[1], f[2]), f[3]); break;
    case ORC_MAT_GLOSSY_HIGHLIGHT:
        m = std::make_shared<GlossyWithHighLight>(Vector3f(f[0], f[1], f[2]), Vector3f(f[3], f[4], f[5]), f[6], f[7], f[8]);
        break;
    case ORC_MAT_EMISSION: m = std::make_shared<Emission>(Vector3f(f[0], f[1], f[2])); break;
    case ORC_MAT_SPECULAR_REFLECTION: m = std::make_shared<SpecularReflection>(); break;
    case ORC_MAT_SPECULAR_REFRACTION: {
        auto r = std::make_shared<SpecularRefraction>();
        r->index = f[0];
        m = r;
        break;
    }
    case ORC_MAT_SPECULAR_FRESNEL: {
        auto r = std::make_shared<SpecularFresnel>();
        r->index = f[0];
        m = r;
        break;
    }
    case ORC_MAT_MF_NORMALMAP:
        if (base < 0 || base >= (int)s->materials.size()) return -1;
        m = std::make_shared<MicrofacetNormalMapping>(s->materials[base]);
        break;
    case ORC_MAT_MULTILOBE_SVBRDF:
        if (base < 0 || base >= (int)s->materials.size() || tex < 0 || tex >= (int)s->svndfs.size()) return -1;
        m = std::make_shared<MultiLobeSVBRDF>(s->materials[base], s->svndfLow[tex], s->svndfScale[tex], s->svndfs[tex]);
        break;
    default: return -1;
    }
    if (normalmap >= 0) m->normalmap = s->textures[normalmap];
    s->materials.push_back(m);
    return (int)s->materials.size() - 1;
}

int xref_add_object(void* p, int mesh, int material, const float* mat, const float* matInv) {
    RefScene* s = (RefScene*)p;
    if (mesh < 0 || mesh >= (int)s->meshes.size() || material < 0 || material >= (int)s->materials.size()) return -1;
    auto obj = std::make_shared<Object>(s->meshes[mesh], s->materials[material], toTransform(mat, matInv));
    s->objects.push_back(obj.get());
    s->scene.addObject(obj);
    return 0;
}

int xref_set_camera(void* p, const float* c2w, const float* c2wInv, float fov, float aspect) {
    RefScene* s = (RefScene*)p;
    s->scene.camera = std::make_shared<PinholeCamera>(toTransform(c2w, c2wInv), fov, aspect);
    return 0;
}

int xref_set_sky(void* p, int type, const float* rgb, int tex) {
    RefScene* s = (RefScene*)p;
    switch (type) {
    case ORC_SKY_NONE: s->scene.skySphere = nullptr; return 0;
    case ORC_SKY_UNIFORM: s->scene.skySphere = std::make_shared<SkySphereUniform>(Vector3f(rgb[0], rgb[1], rgb[2])); return 0;
    case ORC_SKY_PROBE:
        if (tex < 0 || tex >= (int)s->textures.size()) return -1;
        s->scene.skySphere = std::make_shared<SkySphereFromImage>(s->textureNames[tex]);
        return 0;
    case ORC_SKY_LATLONG:
        if (tex < 0 || tex >= (int)s->textures.size()) return -1;
        s->scene.skySphere = std::make_shared<SkySphereLatLong>(s->textures[tex]);
        return 0;
    }
    return -1;
}

// The reference has no quirk fixes: only 0 is accepted.
int xref_set_fixes(void* p, int fixes) {
    (void)p;
    return fixes == 0 ? 0 : -1;
}

int xref_build(void* p) {
    RefScene* s = (RefScene*)p;
    s->scene.buildAccelerationStructure();
    s->built = true;
    return 0;
}

// Per-(pixel, sample) PCG render. Only the reference's defaults are available
// (its Russian-roulette constants are private, PathTracer.h:253-257, and it has
// no depth limit), so other parameter values are rejected.
static int renderPcg(void* p, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                     int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                     float* aov, int nthreads) {
    RefScene* s = (RefScene*)p;
    if (!s->built || !s->scene.camera) return -1;
    if (max_depth != 0 || rr_start != 5 || rr_prob != 0.9f) return -2;
    RenderTarget<Vector3f> target(W, H);
    StandardPathTracer standard;
    NaivePathTracer naive;
    const PathTracer& pt = integrator == ORC_INTEGRATOR_NAIVE ? (const PathTracer&)naive : (const PathTracer&)standard;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; ++y) {
        PcgSampler sampler;
        RenderTargetTile<Vector3f> tile;
        tile.image = &target;
        tile.sampler = std::shared_ptr<Sampler>(&sampler, [](Sampler*) {});
        for (int x = x0; x < x1; ++x) {
            uint32_t pixel = (uint32_t)(x + y * W);
            tile.offset = Vector2i((x / RenderTargetTile<Vector3f>::Width) * RenderTargetTile<Vector3f>::Width,
                                   (y / RenderTargetTile<Vector3f>::Height) * RenderTargetTile<Vector3f>::Height);
            Vector2i local(x - tile.offset.x, y - tile.offset.y);
            DenoisableRenderTargetPixel px;  // sum accumulation as in SimplePathTracerWithDenoiser/Main.cpp:144-151
            for (uint32_t k = 0; k < spp_count; ++k) {
                sampler.seedPath(pixel, spp_begin + k, seed);
                Vector2f pFilm = tile.GenerateFilmPosition(local, true);
                Ray ray = s->scene.camera->generateRay(pFilm, sampler);
                PathTracerEvalResult res = pt.eval(s->scene, sampler, ray);
                px.color += res.color;
                px.albedo += res.albedo;
                px.normal += res.normal;
            }
            float* f = film + 3 * (size_t)pixel;
            f[0] += px.color.x; f[1] += px.color.y; f[2] += px.color.z;
            if (aov) {
                float* q = aov + 6 * (size_t)pixel;
                q[0] += px.albedo.x; q[1] += px.albedo.y; q[2] += px.albedo.z;
                q[3] += px.normal.x; q[4] += px.normal.y; q[5] += px.normal.z;
            }
        }
    }
    return 0;
}

// Per-(pixel, sample) PCG render. Only the reference's defaults are available
// (its Russian-roulette constants are private, PathTracer.h:253-257, and it has
// no depth limit), so other parameter values are rejected.
int xref_render_pcg(void* p, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                    int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                    int nthreads) {
    return renderPcg(p, W, H, spp_begin, spp_count, seed, integrator, max_depth, rr_start, rr_prob, x0, y0, x1, y1,
                     film, nullptr, nthreads);
}

// The same render with DenoisableRenderTargetPixel's albedo and normal sums
// (RenderTarget.h:131-145): aov is float[H][W][6].
int xref_render_pcg_aov(void* p, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                        int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                        float* aov, int nthreads) {
    return renderPcg(p, W, H, spp_begin, spp_count, seed, integrator, max_depth, rr_start, rr_prob, x0, y0, x1, y1,
                     film, aov, nthreads);
}

// The reference's stock render call exactly as the sandboxes drive it
// (SimplePathTracer/Main.cpp:134-138): RenderTarget::render over 16x16 tiles,
// one Mersenne-Twister sampler per tile, OpenMP over tiles. Returns the wall
// time in seconds; the film receives the radiance sums.
double xref_render_stock(void* p, int W, int H, int spp, int integrator, float* film, int nthreads) {
    RefScene* s = (RefScene*)p;
    if (!s->built || !s->scene.camera) return -1.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    SimpleRenderTarget target(W, H);
    target.clear();
    StandardPathTracer standard;
    NaivePathTracer naive;
    const PathTracer& pt = integrator == ORC_INTEGRATOR_NAIVE ? (const PathTracer&)naive : (const PathTracer&)standard;
    auto t0 = std::chrono::steady_clock::now();
    target.render(s->scene, spp, [&](const Vector2f& pFilm, Sampler& sampler, Vector3f& color) {
        auto ray = s->scene.camera->generateRay(pFilm, sampler);
        color += pt.eval(s->scene, sampler, ray).color;
    });
    auto t1 = std::chrono::steady_clock::now();
    for (int i = 0; i < W * H; ++i) {
        film[3 * i] = target.data[i].x;
        film[3 * i + 1] = target.data[i].y;
        film[3 * i + 2] = target.data[i].z;
    }
    return std::chrono::duration<double>(t1 - t0).count();
}

// vMF mixture (VonMisesFisherDistribution.h) for L = 8 lobes: the fit
// (approximateBySEM, :68-160), the mixture pdf (eval, :60-66) and sampling
// (sample, :162-201). Encoded parameters follow encode() (:37-45).
int xref_vmf8_fit(const float* samples, int n, uint32_t seed, float* encoded) {
    std::vector<Vector3f> v(n);
    for (int i = 0; i < n; ++i) v[i] = Vector3f(samples[3 * i], samples[3 * i + 1], samples[3 * i + 2]);
    Sampler sampler((int)seed);
    auto vmf = VonMisesFisherDistribution<8>::approximateBySEM(v, sampler);
    vmf.encode(encoded);
    return 0;
}
int xref_vmf8_eval(const float* encoded, int n, const float* dirs, float* pdf) {
    VonMisesFisherDistribution<8> vmf;
    vmf.decode(encoded);
    for (int i = 0; i < n; ++i) pdf[i] = vmf.eval(Vector3f(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
    return 0;
}
int xref_vmf8_sample_pcg(const float* encoded, int n, uint32_t seed, float* dirs) {
    VonMisesFisherDistribution<8> vmf;
    vmf.decode(encoded);
    PcgSampler sampler;
    for (int i = 0; i < n; ++i) {
        sampler.seedPath((uint32_t)i, 0, seed);
        Vector3f d = vmf.sample(sampler);
        dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    }
    return 0;
}
}  // extern "C"
