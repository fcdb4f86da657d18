/* Scene-building API shared by the two CPU checkers.
 *
 * TEST INFRASTRUCTURE ONLY. Two libraries export this API:
 *   - liboracle.so  (prefix xcpu_): oracle/xgb_cpu.cpp, the project's own CPU
 *     restatement of Xitils' StandardPathTracer and everything it calls;
 *   - oracle/_ref/libxref.so (prefix xref_): oracle/ref_harness.cpp, which runs
 *     the reference's own headers (a patched copy, see oracle/build_ref.py).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
 * either library. The product (libxgb.so) never links or calls them.
 *
 * Conventions (identical to the product's C ABI in include/xgb.h):
 *   positions / normals / tangents / bitangents: packed float[nV][3];
 *   texcoords: packed float[nV][2]; indices: int32[nIdx];
 *   matrices: float[16] row-major m[r][c] (Xitils Matrix4x4 layout);
 *   textures: packed float RGB [h][w][3], row y = 0 first (Texture.h:41-80);
 *   films: float RGB sums [H][W][3], pixel (x, y) at (x + y * W) (RenderTarget.h:25-27).
 *
 * Per-material BSDF queries (the materials' unit tests): a flat shading point at the
 * origin with n = shading.n = +z, tangent +x, bitangent +y, texcoord (0.5, 0.5) and the
 * given wo (unit, any side).
 *   bsdf_sample_pcg: n draws of Material::evalAndSample, draw k on the PCG stream
 *     (k, 0, seed): out[k] = wi.xyz, returned weight rgb, pdf (7 floats; a zero
 *     weight leaves wi and pdf undefined, as in Material.h:21-25).
 *   bsdf_eval_pcg: for each wi[k], getPDF and bsdfCos (a stochastic bsdfCos draws on
 *     the stream (k, 1, seed)): out[k] = pdf, rgb (4 floats). Specular materials
 *     have neither; the call returns -2 for them.
 *
 * light_sample_pcg (built scenes only, -3 otherwise): n draws of Scene::sampleSurface
 * (Scene.h:40-47), draw k on the PCG stream (k, 2, seed): out[k] = p.xyz, geometric
 * normal n.xyz, pdf (area measure) (7 floats).
 *
 * intersect / intersect_any (built scenes only, -3 otherwise): Scene::intersect and
 * Scene::intersectAny (Scene.h:30-36) for rays float[n][7] (o, d, tMax):
 * out[k] = t (the shrunk tMax), object index (-1: miss), p.xyz, shading normal xyz
 * (8 floats); any-hit: out[k] = 0 / 1.
 */
#ifndef XGB_ORACLE_SCENE_API_H
#define XGB_ORACLE_SCENE_API_H
#include <stdint.h>

enum {
    ORC_MAT_DIFFUSE = 0,          /* f: albedo rgb;                      tex: albedo texture      */
    ORC_MAT_METAL = 1,            /* f: roughness, f0 rgb;               tex: roughness texture (nearest, .r) */
    ORC_MAT_GLOSSY = 2,           /* f: albedo rgb, sharpness                                      */
    ORC_MAT_GLOSSY_HIGHLIGHT = 3, /* f: albedo rgb, highlight rgb, sharpness, sharpnessHL, rate    */
    ORC_MAT_GLOSSY_CLAMPED = 4,   /* f: albedo rgb, sharpness (MicrofacetBasedNormalMapping sandbox) */
    ORC_MAT_EMISSION = 5,         /* f: power rgb                                                  */
    ORC_MAT_SPECULAR_REFLECTION = 6,
    ORC_MAT_SPECULAR_REFRACTION = 7, /* f: index */
    ORC_MAT_SPECULAR_FRESNEL = 8,    /* f: index */
    ORC_MAT_MF_NORMALMAP = 9,        /* base: material id of the facet material                   */
    ORC_MAT_MULTILOBE_SVBRDF = 10    /* base: material id; tex: SVNDF id (add_svndf)              */
};

enum { ORC_SKY_NONE = 0, ORC_SKY_UNIFORM = 1, ORC_SKY_PROBE = 2, ORC_SKY_LATLONG = 3 };

enum { ORC_INTEGRATOR_STANDARD = 0, ORC_INTEGRATOR_NAIVE = 1 };

#define ORC_DECLARE_SCENE_API(P)                                                                   \
    void* P##scene_new(void);                                                                      \
    void P##scene_free(void* s);                                                                   \
    int P##add_texture(void* s, int w, int h, const float* rgb, int wrap_clamp, int filter);       \
    int P##add_mesh(void* s, int nV, const float* pos, const float* uv, const float* nrm,          \
                    const float* tan, const float* bit, int nIdx, const int32_t* idx);             \
    int P##add_mesh_shell(void* s, int nV, const float* pos, const float* uv, const float* nrm,    \
                          const float* tan, const float* bit, int nIdx, const int32_t* idx,        \
                          int tex, float scale, int layers);                                       \
    int P##add_svndf(void* s, int tex, float scale, int rate, uint32_t seed, int* low_tex);         \
    int P##svndf_fit(const float* rgb, int w, int h, int wrap_clamp, float scale, int rate,          \
                     uint32_t seed, float* low_r, float* lobes);                                     \
    int P##vmf4_sample_pcg(const float* lobes, int n, uint32_t seed, float* dirs);                  \
    int P##add_material(void* s, int type, const float* f, int base, int tex, int normalmap);      \
    int P##bsdf_sample_pcg(void* s, int material, const float* wo, int n, uint32_t seed,           \
                           float* out);                                                            \
    int P##bsdf_eval_pcg(void* s, int material, const float* wo, int n, const float* wi,           \
                         uint32_t seed, float* out);                                               \
    int P##light_sample_pcg(void* s, int n, uint32_t seed, float* out);                            \
    int P##intersect(void* s, int n, const float* rays, float* out);                               \
    int P##intersect_any(void* s, int n, const float* rays, int32_t* out);                         \
    int P##add_object(void* s, int mesh, int material, const float* mat, const float* matInv);     \
    int P##set_camera(void* s, const float* c2w, const float* c2wInv, float fov, float aspect);    \
    int P##set_sky(void* s, int type, const float* rgb, int tex);                                  \
    int P##set_fixes(void* s, int fixes);                                                          \
    int P##build(void* s);                                                                         \
    int P##render_pcg(void* s, int W, int H, uint32_t spp_begin, uint32_t spp_count,               \
                      uint32_t seed, int integrator, int max_depth, int rr_start, float rr_prob,   \
                      int x0, int y0, int x1, int y1, float* film, int nthreads);              \
    int P##render_pcg_aov(void* s, int W, int H, uint32_t spp_begin, uint32_t spp_count,           \
                          uint32_t seed, int integrator, int max_depth, int rr_start,              \
                          float rr_prob, int x0, int y0, int x1, int y1, float* film, float* aov,  \
                          int nthreads);

#endif
