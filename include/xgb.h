/* xgb.h -- C ABI of the GB300 path tracer (libxgb.so).
 *
 * A drop-in for the render call of Xitils: the same scene-construction calls
 * (meshes, materials, objects with transforms, camera, sky) go in, and a film
 * of per-pixel radiance SUMS comes out, as RenderTarget::render leaves it.
 * Plain C types only: handles are opaque, arrays are host pointers with sizes,
 * CUDA streams travel as void* (cudaStream_t; NULL = the context's stream).
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the Xitils repository). Every call returns an xgb_status; on failure
 * xgb_get_last_error() holds a message. Work is enqueued on the given stream;
 * xgb_film_download() and xgb_render_stats() synchronise it.
 */
#ifndef XGB_H
#define XGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    XGB_OK = 0,
    XGB_INVALID_ARG = 1,     /* bad handle, size, index or parameter            */
    XGB_OOM = 2,             /* device or host allocation failed                */
    XGB_CUDA_ERROR = 3,      /* a CUDA runtime call failed                      */
    XGB_QUEUE_OVERFLOW = 4,  /* a device work queue or traversal stack overflowed */
    XGB_DEVICE_TIMEOUT = 5,  /* a bounded device wait gave up                   */
    XGB_NOT_BUILT = 6,       /* scene used before xgb_scene_build               */
    XGB_UNSUPPORTED = 7      /* feature not available in this build             */
} xgb_status;

typedef struct xgb_ctx xgb_ctx;
typedef struct xgb_texture xgb_texture;
typedef struct xgb_mesh xgb_mesh;
typedef struct xgb_material xgb_material;
typedef struct xgb_scene xgb_scene;
typedef struct xgb_film xgb_film;

/* ---------------------------------------------------------------- context */
/* One context per GPU (and per host thread, or serialise calls on it). */
xgb_status xgb_ctx_create(int device, xgb_ctx** out);
xgb_status xgb_ctx_destroy(xgb_ctx* ctx);
/* Builder of the per-mesh BVH for meshes created afterwards (the tree shape
 * changes speed only, never the image): XGB_BVH_PLOC (default, locally-ordered
 * clustering by surface area) or XGB_BVH_LBVH (Morton-code splits). The
 * reference builds a single-threaded top-down tree (AccelerationStructure.h:163-291). */
#define XGB_BVH_PLOC 0
#define XGB_BVH_LBVH 1
xgb_status xgb_ctx_set_bvh_builder(xgb_ctx* ctx, int builder);
/* Node layout of the per-mesh BVH for meshes created afterwards: XGB_BVH_BINARY
 * (default; 64-byte nodes with two float boxes) or XGB_BVH_WIDE8 (80-byte nodes
 * with eight 8-bit quantised boxes, leaves of up to 3 triangles). */
#define XGB_BVH_BINARY 0
#define XGB_BVH_WIDE8 1
xgb_status xgb_ctx_set_bvh_layout(xgb_ctx* ctx, int layout);
/* Order in which xgb_render fills its wavefront with camera paths: pixel blocks
 * of tile_w x tile_h (rows in bands of tile_h, a band block by block), so that
 * neighbouring paths start close together; 0, 0 = scanline rows (default). The
 * per-pixel random streams make the image independent of the order: this
 * changes speed only. The reference renders 16 x 16 tiles on OpenMP threads
 * (Include/Xitils/RenderTarget.h:58-59, :110-113). */
xgb_status xgb_ctx_set_path_order(xgb_ctx* ctx, int tile_w, int tile_h);
/* Sample order of this context's renders: with samples > 1, consecutive camera
 * paths are `samples` consecutive samples of one pixel (passes of that many
 * samples over the film, the remainder of a call's samples one pass after the
 * other); 0 or 1 = one sample pass over the film after the other. Default 64:
 * a warp's camera rays then leave one or a few pixels, traverse the same nodes
 * and reuse them in L1 and L2. Every
 * (pixel, sample) keeps its own random stream, so this changes speed only. The
 * reference renders one 16 x 16 tile per thread, the tile's pixels once per
 * sample, sample after sample (Include/Xitils/RenderTarget.h:108-127). */
xgb_status xgb_ctx_set_sample_grouping(xgb_ctx* ctx, int samples);
/* Waits for the work enqueued on stream (NULL = the context's own stream). */
xgb_status xgb_ctx_synchronize(xgb_ctx* ctx, void* stream);
/* Last error message of this context ("" when none). Never NULL. */
const char* xgb_get_last_error(const xgb_ctx* ctx);
/* Library version string, e.g. "xgb 0.1 sm_103a". */
const char* xgb_version(void);

/* ---------------------------------------------------------------- texture */
/* Texture(int w, int h) filled with float RGB texels, row y = 0 first
 * (Include/Xitils/Texture.h:25-32, :77-103). wrap_clamp: 1 = clamp
 * (Texture::warpClamp, default), 0 = wrap. filter: 1 = bilinear (default),
 * 0 = nearest. channels: 3 (RGB) or 4 (RGBA, alpha ignored). The data is copied. */
xgb_status xgb_texture_create(xgb_ctx* ctx, int width, int height, int channels, const float* texels,
                              int wrap_clamp, int filter, xgb_texture** out);
xgb_status xgb_texture_destroy(xgb_texture* tex);

/* ------------------------------------------------------------------ meshes */
/* TriangleMesh::setGeometry(vertexNum, positions, texCoords, normals, tangents,
 * bitangents, indexNum, indices) (Include/Xitils/TriangleMesh.h:151-161).
 * vec3_stride: byte stride of positions/normals/tangents/bitangents, 12 (packed
 * float3) or 16 (xitils::Vector3f). uv_stride: 8 (packed float2) or 16
 * (xitils::Vector2f). Optional arrays may be NULL; tangents need bitangents.
 * Indices must lie in [0, vertex_count). All arrays are copied. */
xgb_status xgb_mesh_create(xgb_ctx* ctx, int vertex_count, const float* positions, const float* texcoords,
                           const float* normals, const float* tangents, const float* bitangents, int vec3_stride,
                           int uv_stride, int index_count, const int32_t* indices, xgb_mesh** out);
xgb_status xgb_mesh_destroy(xgb_mesh* mesh);
xgb_status xgb_mesh_triangle_count(const xgb_mesh* mesh, int* out);
/* TriangleMesh::setGeometryWithShellMapping(vertexNum, positions, texCoords,
 * normals, tangents, bitangents, indexNum, indices, displacement, scale,
 * layerNum) (Include/Xitils/TriangleMesh.h:163-177, :279-324): layer_count
 * copies of the mesh, copy l offset along the vertex normals by
 * scale * l / (layer_count - 1); a hit on copy l is discarded where the red
 * channel of the displacement texture at the hit's texcoord is below
 * l / (layer_count - 1), for closest-hit and any-hit rays alike, and a kept
 * hit's shading normal is tilted by the texture's central differences
 * (TriangleIndexedWithShellMapping, TriangleIndexed.h:220-256). Every
 * attribute array is required (the reference replicates all of them). The
 * displacement texture must outlive the mesh. The mesh has
 * layer_count x index_count / 3 triangles. */
xgb_status xgb_mesh_create_shell(xgb_ctx* ctx, int vertex_count, const float* positions, const float* texcoords,
                                 const float* normals, const float* tangents, const float* bitangents,
                                 int vec3_stride, int uv_stride, int index_count, const int32_t* indices,
                                 const xgb_texture* displacement, float displacement_scale, int layer_count,
                                 xgb_mesh** out);

/* --------------------------------------------------------------- materials */
/* Diffuse(albedo) (Include/Xitils/Material.h:50-86); albedo_tex optional (Diffuse::texture). */
xgb_status xgb_material_diffuse(xgb_ctx* ctx, const float albedo[3], const xgb_texture* albedo_tex,
                                xgb_material** out);
/* Metal(roughness, f0): GGX conductor with VNDF sampling (Material.h:275-384).
 * roughness_tex optional: per-hit roughness = red channel of a nearest lookup. */
xgb_status xgb_material_metal(xgb_ctx* ctx, float roughness, const float f0[3], const xgb_texture* roughness_tex,
                              xgb_material** out);
/* Opt-in fixes of reference quirks (the reference has none of them; off by
 * default so that renders match it). XGB_FIX_METAL_HORIZON: Metal reflects
 * nothing when wo or wi lies below its shading normal and samples nothing for
 * wo below it (the reference divides by a clamped zero there and returns
 * inf / NaN, which microfacet normal mapping's random walk over a Metal base
 * reaches). Applies to materials whose scene is built afterwards. */
#define XGB_FIX_METAL_HORIZON 1u
/* Scene-level fix (xgb_scene_set_fixes): XGB_FIX_DROP_NONFINITE skips a
 * radiance contribution with an inf or NaN component instead of adding it to the
 * film (the reference adds it, and one such sample turns the pixel to NaN). */
#define XGB_FIX_DROP_NONFINITE 2u
xgb_status xgb_material_set_fixes(xgb_material* material, uint32_t fixes);
/* Glossy(albedo, sharpness) (Material.h:88-132). */
xgb_status xgb_material_glossy(xgb_ctx* ctx, const float albedo[3], float sharpness, xgb_material** out);
/* GlossyWithHighLight(albedo, highlight, sharpness, sharpnessHighLight, rate) (Material.h:134-175). */
xgb_status xgb_material_glossy_highlight(xgb_ctx* ctx, const float albedo[3], const float highlight[3],
                                         float sharpness, float sharpness_highlight, float rate, xgb_material** out);
/* GlossyClamped(albedo, sharpness) (Sandbox/MicrofacetBasedNormalMapping/Main.cpp:34-84). */
xgb_status xgb_material_glossy_clamped(xgb_ctx* ctx, const float albedo[3], float sharpness, xgb_material** out);
/* Emission(power) (Material.h:386-411): one-sided, emits where dot(wo, n) > 0. */
xgb_status xgb_material_emission(xgb_ctx* ctx, const float power[3], xgb_material** out);
/* SpecularReflection / SpecularRefraction(index) / SpecularFresnel(index) (Material.h:177-273). */
xgb_status xgb_material_specular_reflection(xgb_ctx* ctx, xgb_material** out);
xgb_status xgb_material_specular_refraction(xgb_ctx* ctx, float index, xgb_material** out);
xgb_status xgb_material_specular_fresnel(xgb_ctx* ctx, float index, xgb_material** out);
/* MicrofacetNormalMapping(base) (Sandbox/MicrofacetBasedNormalMapping/Main.cpp:86-340). */
xgb_status xgb_material_mf_normalmap(xgb_ctx* ctx, const xgb_material* base, xgb_material** out);
/* Material::normalmap (Material.h:13; applied in Object.h:58-68). NULL clears it. */
xgb_status xgb_material_set_normalmap(xgb_material* mat, const xgb_texture* normalmap);
xgb_status xgb_material_destroy(xgb_material* mat);

/* ------------------------------------------ SVNDF (prefiltered displacement) */
/* downsampleDisplacementTexture(displacement, scale, svndf) and SVNDF
 * (Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/Main.cpp:361-470), on
 * the GPU: low texel (px, py) covers the rate x rate source texels from
 * (px * rate, py * rate); its height is their mean red value and its normal
 * distribution a 4-lobe vMF mixture fitted by the reference's EM
 * (VonMisesFisherDistribution<4>::approximateBySEM, VonMisesFisherDistribution.h:68-160)
 * to their normals normalize(-dh/du * scale, -dh/dv * scale, 1) (central
 * differences, Texture.h:105-111). The fit of low texel t starts from lobes drawn
 * from the PCG stream (t, 0, seed); the reference draws them from one sampler per
 * OpenMP thread. rate in [1, 16]. *low receives the low-resolution height texture
 * (red channel; bilinear; the source's clamp / wrap mode), which the caller
 * destroys with xgb_texture_destroy. */
typedef struct xgb_svndf xgb_svndf;
xgb_status xgb_svndf_create(xgb_ctx* ctx, const xgb_texture* displacement, float displacement_scale, int rate,
                            uint32_t seed, xgb_svndf** out, xgb_texture** low);
xgb_status xgb_svndf_destroy(xgb_svndf* svndf);
/* Size of the SVNDF (the low texture's width and height). */
xgb_status xgb_svndf_size(const xgb_svndf* svndf, int* width, int* height);
/* Fitted lobes, float[height][width][4][5] = mu.xyz, kappa, alpha. */
xgb_status xgb_svndf_get_lobes(const xgb_svndf* svndf, float* host);
/* Replaces the lobes (same layout), e.g. with a fit stored earlier; scenes built
 * with materials on this SVNDF see the new lobes at their next render. */
xgb_status xgb_svndf_set_lobes(xgb_svndf* svndf, const float* host);
/* MultiLobeSVBRDF(base, lowDisplacement, scale, svndf) (Main.cpp:472-517): at each
 * evaluation and each sample the shading normal is replaced by a normal drawn from
 * the SVNDF at the hit's texcoord (SVNDF::sampleNormal: a stochastic bilinear
 * choice of the texel, then the texel's mixture sampled as
 * VonMisesFisherDistribution::sample does), in the frame of the hit's normal,
 * tangent and bitangent; the base material is evaluated with it. getPDF is the
 * cosine density about the unperturbed shading normal, as in the reference. The
 * base must be a non-emissive material other than microfacet normal mapping or
 * another MultiLobeSVBRDF; the SVNDF must outlive the material. */
xgb_status xgb_material_multilobe_svbrdf(xgb_ctx* ctx, const xgb_material* base, const xgb_svndf* svndf,
                                         xgb_material** out);

/* ------------------------------------------------------------------- scene */
xgb_status xgb_scene_create(xgb_ctx* ctx, xgb_scene** out);
xgb_status xgb_scene_destroy(xgb_scene* scene);
/* Scene::addObject(make_shared<Object>(mesh, material, Transform(mat, matInv)))
 * (Include/Xitils/Scene.h:17-22, Object.h:32-34). mat / mat_inv: float[16]
 * row-major m[r][c] (Matrix4x4). Emissive materials make the object a light,
 * in insertion order. Meshes and materials must outlive the scene. */
xgb_status xgb_scene_add_object(xgb_scene* scene, const xgb_mesh* mesh, const xgb_material* material,
                                const float mat[16], const float mat_inv[16]);
/* scene->camera = make_shared<PinholeCamera>(Transform(c2w, c2w_inv), fov, aspect)
 * (Include/Xitils/Camera.h:32-55). fov in radians; aspect as the reference uses it
 * (tan(fov/2 * aspect) for the vertical extent). */
xgb_status xgb_scene_set_camera_pinhole(xgb_scene* scene, const float c2w[16], const float c2w_inv[16], float fov,
                                        float aspect);
/* scene->skySphere (Include/Xitils/SkySphere.h): none, SkySphereUniform(color),
 * SkySphereFromImage (angular light probe), or a lat-long map
 * (u = atan2(x, -z)/2pi + 1/2, v = acos(y)/pi). */
xgb_status xgb_scene_set_sky_none(xgb_scene* scene);
xgb_status xgb_scene_set_sky_uniform(xgb_scene* scene, const float rgb[3]);
xgb_status xgb_scene_set_sky_probe(xgb_scene* scene, const xgb_texture* probe);
xgb_status xgb_scene_set_sky_latlong(xgb_scene* scene, const xgb_texture* latlong);
/* Scene::buildAccelerationStructure (Scene.h:24-28): uploads the scene and
 * builds the bounding-volume hierarchies on the GPU. stream may be NULL. */
xgb_status xgb_scene_build(xgb_scene* scene, void* stream);

/* -------------------------------------------------------------------- film */
/* RenderTarget<Vector3f>(width, height) (Include/Xitils/RenderTarget.h:13-23):
 * per-pixel radiance sums in device memory, pixel (x, y) at x + y * width.
 * fp64 = 1 accumulates in double (for very high sample counts). */
xgb_status xgb_film_create(xgb_ctx* ctx, int width, int height, int fp64, xgb_film** out);
xgb_status xgb_film_destroy(xgb_film* film);
/* RenderTarget::clear (RenderTarget.h:29-31). */
xgb_status xgb_film_clear(xgb_film* film, void* stream);
/* Copies the sums to host memory as float RGB with the given pixel stride in
 * bytes (12 = packed, 16 = xitils::Vector3f layout). Synchronises the stream. */
xgb_status xgb_film_download(xgb_film* film, float* host, int pixel_stride_bytes, void* stream);
/* Device address of the film (float4 or double4 per pixel, w unused). */
xgb_status xgb_film_device_pointer(xgb_film* film, void** out, int* is_fp64);
/* DenoisableRenderTarget (RenderTarget.h:131-145): xgb_render also sums the
 * first hit's Material::getAlbedo and geometric normal (PathTracer.h:76-80,
 * 138-139; zero for a camera ray that misses) into two more planes of the
 * film's element type. Cleared by xgb_film_clear. */
#define XGB_AOV_ALBEDO 0
#define XGB_AOV_NORMAL 1
xgb_status xgb_film_enable_aovs(xgb_film* film);
xgb_status xgb_film_download_aov(xgb_film* film, int which, float* host, int pixel_stride_bytes, void* stream);

/* ---------------------------------------------------------- image output */
/* Display mapping of RTCamp8/Main.cpp:669-682 on the GPU: per channel
 * clamp((int)(pow(v * exposure, 1 / gamma) * 255), 0, 255) with v = sum * scale
 * (scale = 1 / spp; the reference uses exposure 0.3, gamma 2.2); NaN -> 0.
 * rgb: host array of width * height * 3 bytes, film row 0 first. */
xgb_status xgb_film_tonemap(xgb_film* film, float scale, float exposure, float gamma, unsigned char* rgb, void* stream);
/* VisualizeError/Main.cpp:64-82 on two films of one size: t = (lum(a * scale_a)
 * - lum(b * scale_b))^2 / max_value (rgbToLuminance weights, Vector.h:828-830),
 * coloured by the Jet colormap; rgb as above. */
xgb_status xgb_film_error_map(xgb_film* a, float scale_a, xgb_film* b, float scale_b, float max_value,
                              unsigned char* rgb, void* stream);
/* Writes an 8-bit RGB PNG (rows top to bottom), as stbi_write_png does for
 * RTCamp8/Main.cpp:385-390; uncompressed deflate blocks. */
xgb_status xgb_write_png(const char* path, int width, int height, const unsigned char* rgb);

/* --------------------------------------------------------------- rendering */
typedef enum { XGB_INTEGRATOR_STANDARD = 0, XGB_INTEGRATOR_NAIVE = 1 } xgb_integrator;

typedef struct {
    int integrator;   /* StandardPathTracer (NEE + BSDF sampling, power-heuristic MIS) or NaivePathTracer */
    int max_depth;    /* 0 = unlimited (reference); else the loop stops when pathLength > max_depth */
    int rr_start;     /* Russian roulette when pathLength > rr_start (reference: 5) */
    float rr_prob;    /* survival probability (reference: 0.9) */
    uint32_t seed;    /* PCG stream seed: stream(pixel, sample) = pcg32(splitmix64(seed<<32 ^ sample), pixel) */
    int queue_capacity; /* paths in flight, 0 = automatic (2^23, or the call's path count if smaller) */
} xgb_integrator_params;

/* Fills the reference's defaults (PathTracer.h:253-257). */
void xgb_integrator_params_default(xgb_integrator_params* p);

/* RenderTarget::render(scene, spp, [&](pFilm, sampler, color) {
 *     color += pathTracer.eval(scene, sampler, camera.generateRay(pFilm, sampler)).color; })
 * (Include/Xitils/RenderTarget.h:109-127, PathTracer.h:117-251,
 *  Sandbox/SimplePathTracer/Main.cpp:134-138). Adds the radiance of samples
 * [spp_begin, spp_begin + spp_count) of every pixel to the film. Sample k of a
 * pixel always draws from the same PCG stream, so disjoint sample ranges can be
 * rendered separately (and on different GPUs) and summed. */
xgb_status xgb_render(xgb_scene* scene, const xgb_integrator_params* params, xgb_film* film, uint32_t spp_begin,
                      uint32_t spp_count, void* stream);

typedef struct {
    uint64_t paths;          /* camera paths completed */
    uint64_t extension_rays; /* closest-hit rays traced */
    uint64_t shadow_rays;    /* any-hit rays traced */
    uint64_t iterations;     /* wavefront iterations that had work */
    uint64_t kernel_launches;/* kernels launched by the call */
    uint64_t node_visits;    /* BVH nodes visited by extension rays (profiling only) */
    uint64_t tri_tests;      /* triangle tests of extension rays (profiling only) */
    uint32_t error_flags;    /* device error bits: 1 traversal stack overflow, 4 traversal step bound */
    uint32_t profiled;       /* 1 when the timings below were recorded */
    /* summed device time per kernel stage, CUDA events on the render stream:
       [0] plan, [1] generate, [2] extend (closest hit), [3] shade, [4] shadow (any hit) */
    double kernel_ms[5];
    uint64_t stage_launches[5];
    uint64_t guide_train_steps; /* Adam steps of the learned proposal taken by the call */
    /* profiled calls with a learned proposal: device time of its per-path network
       inference (not part of kernel_ms) and of the end-of-call training (record
       finalisation, pooling, Adam steps) */
    double guide_infer_ms;
    double guide_train_ms;
} xgb_render_stats;

/* ------------------------------------------------------- batched renders */
/* No counterpart in the reference (which renders one RenderTarget at a time):
 * many render jobs -- each a built scene, its own film, integrator parameters and
 * sample range -- advanced by one wavefront, so small films keep the GPU busy
 * next to large ones. Every job's film receives what xgb_render(scene, params,
 * film, spp_begin, spp_count) would add (same per-path random streams; sums in
 * another order). At most 255 jobs, films below 2^24 pixels, all scenes of one
 * context; learned-proposal guiding and AOV planes are not applied here. */
typedef struct {
    xgb_scene* scene;
    xgb_film* film;
    xgb_integrator_params params;
    uint32_t spp_begin;
    uint32_t spp_count;
} xgb_batch_job;
typedef struct {
    int queue_capacity;       /* camera paths in flight; 0 = autotuned */
    int iterations_per_sync;  /* wavefront iterations between host checks (even); 0 = autotuned */
    int use_graph;            /* 1: the iterations between checks replay as one CUDA graph */
} xgb_batch_options;
/* options = NULL: autotuned values (cached per batch shape: scenes, film sizes,
 * sample counts; the first call of a new shape runs the autotuner) with graphs. */
xgb_status xgb_render_batch(const xgb_batch_job* jobs, int n, const xgb_batch_options* options, void* stream);
/* Times short trial renders (1 sample per pixel of every job, into scratch films)
 * for queue capacities 2^18 .. 2^23 and 4 / 8 / 16 iterations per check; writes
 * the fastest to *out and caches it for this batch shape. */
xgb_status xgb_batch_autotune(const xgb_batch_job* jobs, int n, void* stream, xgb_batch_options* out);
/* Counters of the last xgb_render_batch of this context. */
xgb_status xgb_batch_stats_get(xgb_ctx* ctx, xgb_render_stats* out);

/* Counters of the last xgb_render on this scene. Synchronises the stream. */
xgb_status xgb_render_stats_get(xgb_scene* scene, xgb_render_stats* out, void* stream);

/* No counterpart in the reference. The same render as xgb_render, for callers
 * that cannot allocate GPU memory (a host that owns all device memory through
 * its own pool, a frame loop that must not hit cudaMalloc's implicit device
 * synchronisation, a plug-in given only a stream): the path queues, hit records,
 * shadow queue and counters live in a fixed ~6 MB static __device__ array inside
 * the library (held by every GPU that loads it), and the call makes no
 * cudaMalloc, cudaFree or other allocation. At most XGB_NOALLOC_MAX_PATHS paths
 * are in flight: params->queue_capacity above that returns XGB_INVALID_ARG
 * (0 = the maximum); sample counts are not limited. Every call shares the array
 * and re-initialises its counters, so calls whose GPU work overlaps (other
 * streams or threads) race and must be serialised. Every call looks up the
 * array's address with the scene's device current (cudaGetSymbolAddress, no
 * allocation): make the first call on a device before any stream capture.
 * Radiance only: a film with AOV planes or a scene with a learned proposal
 * returns XGB_UNSUPPORTED (both need per-call device memory), and the scene's
 * xgb_render_stats_get counters are not updated. Errors are reported through
 * the return code only (the context's error text is not touched). */
#define XGB_NOALLOC_MAX_PATHS 32768
xgb_status xgb_render_noalloc(xgb_scene* scene, const xgb_integrator_params* params, xgb_film* film,
                              uint32_t spp_begin, uint32_t spp_count, void* stream);

/* ------------------------------------------------------ learned proposal */
/* A 64-64-64-64-40 MLP (BF16 tensor-core kernels, FP32 accumulation, FP32 Adam
 * master weights) mapping a shading point to an 8-lobe von Mises-Fisher mixture
 * with the reference's lobe pdf and sampling (Include/Xitils/VonMisesFisherDistribution.h:
 * pdf :205-211, sample :162-201). Inputs: 6-band sin/cos frequency encoding of the
 * position normalised to the guide bounds, the position, the shading normal, wo.
 * Outputs per lobe: m.xyz (mu = m/|m|), k (kappa = exp(clamp(k, -6, 8))), l
 * (alpha = softmax(l)). No counterpart in the reference path tracer. */
typedef struct xgb_guide xgb_guide;
xgb_status xgb_guide_create(xgb_ctx* ctx, uint32_t seed, xgb_guide** out);
xgb_status xgb_guide_destroy(xgb_guide* guide);
xgb_status xgb_guide_param_count(size_t* out);  /* 15,080 */
/* Save / load: the FP32 master parameters (setting them resets Adam's moments). */
xgb_status xgb_guide_get_params(xgb_guide* guide, float* host, size_t n);
xgb_status xgb_guide_set_params(xgb_guide* guide, const float* host, size_t n);
/* Gradients of the last xgb_guide_train_batch (or in-render training step). */
xgb_status xgb_guide_get_grads(xgb_guide* guide, float* host, size_t n);
/* Box the positions are normalised to (defaults to the scene bounds when rendering). */
xgb_status xgb_guide_set_bounds(xgb_guide* guide, const float lo[3], const float hi[3]);
/* Network outputs (n x 40) for host arrays of positions, normals and wo (n x 3 each). */
xgb_status xgb_guide_infer(xgb_guide* guide, int n, const float* pos, const float* nrm, const float* wo, float* out);
/* Draws one direction per point from the network's mixture with a PCG stream per
 * index (seed), returning the directions (n x 3) and the mixture pdf (n). */
xgb_status xgb_guide_sample(xgb_guide* guide, int n, const float* pos, const float* nrm, const float* wo, uint32_t seed,
                            float* dirs, float* pdf);
/* One Adam step (lr > 0; lr = 0 computes gradients only) on n <= 65536 samples of
 * the loss sum_i -(w_i / sum w) log q(wi_i), w_i = radiance_i / pdf_i. *loss = the loss. */
xgb_status xgb_guide_train_batch(xgb_guide* guide, int n, const float* pos, const float* nrm, const float* wo,
                                 const float* wi, const float* pdf, const float* radiance, float lr, float* loss);
/* In-render training (xgb_scene_set_guide with train = 1): a guided vertex of a
 * camera path becomes a training record (at a rate that spreads about 2^22
 * records over the call); when every path of the call has finished, a record's
 * target is the incident radiance along its sampled direction (the path's
 * later contributions divided by its throughput after the vertex), times the
 * luminance of bsdfCos there when product_target = 1 (default). Records that
 * carry radiance are pooled and consumed in Adam steps of batch_rows records
 * (default 8192, a multiple of 64, at most 65536), at most max_steps_per_call
 * (default 512) at the end of each call; a remainder smaller than a batch stays
 * pooled for the next call. The pool holds 2^22 records; a call that finds more
 * than max_steps_per_call batches drops the excess. */
xgb_status xgb_guide_set_training(xgb_guide* guide, int batch_rows, int max_steps_per_call, int product_target);
/* Polls of each mbarrier wait of the network's tensor-core inference before it
 * gives up (default 2^22; no counterpart in the reference). A wait that gives
 * up makes the call return XGB_DEVICE_TIMEOUT after the kernel has waited
 * (with the default bound) for its matrix operations in flight and freed its
 * tensor memory; the context stays usable. Tests set 0 to take that path. */
xgb_status xgb_guide_set_wait_limit(xgb_guide* guide, int polls);
/* Adam steps taken so far (explicit and in-render). */
xgb_status xgb_guide_train_steps(xgb_guide* guide, uint64_t* out);
/* Guided rendering: at Diffuse / Metal / Glossy vertices xgb_render samples the BSDF
 * with probability bsdf_fraction and the learned mixture otherwise, weighting by
 * the mixture density (one-sample MIS, unbiased at any network state); NEE's MIS
 * uses the same density. train = 1 also trains the network online (see
 * xgb_guide_set_training; standard integrator only; the call then holds 16
 * bytes of device memory per camera path). guide = NULL turns guiding off. */
xgb_status xgb_scene_set_guide(xgb_scene* scene, xgb_guide* guide, float bsdf_fraction, int train, float learning_rate);

/* Opt-in quirk fixes of the render (XGB_FIX_DROP_NONFINITE); 0 = reference behaviour. */
xgb_status xgb_scene_set_fixes(xgb_scene* scene, uint32_t fixes);

/* Scene::intersect / Scene::intersectAny (Scene.h:30-38) for host arrays of n
 * rays, float[n][7] = origin, direction, tMax. xgb_scene_intersect writes
 * float[n][5] = (t of the closest hit, object index in xgb_scene_add_object
 * order, triangle index within its mesh, barycentrics b0, b1); a miss gives
 * (tMax, -1, -1, 0, 0). xgb_scene_occluded writes 1 where something is hit
 * within tMax, else 0. Synchronises the stream. */
xgb_status xgb_scene_intersect(xgb_scene* scene, int n, const float* rays, float* hits, void* stream);
xgb_status xgb_scene_occluded(xgb_scene* scene, int n, const float* rays, int32_t* occluded, void* stream);

/* Device-side bounds of ray traversal on this scene (no counterpart in the
 * reference, whose recursive traversal has none): a ray that takes more than
 * max_steps traversal loop steps ends and the render returns
 * XGB_DEVICE_TIMEOUT; a ray whose traversal would push onto a stack already
 * holding max_stack entries ends and the render returns XGB_QUEUE_OVERFLOW.
 * Either way the film is incomplete, the error bit is in
 * xgb_render_stats.error_flags (4 and 1), the context stays usable and the
 * next call starts with clear bits. 0 restores a default: 2^22 steps, 64
 * entries (the stacks' size; max_stack above 64 is XGB_INVALID_ARG). A
 * well-formed BVH never reaches the defaults; lower values are for testing
 * the error paths. Applies to xgb_render, xgb_render_batch,
 * xgb_render_noalloc and the ray queries on this scene. */
xgb_status xgb_scene_set_traversal_limits(xgb_scene* scene, int max_steps, int max_stack);

/* enable = 1: later xgb_render calls on this scene record CUDA events around
 * every kernel on the render stream and count BVH work (for profiling; adds a
 * few microseconds per wavefront iteration). */
xgb_status xgb_scene_set_profiling(xgb_scene* scene, int enable);

#ifdef __cplusplus
}
#endif
#endif /* XGB_H */
