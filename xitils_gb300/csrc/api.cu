// Host implementation of the C ABI declared in include/xgb.h.
//
// Scene flattening follows the reference's object model: Scene::addObject
// (Scene.h:17-22) appends objects and collects emissive ones as lights in
// insertion order; light-sampling constants are computed here once with the
// reference's float arithmetic (TriangleMesh.h:193-235, Object.h:91-110,
// Scene.h:40-55) instead of per sample. This file is compiled with
// -ffp-contract=off so the host float arithmetic matches the reference's.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/xgb.h"
#include "guide_kernels.h"
#include "xgb_kernels.h"

using namespace xgb;

// ------------------------------------------------------------ host helpers --
namespace {

struct H3 {
    float x = 0, y = 0, z = 0;
};
inline H3 h3(float a, float b, float c) { H3 r; r.x = a; r.y = b; r.z = c; return r; }
inline H3 sub(H3 a, H3 b) { return h3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float dotH(H3 a, H3 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + 0.0f * 0.0f); }
inline H3 scaleH(H3 a, float s) { return h3(a.x * s, a.y * s, a.z * s); }
inline H3 normalizeH(H3 a) { float inv = 1.0f / std::sqrt(dotH(a, a)); return scaleH(a, inv); }
inline H3 crossH(H3 a, H3 b) {  // Vector.h:637-654
    double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return h3((float)(ay * bz - az * by), (float)(az * bx - ax * bz), (float)(ax * by - ay * bx));
}
inline H3 pointH(const float* m, H3 v) {  // Transform.h:61-72
    float xp = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
    float yp = m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7];
    float zp = m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11];
    float wp = m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15];
    if (wp == 1) return h3(xp, yp, zp);
    float inv = 1.0f / wp;
    return h3(xp * inv, yp * inv, zp * inv);
}
inline H3 normalH(const float* m, H3 v) {  // Transform.h:121-127
    return normalizeH(h3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                         m[8] * v.x + m[9] * v.y + m[10] * v.z));
}
inline float lengthH(H3 a) { return std::sqrt(dotH(a, a)); }

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void add(H3 p) {
        lo[0] = std::min(lo[0], p.x); lo[1] = std::min(lo[1], p.y); lo[2] = std::min(lo[2], p.z);
        hi[0] = std::max(hi[0], p.x); hi[1] = std::max(hi[1], p.y); hi[2] = std::max(hi[2], p.z);
    }
    void add(const Box& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
};

bool isIdentity(const float* m) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
            if (m[4 * r + c] != (r == c ? 1.0f : 0.0f)) return false;
    return true;
}

template <class T>
cudaError_t upload(T** dptr, const T* host, size_t count, cudaStream_t s) {
    *dptr = nullptr;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)dptr, sizeof(T) * count);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(*dptr, host, sizeof(T) * count, cudaMemcpyHostToDevice, s);
}

void dfree(const void* p) {
    if (p) cudaFree((void*)p);
}

}  // namespace

// ------------------------------------------------------------------ handles --
struct xgb_ctx {
    int device = 0;
    int numSMs = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    int bvhBuilder = kBuilderPloc;
    int bvhLayout = kLayoutBinary;
    int tileW = 0, tileH = 0;  // camera-path order (xgb_ctx_set_path_order)
    // consecutive samples of a pixel among the camera paths (xgb_ctx_set_sample_grouping);
    // 64 by default: the terrain's 64-spp render took 44.8 ms in sample passes, 38.5 ms
    // in runs of 32 samples, 38.1 ms in runs of 64
    int sampleGroup = 64;
};

struct xgb_texture {
    xgb_ctx* ctx;
    int w = 0, h = 0, clamp = 1, filter = 1;
    float4* d = nullptr;
};

struct xgb_mesh {
    xgb_ctx* ctx;
    int nV = 0, nTris = 0;
    std::vector<H3> pos, nrm;  // host copies for light tables and bounds
    std::vector<int> idx;
    bool hasUV = false, hasN = false, hasT = false;
    float4 *dPos = nullptr, *dNrm = nullptr, *dTan = nullptr, *dBit = nullptr, *dGnrm = nullptr;
    float2* dUV = nullptr;
    int* dIdx = nullptr;
    float* dArea = nullptr;
    WNode* dNodes = nullptr;   // 8-wide BVH (allocated by buildBlas)
    Node2* dNodes2 = nullptr;  // binary BVH (allocated by buildBlas)
    int wide = 0;
    TriV* dTris = nullptr;
    int rootIsLeaf = 1, rootLeaf = 0;
    std::vector<float> triArea;  // TriangleIndexed::surfaceArea
    float area = 0;              // TriangleMesh::calcSurfaceArea
    Box bound;                   // TriangleMesh::bound over all vertices
    // shell mapping (xgb_mesh_create_shell): layers of shellFaces triangles each
    const xgb_texture* shellTex = nullptr;
    float shellScale = 0.0f;
    int shellLayers = 0, shellFaces = 0;
};

struct xgb_svndf {
    xgb_ctx* ctx;
    int resU = 0, resV = 0;
    float4* lobes = nullptr;  // 5 float4 per low texel (SvndfDev)
};

struct xgb_material {
    xgb_ctx* ctx;
    Material m;
    const xgb_texture* tex = nullptr;
    const xgb_texture* normalmap = nullptr;
    const xgb_material* base = nullptr;
    const xgb_svndf* svndf = nullptr;  // MultiLobeSVBRDF
};

struct xgb_film {
    xgb_ctx* ctx;
    int w = 0, h = 0, fp64 = 0;
    void* d = nullptr;
    void* aov = nullptr;  // albedo plane then normal plane, same element type as d
    float* stage = nullptr;  // packed float RGB(A) of one plane for downloads (allocated at the first one)
};

struct xgb_guide {
    xgb_ctx* ctx;
    GuideDevice g;
    GuideBounds bounds;
    bool hasBounds = false;
    std::vector<void*> allocations;
    GuideRecord* arena = nullptr;           // training records of one render call
    int arenaCap = 0;
    unsigned int* recCount = nullptr;       // [0] arena count, [3] pool count
    GuideRecord* batchRec = nullptr;        // device staging for xgb_guide_train_batch
    unsigned int* hostPoolCount = nullptr;  // pinned copy of the pool count
    int maxStepsPerCall = 512;
    int product = 1;                        // target: radiance x bsdfCos (1) or radiance (0)
};

struct SceneObject {
    const xgb_mesh* mesh;
    const xgb_material* material;
    float mat[16], matInv[16];
};

struct RenderBuffers {
    unsigned int capacity = 0;
    PathQueue q[2];
    HitQueue hits;
    ShadowQueue shadow;
    void* block = nullptr;
};

struct xgb_scene {
    xgb_ctx* ctx;
    std::vector<SceneObject> objects;
    bool hasCamera = false;
    float c2w[16], c2wInv[16];
    float fov = 1, aspect = 1;
    int skyKind = SKY_NONE;
    float skyRGB[3] = {0, 0, 0};
    const xgb_texture* skyTex = nullptr;
    bool built = false;
    // device copies
    SceneDev sd;
    std::vector<void*> allocations;
    RenderBuffers rb;
    Ctrl* ctrl = nullptr;
    Ctrl* ctrlHost = nullptr;  // pinned
    xgb_render_stats last{};
    bool profiling = false;
    std::vector<cudaEvent_t> events;  // profiling: 6 per wavefront iteration
    float boundsLo[3] = {0, 0, 0}, boundsHi[3] = {1, 1, 1};  // world bounds of the built scene
    xgb_guide* guide = nullptr;
    float bsdfFrac = 0.5f;
    int guideTrain = 0;
    float guideLr = 1e-3f;
    float4* mix = nullptr;  // per-path mixtures (capacity x 10 float4)
    unsigned int mixCapacity = 0;
    unsigned int fixes = 0;     // opt-in quirk fixes (xgb_scene_set_fixes)
    int maxSteps = kDefaultMaxSteps;   // traversal bounds (xgb_scene_set_traversal_limits)
    int stackLimit = kMaxStackLimit;
    bool guidable = false;      // some object's material takes the learned proposal
    float4* pathAcc = nullptr;  // guide training: per-path contributions of a call
    unsigned long long pathAccCapacity = 0;
    double vertsPerPath = 4.0;  // extension rays per path of the last call (sizes the record rate)
};

static xgb_status fail(xgb_ctx* ctx, xgb_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}
static xgb_status cudaFail(xgb_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, XGB_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
#define XGB_CUDA(ctx, call)                                         \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cudaFail((ctx), e_, #call);   \
    } while (0)

static cudaStream_t pick(xgb_ctx* ctx, void* s) { return s ? (cudaStream_t)s : ctx->stream; }

namespace xgb {
void batchRelease(xgb_ctx* ctx);  // batch.cu: the context's batch queues, arrays and graph
}

extern "C" {

const char* xgb_version(void) { return "xgb 0.1 sm_103a"; }

const char* xgb_get_last_error(const xgb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

xgb_status xgb_ctx_create(int device, xgb_ctx** out) {
    if (!out) return XGB_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) return XGB_CUDA_ERROR;
    if (cudaSetDevice(device) != cudaSuccess) return XGB_CUDA_ERROR;
    auto* c = new xgb_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return XGB_CUDA_ERROR;
    }
    *out = c;
    return XGB_OK;
}

xgb_status xgb_ctx_destroy(xgb_ctx* ctx) {
    if (!ctx) return XGB_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    batchRelease(ctx);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return XGB_OK;
}

xgb_status xgb_ctx_set_bvh_builder(xgb_ctx* ctx, int builder) {
    if (!ctx) return XGB_INVALID_ARG;
    if (builder != XGB_BVH_PLOC && builder != XGB_BVH_LBVH)
        return fail(ctx, XGB_INVALID_ARG, "xgb_ctx_set_bvh_builder: unknown builder");
    ctx->bvhBuilder = builder == XGB_BVH_PLOC ? kBuilderPloc : kBuilderLbvh;
    return XGB_OK;
}

xgb_status xgb_ctx_set_path_order(xgb_ctx* ctx, int tile_w, int tile_h) {
    if (!ctx) return XGB_INVALID_ARG;
    if (tile_w < 0 || tile_h < 0 || tile_w > 256 || tile_h > 256 || (tile_w == 0) != (tile_h == 0))
        return fail(ctx, XGB_INVALID_ARG, "xgb_ctx_set_path_order: tile sides in [1, 256], or both 0");
    ctx->tileW = tile_w;
    ctx->tileH = tile_h;
    return XGB_OK;
}

xgb_status xgb_ctx_set_sample_grouping(xgb_ctx* ctx, int samples) {
    if (!ctx) return XGB_INVALID_ARG;
    if (samples < 0 || samples > 4096)
        return fail(ctx, XGB_INVALID_ARG, "xgb_ctx_set_sample_grouping: samples in [0, 4096]");
    ctx->sampleGroup = samples;
    return XGB_OK;
}

xgb_status xgb_ctx_set_bvh_layout(xgb_ctx* ctx, int layout) {
    if (!ctx) return XGB_INVALID_ARG;
    if (layout != XGB_BVH_BINARY && layout != XGB_BVH_WIDE8)
        return fail(ctx, XGB_INVALID_ARG, "xgb_ctx_set_bvh_layout: unknown layout");
    ctx->bvhLayout = layout == XGB_BVH_WIDE8 ? kLayoutWide : kLayoutBinary;
    return XGB_OK;
}

xgb_status xgb_ctx_synchronize(xgb_ctx* ctx, void* stream) {
    if (!ctx) return XGB_INVALID_ARG;
    XGB_CUDA(ctx, cudaStreamSynchronize(pick(ctx, stream)));
    return XGB_OK;
}

// ---------------------------------------------------------------- textures --
xgb_status xgb_texture_create(xgb_ctx* ctx, int width, int height, int channels, const float* texels, int wrap_clamp,
                              int filter, xgb_texture** out) {
    if (!ctx || !out || !texels || width <= 0 || height <= 0 || (channels != 3 && channels != 4))
        return fail(ctx, XGB_INVALID_ARG, "xgb_texture_create: bad arguments");
    cudaSetDevice(ctx->device);
    size_t n = (size_t)width * height;
    std::vector<float4> t(n);
    for (size_t i = 0; i < n; ++i)
        t[i] = make_float4(texels[channels * i], texels[channels * i + 1], texels[channels * i + 2], 0.0f);
    auto* tex = new xgb_texture();
    tex->ctx = ctx;
    tex->w = width; tex->h = height; tex->clamp = wrap_clamp ? 1 : 0; tex->filter = filter ? 1 : 0;
    cudaError_t e = upload(&tex->d, t.data(), n, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        dfree(tex->d);
        delete tex;
        return cudaFail(ctx, e, "xgb_texture_create");
    }
    *out = tex;
    return XGB_OK;
}

xgb_status xgb_texture_destroy(xgb_texture* tex) {
    if (!tex) return XGB_INVALID_ARG;
    dfree(tex->d);
    delete tex;
    return XGB_OK;
}

// ------------------------------------------------------------------ meshes --
static void freeMesh(xgb_mesh* m) {
    for (const void* p : {(const void*)m->dPos, (const void*)m->dNrm, (const void*)m->dTan, (const void*)m->dBit,
                          (const void*)m->dGnrm, (const void*)m->dUV, (const void*)m->dIdx, (const void*)m->dArea,
                          (const void*)m->dNodes, (const void*)m->dNodes2, (const void*)m->dTris})
        dfree(p);
}

static xgb_status createMesh(xgb_ctx* ctx, int vertex_count, const float* positions, const float* texcoords,
                             const float* normals, const float* tangents, const float* bitangents, int vec3_stride,
                             int uv_stride, int index_count, const int32_t* indices, xgb_mesh** out) {
    if (!ctx || !out) return XGB_INVALID_ARG;
    if (vertex_count <= 0 || !positions || index_count <= 0 || index_count % 3 || !indices)
        return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create: need positions and a multiple of 3 indices");
    if (vec3_stride != 12 && vec3_stride != 16) return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create: vec3_stride must be 12 or 16");
    if (uv_stride != 8 && uv_stride != 16) return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create: uv_stride must be 8 or 16");
    if ((tangents == nullptr) != (bitangents == nullptr))
        return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create: tangents and bitangents go together");
    for (int i = 0; i < index_count; ++i)
        if (indices[i] < 0 || indices[i] >= vertex_count)
            return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create: index out of range");
    cudaSetDevice(ctx->device);
    const int vs = vec3_stride / 4, us = uv_stride / 4;
    auto* m = new xgb_mesh();
    m->ctx = ctx;
    m->nV = vertex_count;
    m->nTris = index_count / 3;
    m->idx.assign(indices, indices + index_count);
    m->pos.resize(vertex_count);
    std::vector<float4> p4(vertex_count), n4, t4, b4;
    std::vector<float2> uv;
    for (int i = 0; i < vertex_count; ++i) {
        const float* p = positions + (size_t)vs * i;
        m->pos[i] = h3(p[0], p[1], p[2]);
        p4[i] = make_float4(p[0], p[1], p[2], 0.0f);
        m->bound.add(m->pos[i]);
    }
    auto fill4 = [&](const float* a, std::vector<float4>& v) {
        v.resize(vertex_count);
        for (int i = 0; i < vertex_count; ++i) {
            const float* q = a + (size_t)vs * i;
            v[i] = make_float4(q[0], q[1], q[2], 0.0f);
        }
    };
    if (normals) {
        fill4(normals, n4);
        m->hasN = true;
        m->nrm.resize(vertex_count);
        for (int i = 0; i < vertex_count; ++i) m->nrm[i] = h3(n4[i].x, n4[i].y, n4[i].z);
    }
    if (tangents) { fill4(tangents, t4); fill4(bitangents, b4); m->hasT = true; }
    if (texcoords) {
        uv.resize(vertex_count);
        for (int i = 0; i < vertex_count; ++i) uv[i] = make_float2(texcoords[(size_t)us * i], texcoords[(size_t)us * i + 1]);
        m->hasUV = true;
    }
    // TriangleIndexed::surfaceArea (TriangleIndexed.h:56-62), TriangleMesh::calcSurfaceArea (:253-258)
    m->triArea.resize(m->nTris);
    m->area = 0.0f;
    for (int t = 0; t < m->nTris; ++t) {
        H3 a = m->pos[m->idx[3 * t]], b = m->pos[m->idx[3 * t + 1]], c = m->pos[m->idx[3 * t + 2]];
        m->triArea[t] = lengthH(crossH(sub(b, a), sub(c, a))) / 2.0f;
        m->area += m->triArea[t];
    }
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = upload(&m->dPos, p4.data(), p4.size(), s);
    if (e == cudaSuccess && m->hasN) e = upload(&m->dNrm, n4.data(), n4.size(), s);
    if (e == cudaSuccess && m->hasT) e = upload(&m->dTan, t4.data(), t4.size(), s);
    if (e == cudaSuccess && m->hasT) e = upload(&m->dBit, b4.data(), b4.size(), s);
    if (e == cudaSuccess && m->hasUV) e = upload(&m->dUV, uv.data(), uv.size(), s);
    if (e == cudaSuccess) e = upload(&m->dIdx, m->idx.data(), m->idx.size(), s);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->dGnrm, sizeof(float4) * m->nTris);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->dArea, sizeof(float) * m->nTris);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->dTris, sizeof(TriV) * m->nTris);
    if (e == cudaSuccess) {
        BlasBuildInput in{m->dPos, m->dIdx, m->nTris, ctx->bvhBuilder, ctx->bvhLayout};
        BlasBuildOutput o{};
        o.tris = m->dTris; o.gnrm = m->dGnrm; o.triArea = m->dArea;
        e = buildBlas(in, &o, s);
        m->dNodes = o.nodes;
        m->dNodes2 = o.nodes2;
        m->wide = o.wide;
        m->rootIsLeaf = o.rootIsLeaf;
        m->rootLeaf = o.rootLeaf;
    }
    if (e != cudaSuccess) {
        freeMesh(m);
        delete m;
        return e == cudaErrorMemoryAllocation ? fail(ctx, XGB_OOM, "xgb_mesh_create: out of device memory")
                                              : cudaFail(ctx, e, "xgb_mesh_create");
    }
    *out = m;
    return XGB_OK;
}

xgb_status xgb_mesh_create(xgb_ctx* ctx, int vertex_count, const float* positions, const float* texcoords,
                           const float* normals, const float* tangents, const float* bitangents, int vec3_stride,
                           int uv_stride, int index_count, const int32_t* indices, xgb_mesh** out) {
    return createMesh(ctx, vertex_count, positions, texcoords, normals, tangents, bitangents, vec3_stride, uv_stride,
                      index_count, indices, out);
}

// TriangleMesh::setGeometryWithShellMapping + buildTrianglesWithShellMapping
// (TriangleMesh.h:163-177, :279-324): the vertex arrays repeated layer_count
// times, layer l's positions moved by d = scale * l / (layer_count - 1) along
// the vertex normals (in float, unfused: this file is compiled without FP
// contraction), layer l's indices shifted by l * vertex_count. Triangle
// l * faces + f of the result is face f on layer l.
xgb_status xgb_mesh_create_shell(xgb_ctx* ctx, int vertex_count, const float* positions, const float* texcoords,
                                 const float* normals, const float* tangents, const float* bitangents,
                                 int vec3_stride, int uv_stride, int index_count, const int32_t* indices,
                                 const xgb_texture* displacement, float displacement_scale, int layer_count,
                                 xgb_mesh** out) {
    if (!ctx || !out) return XGB_INVALID_ARG;
    if (!positions || !texcoords || !normals || !tangents || !bitangents || !indices || !displacement)
        return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: every vertex attribute and the displacement texture are required");
    if (vertex_count <= 0 || index_count <= 0 || index_count % 3 || layer_count < 1 || !std::isfinite(displacement_scale))
        return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: bad sizes, layer count or scale");
    if ((int64_t)vertex_count * layer_count > INT32_MAX / 2 || (int64_t)index_count * layer_count > INT32_MAX / 2)
        return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: too many layers for this mesh");
    if (vec3_stride != 12 && vec3_stride != 16) return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: vec3_stride must be 12 or 16");
    if (uv_stride != 8 && uv_stride != 16) return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: uv_stride must be 8 or 16");
    const int vs = vec3_stride / 4, us = uv_stride / 4;
    const size_t V = (size_t)vertex_count, L = (size_t)layer_count, I = (size_t)index_count;
    std::vector<float> P(3 * V * L), N(3 * V * L), T(3 * V * L), B(3 * V * L), UV(2 * V * L);
    std::vector<int32_t> idx(I * L);
    for (size_t l = 0; l < L; ++l) {
        // layer 0 keeps the input positions; the reference's loop starts at layer 1
        const float d = l == 0 ? 0.0f : displacement_scale * (float)l / (float)(layer_count - 1);
        for (size_t i = 0; i < V; ++i) {
            const size_t o = l * V + i;
            for (int c = 0; c < 3; ++c) {
                const float p = positions[vs * i + c], n = normals[vs * i + c];
                P[3 * o + c] = l == 0 ? p : p + d * n;
                N[3 * o + c] = n;
                T[3 * o + c] = tangents[vs * i + c];
                B[3 * o + c] = bitangents[vs * i + c];
            }
            UV[2 * o] = texcoords[us * i];
            UV[2 * o + 1] = texcoords[us * i + 1];
        }
        for (size_t k = 0; k < I; ++k) idx[l * I + k] = indices[k] + (int32_t)(l * V);
    }
    for (size_t k = 0; k < I; ++k)
        if (indices[k] < 0 || indices[k] >= vertex_count)
            return fail(ctx, XGB_INVALID_ARG, "xgb_mesh_create_shell: index out of range");
    xgb_mesh* m = nullptr;
    xgb_status st = createMesh(ctx, (int)(V * L), P.data(), UV.data(), N.data(), T.data(), B.data(), 12, 8,
                               (int)(I * L), idx.data(), &m);
    if (st != XGB_OK) return st;
    m->shellTex = displacement;
    m->shellScale = displacement_scale;
    m->shellLayers = layer_count;
    m->shellFaces = index_count / 3;
    *out = m;
    return XGB_OK;
}

xgb_status xgb_mesh_destroy(xgb_mesh* mesh) {
    if (!mesh) return XGB_INVALID_ARG;
    freeMesh(mesh);
    delete mesh;
    return XGB_OK;
}

xgb_status xgb_mesh_triangle_count(const xgb_mesh* mesh, int* out) {
    if (!mesh || !out) return XGB_INVALID_ARG;
    *out = mesh->nTris;
    return XGB_OK;
}

// --------------------------------------------------------------- materials --
static xgb_status newMaterial(xgb_ctx* ctx, int kind, xgb_material** out, xgb_material** made) {
    if (!ctx || !out) return fail(ctx, XGB_INVALID_ARG, "material: null argument");
    auto* m = new xgb_material();
    m->ctx = ctx;
    std::memset(&m->m, 0, sizeof(Material));
    m->m.kind = kind;
    m->m.tex = -1; m->m.normalmap = -1; m->m.base = -1;
    m->m.index = 1.0f;
    *made = m;
    *out = m;
    return XGB_OK;
}
static bool finite3(const float* v) { return v && std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

xgb_status xgb_material_diffuse(xgb_ctx* ctx, const float albedo[3], const xgb_texture* albedo_tex, xgb_material** out) {
    if (!finite3(albedo)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_diffuse: bad albedo");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_DIFFUSE, out, &m);
    if (st) return st;
    m->m.albedo = make_float3(albedo[0], albedo[1], albedo[2]);
    m->tex = albedo_tex;
    return XGB_OK;
}
xgb_status xgb_material_metal(xgb_ctx* ctx, float roughness, const float f0[3], const xgb_texture* roughness_tex,
                              xgb_material** out) {
    if (!finite3(f0) || !std::isfinite(roughness)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_metal: bad parameters");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_METAL, out, &m);
    if (st) return st;
    m->m.roughness = roughness;
    m->m.albedo = make_float3(f0[0], f0[1], f0[2]);
    m->tex = roughness_tex;
    return XGB_OK;
}
xgb_status xgb_material_set_fixes(xgb_material* m, uint32_t fixes) {
    if (!m) return XGB_INVALID_ARG;
    if (fixes & ~(uint32_t)XGB_FIX_METAL_HORIZON) return fail(m->ctx, XGB_INVALID_ARG, "xgb_material_set_fixes: unknown fix");
    if ((fixes & XGB_FIX_METAL_HORIZON) && m->m.kind != MAT_METAL)
        return fail(m->ctx, XGB_INVALID_ARG, "xgb_material_set_fixes: the horizon fix applies to Metal");
    m->m.flags = (int)fixes;
    return XGB_OK;
}
xgb_status xgb_material_glossy(xgb_ctx* ctx, const float albedo[3], float sharpness, xgb_material** out) {
    if (!finite3(albedo)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_glossy: bad albedo");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_GLOSSY, out, &m);
    if (st) return st;
    m->m.albedo = make_float3(albedo[0], albedo[1], albedo[2]);
    m->m.sharpness = sharpness;
    return XGB_OK;
}
xgb_status xgb_material_glossy_highlight(xgb_ctx* ctx, const float albedo[3], const float highlight[3], float sharpness,
                                         float sharpness_highlight, float rate, xgb_material** out) {
    if (!finite3(albedo) || !finite3(highlight)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_glossy_highlight: bad colour");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_GLOSSY_HIGHLIGHT, out, &m);
    if (st) return st;
    m->m.albedo = make_float3(albedo[0], albedo[1], albedo[2]);
    m->m.highlight = make_float3(highlight[0], highlight[1], highlight[2]);
    m->m.sharpness = sharpness;
    m->m.sharpnessHL = sharpness_highlight;
    m->m.rate = rate;
    return XGB_OK;
}
xgb_status xgb_material_glossy_clamped(xgb_ctx* ctx, const float albedo[3], float sharpness, xgb_material** out) {
    if (!finite3(albedo)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_glossy_clamped: bad albedo");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_GLOSSY_CLAMPED, out, &m);
    if (st) return st;
    m->m.albedo = make_float3(albedo[0], albedo[1], albedo[2]);
    m->m.sharpness = sharpness;
    return XGB_OK;
}
xgb_status xgb_material_emission(xgb_ctx* ctx, const float power[3], xgb_material** out) {
    if (!finite3(power)) return fail(ctx, XGB_INVALID_ARG, "xgb_material_emission: bad power");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_EMISSION, out, &m);
    if (st) return st;
    m->m.albedo = make_float3(power[0], power[1], power[2]);
    return XGB_OK;
}
xgb_status xgb_material_specular_reflection(xgb_ctx* ctx, xgb_material** out) {
    xgb_material* m;
    return newMaterial(ctx, MAT_SPECULAR_REFLECTION, out, &m);
}
xgb_status xgb_material_specular_refraction(xgb_ctx* ctx, float index, xgb_material** out) {
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_SPECULAR_REFRACTION, out, &m);
    if (st) return st;
    m->m.index = index;
    return XGB_OK;
}
xgb_status xgb_material_specular_fresnel(xgb_ctx* ctx, float index, xgb_material** out) {
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_SPECULAR_FRESNEL, out, &m);
    if (st) return st;
    m->m.index = index;
    return XGB_OK;
}
xgb_status xgb_material_mf_normalmap(xgb_ctx* ctx, const xgb_material* base, xgb_material** out) {
    if (!base || base->m.kind == MAT_MF_NORMALMAP || base->m.kind == MAT_EMISSION)
        return fail(ctx, XGB_INVALID_ARG, "xgb_material_mf_normalmap: base must be a non-emissive, non-MFNM material");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_MF_NORMALMAP, out, &m);
    if (st) return st;
    m->base = base;
    return XGB_OK;
}
xgb_status xgb_material_multilobe_svbrdf(xgb_ctx* ctx, const xgb_material* base, const xgb_svndf* svndf,
                                         xgb_material** out) {
    if (!base || !svndf || base->m.kind == MAT_MF_NORMALMAP || base->m.kind == MAT_EMISSION ||
        base->m.kind == MAT_MULTILOBE_SVBRDF)
        return fail(ctx, XGB_INVALID_ARG,
                    "xgb_material_multilobe_svbrdf: needs an SVNDF and a non-emissive base other than MFNM / SVBRDF");
    xgb_material* m;
    xgb_status st = newMaterial(ctx, MAT_MULTILOBE_SVBRDF, out, &m);
    if (st) return st;
    m->base = base;
    m->svndf = svndf;
    return XGB_OK;
}

xgb_status xgb_svndf_create(xgb_ctx* ctx, const xgb_texture* displacement, float displacement_scale, int rate,
                            uint32_t seed, xgb_svndf** out, xgb_texture** low) {
    if (!ctx || !out || !low) return XGB_INVALID_ARG;
    if (!displacement || rate < 1 || rate > 16 || !std::isfinite(displacement_scale))
        return fail(ctx, XGB_INVALID_ARG, "xgb_svndf_create: needs a displacement texture and rate in [1, 16]");
    cudaSetDevice(ctx->device);
    const int W = (displacement->w + rate - 1) / rate, H = (displacement->h + rate - 1) / rate;
    auto* sv = new xgb_svndf();
    sv->ctx = ctx;
    sv->resU = W;
    sv->resV = H;
    auto* tex = new xgb_texture();
    tex->ctx = ctx;
    tex->w = W; tex->h = H; tex->clamp = displacement->clamp; tex->filter = 1;  // Texture(w, h): bilinear
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMalloc((void**)&sv->lobes, sizeof(float4) * 5 * (size_t)W * H);
    if (e == cudaSuccess) e = cudaMalloc((void**)&tex->d, sizeof(float4) * (size_t)W * H);
    if (e == cudaSuccess) {
        const TextureDev src{displacement->d, displacement->w, displacement->h, displacement->clamp, displacement->filter};
        e = svndfFit(src, displacement_scale, rate, seed, W, H, sv->lobes, tex->d, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        dfree(sv->lobes);
        dfree(tex->d);
        delete sv;
        delete tex;
        return e == cudaErrorMemoryAllocation ? fail(ctx, XGB_OOM, "xgb_svndf_create: out of device memory")
                                              : cudaFail(ctx, e, "xgb_svndf_create");
    }
    *out = sv;
    *low = tex;
    return XGB_OK;
}

xgb_status xgb_svndf_destroy(xgb_svndf* svndf) {
    if (!svndf) return XGB_INVALID_ARG;
    dfree(svndf->lobes);
    delete svndf;
    return XGB_OK;
}

xgb_status xgb_svndf_size(const xgb_svndf* svndf, int* width, int* height) {
    if (!svndf || !width || !height) return XGB_INVALID_ARG;
    *width = svndf->resU;
    *height = svndf->resV;
    return XGB_OK;
}

xgb_status xgb_svndf_get_lobes(const xgb_svndf* svndf, float* host) {
    if (!svndf || !host) return XGB_INVALID_ARG;
    xgb_ctx* ctx = svndf->ctx;
    cudaSetDevice(ctx->device);
    const size_t T = (size_t)svndf->resU * svndf->resV;
    std::vector<float4> raw(5 * T);
    XGB_CUDA(ctx, cudaMemcpyAsync(raw.data(), svndf->lobes, sizeof(float4) * raw.size(), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    XGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t t = 0; t < T; ++t) {
        const float4 al = raw[5 * t + 4];
        const float alpha[4] = {al.x, al.y, al.z, al.w};
        for (int j = 0; j < 4; ++j) {
            float* o = host + (t * 4 + j) * 5;
            const float4 l = raw[5 * t + j];
            o[0] = l.x; o[1] = l.y; o[2] = l.z; o[3] = l.w; o[4] = alpha[j];
        }
    }
    return XGB_OK;
}

xgb_status xgb_svndf_set_lobes(xgb_svndf* svndf, const float* host) {
    if (!svndf || !host) return XGB_INVALID_ARG;
    xgb_ctx* ctx = svndf->ctx;
    cudaSetDevice(ctx->device);
    const size_t T = (size_t)svndf->resU * svndf->resV;
    std::vector<float4> raw(5 * T);
    for (size_t t = 0; t < T; ++t) {
        float alpha[4];
        for (int j = 0; j < 4; ++j) {
            const float* l = host + (t * 4 + j) * 5;
            raw[5 * t + j] = make_float4(l[0], l[1], l[2], l[3]);
            alpha[j] = l[4];
        }
        raw[5 * t + 4] = make_float4(alpha[0], alpha[1], alpha[2], alpha[3]);
    }
    XGB_CUDA(ctx, cudaMemcpyAsync(svndf->lobes, raw.data(), sizeof(float4) * raw.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
    XGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return XGB_OK;
}

xgb_status xgb_material_set_normalmap(xgb_material* mat, const xgb_texture* normalmap) {
    if (!mat) return XGB_INVALID_ARG;
    mat->normalmap = normalmap;
    return XGB_OK;
}
xgb_status xgb_material_destroy(xgb_material* mat) {
    if (!mat) return XGB_INVALID_ARG;
    delete mat;
    return XGB_OK;
}

// ------------------------------------------------------------------- scene --
static void freeSceneDevice(xgb_scene* s) {
    for (void* p : s->allocations) dfree(p);
    s->allocations.clear();
    s->built = false;
}
static void freeBuffers(xgb_scene* s) {
    dfree(s->rb.block);
    s->rb = RenderBuffers();
}

xgb_status xgb_scene_create(xgb_ctx* ctx, xgb_scene** out) {
    if (!ctx || !out) return XGB_INVALID_ARG;
    cudaSetDevice(ctx->device);
    auto* s = new xgb_scene();
    s->ctx = ctx;
    std::memset(&s->sd, 0, sizeof(SceneDev));
    if (cudaMalloc((void**)&s->ctrl, sizeof(Ctrl)) != cudaSuccess ||
        cudaMallocHost((void**)&s->ctrlHost, sizeof(Ctrl)) != cudaSuccess) {
        dfree(s->ctrl);
        delete s;
        return fail(ctx, XGB_OOM, "xgb_scene_create: allocation failed");
    }
    *out = s;
    return XGB_OK;
}

xgb_status xgb_scene_destroy(xgb_scene* s) {
    if (!s) return XGB_INVALID_ARG;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    freeSceneDevice(s);
    freeBuffers(s);
    dfree(s->mix);
    dfree(s->pathAcc);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    dfree(s->ctrl);
    if (s->ctrlHost) cudaFreeHost(s->ctrlHost);
    delete s;
    return XGB_OK;
}

xgb_status xgb_scene_add_object(xgb_scene* s, const xgb_mesh* mesh, const xgb_material* material, const float mat[16],
                                const float mat_inv[16]) {
    if (!s || !mesh || !material || !mat || !mat_inv) return fail(s ? s->ctx : nullptr, XGB_INVALID_ARG, "xgb_scene_add_object: null argument");
    SceneObject o;
    o.mesh = mesh;
    o.material = material;
    std::memcpy(o.mat, mat, 64);
    std::memcpy(o.matInv, mat_inv, 64);
    s->objects.push_back(o);
    s->built = false;
    return XGB_OK;
}

xgb_status xgb_scene_set_camera_pinhole(xgb_scene* s, const float c2w[16], const float c2w_inv[16], float fov,
                                        float aspect) {
    if (!s || !c2w || !c2w_inv || !(fov > 0.0f) || !std::isfinite(aspect))
        return fail(s ? s->ctx : nullptr, XGB_INVALID_ARG, "xgb_scene_set_camera_pinhole: bad arguments");
    std::memcpy(s->c2w, c2w, 64);
    std::memcpy(s->c2wInv, c2w_inv, 64);
    s->fov = fov;
    s->aspect = aspect;
    s->hasCamera = true;
    // Camera.h:50-51, evaluated once on the host with the reference's float expressions.
    std::memcpy(s->sd.c2w, c2w, 64);
    s->sd.tanHalfX = tanf(fov / 2);
    s->sd.tanHalfY = tanf(fov / 2 * aspect);
    return XGB_OK;
}

xgb_status xgb_scene_set_sky_none(xgb_scene* s) {
    if (!s) return XGB_INVALID_ARG;
    s->skyKind = SKY_NONE;
    s->skyTex = nullptr;
    s->built = false;
    return XGB_OK;
}
xgb_status xgb_scene_set_sky_uniform(xgb_scene* s, const float rgb[3]) {
    if (!s || !finite3(rgb)) return XGB_INVALID_ARG;
    s->skyKind = SKY_UNIFORM;
    std::memcpy(s->skyRGB, rgb, 12);
    s->skyTex = nullptr;
    s->built = false;
    return XGB_OK;
}
xgb_status xgb_scene_set_sky_probe(xgb_scene* s, const xgb_texture* probe) {
    if (!s || !probe) return XGB_INVALID_ARG;
    s->skyKind = SKY_PROBE;
    s->skyTex = probe;
    s->built = false;
    return XGB_OK;
}
xgb_status xgb_scene_set_sky_latlong(xgb_scene* s, const xgb_texture* latlong) {
    if (!s || !latlong) return XGB_INVALID_ARG;
    s->skyKind = SKY_LATLONG;
    s->skyTex = latlong;
    s->built = false;
    return XGB_OK;
}

// Transform::operator()(Bounds3f) (Transform.h:155-178), padded by a relative
// 1e-6 so that rounding never makes an instance box cull its own triangles.
static Box transformBox(const float* m, const Box& b) {
    H3 lo = h3(b.lo[0], b.lo[1], b.lo[2]);
    H3 size = h3(b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]);
    H3 tmin = pointH(m, lo);
    H3 bx = h3(m[0], m[4], m[8]), by = h3(m[1], m[5], m[9]), bz = h3(m[2], m[6], m[10]);
    H3 vx = scaleH(bx, size.x), vy = scaleH(by, size.y), vz = scaleH(bz, size.z);
    auto add = [](H3 a, H3 c) { return h3(a.x + c.x, a.y + c.y, a.z + c.z); };
    Box r;
    r.add(tmin);
    r.add(add(tmin, vx));
    r.add(add(tmin, vy));
    r.add(add(add(tmin, vy), vx));
    r.add(add(tmin, vz));
    r.add(add(add(tmin, vz), vx));
    r.add(add(add(tmin, vz), vy));
    r.add(add(add(add(tmin, vz), vy), vx));
    for (int k = 0; k < 3; ++k) {
        float pad = 1e-6f * (std::fabs(r.lo[k]) + std::fabs(r.hi[k]) + (r.hi[k] - r.lo[k])) + 1e-30f;
        r.lo[k] -= pad;
        r.hi[k] += pad;
    }
    return r;
}

// Top-level BVH over instance boxes: median split on the longest centroid axis.
static int buildTlas(std::vector<Node2>& nodes, std::vector<int>& items, const std::vector<Box>& boxes, int begin,
                     int end, Box* outBox) {
    Box bb;
    for (int i = begin; i < end; ++i) bb.add(boxes[items[i]]);
    *outBox = bb;
    if (end - begin == 1) return leafEncode(items[begin], 1);
    Box cb;
    for (int i = begin; i < end; ++i) {
        const Box& b = boxes[items[i]];
        cb.add(h3(0.5f * (b.lo[0] + b.hi[0]), 0.5f * (b.lo[1] + b.hi[1]), 0.5f * (b.lo[2] + b.hi[2])));
    }
    int axis = 0;
    float ext = -1;
    for (int k = 0; k < 3; ++k)
        if (cb.hi[k] - cb.lo[k] > ext) { ext = cb.hi[k] - cb.lo[k]; axis = k; }
    int mid = (begin + end) / 2;
    std::nth_element(items.begin() + begin, items.begin() + mid, items.begin() + end, [&](int a, int b) {
        return boxes[a].lo[axis] + boxes[a].hi[axis] < boxes[b].lo[axis] + boxes[b].hi[axis];
    });
    int me = (int)nodes.size();
    nodes.push_back(Node2());
    Box l, r;
    int cl = buildTlas(nodes, items, boxes, begin, mid, &l);
    int cr = buildTlas(nodes, items, boxes, mid, end, &r);
    Node2& nd = nodes[me];
    nd.a = make_float4(l.lo[0], l.lo[1], l.lo[2], l.hi[0]);
    nd.b = make_float4(l.hi[1], l.hi[2], r.lo[0], r.lo[1]);
    nd.c = make_float4(r.lo[2], r.hi[0], r.hi[1], r.hi[2]);
    nd.d = make_int4(cl, cr, 0, 0);
    return me;
}

xgb_status xgb_scene_build(xgb_scene* s, void* stream) {
    if (!s) return XGB_INVALID_ARG;
    xgb_ctx* ctx = s->ctx;
    if (s->objects.empty()) return fail(ctx, XGB_INVALID_ARG, "xgb_scene_build: scene has no objects");
    if (!s->hasCamera) return fail(ctx, XGB_INVALID_ARG, "xgb_scene_build: no camera");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    XGB_CUDA(ctx, cudaStreamSynchronize(st));
    freeSceneDevice(s);

    // tables of meshes, materials and textures referenced by the objects
    std::map<const xgb_mesh*, int> meshIds;
    std::vector<const xgb_mesh*> meshes;
    std::map<const xgb_material*, int> matIds;
    std::vector<const xgb_material*> mats;
    std::map<const xgb_texture*, int> texIds;
    std::vector<const xgb_texture*> texs;
    auto texId = [&](const xgb_texture* t) -> int {
        if (!t) return -1;
        auto it = texIds.find(t);
        if (it != texIds.end()) return it->second;
        texIds[t] = (int)texs.size();
        texs.push_back(t);
        return (int)texs.size() - 1;
    };
    std::function<int(const xgb_material*)> matId = [&](const xgb_material* m) -> int {
        auto it = matIds.find(m);
        if (it != matIds.end()) return it->second;
        int base = m->base ? matId(m->base) : -1;
        matIds[m] = (int)mats.size();
        mats.push_back(m);
        (void)base;
        return (int)mats.size() - 1;
    };
    std::vector<Instance> inst(s->objects.size());
    std::vector<Box> boxes(s->objects.size());
    for (size_t i = 0; i < s->objects.size(); ++i) {
        const SceneObject& o = s->objects[i];
        if (!meshIds.count(o.mesh)) { meshIds[o.mesh] = (int)meshes.size(); meshes.push_back(o.mesh); }
        std::memcpy(inst[i].mat, o.mat, 64);
        std::memcpy(inst[i].matInv, o.matInv, 64);
        inst[i].mesh = meshIds[o.mesh];
        inst[i].material = matId(o.material);
        inst[i].lightIndex = -1;
        inst[i].identity = isIdentity(o.mat) && isIdentity(o.matInv) ? 1 : 0;
        boxes[i] = transformBox(o.mat, o.mesh->bound);
    }
    std::map<const xgb_svndf*, int> svIds;
    std::vector<SvndfDev> sv;
    std::vector<Material> dm(mats.size());
    for (size_t i = 0; i < mats.size(); ++i) {
        dm[i] = mats[i]->m;
        dm[i].tex = texId(mats[i]->tex);
        dm[i].normalmap = texId(mats[i]->normalmap);
        dm[i].base = mats[i]->base ? matIds[mats[i]->base] : -1;
        if (const xgb_svndf* d = mats[i]->svndf) {  // MultiLobeSVBRDF: tex = index in the SVNDF table
            if (!svIds.count(d)) { svIds[d] = (int)sv.size(); sv.push_back(SvndfDev{d->lobes, d->resU, d->resV}); }
            dm[i].tex = svIds[d];
        }
    }
    // whether any object's material takes the learned proposal (integrator.cu::guidableBasic)
    s->guidable = false;
    for (const Instance& in : inst) {
        const int k = dm[in.material].kind;
        if (k == MAT_DIFFUSE || k == MAT_METAL || k == MAT_GLOSSY || k == MAT_GLOSSY_CLAMPED || k == MAT_GLOSSY_HIGHLIGHT)
            s->guidable = true;
    }
    int skyTex = texId(s->skyTex);
    std::vector<TextureDev> td(texs.size());
    for (size_t i = 0; i < texs.size(); ++i) td[i] = TextureDev{texs[i]->d, texs[i]->w, texs[i]->h, texs[i]->clamp, texs[i]->filter};
    std::vector<MeshDev> md(meshes.size());
    int nWideMeshes = 0, anyShell = 0;
    for (size_t i = 0; i < meshes.size(); ++i) {
        const xgb_mesh* m = meshes[i];
        md[i] = MeshDev{m->dNodes2, m->dNodes, m->wide, m->dTris, m->dPos, m->dUV, m->dNrm, m->dTan, m->dBit, m->dIdx,
                        m->dGnrm, m->dArea, m->nTris, m->nV, m->rootIsLeaf, m->rootLeaf};
        if (m->shellTex) {
            md[i].shellLayers = m->shellLayers;
            md[i].shellFaces = m->shellFaces;
            md[i].shellScale = m->shellScale;
            md[i].shellTexels = m->shellTex->d;
            md[i].shellW = m->shellTex->w;
            md[i].shellH = m->shellTex->h;
            md[i].shellClamp = m->shellTex->clamp;
            md[i].shellFilter = m->shellTex->filter;
            anyShell = 1;
        }
        nWideMeshes += m->wide;
    }
    const int blasLayout = nWideMeshes == 0 ? 0 : (nWideMeshes == (int)meshes.size() ? 1 : 2);

    // lights (Scene.h:17-22) and their sampling constants
    std::vector<LightDev> lights;
    std::vector<float4> lightNormal;
    std::vector<float> lightPdf;
    for (size_t i = 0; i < s->objects.size(); ++i)
        if (s->objects[i].material->m.kind == MAT_EMISSION) {
            inst[i].lightIndex = (int)lights.size();
            lights.push_back(LightDev{(int)i, inst[i].mesh, s->objects[i].mesh->nTris, 0});
        }
    for (auto& L : lights) {
        const SceneObject& o = s->objects[L.instance];
        const xgb_mesh* m = o.mesh;
        L.triOffset = (int)lightPdf.size();
        // TriangleMesh::surfaceAreaScaling (TriangleMesh.h:193-200, TriangleIndexed.h:64-72)
        float scaled = 0.0f;
        for (int t = 0; t < m->nTris; ++t) {
            H3 a = pointH(o.mat, m->pos[m->idx[3 * t]]), b = pointH(o.mat, m->pos[m->idx[3 * t + 1]]),
               c = pointH(o.mat, m->pos[m->idx[3 * t + 2]]);
            float sc = lengthH(crossH(sub(b, a), sub(c, a))) / 2.0f / m->triArea[t];
            scaled += m->triArea[t] * sc;
        }
        float scaling = scaled / m->area;
        for (int t = 0; t < m->nTris; ++t) {
            // pdf: TriangleIndexed.h:189 / TriangleMesh.h:221 / Object.h:96 / Scene.h:45
            float pdf = 1.0f / m->triArea[t];
            pdf /= m->nTris;
            pdf /= scaling;
            pdf /= lights.size();
            lightPdf.push_back(pdf);
            H3 a = m->pos[m->idx[3 * t]], b = m->pos[m->idx[3 * t + 1]], c = m->pos[m->idx[3 * t + 2]];
            H3 n = normalH(o.mat, normalizeH(crossH(sub(b, a), sub(c, a))));
            lightNormal.push_back(make_float4(n.x, n.y, n.z, 0.0f));
        }
    }

    Box sceneBox;
    for (const Box& b : boxes) sceneBox.add(b);
    for (int k = 0; k < 3; ++k) { s->boundsLo[k] = sceneBox.lo[k]; s->boundsHi[k] = sceneBox.hi[k]; }

    // top-level hierarchy
    std::vector<Node2> tlas;
    int tlasRootIsLeaf = 0;
    if (inst.size() == 1) {
        tlasRootIsLeaf = 1;
        tlas.push_back(Node2());
    } else {
        std::vector<int> items(inst.size());
        for (size_t i = 0; i < items.size(); ++i) items[i] = (int)i;
        Box root;
        buildTlas(tlas, items, boxes, 0, (int)items.size(), &root);
    }

    auto up = [&](auto** dptr, const auto& vec) -> cudaError_t {
        cudaError_t e = upload(dptr, vec.data(), vec.size(), st);
        if (*dptr) s->allocations.push_back((void*)*dptr);
        return e;
    };
    SceneDev& sd = s->sd;
    MeshDev* dMeshes; Instance* dInst; Node2* dTlas; Material* dMat; TextureDev* dTex = nullptr; LightDev* dLights = nullptr;
    SvndfDev* dSv = nullptr;
    float4* dLN = nullptr; float* dLP = nullptr; float4* dBox = nullptr;
    std::vector<float4> instBox(2 * inst.size());
    for (size_t i = 0; i < inst.size(); ++i) {
        instBox[2 * i] = make_float4(boxes[i].lo[0], boxes[i].lo[1], boxes[i].lo[2], 0.0f);
        instBox[2 * i + 1] = make_float4(boxes[i].hi[0], boxes[i].hi[1], boxes[i].hi[2], 0.0f);
    }
    XGB_CUDA(ctx, up(&dMeshes, md));
    XGB_CUDA(ctx, up(&dInst, inst));
    XGB_CUDA(ctx, up(&dTlas, tlas));
    XGB_CUDA(ctx, up(&dMat, dm));
    XGB_CUDA(ctx, up(&dTex, td));
    XGB_CUDA(ctx, up(&dSv, sv));
    XGB_CUDA(ctx, up(&dLights, lights));
    XGB_CUDA(ctx, up(&dLN, lightNormal));
    XGB_CUDA(ctx, up(&dLP, lightPdf));
    XGB_CUDA(ctx, up(&dBox, instBox));
    sd.meshes = dMeshes;
    sd.instances = dInst;
    sd.tlas = dTlas;
    sd.nInstances = (int)inst.size();
    sd.tlasRootIsLeaf = tlasRootIsLeaf;
    sd.blasLayout = blasLayout;
    sd.fixes = (int)s->fixes;
    sd.maxSteps = s->maxSteps;
    sd.stackLimit = s->stackLimit;
    sd.shell = anyShell;
    sd.nested = 0;
    sd.kinds = 0;
    for (const Material& m : dm) {
        sd.nested |= (m.kind == MAT_MF_NORMALMAP ? 1 : 0) | (m.kind == MAT_MULTILOBE_SVBRDF ? 2 : 0);
        sd.kinds |= 1 << m.kind;
    }
    sd.instBox = dBox;
    sd.materials = dMat;
    sd.textures = dTex;
    sd.svndfs = dSv;
    sd.lights = dLights;
    sd.nLights = (int)lights.size();
    sd.lightNormal = dLN;
    sd.lightPdf = dLP;
    sd.skyKind = s->skyKind;
    sd.skyTex = skyTex;
    sd.skyColor = make_float3(s->skyRGB[0], s->skyRGB[1], s->skyRGB[2]);
    XGB_CUDA(ctx, cudaStreamSynchronize(st));
    s->built = true;
    return XGB_OK;
}

// -------------------------------------------------------------------- film --
xgb_status xgb_film_create(xgb_ctx* ctx, int width, int height, int fp64, xgb_film** out) {
    if (!ctx || !out || width <= 0 || height <= 0) return fail(ctx, XGB_INVALID_ARG, "xgb_film_create: bad size");
    cudaSetDevice(ctx->device);
    auto* f = new xgb_film();
    f->ctx = ctx;
    f->w = width; f->h = height; f->fp64 = fp64 ? 1 : 0;
    size_t bytes = (size_t)width * height * (f->fp64 ? 32 : 16);
    cudaError_t e = cudaMalloc(&f->d, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->d, 0, bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        dfree(f->d);
        delete f;
        return e == cudaErrorMemoryAllocation ? fail(ctx, XGB_OOM, "xgb_film_create: out of memory") : cudaFail(ctx, e, "xgb_film_create");
    }
    *out = f;
    return XGB_OK;
}
xgb_status xgb_film_destroy(xgb_film* f) {
    if (!f) return XGB_INVALID_ARG;
    dfree(f->d);
    dfree(f->aov);
    dfree(f->stage);
    delete f;
    return XGB_OK;
}
static size_t filmPlaneBytes(const xgb_film* f) { return (size_t)f->w * f->h * (f->fp64 ? 32 : 16); }
xgb_status xgb_film_clear(xgb_film* f, void* stream) {
    if (!f) return XGB_INVALID_ARG;
    XGB_CUDA(f->ctx, cudaMemsetAsync(f->d, 0, filmPlaneBytes(f), pick(f->ctx, stream)));
    if (f->aov) XGB_CUDA(f->ctx, cudaMemsetAsync(f->aov, 0, 2 * filmPlaneBytes(f), pick(f->ctx, stream)));
    return XGB_OK;
}
// A plane to host floats: a kernel packs it (FP64 rounded to float, the
// caller's 12- or 16-byte pixel stride) into the film's staging buffer, and one
// linear copy moves it to the host pointer (pinned or pageable).
static xgb_status downloadPlane(xgb_film* f, const void* src, float* host, int stride, cudaStream_t st) {
    const size_t n = (size_t)f->w * f->h;
    cudaSetDevice(f->ctx->device);
    if (!f->stage) {
        cudaError_t e = cudaMalloc((void**)&f->stage, 16 * n);
        if (e != cudaSuccess) {
            f->stage = nullptr;
            return e == cudaErrorMemoryAllocation ? fail(f->ctx, XGB_OOM, "xgb_film_download: out of memory")
                                                  : cudaFail(f->ctx, e, "xgb_film_download");
        }
    }
    const int grid = f->ctx->numSMs * 8;
    launchPackFilm(src, f->fp64, n, stride / 4, f->stage, grid, st);
    XGB_CUDA(f->ctx, cudaGetLastError());
    XGB_CUDA(f->ctx, cudaMemcpyAsync(host, f->stage, (size_t)stride * n, cudaMemcpyDeviceToHost, st));
    XGB_CUDA(f->ctx, cudaStreamSynchronize(st));
    return XGB_OK;
}
xgb_status xgb_film_download(xgb_film* f, float* host, int stride, void* stream) {
    if (!f || !host || (stride != 12 && stride != 16)) return fail(f ? f->ctx : nullptr, XGB_INVALID_ARG, "xgb_film_download: bad arguments");
    return downloadPlane(f, f->d, host, stride, pick(f->ctx, stream));
}
xgb_status xgb_film_enable_aovs(xgb_film* f) {
    if (!f) return XGB_INVALID_ARG;
    if (f->aov) return XGB_OK;
    cudaSetDevice(f->ctx->device);
    cudaError_t e = cudaMalloc(&f->aov, 2 * filmPlaneBytes(f));
    if (e == cudaSuccess) e = cudaMemsetAsync(f->aov, 0, 2 * filmPlaneBytes(f), f->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->ctx->stream);
    if (e != cudaSuccess) {
        dfree(f->aov);
        f->aov = nullptr;
        return e == cudaErrorMemoryAllocation ? fail(f->ctx, XGB_OOM, "xgb_film_enable_aovs: out of memory")
                                              : cudaFail(f->ctx, e, "xgb_film_enable_aovs");
    }
    return XGB_OK;
}
xgb_status xgb_film_download_aov(xgb_film* f, int which, float* host, int stride, void* stream) {
    if (!f || !host || (stride != 12 && stride != 16) || (which != XGB_AOV_ALBEDO && which != XGB_AOV_NORMAL))
        return fail(f ? f->ctx : nullptr, XGB_INVALID_ARG, "xgb_film_download_aov: bad arguments");
    if (!f->aov) return fail(f->ctx, XGB_INVALID_ARG, "xgb_film_download_aov: call xgb_film_enable_aovs first");
    const char* base = (const char*)f->aov + (which == XGB_AOV_NORMAL ? filmPlaneBytes(f) : 0);
    return downloadPlane(f, base, host, stride, pick(f->ctx, stream));
}
xgb_status xgb_film_device_pointer(xgb_film* f, void** out, int* is_fp64) {
    if (!f || !out) return XGB_INVALID_ARG;
    *out = f->d;
    if (is_fp64) *is_fp64 = f->fp64;
    return XGB_OK;
}

// --------------------------------------------------------------- rendering --
void xgb_integrator_params_default(xgb_integrator_params* p) {
    if (!p) return;
    p->integrator = XGB_INTEGRATOR_STANDARD;
    p->max_depth = 0;
    p->rr_start = 5;
    p->rr_prob = 0.9f;
    p->seed = 0;
    p->queue_capacity = 0;
}

static xgb_status ensureBuffers(xgb_scene* s, unsigned int cap) {
    if (s->rb.capacity >= cap && s->rb.block) return XGB_OK;
    freeBuffers(s);
    size_t pathBytes = (size_t)cap * (16 * 3 + 8 + 4 + 4);
    size_t hitBytes = (size_t)cap * (16 + 4);
    size_t shadowBytes = (size_t)cap * (16 * 3 + 8 + 4);
    size_t total = 2 * pathBytes + hitBytes + shadowBytes + 64 * 256;
    void* block = nullptr;
    cudaError_t e = cudaMalloc(&block, total);
    if (e != cudaSuccess) return fail(s->ctx, XGB_OOM, "render: cannot allocate path queues");
    char* p = (char*)block;
    auto take = [&](size_t bytes) { char* r = p; p += (bytes + 255) & ~(size_t)255; return r; };
    for (int k = 0; k < 2; ++k) {
        s->rb.q[k].o = (float4*)take(16 * (size_t)cap);
        s->rb.q[k].d = (float4*)take(16 * (size_t)cap);
        s->rb.q[k].thr = (float4*)take(16 * (size_t)cap);
        s->rb.q[k].rng = (uint2*)take(8 * (size_t)cap);
        s->rb.q[k].grec = (int*)take(4 * (size_t)cap);
        s->rb.q[k].pid = (unsigned int*)take(4 * (size_t)cap);
    }
    s->rb.hits.h = (float4*)take(16 * (size_t)cap);
    s->rb.hits.inst = (int*)take(4 * (size_t)cap);
    s->rb.shadow.o = (float4*)take(16 * (size_t)cap);
    s->rb.shadow.d = (float4*)take(16 * (size_t)cap);
    s->rb.shadow.c = (float4*)take(16 * (size_t)cap);
    s->rb.shadow.rng = (uint2*)take(8 * (size_t)cap);
    s->rb.shadow.pid = (unsigned int*)take(4 * (size_t)cap);
    s->rb.block = block;
    s->rb.capacity = cap;
    return XGB_OK;
}

xgb_status xgb_render(xgb_scene* s, const xgb_integrator_params* params, xgb_film* film, uint32_t spp_begin,
                      uint32_t spp_count, void* stream) {
    if (!s || !film) return XGB_INVALID_ARG;
    xgb_ctx* ctx = s->ctx;
    if (!s->built) return fail(ctx, XGB_NOT_BUILT, "xgb_render: call xgb_scene_build first");
    if (film->ctx != ctx) return fail(ctx, XGB_INVALID_ARG, "xgb_render: film belongs to another context");
    xgb_integrator_params P;
    if (params) P = *params;
    else xgb_integrator_params_default(&P);
    if (P.integrator != XGB_INTEGRATOR_STANDARD && P.integrator != XGB_INTEGRATOR_NAIVE)
        return fail(ctx, XGB_INVALID_ARG, "xgb_render: unknown integrator");
    if (P.rr_start < 1 || !(P.rr_prob > 0.0f && P.rr_prob <= 1.0f) || P.max_depth < 0 || P.queue_capacity < 0)
        return fail(ctx, XGB_INVALID_ARG, "xgb_render: need rr_start >= 1, 0 < rr_prob <= 1, max_depth >= 0");
    if (P.max_depth == 0 && P.rr_prob >= 1.0f)
        return fail(ctx, XGB_INVALID_ARG, "xgb_render: rr_prob = 1 needs a max_depth (paths would never end)");
    if (P.max_depth > 60000) return fail(ctx, XGB_INVALID_ARG, "xgb_render: max_depth must be <= 60000");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    s->last = xgb_render_stats{};
    unsigned long long total = (unsigned long long)film->w * film->h * spp_count;
    if (total == 0) return XGB_OK;
    // 2^23 paths in flight (~1.7 GB of queues) by default: on the terrain 2^21 -> 2^22 -> 2^23
    // gave 1162 -> 1280 -> 1346 Mpaths/s (fewer, fuller wavefront launches)
    unsigned int cap = P.queue_capacity > 0 ? (unsigned int)P.queue_capacity : (1u << 23);
    if ((unsigned long long)cap > total) cap = (unsigned int)std::max<unsigned long long>(total, 1024ull);
    cap = (cap + 255u) & ~255u;
    xgb_status bs = ensureBuffers(s, cap);
    if (bs) return bs;
    cap = s->rb.capacity;

    RenderParams rp{};
    rp.width = film->w; rp.height = film->h;
    rp.sppBegin = spp_begin;
    rp.seed = P.seed;
    rp.integrator = P.integrator;
    rp.maxDepth = P.max_depth;
    rp.rrStart = P.rr_start;
    rp.rrProb = P.rr_prob;
    rp.capacity = cap;
    rp.filmFp64 = film->fp64;
    rp.film = film->d;
    rp.aov = film->aov;
    rp.dropNonFinite = (s->fixes & XGB_FIX_DROP_NONFINITE) ? 1 : 0;
    rp.tileW = ctx->tileW;
    rp.tileH = ctx->tileH;
    rp.sampleGroup = ctx->sampleGroup;
    rp.sppCount = spp_count;
    rp.guided = 0;
    rp.train = 0;
    rp.bsdfFrac = s->bsdfFrac;
    // a scene without guidable materials renders as plain (no inference, no records)
    xgb_guide* gd = s->guidable ? s->guide : nullptr;
    GuideBounds gb;
    if (gd) {
        if (s->mixCapacity < cap) {
            dfree(s->mix);
            s->mix = nullptr;
            s->mixCapacity = 0;
            if (cudaMalloc((void**)&s->mix, sizeof(float4) * 10 * (size_t)cap) != cudaSuccess)
                return fail(ctx, XGB_OOM, "xgb_render: cannot allocate guiding mixtures");
            s->mixCapacity = cap;
        }
        rp.guided = 1;
        rp.mix = s->mix;
        rp.train = s->guideTrain && P.integrator == XGB_INTEGRATOR_STANDARD;
        if (rp.train) {
            if (total > 0xFFFFFFF0ull)
                return fail(ctx, XGB_INVALID_ARG, "xgb_render: guide training needs fewer than 2^32 paths per call");
            if (s->pathAccCapacity < total) {
                dfree(s->pathAcc);
                s->pathAcc = nullptr;
                s->pathAccCapacity = 0;
                if (cudaMalloc((void**)&s->pathAcc, sizeof(float4) * (size_t)total) != cudaSuccess)
                    return fail(ctx, XGB_OOM, "xgb_render: cannot allocate guide training accumulators");
                s->pathAccCapacity = total;
            }
            rp.pathAcc = s->pathAcc;
            rp.arena = gd->arena;
            rp.arenaCount = gd->recCount;
            rp.arenaCap = gd->arenaCap;
            // spread the records over the whole call rather than its first vertices
            double expected = (double)total * std::max(1.0, s->vertsPerPath);
            rp.recordProb = (float)std::min(1.0, (double)gd->arenaCap / expected);
        }
        if (gd->hasBounds) {
            gb = gd->bounds;
        } else {
            for (int k = 0; k < 3; ++k) {
                gb.lo[k] = s->boundsLo[k];
                float e = s->boundsHi[k] - s->boundsLo[k];
                gb.invExtent[k] = e > 0 ? 1.0f / e : 1.0f;
            }
        }
        if (rp.train) XGB_CUDA(ctx, cudaMemsetAsync(gd->recCount, 0, sizeof(unsigned int), st));
    }
    uint64_t guideSteps = 0;

    Ctrl init;
    std::memset(&init, 0, sizeof(init));
    init.totalPaths = total;
    *s->ctrlHost = init;
    XGB_CUDA(ctx, cudaMemcpyAsync(s->ctrl, s->ctrlHost, sizeof(Ctrl), cudaMemcpyHostToDevice, st));
    const int gShade = ctx->numSMs * 8;
    int parity = 0;
    const int kIterPerCheck = 8;
    const bool prof = s->profiling;
    constexpr int kEv = 7;  // per iteration: plan, generate, extend, guide inference, shade, shadow, end
    if (prof && s->events.size() < kEv * kIterPerCheck + 2) {
        while (s->events.size() < kEv * kIterPerCheck + 2) {
            cudaEvent_t ev;
            XGB_CUDA(ctx, cudaEventCreate(&ev));
            s->events.push_back(ev);
        }
    }
    double stageMs[5] = {0, 0, 0, 0, 0};
    double inferMs = 0.0, trainMs = 0.0;
    uint64_t launches = 0;
    for (int guard = 0;; ++guard) {
        for (int k = 0; k < kIterPerCheck; ++k) {
            PathQueue& X = s->rb.q[parity];
            PathQueue& Y = s->rb.q[parity ^ 1];
            cudaEvent_t* ev = prof ? &s->events[kEv * k] : nullptr;
            if (prof) cudaEventRecord(ev[0], st);
            launchPlan(s->ctrl, cap, st);
            if (prof) cudaEventRecord(ev[1], st);
            launchGenerate(s->sd, rp, X, s->ctrl, gShade, st);
            if (prof) cudaEventRecord(ev[2], st);
            launchExtend(s->sd, X, s->rb.hits, s->ctrl, ctx->numSMs, prof, st);
            if (prof) cudaEventRecord(ev[3], st);
            if (gd) {
                guideInferPaths(s->sd, gd->g, gb, X, s->rb.hits, s->ctrl, s->mix, gShade, st);
                ++launches;
            }
            if (prof) cudaEventRecord(ev[4], st);
            launchShade(s->sd, rp, X, s->rb.hits, Y, s->rb.shadow, s->ctrl, ctx->numSMs, st);
            if (prof) cudaEventRecord(ev[5], st);
            launchShadow(s->sd, rp, s->rb.shadow, Y, s->ctrl, ctx->numSMs, st);
            if (prof) cudaEventRecord(ev[6], st);
            launches += 5;
            parity ^= 1;
        }
        XGB_CUDA(ctx, cudaGetLastError());
        XGB_CUDA(ctx, cudaMemcpyAsync(s->ctrlHost, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st));
        XGB_CUDA(ctx, cudaStreamSynchronize(st));
        if (prof) {
            // stages: plan, generate, extend, [guide inference], shade, shadow
            for (int k = 0; k < kIterPerCheck; ++k) {
                float ms[6] = {0, 0, 0, 0, 0, 0};
                for (int j = 0; j < 6; ++j)
                    cudaEventElapsedTime(&ms[j], s->events[kEv * k + j], s->events[kEv * k + j + 1]);
                stageMs[0] += ms[0];
                stageMs[1] += ms[1];
                stageMs[2] += ms[2];
                inferMs += ms[3];
                stageMs[3] += ms[4];
                stageMs[4] += ms[5];
            }
        }
        const Ctrl& c = *s->ctrlHost;
        if (c.errors) break;  // a device bound ran out: the call returns its status below
        if (c.nextPath >= c.totalPaths && c.nOut == 0) break;
        if (guard > (1 << 22)) return fail(ctx, XGB_DEVICE_TIMEOUT, "xgb_render: wavefront did not drain");
    }
    if (gd && rp.train && s->ctrlHost->errors == 0) {
        if (prof) cudaEventRecord(s->events[kEv * kIterPerCheck], st);
        // every path of the call has finished: records take their incident
        // radiance, those that carry some join the pool, and the pool is
        // consumed in fixed-size Adam steps
        guideFinalizeRecords(gd->arena, gd->recCount, gd->arenaCap, s->pathAcc, gd->product, st);
        guideCollect(gd->g, gd->arena, gd->recCount, gd->arenaCap, st);
        XGB_CUDA(ctx, cudaMemcpyAsync(gd->hostPoolCount, gd->g.poolCount, 4, cudaMemcpyDeviceToHost, st));
        XGB_CUDA(ctx, cudaStreamSynchronize(st));
        int n = guidePoolTrain(gd->g, *gd->hostPoolCount, gb, s->guideLr, gd->maxStepsPerCall, st);
        guideSteps += (uint64_t)n;
        launches += 2 + 2 * (uint64_t)n + 1;  // finalize, collect; two per Adam step; pool count
        XGB_CUDA(ctx, cudaGetLastError());
        if (prof) {
            float ms = 0.0f;
            cudaEventRecord(s->events[kEv * kIterPerCheck + 1], st);
            XGB_CUDA(ctx, cudaEventSynchronize(s->events[kEv * kIterPerCheck + 1]));
            cudaEventElapsedTime(&ms, s->events[kEv * kIterPerCheck], s->events[kEv * kIterPerCheck + 1]);
            trainMs = ms;
        }
    }
    const Ctrl& c = *s->ctrlHost;
    if (c.pathsDone > 0) s->vertsPerPath = (double)c.extensionRays / (double)c.pathsDone;
    s->last.paths = c.pathsDone;
    s->last.extension_rays = c.extensionRays;
    s->last.shadow_rays = c.shadowRays;
    s->last.iterations = c.iterations;
    s->last.error_flags = c.errors;
    s->last.kernel_launches = launches;
    s->last.node_visits = c.nodeVisits;
    s->last.tri_tests = c.triTests;
    s->last.guide_train_steps = guideSteps;
    s->last.guide_infer_ms = inferMs;
    s->last.guide_train_ms = trainMs;
    s->last.profiled = prof ? 1 : 0;
    for (int j = 0; j < 5; ++j) {
        s->last.kernel_ms[j] = stageMs[j];
        s->last.stage_launches[j] = launches / 5;
    }
    if (c.errors & ERR_STACK) return fail(ctx, XGB_QUEUE_OVERFLOW, "xgb_render: traversal stack overflow");
    if (c.errors & ERR_LOOP) return fail(ctx, XGB_DEVICE_TIMEOUT, "xgb_render: traversal iteration bound exceeded");
    if (c.errors & ERR_WAIT) return fail(ctx, XGB_DEVICE_TIMEOUT, "xgb_render: guiding network inference wait timed out");
    return XGB_OK;
}

static xgb_status sceneQuery(xgb_scene* s, int n, const float* rays, int any, float* hits, int32_t* occ, void* stream) {
    if (!s || n < 0 || !rays || (!any && !hits) || (any && !occ)) return XGB_INVALID_ARG;
    xgb_ctx* ctx = s->ctx;
    if (!s->built) return fail(ctx, XGB_NOT_BUILT, "xgb_scene_intersect: call xgb_scene_build first");
    if (n == 0) return XGB_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    std::vector<float4> h(2 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 7 * (size_t)i;
        h[i] = make_float4(r[0], r[1], r[2], r[6]);
        h[(size_t)n + i] = make_float4(r[3], r[4], r[5], 0.0f);
    }
    char* dev = nullptr;
    const size_t rayBytes = 32 * (size_t)n, outBytes = any ? 4 * (size_t)n : 32 * (size_t)n;
    if (cudaMallocAsync((void**)&dev, rayBytes + outBytes + 256, st) != cudaSuccess)
        return fail(ctx, XGB_OOM, "xgb_scene_intersect: out of device memory");
    float4* dRays = (float4*)dev;
    char* dOut = dev + rayBytes;
    unsigned int* dErr = (unsigned int*)(dev + rayBytes + outBytes);
    cudaError_t e = cudaMemcpyAsync(dRays, h.data(), rayBytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dErr, 0, 4, st);
    unsigned int err = 0;
    std::vector<float4> out(any ? 0 : 2 * (size_t)n);
    if (e == cudaSuccess) {
        launchQuery(s->sd, dRays, dRays + n, n, any, (float4*)dOut, (int*)dOut, dErr, ctx->numSMs * 8, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = any ? cudaMemcpyAsync(occ, dOut, 4 * (size_t)n, cudaMemcpyDeviceToHost, st)
                                  : cudaMemcpyAsync(out.data(), dOut, 32 * (size_t)n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, dErr, 4, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dev, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cudaFail(ctx, e, "xgb_scene_intersect");
    if (!any)
        for (int i = 0; i < n; ++i) {
            const float4 a = out[2 * (size_t)i], b = out[2 * (size_t)i + 1];
            float* o = hits + 5 * (size_t)i;
            int inst, prim;
            std::memcpy(&inst, &a.y, 4);
            std::memcpy(&prim, &a.z, 4);
            o[0] = a.x; o[1] = (float)inst; o[2] = (float)prim; o[3] = b.x; o[4] = b.y;
        }
    if (err & ERR_STACK) return fail(ctx, XGB_QUEUE_OVERFLOW, "xgb_scene_intersect: traversal stack overflow");
    if (err & ERR_LOOP) return fail(ctx, XGB_DEVICE_TIMEOUT, "xgb_scene_intersect: traversal iteration bound exceeded");
    return XGB_OK;
}

xgb_status xgb_scene_intersect(xgb_scene* s, int n, const float* rays, float* hits, void* stream) {
    return sceneQuery(s, n, rays, 0, hits, nullptr, stream);
}

xgb_status xgb_scene_occluded(xgb_scene* s, int n, const float* rays, int32_t* occluded, void* stream) {
    return sceneQuery(s, n, rays, 1, nullptr, occluded, stream);
}

xgb_status xgb_scene_set_fixes(xgb_scene* s, uint32_t fixes) {
    if (!s) return XGB_INVALID_ARG;
    if (fixes & ~(uint32_t)XGB_FIX_DROP_NONFINITE) return fail(s->ctx, XGB_INVALID_ARG, "xgb_scene_set_fixes: unknown fix");
    s->fixes = fixes;
    s->sd.fixes = (int)fixes;
    return XGB_OK;
}

xgb_status xgb_scene_set_traversal_limits(xgb_scene* s, int max_steps, int max_stack) {
    if (!s) return XGB_INVALID_ARG;
    if (max_steps < 0 || max_stack < 0 || max_stack > kMaxStackLimit)
        return fail(s->ctx, XGB_INVALID_ARG, "xgb_scene_set_traversal_limits: max_steps >= 0, max_stack in [0, 64]");
    s->maxSteps = max_steps ? max_steps : kDefaultMaxSteps;
    s->stackLimit = max_stack ? max_stack : kMaxStackLimit;
    s->sd.maxSteps = s->maxSteps;
    s->sd.stackLimit = s->stackLimit;
    return XGB_OK;
}

xgb_status xgb_scene_set_profiling(xgb_scene* s, int enable) {
    if (!s) return XGB_INVALID_ARG;
    s->profiling = enable != 0;
    return XGB_OK;
}

xgb_status xgb_render_stats_get(xgb_scene* s, xgb_render_stats* out, void* stream) {
    if (!s || !out) return XGB_INVALID_ARG;
    XGB_CUDA(s->ctx, cudaStreamSynchronize(pick(s->ctx, stream)));
    *out = s->last;
    return XGB_OK;
}

}  // extern "C"

// ------------------------------------------------------ internal accessors --
// Read-only views used by other translation units of the library (no allocation).
namespace xgb {
bool sceneView(xgb_scene* s, SceneDev* sd, int* device, int* numSMs, cudaStream_t* stream, int* built) {
    if (!s) return false;
    *sd = s->sd;
    *device = s->ctx->device;
    *numSMs = s->ctx->numSMs;
    *stream = s->ctx->stream;
    *built = s->built ? 1 : 0;
    return true;
}
bool filmView(xgb_film* f, const xgb_scene* s, void** d, int* w, int* h, int* fp64) {
    if (!f || !s || f->ctx != s->ctx) return false;
    *d = f->d;
    *w = f->w;
    *h = f->h;
    *fp64 = f->fp64;
    return true;
}
// What xgb_render would add beyond the plain radiance: AOV planes on the film, a
// learned proposal on the scene.
void renderExtras(const xgb_scene* s, const xgb_film* f, int* filmAovs, int* sceneGuide) {
    *filmAovs = (f && f->aov) ? 1 : 0;
    *sceneGuide = (s && s->guide) ? 1 : 0;
}
xgb_ctx* sceneContext(xgb_scene* s) { return s ? s->ctx : nullptr; }
int sampleGrouping(const xgb_ctx* ctx) { return ctx ? ctx->sampleGroup : 0; }
xgb_status contextFail(xgb_ctx* ctx, xgb_status st, const std::string& msg) { return fail(ctx, st, msg); }
bool filmPlane(xgb_film* f, void** d, int* w, int* h, int* fp64, int* device, cudaStream_t* ctxStream) {
    if (!f) return false;
    *d = f->d;
    *w = f->w;
    *h = f->h;
    *fp64 = f->fp64;
    *device = f->ctx->device;
    *ctxStream = f->ctx->stream;
    return true;
}
}  // namespace xgb

// ------------------------------------------------------------ guiding MLP --
namespace {
// splitmix64-based uniform in [-1, 1) for deterministic initialisation.
float initUniform(uint64_t& state) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((z >> 40) * (1.0 / 8388608.0)) - 1.0f;
}
}  // namespace

extern "C" {

// Reads and clears the error word of the tensor-memory row inference (after the
// stream has been synchronised); XGB_DEVICE_TIMEOUT when one of its waits gave up.
static xgb_status guideRowErrors(xgb_guide* gd, const char* what) {
    unsigned int e = 0;
    unsigned int* word = reinterpret_cast<unsigned int*>(gd->g.scratch.scalars + 2);
    if (cudaMemcpy(&e, word, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return fail(gd->ctx, XGB_CUDA_ERROR, what);
    if (e & ERR_WAIT) {
        cudaMemset(word, 0, 4);
        return fail(gd->ctx, XGB_DEVICE_TIMEOUT, std::string(what) + ": network inference wait timed out");
    }
    return XGB_OK;
}

xgb_status xgb_guide_create(xgb_ctx* ctx, uint32_t seed, xgb_guide** out) {
    if (!ctx || !out) return XGB_INVALID_ARG;
    cudaSetDevice(ctx->device);
    auto* gd = new xgb_guide();
    gd->ctx = ctx;
    GuideDevice& g = gd->g;
    g.maxRows = 65536;
    g.step = 0;
    g.waitLimit = 1 << 22;
    const int R = g.maxRows;
    auto alloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, bytes);
        gd->allocations.push_back(p);
        return p;
    };
    bool ok = true;
    auto A = [&](size_t bytes) { void* p = alloc(bytes); ok = ok && p; return p; };
    g.params = (float*)A(4 * kGuideParams);
    g.grads = (float*)A(4 * kGuideParams);
    g.m = (float*)A(4 * kGuideParams);
    g.v = (float*)A(4 * kGuideParams);
    for (int l = 0; l < 3; ++l) {
        g.w.W[l] = (__nv_bfloat16*)A(2 * 64 * 64);
        g.w.WT[l] = (__nv_bfloat16*)A(2 * 64 * 64);
        g.w.bias[l] = (float*)A(4 * 64);
    }
    g.w.W[3] = (__nv_bfloat16*)A(2 * kGuideOutPad * 64);
    g.w.WT[3] = (__nv_bfloat16*)A(2 * 64 * kGuideOutPad);
    g.w.bias[3] = (float*)A(4 * kGuideOutPad);
    g.scratch.X0 = (__nv_bfloat16*)A(2 * (size_t)R * 64);
    g.scratch.Y = (float*)A(4 * (size_t)R * kGuideOutPad);
    g.scratch.partial = (float*)A(guidePartialBytes());
    g.scratch.scalars = (float*)A(16);
    gd->arenaCap = 1 << 22;
    gd->arena = (GuideRecord*)A(sizeof(GuideRecord) * (size_t)gd->arenaCap);
    gd->recCount = (unsigned int*)A(4 * 4);
    gd->batchRec = (GuideRecord*)A(sizeof(GuideRecord) * (size_t)R);
    g.poolCap = 1 << 22;
    g.batch = 8192;
    g.pool = (GuideRecord*)A(sizeof(GuideRecord) * (size_t)g.poolCap);
    g.poolCount = gd->recCount + 3;
    if (ok && cudaMallocHost((void**)&gd->hostPoolCount, 4) != cudaSuccess) {
        gd->hostPoolCount = nullptr;
        ok = false;
    }
    if (!ok) {
        if (gd->hostPoolCount) cudaFreeHost(gd->hostPoolCount);
        for (void* p : gd->allocations) dfree(p);
        delete gd;
        return fail(ctx, XGB_OOM, "xgb_guide_create: out of device memory");
    }
    // He-uniform hidden layers, zero biases; a small output layer whose biases
    // spread 8 broad lobes (kappa = 1, equal weights) over the sphere.
    std::vector<float> p(kGuideParams, 0.0f);
    uint64_t st = 0x1234567ull ^ ((uint64_t)seed << 20);
    const float hs = std::sqrt(6.0f / 64.0f);
    for (int i = kGuideW0; i < kGuideB0; ++i) p[i] = hs * initUniform(st);
    for (int i = kGuideW1; i < kGuideB1; ++i) p[i] = hs * initUniform(st);
    for (int i = kGuideW2; i < kGuideB2; ++i) p[i] = hs * initUniform(st);
    for (int i = kGuideW3; i < kGuideB3; ++i) p[i] = 0.01f * initUniform(st);
    const float dirs[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    for (int j = 0; j < kGuideLobes; ++j) {
        p[kGuideB3 + 5 * j + 0] = dirs[j][0];
        p[kGuideB3 + 5 * j + 1] = dirs[j][1];
        p[kGuideB3 + 5 * j + 2] = dirs[j][2];
        p[kGuideB3 + 5 * j + 3] = 0.0f;
        p[kGuideB3 + 5 * j + 4] = 0.0f;
    }
    cudaMemcpy(g.params, p.data(), 4 * kGuideParams, cudaMemcpyHostToDevice);
    guideRefresh(g, ctx->stream);
    if (guideTcPrepare() != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        for (void* q : gd->allocations) dfree(q);
        delete gd;
        return fail(ctx, XGB_CUDA_ERROR, "xgb_guide_create: initialisation failed");
    }
    *out = gd;
    return XGB_OK;
}

xgb_status xgb_guide_destroy(xgb_guide* gd) {
    if (!gd) return XGB_INVALID_ARG;
    cudaSetDevice(gd->ctx->device);
    cudaStreamSynchronize(gd->ctx->stream);
    for (void* p : gd->allocations) dfree(p);
    if (gd->hostPoolCount) cudaFreeHost(gd->hostPoolCount);
    delete gd;
    return XGB_OK;
}

xgb_status xgb_guide_param_count(size_t* out) {
    if (!out) return XGB_INVALID_ARG;
    *out = kGuideParams;
    return XGB_OK;
}

xgb_status xgb_guide_get_params(xgb_guide* gd, float* host, size_t n) {
    if (!gd || !host || n != (size_t)kGuideParams) return XGB_INVALID_ARG;
    XGB_CUDA(gd->ctx, cudaStreamSynchronize(gd->ctx->stream));
    XGB_CUDA(gd->ctx, cudaMemcpy(host, gd->g.params, 4 * n, cudaMemcpyDeviceToHost));
    return XGB_OK;
}

xgb_status xgb_guide_set_params(xgb_guide* gd, const float* host, size_t n) {
    if (!gd || !host || n != (size_t)kGuideParams) return XGB_INVALID_ARG;
    xgb_ctx* ctx = gd->ctx;
    XGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    XGB_CUDA(ctx, cudaMemcpy(gd->g.params, host, 4 * n, cudaMemcpyHostToDevice));
    XGB_CUDA(ctx, cudaMemset(gd->g.m, 0, 4 * n));
    XGB_CUDA(ctx, cudaMemset(gd->g.v, 0, 4 * n));
    gd->g.step = 0;
    guideRefresh(gd->g, ctx->stream);
    XGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return XGB_OK;
}

xgb_status xgb_guide_get_grads(xgb_guide* gd, float* host, size_t n) {
    if (!gd || !host || n != (size_t)kGuideParams) return XGB_INVALID_ARG;
    XGB_CUDA(gd->ctx, cudaStreamSynchronize(gd->ctx->stream));
    XGB_CUDA(gd->ctx, cudaMemcpy(host, gd->g.grads, 4 * n, cudaMemcpyDeviceToHost));
    return XGB_OK;
}

xgb_status xgb_guide_set_bounds(xgb_guide* gd, const float lo[3], const float hi[3]) {
    if (!gd || !lo || !hi) return XGB_INVALID_ARG;
    for (int k = 0; k < 3; ++k) {
        if (!(hi[k] > lo[k])) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_set_bounds: need hi > lo");
        gd->bounds.lo[k] = lo[k];
        gd->bounds.invExtent[k] = 1.0f / (hi[k] - lo[k]);
    }
    gd->hasBounds = true;
    return XGB_OK;
}

xgb_status xgb_guide_infer(xgb_guide* gd, int n, const float* pos, const float* nrm, const float* wo, float* out) {
    if (!gd || n < 0 || (n > 0 && (!pos || !nrm || !wo || !out))) return XGB_INVALID_ARG;
    if (!gd->hasBounds) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_infer: call xgb_guide_set_bounds first");
    xgb_ctx* ctx = gd->ctx;
    cudaStream_t st = ctx->stream;
    const int R = gd->g.maxRows;
    float* dIn = nullptr;
    XGB_CUDA(ctx, cudaMalloc((void**)&dIn, 4 * 9 * (size_t)R));
    std::vector<float> y((size_t)R * kGuideOutPad);
    for (int b = 0; b < n; b += R) {
        int cnt = std::min(R, n - b);
        int rows = ((cnt + 63) / 64) * 64;
        cudaMemcpyAsync(dIn, pos + 3 * (size_t)b, 12 * (size_t)cnt, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dIn + 3 * R, nrm + 3 * (size_t)b, 12 * (size_t)cnt, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dIn + 6 * R, wo + 3 * (size_t)b, 12 * (size_t)cnt, cudaMemcpyHostToDevice, st);
        guideFeaturesFromPoints(dIn, dIn + 3 * R, dIn + 6 * R, cnt, rows, gd->bounds, gd->g.scratch.X0, st);
        guideInferRows(gd->g, gd->g.scratch.X0, rows, gd->g.scratch.Y, st);
        cudaMemcpyAsync(y.data(), gd->g.scratch.Y, 4 * (size_t)rows * kGuideOutPad, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            cudaFree(dIn);
            return fail(ctx, XGB_CUDA_ERROR, "xgb_guide_infer failed");
        }
        for (int r = 0; r < cnt; ++r)
            std::memcpy(out + (size_t)(b + r) * kGuideOut, y.data() + (size_t)r * kGuideOutPad, 4 * kGuideOut);
    }
    cudaFree(dIn);
    return guideRowErrors(gd, "xgb_guide_infer");
}

xgb_status xgb_guide_sample(xgb_guide* gd, int n, const float* pos, const float* nrm, const float* wo, uint32_t seed,
                            float* dirs, float* pdf) {
    if (!gd || n < 0 || (n > 0 && (!pos || !nrm || !wo || !dirs || !pdf))) return XGB_INVALID_ARG;
    if (n > gd->g.maxRows) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_sample: at most 65536 points");
    if (!gd->hasBounds) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_sample: call xgb_guide_set_bounds first");
    if (n == 0) return XGB_OK;
    xgb_ctx* ctx = gd->ctx;
    cudaStream_t st = ctx->stream;
    const int R = gd->g.maxRows;
    float* dIn = nullptr;
    XGB_CUDA(ctx, cudaMalloc((void**)&dIn, 4 * 13 * (size_t)R));
    int rows = ((n + 63) / 64) * 64;
    cudaMemcpyAsync(dIn, pos, 12 * (size_t)n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dIn + 3 * R, nrm, 12 * (size_t)n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dIn + 6 * R, wo, 12 * (size_t)n, cudaMemcpyHostToDevice, st);
    guideFeaturesFromPoints(dIn, dIn + 3 * R, dIn + 6 * R, n, rows, gd->bounds, gd->g.scratch.X0, st);
    guideInferRows(gd->g, gd->g.scratch.X0, rows, gd->g.scratch.Y, st);
    guideSampleRows(gd->g.scratch.Y, n, seed, dIn + 9 * R, dIn + 12 * R, st);
    cudaMemcpyAsync(dirs, dIn + 9 * R, 12 * (size_t)n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(pdf, dIn + 12 * R, 4 * (size_t)n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(dIn);
    if (e != cudaSuccess) return cudaFail(ctx, e, "xgb_guide_sample");
    return guideRowErrors(gd, "xgb_guide_sample");
}

xgb_status xgb_guide_train_batch(xgb_guide* gd, int n, const float* pos, const float* nrm, const float* wo,
                                 const float* wi, const float* pdf, const float* radiance, float lr, float* loss) {
    if (!gd || n <= 0 || !pos || !nrm || !wo || !wi || !pdf || !radiance || lr < 0) return XGB_INVALID_ARG;
    if (n > gd->g.maxRows) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_train_batch: at most 65536 samples");
    if (!gd->hasBounds) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_train_batch: call xgb_guide_set_bounds first");
    xgb_ctx* ctx = gd->ctx;
    cudaStream_t st = ctx->stream;
    std::vector<GuideRecord> rec(n);
    for (int i = 0; i < n; ++i) {
        rec[i].p = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        rec[i].n = make_float3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        rec[i].wo = make_float3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        rec[i].wi = make_float3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        rec[i].pdf = pdf[i];
        rec[i].radiance = radiance[i];
    }
    XGB_CUDA(ctx, cudaMemcpyAsync(gd->batchRec, rec.data(), sizeof(GuideRecord) * n, cudaMemcpyHostToDevice, st));
    guideTrainStep(gd->g, gd->batchRec, n, gd->bounds, lr, st);
    float sc[2];
    XGB_CUDA(ctx, cudaMemcpyAsync(sc, gd->g.scratch.scalars, 8, cudaMemcpyDeviceToHost, st));
    XGB_CUDA(ctx, cudaStreamSynchronize(st));
    XGB_CUDA(ctx, cudaGetLastError());
    if (loss) *loss = sc[1];
    return XGB_OK;
}

xgb_status xgb_guide_set_wait_limit(xgb_guide* gd, int polls) {
    if (!gd) return XGB_INVALID_ARG;
    if (polls < 0) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_set_wait_limit: polls >= 0");
    XGB_CUDA(gd->ctx, cudaStreamSynchronize(gd->ctx->stream));
    gd->g.waitLimit = polls;
    return XGB_OK;
}

xgb_status xgb_guide_set_training(xgb_guide* gd, int batch_rows, int max_steps_per_call, int product_target) {
    if (!gd) return XGB_INVALID_ARG;
    if (batch_rows < 64 || batch_rows > gd->g.maxRows || (batch_rows & 63))
        return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_set_training: batch_rows must be a multiple of 64 in [64, 65536]");
    if (max_steps_per_call < 1) return fail(gd->ctx, XGB_INVALID_ARG, "xgb_guide_set_training: max_steps_per_call >= 1");
    XGB_CUDA(gd->ctx, cudaStreamSynchronize(gd->ctx->stream));
    gd->g.batch = batch_rows;
    gd->maxStepsPerCall = max_steps_per_call;
    gd->product = product_target ? 1 : 0;
    return XGB_OK;
}

xgb_status xgb_guide_train_steps(xgb_guide* gd, uint64_t* out) {
    if (!gd || !out) return XGB_INVALID_ARG;
    *out = (uint64_t)gd->g.step;
    return XGB_OK;
}

xgb_status xgb_scene_set_guide(xgb_scene* s, xgb_guide* gd, float bsdf_fraction, int train, float learning_rate) {
    if (!s) return XGB_INVALID_ARG;
    if (gd && gd->ctx != s->ctx) return fail(s->ctx, XGB_INVALID_ARG, "xgb_scene_set_guide: guide of another context");
    if (gd && !(bsdf_fraction > 0.0f && bsdf_fraction < 1.0f))
        return fail(s->ctx, XGB_INVALID_ARG, "xgb_scene_set_guide: bsdf_fraction must be in (0, 1)");
    if (gd && train && !(learning_rate > 0.0f)) return fail(s->ctx, XGB_INVALID_ARG, "xgb_scene_set_guide: learning rate");
    s->guide = gd;
    s->bsdfFrac = bsdf_fraction;
    s->guideTrain = (gd && train) ? 1 : 0;
    s->guideLr = learning_rate;
    return XGB_OK;
}

}  // extern "C"
