// Launch wrappers shared between the host API (api.cu) and the kernel
// translation units. No CUDA types beyond cudaStream_t cross this boundary.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "xgb_types.h"

namespace xgb {

// ---- BVH build (bvh_build.cu) ------------------------------------------------
constexpr int kBuilderPloc = 0;  // locally-ordered clustering (default)
constexpr int kBuilderLbvh = 1;  // Morton-split linear BVH
constexpr int kLayoutBinary = 0;  // Node2, two children per 64-byte node
constexpr int kLayoutWide = 1;    // WNode, eight quantised children per 80-byte node
struct BlasBuildInput {
    const float4* pos;  // device, object space
    const int* idx;     // device, 3 per triangle
    int nTris;
    int builder;        // kBuilderPloc or kBuilderLbvh
    int layout;         // kLayoutBinary or kLayoutWide
};
struct BlasBuildOutput {
    WNode* nodes;       // wide layout: device, allocated by buildBlas (cudaMalloc, nWide entries; the caller frees it)
    int nWide;
    Node2* nodes2;      // binary layout: device, allocated by buildBlas (nTris - 1 entries; the caller frees it)
    int wide;
    TriV* tris;         // device, nTris entries (leaf order), allocated by the caller
    float4* gnrm;       // device, nTris entries (original order)
    float* triArea;     // device, nTris entries (original order)
    int rootIsLeaf;
    int rootLeaf;
    float boundsLo[3], boundsHi[3];  // object-space bounds of the vertices used
};
// Builds a binary BVH over the triangles (PLOC or LBVH), in the binary layout or
// converted into an 8-wide compressed BVH, on `stream`, and synchronises it.
// Returns a CUDA error code (cudaSuccess on success).
cudaError_t buildBlas(const BlasBuildInput& in, BlasBuildOutput* out, cudaStream_t stream);

// SVNDF fit of a displacement map (svndf.cu): lobes [resV][resU][5] float4, low
// heights [resV][resU] float4 (red channel). rate in [1, 16].
cudaError_t svndfFit(const TextureDev& src, float scale, int rate, uint32_t seed, int resU, int resV, float4* lobes,
                     float4* low, cudaStream_t s);

// ---- wavefront (integrator.cu / trace.cu) --------------------------------------
struct Ctrl {
    unsigned long long nextPath;   // next camera path id to generate
    unsigned long long totalPaths;
    unsigned long long firstNew;   // id of the first path generated this iteration
    unsigned int nCont;            // paths carried over into this iteration's input queue
    unsigned int nActive;          // paths in this iteration's input queue
    unsigned int nOut;             // paths written to the output queue by shade
    unsigned int nShadow;          // shadow rays written by shade
    unsigned int extendHead;       // persistent work counters
    unsigned int shadowHead;
    unsigned int errors;           // bit 0: traversal stack overflow
    unsigned int pad;
    unsigned long long extensionRays;
    unsigned long long shadowRays;
    unsigned long long iterations;
    unsigned long long pathsDone;
    unsigned long long nodeVisits;  // profiling counters (extension rays)
    unsigned long long triTests;
};

// ERR_WAIT: a bounded mbarrier wait of the tensor-memory inference kernels gave up.
enum ErrorBits : unsigned int { ERR_STACK = 1u, ERR_QUEUE = 2u, ERR_LOOP = 4u, ERR_WAIT = 8u };

struct PathQueue {
    float4* o;          // o.xyz, w = pdf of the BSDF sample that produced this ray (-1: specular)
    float4* d;          // d.xyz, w = bits: pathLength | flags << 16
    float4* thr;        // throughput.xyz, w = bits: pixel index
    uint2* rng;         // PCG state
    int* grec;          // guide training: record of the vertex this ray left (-1: none)
    unsigned int* pid;  // guide training: index of the path within the render call
};

// One training sample of the guiding network: a guided vertex, the direction
// sampled there and, once the path has finished, the incident radiance found
// along it: (contributions of the later vertices) / (throughput after this vertex).
struct __align__(16) GuideRecord {
    float3 p;
    float pdf;        // density wi was sampled with (mixture of BSDF and network)
    float3 n;
    float fcos;       // luminance of bsdfCos(wi) (product target)
    float3 wo;
    unsigned int pid; // path index within the render call
    float3 wi;
    float radiance;   // training target (luminance), filled in when the call ends
    float3 snap;      // the path's accumulated contribution before the next vertex (NaN: none)
    float pad0;
    float3 thr;       // path throughput after this vertex
    float pad1;
};
static_assert(sizeof(GuideRecord) == 96, "GuideRecord size");

struct HitQueue {
    float4* h;    // t, b0, b1, bits(prim); prim = -1 on a miss
    int* inst;
};
struct ShadowQueue {
    float4* o;          // o.xyz, tMax
    float4* d;          // d.xyz, bits(pixel)
    float4* c;          // contribution rgb, bits(output-queue index of the path or -1)
    uint2* rng;         // PCG state after a stochastic bsdfCos (committed if visible)
    unsigned int* pid;  // guide training: path credited with the contribution
};

enum PathFlags : int { FLAG_PRIMARY = 1, FLAG_STOCHASTIC_NEE = 2 };

struct RenderParams {
    int width, height;
    uint32_t sppBegin;
    uint32_t seed;
    int integrator;
    int maxDepth;
    int rrStart;
    float rrProb;
    unsigned int capacity;
    int filmFp64;
    void* film;  // float4* or double4*
    void* aov;   // first-hit albedo plane then normal plane (same type as film), nullptr: off
    int dropNonFinite;  // film additions with a non-finite component are skipped (opt-in fix)
    // learned proposal (0 / nullptr when off)
    int guided;
    int train;
    float bsdfFrac;           // one-sample MIS: probability of sampling the BSDF
    const float4* mix;        // per input path: 8 x (mu, kappa) then 8 weights
    GuideRecord* arena;       // training records of this call
    unsigned int* arenaCount; // may run past arenaCap (writers drop)
    int arenaCap;
    float recordProb;         // probability that a guided vertex becomes a record
    float4* pathAcc;          // per path of the call: contributions so far (rgb)
    // order of the camera paths of a sample pass: tileW x tileH pixel blocks
    // (k_generate), 0 = scanline rows
    int tileW, tileH;
    // order of the samples: sampleGroup (> 1) consecutive camera paths are
    // consecutive samples of one pixel, in passes of sampleGroup samples over
    // the film; 0 or 1 = one sample pass over the film after the other.
    // sppCount = samples of this call.
    int sampleGroup;
    unsigned int sppCount;
};

// Device arrays of a batch of render jobs sharing one wavefront (xgb_render_batch):
// a path of job j carries j << 24 | pixel in its pixel field.
constexpr int kBatchFlat = 1, kBatchSingle = 2;
struct BatchView {
    const SceneDev* scenes;
    const RenderParams* params;
    const unsigned long long* start;  // nJobs + 1 prefix sums of the jobs' path counts
    int nJobs;
    int flat;    // kBatchFlat: every scene has <= 16 instances and binary mesh BVHs (the persistent per-lane
                 // kernels); kBatchSingle: every scene is one instance of a binary mesh BVH; 0: general
    int nested;  // some scene has a material that evaluates another (the shade kernel with that code)
};
void launchGenerateBatch(const BatchView& b, PathQueue q, Ctrl* ctrl, int grid, cudaStream_t s);
void launchShadeBatch(const BatchView& b, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl,
                      int numSMs, cudaStream_t s);
void launchExtendBatch(const BatchView& b, PathQueue q, HitQueue h, Ctrl* ctrl, int numSMs, cudaStream_t s);
void launchShadowBatch(const BatchView& b, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int numSMs, cudaStream_t s);

void launchPlan(Ctrl* ctrl, unsigned int capacity, cudaStream_t s);
void launchGenerate(const SceneDev& sc, const RenderParams& rp, PathQueue q, Ctrl* ctrl, int grid, cudaStream_t s);
// Extension / shadow rays and shading of the wavefront; grids sized from the
// launched kernel's occupancy on numSMs SMs (one full wave).
void launchExtend(const SceneDev& sc, PathQueue q, HitQueue h, Ctrl* ctrl, int numSMs, bool count, cudaStream_t s);
void launchShade(const SceneDev& sc, const RenderParams& rp, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq,
                 Ctrl* ctrl, int numSMs, cudaStream_t s);
void launchShadow(const SceneDev& sc, const RenderParams& rp, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int numSMs,
                  cudaStream_t s);
// Film plane (float4 or double4 per pixel) -> packed float RGB, strideFloats 3 or 4 (image.cu).
void launchPackFilm(const void* film, int fp64, size_t n, int strideFloats, float* out, int grid, cudaStream_t s);
// Ray queries on a built scene: rays o (xyz, w = tMax) and d; closest hits as 2 float4
// per ray (t, bits(instance), bits(triangle), -; b0, b1, -, -) or any-hit flags.
void launchQuery(const SceneDev& sc, const float4* o, const float4* d, int n, int any, float4* hits, int* occluded,
                 unsigned int* errors, int grid, cudaStream_t s);

}  // namespace xgb
