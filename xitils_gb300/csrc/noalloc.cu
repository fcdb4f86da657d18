// xgb_render_noalloc: the render call of xgb_render for callers that must not
// allocate GPU memory.
//
// xgb_render sizes its path queues to the work and allocates them with
// cudaMalloc on first use. Some hosts cannot allow that: an engine that reserves
// all device memory through its own pool at start-up, a frame loop where the
// implicit device synchronisation of cudaMalloc/cudaFree would stall the other
// streams, or a plug-in host that hands the renderer a stream and nothing else.
// This entry point keeps every byte of its working memory -- two path queues,
// the hit records, the shadow-ray queue and the counters -- in one file-scope
// __device__ array of fixed size, so it calls no cudaMalloc, cudaFree or other
// allocating routine. The caller still owns the inputs (a built scene) and the
// output (a film).
//
// Limits and rules:
//  * at most kNoAllocMaxPaths = 32768 paths are in flight; a larger
//    params->queue_capacity is rejected with XGB_INVALID_ARG (0 selects the
//    maximum). The number of samples is not limited: the queue refills.
//  * the array (about 6 MB) is part of the library image: every GPU that loads
//    the library holds it until the process exits.
//  * all calls share the one array per device and every call re-initialises the
//    counters it needs; calls whose GPU work overlaps (other streams, other host
//    threads) race on it and must be serialised by the caller.
//  * every call looks up the array's device address (cudaGetSymbolAddress,
//    with the scene's device current), so the address stays right after a
//    context reset; make the first call on a device before any stream capture.
//  * the film receives the radiance only: a film with AOV planes
//    (xgb_film_enable_aovs) or a scene with a learned proposal
//    (xgb_scene_set_guide) is refused with XGB_UNSUPPORTED, since both need
//    per-call device memory. The scene's last-render statistics
//    (xgb_render_stats_get) are not updated.
#include <cstring>

#include "../../include/xgb.h"
#include "xgb_kernels.h"

namespace xgb {
bool sceneView(xgb_scene* s, SceneDev* sd, int* device, int* numSMs, cudaStream_t* stream, int* built);
bool filmView(xgb_film* f, const xgb_scene* s, void** d, int* w, int* h, int* fp64);
void renderExtras(const xgb_scene* s, const xgb_film* f, int* filmAovs, int* sceneGuide);
xgb_ctx* sceneContext(xgb_scene* s);
int sampleGrouping(const xgb_ctx* ctx);
}  // namespace xgb

using namespace xgb;

namespace {

constexpr unsigned int kNoAllocMaxPaths = 32768;
constexpr size_t kAlign = 256;
constexpr size_t up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }
constexpr size_t kV4 = up(16ull * kNoAllocMaxPaths);  // one float4 per path
constexpr size_t kU2 = up(8ull * kNoAllocMaxPaths);   // one uint2 per path
constexpr size_t kI1 = up(4ull * kNoAllocMaxPaths);   // one int per path
constexpr size_t kQueueBytes = 3 * kV4 + kU2;         // o, d, thr, rng
constexpr size_t kScratchBytes = 2 * kQueueBytes      // path queues (in, out)
                                 + kV4 + kI1          // hit records
                                 + 3 * kV4 + kU2      // shadow queue
                                 + up(sizeof(Ctrl));  // counters

}  // namespace

// The scratch of xgb_render_noalloc (see the header of this file).
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

namespace {

// Device address of g_noallocScratch on the current device. In host code the
// array's name is only a host-side stand-in, never a device address; the
// lookup allocates nothing and is repeated on every call, so a context
// recreated by the host application (cudaDeviceReset) is picked up.
cudaError_t scratchAddress(unsigned char** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return e;
    *out = (unsigned char*)p;
    return cudaSuccess;
}

}  // namespace

extern "C" xgb_status xgb_render_noalloc(xgb_scene* scene, const xgb_integrator_params* params, xgb_film* film,
                                         uint32_t spp_begin, uint32_t spp_count, void* stream) {
    SceneDev sd;
    int device = 0, numSMs = 1, built = 0;
    cudaStream_t ctxStream = nullptr;
    if (!sceneView(scene, &sd, &device, &numSMs, &ctxStream, &built)) return XGB_INVALID_ARG;
    if (!built) return XGB_NOT_BUILT;
    void* filmPtr = nullptr;
    int W = 0, H = 0, fp64 = 0;
    if (!filmView(film, scene, &filmPtr, &W, &H, &fp64)) return XGB_INVALID_ARG;
    int filmAovs = 0, sceneGuide = 0;
    renderExtras(scene, film, &filmAovs, &sceneGuide);
    if (filmAovs || sceneGuide) return XGB_UNSUPPORTED;
    xgb_integrator_params P;
    if (params) P = *params;
    else xgb_integrator_params_default(&P);
    if (P.integrator != XGB_INTEGRATOR_STANDARD && P.integrator != XGB_INTEGRATOR_NAIVE) return XGB_INVALID_ARG;
    if (P.rr_start < 1 || !(P.rr_prob > 0.0f && P.rr_prob <= 1.0f) || P.max_depth < 0 || P.max_depth > 60000)
        return XGB_INVALID_ARG;
    if (P.max_depth == 0 && P.rr_prob >= 1.0f) return XGB_INVALID_ARG;
    if (P.queue_capacity < 0 || (unsigned int)P.queue_capacity > kNoAllocMaxPaths) return XGB_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return XGB_CUDA_ERROR;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctxStream;
    unsigned long long total = (unsigned long long)W * H * spp_count;
    if (total == 0) return XGB_OK;
    const unsigned int cap = P.queue_capacity > 0 ? (unsigned int)P.queue_capacity : kNoAllocMaxPaths;

    unsigned char* base = nullptr;
    if (scratchAddress(&base) != cudaSuccess) return XGB_CUDA_ERROR;
    unsigned char* p = base;
    auto take = [&](size_t bytes) { unsigned char* r = p; p += bytes; return r; };
    PathQueue q[2]{};  // training fields (grec, pid) stay null: guiding is refused above
    for (int k = 0; k < 2; ++k) {
        q[k].o = (float4*)take(kV4);
        q[k].d = (float4*)take(kV4);
        q[k].thr = (float4*)take(kV4);
        q[k].rng = (uint2*)take(kU2);
    }
    HitQueue hits{};
    hits.h = (float4*)take(kV4);
    hits.inst = (int*)take(kI1);
    ShadowQueue sq{};
    sq.o = (float4*)take(kV4);
    sq.d = (float4*)take(kV4);
    sq.c = (float4*)take(kV4);
    sq.rng = (uint2*)take(kU2);
    Ctrl* ctrl = (Ctrl*)take(up(sizeof(Ctrl)));

    RenderParams rp{};  // learned-proposal fields stay off (0 / nullptr)
    rp.width = W; rp.height = H;
    rp.sppBegin = spp_begin;
    rp.sampleGroup = sampleGrouping(sceneContext(scene));
    rp.sppCount = spp_count;
    rp.seed = P.seed;
    rp.integrator = P.integrator;
    rp.maxDepth = P.max_depth;
    rp.rrStart = P.rr_start;
    rp.rrProb = P.rr_prob;
    rp.capacity = cap;
    rp.filmFp64 = fp64;
    rp.film = filmPtr;
    rp.dropNonFinite = (sd.fixes & XGB_FIX_DROP_NONFINITE) ? 1 : 0;

    // The counters keep the previous call's values: start from zero.
    Ctrl host;
    std::memset(&host, 0, sizeof(host));
    host.totalPaths = total;
    if (cudaMemcpyAsync(ctrl, &host, sizeof(Ctrl), cudaMemcpyHostToDevice, st) != cudaSuccess) return XGB_CUDA_ERROR;
    const int gShade = numSMs * 8;
    int parity = 0;
    for (int guard = 0;; ++guard) {
        for (int k = 0; k < 8; ++k) {
            PathQueue& X = q[parity];
            PathQueue& Y = q[parity ^ 1];
            launchPlan(ctrl, cap, st);
            launchGenerate(sd, rp, X, ctrl, gShade, st);
            launchExtend(sd, X, hits, ctrl, numSMs, false, st);
            launchShade(sd, rp, X, hits, Y, sq, ctrl, numSMs, st);
            launchShadow(sd, rp, sq, Y, ctrl, numSMs, st);
            parity ^= 1;
        }
        if (cudaGetLastError() != cudaSuccess) return XGB_CUDA_ERROR;
        if (cudaMemcpyAsync(&host, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st) != cudaSuccess) return XGB_CUDA_ERROR;
        if (cudaStreamSynchronize(st) != cudaSuccess) return XGB_CUDA_ERROR;
        if (host.nextPath >= host.totalPaths && host.nOut == 0) break;
        if (guard > (1 << 24)) return XGB_DEVICE_TIMEOUT;
    }
    if (host.errors & ERR_STACK) return XGB_QUEUE_OVERFLOW;
    if (host.errors & ERR_LOOP) return XGB_DEVICE_TIMEOUT;
    return XGB_OK;
}
