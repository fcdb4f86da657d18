// xgb_render_batch: many independent render jobs (scene, film, parameters,
// sample range) in one wavefront.
//
// The jobs' camera paths are numbered one after the other (job j owns the ids
// [start[j], start[j + 1])), so a single queue of paths in flight serves every
// scene: small films do not leave the GPU idle and large ones do not need their
// own launches. Each path carries its job in the high byte of its pixel field;
// the kernels look the scene and the render parameters up per path (the
// two-level traversal per ray, the same shading as xgb_render). Per-path random
// streams are those of xgb_render, so a job's film equals the film xgb_render
// makes for it, up to the order of the floating-point sums.
//
// The wavefront iterations between host checks are recorded once as a CUDA graph
// and replayed (kernel arguments are device pointers whose contents are updated
// before each call, so one graph serves later calls of the same shape). The
// number of paths in flight and the iterations per check come from an
// autotuner: short trial renders (one sample per pixel of every job into scratch
// films) of each candidate, the fastest kept per batch shape.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/xgb.h"
#include "xgb_kernels.h"

namespace xgb {
bool sceneView(xgb_scene* s, SceneDev* sd, int* device, int* numSMs, cudaStream_t* stream, int* built);
bool filmPlane(xgb_film* f, void** d, int* w, int* h, int* fp64, int* device, cudaStream_t* ctxStream);
xgb_ctx* sceneContext(xgb_scene* s);
int sampleGrouping(const xgb_ctx* ctx);
xgb_status contextFail(xgb_ctx* ctx, xgb_status st, const std::string& msg);
}  // namespace xgb

using namespace xgb;

namespace {

constexpr int kMaxJobs = 255;  // the job travels in 8 bits of the pixel field

struct BatchState {
    unsigned int capacity = 0;
    PathQueue q[2];
    HitQueue hits;
    ShadowQueue shadow;
    void* block = nullptr;
    Ctrl* ctrl = nullptr;
    Ctrl* ctrlHost = nullptr;
    int jobCap = 0;
    SceneDev* dScenes = nullptr;
    RenderParams* dParams = nullptr;
    unsigned long long* dStart = nullptr;
    // staging (pinned) for the per-call arrays
    SceneDev* hScenes = nullptr;
    RenderParams* hParams = nullptr;
    unsigned long long* hStart = nullptr;
    // replayed iteration block
    cudaGraphExec_t graph = nullptr;
    unsigned int graphCap = 0;
    int graphIters = 0;
    int graphJobs = 0;
    int graphFlat = -1;
    std::map<std::string, xgb_batch_options> tuned;
    xgb_render_stats last{};
};

std::mutex g_mu;
std::map<xgb_ctx*, BatchState*> g_states;

void freeState(BatchState* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : {(void*)b->block, (void*)b->ctrl, (void*)b->dScenes, (void*)b->dParams, (void*)b->dStart})
        if (p) cudaFree(p);
    for (void* p : {(void*)b->ctrlHost, (void*)b->hScenes, (void*)b->hParams, (void*)b->hStart})
        if (p) cudaFreeHost(p);
    delete b;
}

BatchState* stateOf(xgb_ctx* ctx) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_states.find(ctx);
    if (it != g_states.end()) return it->second;
    auto* b = new BatchState();
    g_states[ctx] = b;
    return b;
}

cudaError_t ensureQueues(BatchState* b, unsigned int cap) {
    if (b->capacity >= cap && b->block) return cudaSuccess;
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    if (b->block) { cudaFree(b->block); b->block = nullptr; b->capacity = 0; }
    const size_t pathBytes = (size_t)cap * (16 * 3 + 8);
    const size_t total = 2 * pathBytes + (size_t)cap * (16 + 4) + (size_t)cap * (16 * 3 + 8) + 64 * 256;
    void* block = nullptr;
    cudaError_t e = cudaMalloc(&block, total);
    if (e != cudaSuccess) return e;
    char* p = (char*)block;
    auto take = [&](size_t bytes) { char* r = p; p += (bytes + 255) & ~(size_t)255; return r; };
    for (int k = 0; k < 2; ++k) {
        b->q[k] = PathQueue{};
        b->q[k].o = (float4*)take(16 * (size_t)cap);
        b->q[k].d = (float4*)take(16 * (size_t)cap);
        b->q[k].thr = (float4*)take(16 * (size_t)cap);
        b->q[k].rng = (uint2*)take(8 * (size_t)cap);
    }
    b->hits.h = (float4*)take(16 * (size_t)cap);
    b->hits.inst = (int*)take(4 * (size_t)cap);
    b->shadow = ShadowQueue{};
    b->shadow.o = (float4*)take(16 * (size_t)cap);
    b->shadow.d = (float4*)take(16 * (size_t)cap);
    b->shadow.c = (float4*)take(16 * (size_t)cap);
    b->shadow.rng = (uint2*)take(8 * (size_t)cap);
    b->block = block;
    b->capacity = cap;
    return cudaSuccess;
}

cudaError_t ensureJobs(BatchState* b, int n) {
    if (!b->ctrl) {
        cudaError_t e = cudaMalloc((void**)&b->ctrl, sizeof(Ctrl));
        if (e == cudaSuccess) e = cudaMallocHost((void**)&b->ctrlHost, sizeof(Ctrl));
        if (e != cudaSuccess) return e;
    }
    if (b->jobCap >= n) return cudaSuccess;
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    for (void* p : {(void*)b->dScenes, (void*)b->dParams, (void*)b->dStart}) if (p) cudaFree(p);
    for (void* p : {(void*)b->hScenes, (void*)b->hParams, (void*)b->hStart}) if (p) cudaFreeHost(p);
    b->dScenes = nullptr; b->dParams = nullptr; b->dStart = nullptr;
    b->hScenes = nullptr; b->hParams = nullptr; b->hStart = nullptr;
    b->jobCap = 0;
    const int cap = std::max(n, 16);
    cudaError_t e = cudaMalloc((void**)&b->dScenes, sizeof(SceneDev) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->dParams, sizeof(RenderParams) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->dStart, sizeof(unsigned long long) * (cap + 1));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hScenes, sizeof(SceneDev) * cap);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hParams, sizeof(RenderParams) * cap);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hStart, sizeof(unsigned long long) * (cap + 1));
    if (e == cudaSuccess) b->jobCap = cap;
    return e;
}

// One block of `iters` wavefront iterations (an even count: the queues come back to parity 0).
void enqueueBlock(BatchState* b, const BatchView& v, unsigned int cap, int iters, int numSMs, cudaStream_t st) {
    for (int k = 0; k < iters; ++k) {
        PathQueue& X = b->q[k & 1];
        PathQueue& Y = b->q[(k & 1) ^ 1];
        launchPlan(b->ctrl, cap, st);
        launchGenerateBatch(v, X, b->ctrl, numSMs * 8, st);
        launchExtendBatch(v, X, b->hits, b->ctrl, numSMs, st);
        launchShadeBatch(v, X, b->hits, Y, b->shadow, b->ctrl, numSMs, st);
        launchShadowBatch(v, b->shadow, Y, b->ctrl, numSMs, st);
    }
}

std::string shapeKey(const xgb_batch_job* jobs, int n) {
    std::string k;
    for (int i = 0; i < n; ++i) {
        void* d; int w, h, f64, dev; cudaStream_t cs;
        filmPlane(jobs[i].film, &d, &w, &h, &f64, &dev, &cs);
        k += std::to_string((uintptr_t)jobs[i].scene) + ":" + std::to_string(w) + "x" + std::to_string(h) + "x" +
             std::to_string(jobs[i].spp_count) + ";";
    }
    return k;
}

// The wavefront over all jobs. Returns XGB_OK or an error (with the context's message set).
xgb_status runBatch(xgb_ctx* ctx, BatchState* b, const xgb_batch_job* jobs, int n, const xgb_batch_options& o,
                    cudaStream_t st, int device, int numSMs, double* seconds) {
    unsigned long long total = 0;
    int flat = 1, single = 1, nested = 0;
    for (int i = 0; i < n; ++i) {
        SceneDev sd; int dev, sms, built; cudaStream_t cs;
        sceneView(jobs[i].scene, &sd, &dev, &sms, &cs, &built);
        if (sd.nInstances > 16 || sd.blasLayout != 0 || sd.shell) flat = 0;
        if (sd.nInstances != 1 || sd.blasLayout != 0 || sd.shell) single = 0;
        nested |= sd.nested ? 1 : 0;
        void* fd; int w, h, f64, fdev; cudaStream_t fcs;
        filmPlane(jobs[i].film, &fd, &w, &h, &f64, &fdev, &fcs);
        const xgb_integrator_params& P = jobs[i].params;
        RenderParams rp{};
        rp.width = w; rp.height = h;
        rp.sppBegin = jobs[i].spp_begin;
        rp.sampleGroup = sampleGrouping(ctx);
        rp.sppCount = jobs[i].spp_count;
        rp.seed = P.seed;
        rp.integrator = P.integrator;
        rp.maxDepth = P.max_depth;
        rp.rrStart = P.rr_start;
        rp.rrProb = P.rr_prob;
        rp.capacity = o.queue_capacity;
        rp.filmFp64 = f64;
        rp.film = fd;
        rp.dropNonFinite = (sd.fixes & XGB_FIX_DROP_NONFINITE) ? 1 : 0;
        b->hScenes[i] = sd;
        b->hParams[i] = rp;
        b->hStart[i] = total;
        total += (unsigned long long)w * h * jobs[i].spp_count;
    }
    b->hStart[n] = total;
    if (total == 0) return XGB_OK;
    const unsigned int cap = (unsigned int)std::min<unsigned long long>((unsigned long long)o.queue_capacity,
                                                                        std::max<unsigned long long>(total, 1024ull));
    const unsigned int capR = (cap + 255u) & ~255u;
    for (int i = 0; i < n; ++i) b->hParams[i].capacity = capR;
    if (ensureQueues(b, capR) != cudaSuccess) return contextFail(ctx, XGB_OOM, "xgb_render_batch: cannot allocate queues");
    Ctrl init;
    std::memset(&init, 0, sizeof(init));
    init.totalPaths = total;
    *b->ctrlHost = init;
    cudaError_t e = cudaMemcpyAsync(b->dScenes, b->hScenes, sizeof(SceneDev) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->dParams, b->hParams, sizeof(RenderParams) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->dStart, b->hStart, sizeof(unsigned long long) * (n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->ctrl, b->ctrlHost, sizeof(Ctrl), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return contextFail(ctx, XGB_CUDA_ERROR, std::string("xgb_render_batch: ") + cudaGetErrorString(e));
    const int layout = single ? kBatchSingle : flat ? kBatchFlat : 0;
    const BatchView v{b->dScenes, b->dParams, b->dStart, n, layout, nested};
    const int kernels = layout | (nested << 2);  // which kernels a captured graph holds
    const int iters = std::max(2, (o.iterations_per_sync + 1) & ~1);
    const auto t0 = std::chrono::steady_clock::now();
    uint64_t launches = 0;
    for (int block = 0;; ++block) {
        const bool replay = o.use_graph && block > 0;  // the first block runs direct (and primes the occupancy cache)
        if (replay && !(b->graph && b->graphCap == capR && b->graphIters == iters && b->graphJobs == n &&
                        b->graphFlat == kernels)) {
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            cudaGraph_t g = nullptr;
            e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                enqueueBlock(b, v, capR, iters, numSMs, st);
                e = cudaStreamEndCapture(st, &g);
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->graph = nullptr;
                return contextFail(ctx, XGB_CUDA_ERROR, std::string("xgb_render_batch: graph capture: ") + cudaGetErrorString(e));
            }
            b->graphCap = capR; b->graphIters = iters; b->graphJobs = n; b->graphFlat = kernels;
        }
        if (replay) e = cudaGraphLaunch(b->graph, st);
        else { enqueueBlock(b, v, capR, iters, numSMs, st); e = cudaGetLastError(); }
        launches += 5 * (uint64_t)iters;
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->ctrlHost, b->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return contextFail(ctx, XGB_CUDA_ERROR, std::string("xgb_render_batch: ") + cudaGetErrorString(e));
        const Ctrl& c = *b->ctrlHost;
        if (c.errors & ERR_STACK) return contextFail(ctx, XGB_QUEUE_OVERFLOW, "xgb_render_batch: traversal stack overflow");
        if (c.errors & ERR_LOOP) return contextFail(ctx, XGB_DEVICE_TIMEOUT, "xgb_render_batch: traversal iteration bound exceeded");
        if (c.nextPath >= c.totalPaths && c.nOut == 0) break;
        if (block > (1 << 22)) return contextFail(ctx, XGB_DEVICE_TIMEOUT, "xgb_render_batch: wavefront did not drain");
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const Ctrl& c = *b->ctrlHost;
    b->last = xgb_render_stats{};
    b->last.paths = c.pathsDone;
    b->last.extension_rays = c.extensionRays;
    b->last.shadow_rays = c.shadowRays;
    b->last.iterations = c.iterations;
    b->last.kernel_launches = launches;
    b->last.error_flags = c.errors;
    return XGB_OK;
}

xgb_status checkJobs(const xgb_batch_job* jobs, int n, xgb_ctx** ctxOut, int* device, int* numSMs, cudaStream_t* st) {
    if (!jobs || n <= 0) return XGB_INVALID_ARG;
    xgb_ctx* ctx = sceneContext(jobs[0].scene);
    if (!ctx) return XGB_INVALID_ARG;
    if (n > kMaxJobs) return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: at most 255 jobs");
    for (int i = 0; i < n; ++i) {
        const xgb_batch_job& j = jobs[i];
        if (!j.scene || !j.film || sceneContext(j.scene) != ctx)
            return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: every job needs a scene and a film of one context");
        SceneDev sd; int dev, sms, built; cudaStream_t cs;
        sceneView(j.scene, &sd, &dev, &sms, &cs, &built);
        if (!built) return contextFail(ctx, XGB_NOT_BUILT, "xgb_render_batch: call xgb_scene_build first");
        void* fd; int w, h, f64, fdev; cudaStream_t fcs;
        if (!filmPlane(j.film, &fd, &w, &h, &f64, &fdev, &fcs) || fdev != dev)
            return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: film of another device");
        if ((long long)w * h >= (1ll << 24))
            return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: films of at most 2^24 - 1 pixels");
        const xgb_integrator_params& P = j.params;
        if (P.integrator != XGB_INTEGRATOR_STANDARD && P.integrator != XGB_INTEGRATOR_NAIVE)
            return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: unknown integrator");
        if (P.rr_start < 1 || !(P.rr_prob > 0.0f && P.rr_prob <= 1.0f) || P.max_depth < 0 || P.max_depth > 60000 ||
            (P.max_depth == 0 && P.rr_prob >= 1.0f))
            return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: bad integrator parameters");
        *device = dev;
        *numSMs = sms;
        *st = cs;
    }
    *ctxOut = ctx;
    return XGB_OK;
}

}  // namespace

namespace xgb {
void batchRelease(xgb_ctx* ctx) {
    BatchState* b = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_states.find(ctx);
        if (it == g_states.end()) return;
        b = it->second;
        g_states.erase(it);
    }
    freeState(b);
}
}  // namespace xgb

extern "C" {

xgb_status xgb_batch_autotune(const xgb_batch_job* jobs, int n, void* stream, xgb_batch_options* out) {
    xgb_ctx* ctx = nullptr;
    int device = 0, numSMs = 1;
    cudaStream_t st = nullptr;
    xgb_status s = checkJobs(jobs, n, &ctx, &device, &numSMs, &st);
    if (s != XGB_OK) return s;
    if (!out) return contextFail(ctx, XGB_INVALID_ARG, "xgb_batch_autotune: out is NULL");
    cudaSetDevice(device);
    if (stream) st = (cudaStream_t)stream;
    BatchState* b = stateOf(ctx);
    if (ensureJobs(b, n) != cudaSuccess) return contextFail(ctx, XGB_OOM, "xgb_batch_autotune: out of memory");
    // trial jobs: one sample per pixel of every job, into scratch films
    std::vector<xgb_batch_job> trial(jobs, jobs + n);
    std::vector<xgb_film*> films(n, nullptr);
    xgb_status st2 = XGB_OK;
    for (int i = 0; i < n && st2 == XGB_OK; ++i) {
        void* fd; int w, h, f64, fdev; cudaStream_t fcs;
        filmPlane(jobs[i].film, &fd, &w, &h, &f64, &fdev, &fcs);
        st2 = xgb_film_create(ctx, w, h, 0, &films[i]);
        trial[i].film = films[i];
        trial[i].spp_count = 1;
    }
    xgb_batch_options best{1 << 20, 8, 1};
    double bestT = 1e30;
    if (st2 == XGB_OK) {
        const unsigned int caps[] = {1u << 18, 1u << 19, 1u << 20, 1u << 21, 1u << 22, 1u << 23};
        for (unsigned int cap : caps) {
            xgb_batch_options o{(int)cap, 8, 1};
            double t = 0;
            for (int rep = 0; rep < 2 && st2 == XGB_OK; ++rep) st2 = runBatch(ctx, b, trial.data(), n, o, st, device, numSMs, &t);
            if (st2 != XGB_OK) break;
            if (t < bestT) { bestT = t; best = o; }
        }
        const int itersList[] = {4, 16};
        for (int it : itersList) {
            if (st2 != XGB_OK) break;
            xgb_batch_options o{best.queue_capacity, it, 1};
            double t = 0;
            for (int rep = 0; rep < 2 && st2 == XGB_OK; ++rep) st2 = runBatch(ctx, b, trial.data(), n, o, st, device, numSMs, &t);
            if (st2 == XGB_OK && t < bestT) { bestT = t; best = o; }
        }
    }
    for (xgb_film* f : films) if (f) xgb_film_destroy(f);
    if (st2 != XGB_OK) return st2;
    b->tuned[shapeKey(jobs, n)] = best;
    *out = best;
    return XGB_OK;
}

xgb_status xgb_render_batch(const xgb_batch_job* jobs, int n, const xgb_batch_options* options, void* stream) {
    xgb_ctx* ctx = nullptr;
    int device = 0, numSMs = 1;
    cudaStream_t st = nullptr;
    xgb_status s = checkJobs(jobs, n, &ctx, &device, &numSMs, &st);
    if (s != XGB_OK) return s;
    cudaSetDevice(device);
    if (stream) st = (cudaStream_t)stream;
    BatchState* b = stateOf(ctx);
    if (ensureJobs(b, n) != cudaSuccess) return contextFail(ctx, XGB_OOM, "xgb_render_batch: out of memory");
    xgb_batch_options o = options ? *options : xgb_batch_options{0, 0, 1};
    if (o.queue_capacity < 0 || o.iterations_per_sync < 0)
        return contextFail(ctx, XGB_INVALID_ARG, "xgb_render_batch: negative option");
    if (o.queue_capacity == 0 || o.iterations_per_sync == 0) {
        auto it = b->tuned.find(shapeKey(jobs, n));
        xgb_batch_options t{};
        if (it != b->tuned.end()) t = it->second;
        else if ((s = xgb_batch_autotune(jobs, n, stream, &t)) != XGB_OK) return s;
        if (o.queue_capacity == 0) o.queue_capacity = t.queue_capacity;
        if (o.iterations_per_sync == 0) o.iterations_per_sync = t.iterations_per_sync;
    }
    return runBatch(ctx, b, jobs, n, o, st, device, numSMs, nullptr);
}

xgb_status xgb_batch_stats_get(xgb_ctx* ctx, xgb_render_stats* out) {
    if (!ctx || !out) return XGB_INVALID_ARG;
    *out = stateOf(ctx)->last;
    return XGB_OK;
}

}  // extern "C"
