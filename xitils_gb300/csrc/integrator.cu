// Wavefront integrator: plan -> generate -> (extend, trace.cu) -> shade ->
// (shadow, trace.cu), repeated until every camera path has finished.
//
// One iteration advances every path in flight by one vertex of
// StandardPathTracer::eval (PathTracer.h:117-251) or NaivePathTracer::eval
// (PathTracer.h:50-104). Paths are carried between iterations in a compacted
// queue (warp ballot + one atomicAdd per warp); freed slots are refilled with
// new camera paths, so the queue stays full until the work runs out.
//
// Per-path random numbers come from a PCG32 stream keyed by (pixel, sample),
// drawn in the reference's order: film jitter x, y; then per vertex the
// Russian-roulette draw, the BSDF sample, the light sample (object, triangle,
// barycentrics) and, only when the light is visible, a stochastic bsdfCos.
// This translation unit is compiled with -fmad=false.
#include "shade.cuh"

namespace xgb {

__global__ void k_plan(Ctrl* c, unsigned int capacity) {
    unsigned int nCont = c->nOut;
    unsigned long long remain = c->totalPaths - c->nextPath;
    unsigned long long room = capacity - nCont;
    unsigned int nNew = (unsigned int)(remain < room ? remain : room);
    c->firstNew = c->nextPath;
    c->nextPath += nNew;
    c->nCont = nCont;
    c->nActive = nCont + nNew;
    c->nOut = 0;
    c->nShadow = 0;
    c->extendHead = 0;
    c->shadowHead = 0;
    if (c->nActive) c->iterations += 1;
}

// Camera paths: RenderTargetTile::GenerateFilmPosition (RenderTarget.h:68-80)
// then PinholeCamera::generateRay (Camera.h:45-55).
// Pixel of the i-th camera path of a sample pass when paths are ordered in
// tw x th pixel blocks: rows in bands of th, a band's pixels block by block
// (row-major inside a block, the last block of a band as wide as what is left),
// so that a warp's 32 paths start from a compact patch of the film. Bijective on
// [0, W H) for any W, H; the per-pixel random streams make the image
// independent of the order.
__device__ __forceinline__ unsigned int tiledPixel(unsigned int i, unsigned int W, unsigned int H, unsigned int tw,
                                                   unsigned int th) {
    const unsigned int band = i / (W * th);
    const unsigned int y0 = band * th;
    const unsigned int hb = min(th, H - y0);
    const unsigned int j = i - band * W * th;
    const unsigned int blockSize = tw * hb;
    const unsigned int full = W / tw;
    unsigned int x, y;
    if (j < full * blockSize) {
        const unsigned int b = j / blockSize, k = j - b * blockSize;
        x = b * tw + k % tw;
        y = y0 + k / tw;
    } else {
        const unsigned int rem = W - full * tw;
        const unsigned int k = j - full * blockSize;
        x = full * tw + k % rem;
        y = y0 + k / rem;
    }
    return x + y * W;
}

// Sample and pixel index of the call's local-th camera path when groups of G
// consecutive paths are G samples of one pixel: passes of G samples over the
// film, then (when G does not divide the call's sample count) the remaining
// samples one pass after the other. Bijective on [0, px spp).
__device__ __forceinline__ void groupedSample(unsigned long long local, unsigned int px, unsigned int spp,
                                              unsigned int G, unsigned int& sample, unsigned int& pix) {
    const unsigned int full = (spp / G) * G;
    const unsigned long long grouped = (unsigned long long)full * px;
    if (local < grouped) {
        const unsigned long long pass = (unsigned long long)px * G;  // may exceed 2^32
        const unsigned int grp = (unsigned int)(local / pass);
        const unsigned long long r = local - (unsigned long long)grp * pass;
        pix = (unsigned int)(r / G);
        sample = grp * G + (unsigned int)(r % G);
    } else {
        const unsigned long long t = local - grouped;
        sample = full + (unsigned int)(t / px);
        pix = (unsigned int)(t % px);
    }
}

template <class J>
__global__ void __launch_bounds__(kShadeBlock) k_generate(J jobs, PathQueue q, const Ctrl* ctrl) {
    const unsigned int nCont = ctrl->nCont, nActive = ctrl->nActive;
    const unsigned long long firstNew = ctrl->firstNew;
    for (unsigned int s = nCont + blockIdx.x * blockDim.x + threadIdx.x; s < nActive; s += gridDim.x * blockDim.x) {
        const unsigned long long g = firstNew + (s - nCont);
        unsigned long long local;
        const int job = jobs.locate(g, local);
        const SceneDev& sc = jobs.scene(job);
        const RenderParams& rp = jobs.params(job);
        const unsigned int px = (unsigned int)rp.width * (unsigned int)rp.height;
        unsigned int sample, pix;
        if (rp.sampleGroup > 1 && rp.sppCount > 1) {
            groupedSample(local, px, rp.sppCount, min((unsigned int)rp.sampleGroup, rp.sppCount), sample, pix);
            sample += rp.sppBegin;
        } else {
            sample = rp.sppBegin + (unsigned int)(local / px);
            pix = (unsigned int)(local % px);
        }
        if (rp.tileW > 0) pix = tiledPixel(pix, (unsigned int)rp.width, (unsigned int)rp.height, (unsigned int)rp.tileW,
                                           (unsigned int)rp.tileH);
        int x = (int)(pix % (unsigned int)rp.width), y = (int)(pix / (unsigned int)rp.width);
        Pcg rng;
        rng.seed(pix, sample, rp.seed);
        float fx = (float)x / (float)rp.width;
        float fy = (float)y / (float)rp.height;
        fy = 1.0f - fy;
        fx = fx + (rng.randf() - 0.5f) / (float)rp.width;
        fy = fy + (rng.randf() - 0.5f) / (float)rp.height;
        V3 d = normalize(V3(sc.tanHalfX * (fx - 0.5f) * 2.0f, sc.tanHalfY * (fy - 0.5f) * 2.0f, 1.0f));
        V3 o = xformPoint(sc.c2w, V3(0.0f, 0.0f, 0.0f));
        d = xformVector(sc.c2w, d);
        // Standard: the first loop vertex has pathLength 2; Naive counts from 1.
        int len = rp.integrator == 0 ? 2 : 1;
        // streaming stores: the queue is read once, by the next traversal
        __stcs(&q.o[s], make_float4(o.x, o.y, o.z, 0.0f));
        __stcs(&q.d[s], make_float4(d.x, d.y, d.z, __int_as_float(len | (FLAG_PRIMARY << 16))));
        __stcs(&q.thr[s], make_float4(1.0f, 1.0f, 1.0f, __int_as_float(jobs.encode(job, (int)pix))));
        __stcs(&q.rng[s], make_uint2((unsigned int)rng.state, (unsigned int)(rng.state >> 32)));
        if (rp.train) {
            q.grec[s] = -1;
            q.pid[s] = (unsigned int)g;
            rp.pathAcc[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

void launchPlan(Ctrl* ctrl, unsigned int capacity, cudaStream_t s) { k_plan<<<1, 1, 0, s>>>(ctrl, capacity); }

void launchGenerate(const SceneDev& sc, const RenderParams& rp, PathQueue q, Ctrl* ctrl, int grid, cudaStream_t s) {
    k_generate<OneJob><<<grid, kShadeBlock, 0, s>>>(OneJob{sc, rp}, q, ctrl);
}

void launchShade(const SceneDev& sc, const RenderParams& rp, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq,
                 Ctrl* ctrl, int numSMs, cudaStream_t s) {
    const OneJob job{sc, rp};
    switch (sc.nested & 3) {
    case 1: launchShadeMask1(job, in, h, out, sq, ctrl, numSMs, s); break;
    case 2: launchShadeMask2(job, in, h, out, sq, ctrl, numSMs, s); break;
    case 3: launchShadeMask3(job, in, h, out, sq, ctrl, numSMs, s); break;
    default: {
        // plain renders (standard integrator) of scenes whose non-emissive materials are all
        // Lambert or all GGX metal take a variant with only that material's code
        const int basic = sc.kinds & ~(1 << MAT_EMISSION);
        const bool emitters = (sc.kinds & (1 << MAT_EMISSION)) != 0 || sc.nLights > 0;
        if (rp.guided || rp.train || rp.aov) launchShadeVariant<OneJob, 0, true>(job, in, h, out, sq, ctrl, numSMs, s);
        else if (rp.integrator != 0) launchShadeVariant<OneJob, 0, false>(job, in, h, out, sq, ctrl, numSMs, s);
        else if (basic == (1 << MAT_METAL) && !emitters)
            launchShadeVariant<OneJob, kOnlyMetal | kNoEmitters, false>(job, in, h, out, sq, ctrl, numSMs, s);
        else if (basic == (1 << MAT_METAL)) launchShadeVariant<OneJob, kOnlyMetal, false>(job, in, h, out, sq, ctrl, numSMs, s);
        else if (basic == (1 << MAT_DIFFUSE))
            launchShadeVariant<OneJob, kOnlyDiffuse, false>(job, in, h, out, sq, ctrl, numSMs, s);
        else launchShadeVariant<OneJob, 0, false>(job, in, h, out, sq, ctrl, numSMs, s);
        break;
    }
    }
}

void launchGenerateBatch(const BatchView& b, PathQueue q, Ctrl* ctrl, int grid, cudaStream_t s) {
    k_generate<ManyJobs><<<grid, kShadeBlock, 0, s>>>(ManyJobs{b.scenes, b.params, b.start, b.nJobs}, q, ctrl);
}

void launchShadeBatch(const BatchView& b, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl,
                      int numSMs, cudaStream_t s) {
    const ManyJobs jobs{b.scenes, b.params, b.start, b.nJobs};
    if (b.nested) launchShadeMask3Batch(jobs, in, h, out, sq, ctrl, numSMs, s);
    else launchShadeVariant<ManyJobs, 0, false>(jobs, in, h, out, sq, ctrl, numSMs, s);
}

}  // namespace xgb
