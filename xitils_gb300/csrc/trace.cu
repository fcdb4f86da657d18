// Extension (closest-hit) and shadow (any-hit) kernels of the wavefront.
//
// Both are persistent: a grid of (SMs x resident blocks) threads where each
// warp claims 32 queue entries at a time with one atomicAdd, so the grid drains
// queues of any length without a relaunch per batch.
#include "trace.cuh"
#include "xgb_kernels.h"

namespace xgb {

__device__ __forceinline__ void filmAdd(const RenderParams& rp, int pix, V3 c) {
    if (rp.filmFp64) {
        double* f = (double*)rp.film + 4 * (size_t)pix;
        atomicAdd(f, (double)c.x);
        atomicAdd(f + 1, (double)c.y);
        atomicAdd(f + 2, (double)c.z);
    } else {
        float4* f = (float4*)rp.film + pix;
        atomicAdd(f, make_float4(c.x, c.y, c.z, 0.0f));
    }
}

constexpr int kTraceBlock = 128;

template <bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_extend(SceneDev sc, PathQueue q, HitQueue h, Ctrl* ctrl) {
    const unsigned int n = ctrl->nActive;
    const int lane = threadIdx.x & 31;
    WorkCount wc;
    for (;;) {
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&ctrl->extendHead, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        unsigned int i = base + lane;
        if (i < n) {
            float4 o = q.o[i], d = q.d[i];
            TraceHit hit;
            traceScene<false, COUNT>(sc, V3(o.x, o.y, o.z), V3(d.x, d.y, d.z), __int_as_float(0x7f800000), hit,
                                     &ctrl->errors, wc);
            h.h[i] = make_float4(hit.t, hit.b0, hit.b1, __int_as_float(hit.prim));
            h.inst[i] = hit.inst;
        }
    }
    if (COUNT) {
        unsigned long long nv = wc.nodes, nt = wc.tris;
        for (int off = 16; off > 0; off >>= 1) {
            nv += __shfl_down_sync(0xFFFFFFFFu, nv, off);
            nt += __shfl_down_sync(0xFFFFFFFFu, nt, off);
        }
        if (lane == 0) {
            atomicAdd(&ctrl->nodeVisits, nv);
            atomicAdd(&ctrl->triTests, nt);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctrl->extensionRays, (unsigned long long)n);
}

__global__ void __launch_bounds__(kTraceBlock) k_shadow(SceneDev sc, RenderParams rp, ShadowQueue s, PathQueue out,
                                                        Ctrl* ctrl) {
    const unsigned int n = ctrl->nShadow;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&ctrl->shadowHead, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        unsigned int i = base + lane;
        if (i < n) {
            float4 o = s.o[i], d = s.d[i];
            TraceHit hit;
            WorkCount wc;
            bool occluded = traceScene<true>(sc, V3(o.x, o.y, o.z), V3(d.x, d.y, d.z), o.w, hit, &ctrl->errors, wc);
            if (!occluded) {
                float4 c = s.c[i];
                filmAdd(rp, __float_as_int(d.w), V3(c.x, c.y, c.z));
                int target = __float_as_int(c.w);
                // A stochastic bsdfCos (MicrofacetNormalMapping) drew from the path's
                // stream only because the light was visible (PathTracer.h:209-227):
                // commit the stream position it left.
                if (target >= 0) out.rng[target] = s.rng[i];
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctrl->shadowRays, (unsigned long long)n);
}

static int g_extendBlocks = 0, g_shadowBlocks = 0;

int extendBlocksPerSM() {
    if (!g_extendBlocks) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_extendBlocks, k_extend<false>, kTraceBlock, 0);
    return g_extendBlocks > 0 ? g_extendBlocks : 1;
}
int shadowBlocksPerSM() {
    if (!g_shadowBlocks) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_shadowBlocks, k_shadow, kTraceBlock, 0);
    return g_shadowBlocks > 0 ? g_shadowBlocks : 1;
}

void launchExtend(const SceneDev& sc, PathQueue q, HitQueue h, Ctrl* ctrl, int grid, bool count, cudaStream_t s) {
    if (count) k_extend<true><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
    else k_extend<false><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
}
void launchShadow(const SceneDev& sc, const RenderParams& rp, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int grid,
                  cudaStream_t s) {
    k_shadow<<<grid, kTraceBlock, 0, s>>>(sc, rp, sq, out, ctrl);
}

}  // namespace xgb
