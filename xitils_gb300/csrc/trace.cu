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

// ---- single-mesh scenes ------------------------------------------------------
// When the scene is one instance, traversal runs as a persistent per-lane state
// machine in the style of Aila & Laine ("Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009): a lane whose ray is finished fetches the next
// one at once (one atomicAdd per group of lanes), inner nodes and leaves are
// processed in separate inner loops, and the first leaf a lane reaches is
// postponed until every lane of the warp holds one, so that the warp tests
// triangles together. Results are identical to traceScene: the same slab and
// watertight tests, the same closest-hit acceptance.
constexpr int kSentinel = 0x7FFFFFFF;

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_trace_single(SceneDev sc, RenderParams rp, PathQueue q, HitQueue h,
                                                              ShadowQueue s, PathQueue out, Ctrl* ctrl) {
    const unsigned int n = ANY ? ctrl->nShadow : ctrl->nActive;
    unsigned int* head = ANY ? &ctrl->shadowHead : &ctrl->extendHead;
    const Instance& in = sc.instances[0];
    const MeshDev m = sc.meshes[in.mesh];
    const bool identity = in.identity != 0;
    const int lane = threadIdx.x & 31;
    const unsigned int ltMask = (1u << lane) - 1u;
    int stack[kStackDepth];
    int sp = 0;
    int nodeAddr = kSentinel, leafAddr = 0;
    unsigned int ray = 0;
    WRay r;
    float tMax = 0.0f;
    TraceHit hit;
    hit.prim = -1;
    hit.t = 0.0f;
    hit.b0 = hit.b1 = 0.0f;
    bool occluded = false;
    WorkCount wc;
    for (int guard = 0;; ++guard) {
        if (nodeAddr == kSentinel) {
            // lanes without a ray fetch the next ones together
            const unsigned int act = __activemask();
            const int leader = __ffs(act) - 1;
            unsigned int base = 0;
            if (lane == leader) base = atomicAdd(head, (unsigned int)__popc(act));
            base = __shfl_sync(act, base, leader);
            ray = base + __popc(act & ltMask);
            if (ray >= n) break;
            float4 o4, d4;
            if (ANY) { o4 = s.o[ray]; d4 = s.d[ray]; tMax = o4.w; }
            else { o4 = q.o[ray]; d4 = q.d[ray]; tMax = __int_as_float(0x7f800000); }
            V3 o(o4.x, o4.y, o4.z), d(d4.x, d4.y, d4.z);
            if (!identity) {
                o = xformPointRn(in.matInv, o);
                d = xformVectorRn(in.matInv, d);
            }
            r = makeWRay(o, d);
            hit.prim = -1;
            hit.t = tMax;
            occluded = false;
            sp = 0;
            guard = 0;
            if (m.rootIsLeaf) { leafAddr = m.rootLeaf; nodeAddr = kSentinel; }
            else { leafAddr = 0; nodeAddr = 0; }
        }
        if (guard > kMaxVisits) { atomicOr(&ctrl->errors, 4u); nodeAddr = kSentinel; leafAddr = 0; }
        bool searching = true;
        while ((unsigned int)nodeAddr < (unsigned int)kSentinel) {
            if (COUNT) wc.nodes++;
            const Node2* nd = m.nodes + nodeAddr;
            float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
            int4 dd = __ldg(&nd->d);
            float t0, t1;
            bool h0 = slab(r, a.x, a.y, a.z, a.w, b.x, b.y, tMax, t0);
            bool h1 = slab(r, b.z, b.w, c.x, c.y, c.z, c.w, tMax, t1);
            if (h0 && h1) {
                int near = dd.x, far = dd.y;
                if (t1 < t0) { near = dd.y; far = dd.x; }
                if (sp >= kStackDepth) { atomicOr(&ctrl->errors, 1u); sp = 0; nodeAddr = kSentinel; break; }
                stack[sp++] = far;
                nodeAddr = near;
            } else if (h0) {
                nodeAddr = dd.x;
            } else if (h1) {
                nodeAddr = dd.y;
            } else {
                nodeAddr = sp > 0 ? stack[--sp] : kSentinel;
            }
            if (nodeAddr < 0 && leafAddr >= 0) {  // first leaf: postpone it, keep descending
                searching = false;
                leafAddr = nodeAddr;
                nodeAddr = sp > 0 ? stack[--sp] : kSentinel;
            }
            if (!__any_sync(__activemask(), searching)) break;
        }
        while (leafAddr < 0) {
            int first = leafFirst(leafAddr), cnt = leafCount(leafAddr);
            if (COUNT) wc.tris += cnt;
            for (int k = 0; k < cnt; ++k) {
                const TriV* tv = m.tris + first + k;
                float4 p0 = __ldg(&tv->p0), p1 = __ldg(&tv->p1), p2 = __ldg(&tv->p2);
                float t, b0, b1;
                if (watertight(r, p0, p1, p2, tMax, t, b0, b1)) {
                    tMax = t;
                    if (ANY) { occluded = true; break; }
                    hit.t = t; hit.b0 = b0; hit.b1 = b1;
                    hit.prim = __float_as_int(p0.w);
                }
            }
            if (ANY && occluded) { leafAddr = 0; nodeAddr = kSentinel; break; }
            leafAddr = nodeAddr;  // another leaf was postponed: take it next
            if (nodeAddr < 0) nodeAddr = sp > 0 ? stack[--sp] : kSentinel;
        }
        if (nodeAddr == kSentinel && leafAddr >= 0) {  // ray finished
            if (ANY) {
                if (!occluded) {
                    float4 cc = s.c[ray];
                    filmAdd(rp, __float_as_int(s.d[ray].w), V3(cc.x, cc.y, cc.z));
                    int target = __float_as_int(cc.w);
                    if (target >= 0) out.rng[target] = s.rng[ray];
                }
            } else {
                h.h[ray] = make_float4(hit.prim >= 0 ? hit.t : tMax, hit.b0, hit.b1, __int_as_float(hit.prim));
                h.inst[ray] = hit.prim >= 0 ? 0 : -1;
            }
        }
    }
    if (COUNT) {
        unsigned long long nv = wc.nodes, nt = wc.tris;
        for (int off = 16; off > 0; off >>= 1) {
            nv += __shfl_down_sync(__activemask(), nv, off);
            nt += __shfl_down_sync(__activemask(), nt, off);
        }
        if (lane == 0) {
            atomicAdd(&ctrl->nodeVisits, nv);
            atomicAdd(&ctrl->triTests, nt);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(ANY ? &ctrl->shadowRays : &ctrl->extensionRays, (unsigned long long)n);
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
    RenderParams none{};
    if (sc.nInstances == 1) {
        if (count) k_trace_single<false, true><<<grid, kTraceBlock, 0, s>>>(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        else k_trace_single<false, false><<<grid, kTraceBlock, 0, s>>>(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        return;
    }
    if (count) k_extend<true><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
    else k_extend<false><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
}
void launchShadow(const SceneDev& sc, const RenderParams& rp, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int grid,
                  cudaStream_t s) {
    if (sc.nInstances == 1) {
        k_trace_single<true, false><<<grid, kTraceBlock, 0, s>>>(sc, rp, PathQueue{}, HitQueue{}, sq, out, ctrl);
        return;
    }
    k_shadow<<<grid, kTraceBlock, 0, s>>>(sc, rp, sq, out, ctrl);
}

}  // namespace xgb
