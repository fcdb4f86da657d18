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

// Guide training: a visible light's contribution also goes to its path's accumulator.
__device__ __forceinline__ void creditPath(const RenderParams& rp, unsigned int pid, float4 c) {
    float4 a = rp.pathAcc[pid];
    rp.pathAcc[pid] = make_float4(a.x + c.x, a.y + c.y, a.z + c.z, a.w);
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
                if (rp.train) creditPath(rp, s.pid[i], c);
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctrl->shadowRays, (unsigned long long)n);
}

// ---- scenes of a few instances ------------------------------------------------
// With at most kFlatInstances instances the top level is a short list: a lane
// walks the instances in order (those whose world box the ray still reaches
// within tMax) and traverses each mesh BVH as a persistent per-lane state machine
// in the style of Aila & Laine ("Understanding the Efficiency of Ray Traversal
// on GPUs", HPG 2009): a lane whose ray is finished fetches the next one at once
// (one atomicAdd per group of lanes), inner nodes and leaves are processed in
// separate inner loops, and the first leaf a lane reaches is postponed until
// every lane of the warp holds one, so that the warp tests triangles together.
// Results are those of traceScene: the same slab and watertight tests and the
// same closest-hit acceptance (tMax shrinks across instances).
constexpr int kSentinel = 0x7FFFFFFF;
constexpr int kFlatInstances = 16;

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_trace_flat(SceneDev sc, RenderParams rp, PathQueue q, HitQueue h,
                                                            ShadowQueue s, PathQueue out, Ctrl* ctrl) {
    const unsigned int n = ANY ? ctrl->nShadow : ctrl->nActive;
    unsigned int* head = ANY ? &ctrl->shadowHead : &ctrl->extendHead;
    const int nInst = sc.nInstances;
    const int lane = threadIdx.x & 31;
    const unsigned int ltMask = (1u << lane) - 1u;
    int stack[kStackDepth];
    int sp = 0;
    int nodeAddr = kSentinel, leafAddr = 0;
    int inst = nInst;  // instance being traversed; nInst = ray finished
    unsigned int ray = 0;
    V3 wo(0.f, 0.f, 0.f), wd(0.f, 0.f, 1.f);
    WRay r;
    const Node2* nodes = nullptr;
    const TriV* tris = nullptr;
    float tMax = 0.0f;
    TraceHit hit;
    hit.prim = -1;
    hit.inst = -1;
    hit.t = 0.0f;
    hit.b0 = hit.b1 = 0.0f;
    bool occluded = false;
    bool fetch = true;
    WorkCount wc;
    for (int guard = 0;; ++guard) {
        if (fetch) {
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
            wo = V3(o4.x, o4.y, o4.z);
            wd = V3(d4.x, d4.y, d4.z);
            hit.prim = -1;
            hit.inst = -1;
            hit.t = tMax;
            occluded = false;
            guard = 0;
            inst = -1;
            nodeAddr = kSentinel;
            leafAddr = 0;
            fetch = false;
        }
        if (nodeAddr == kSentinel && leafAddr >= 0) {
            // next instance whose world box the ray still reaches
            WRay wr = makeWRay(wo, wd);
            for (++inst; inst < nInst; ++inst) {
                float4 lo = __ldg(&sc.instBox[2 * inst]), hi = __ldg(&sc.instBox[2 * inst + 1]);
                float tn;
                if (slab(wr, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, tMax, tn)) break;
            }
            if (ANY && occluded) inst = nInst;
            if (inst >= nInst) {  // ray finished
                if (ANY) {
                    if (!occluded) {
                        float4 cc = s.c[ray];
                        filmAdd(rp, __float_as_int(s.d[ray].w), V3(cc.x, cc.y, cc.z));
                        int target = __float_as_int(cc.w);
                        if (target >= 0) out.rng[target] = s.rng[ray];
                        if (rp.train) creditPath(rp, s.pid[ray], cc);
                    }
                } else {
                    h.h[ray] = make_float4(hit.prim >= 0 ? hit.t : tMax, hit.b0, hit.b1, __int_as_float(hit.prim));
                    h.inst[ray] = hit.inst;
                }
                fetch = true;
                continue;
            }
            const Instance& in = sc.instances[inst];
            const MeshDev& m = sc.meshes[in.mesh];
            nodes = m.nodes;
            tris = m.tris;
            if (in.identity) r = wr;
            else r = makeWRay(xformPointRn(in.matInv, wo), xformVectorRn(in.matInv, wd));
            sp = 0;
            if (m.rootIsLeaf) { leafAddr = m.rootLeaf; nodeAddr = kSentinel; }
            else { leafAddr = 0; nodeAddr = 0; }
        }
        if (guard > kMaxVisits) { atomicOr(&ctrl->errors, 4u); nodeAddr = kSentinel; leafAddr = 0; inst = nInst; }
        bool searching = true;
        while ((unsigned int)nodeAddr < (unsigned int)kSentinel) {
            if (COUNT) wc.nodes++;
            const Node2* nd = nodes + nodeAddr;
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
                const TriV* tv = tris + first + k;
                float4 p0 = __ldg(&tv->p0), p1 = __ldg(&tv->p1), p2 = __ldg(&tv->p2);
                float t, b0, b1;
                if (watertight(r, p0, p1, p2, tMax, t, b0, b1)) {
                    tMax = t;
                    if (ANY) { occluded = true; break; }
                    hit.t = t; hit.b0 = b0; hit.b1 = b1;
                    hit.prim = __float_as_int(p0.w);
                    hit.inst = inst;
                }
            }
            if (ANY && occluded) { leafAddr = 0; nodeAddr = kSentinel; sp = 0; break; }
            leafAddr = nodeAddr;  // another leaf was postponed: take it next
            if (nodeAddr < 0) nodeAddr = sp > 0 ? stack[--sp] : kSentinel;
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

// ---- ray queries (xgb_scene_intersect / xgb_scene_occluded) -------------------
__global__ void __launch_bounds__(kTraceBlock) k_query(SceneDev sc, const float4* o, const float4* d, int n, int any,
                                                       float4* hits, int* occluded, unsigned int* errors) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 oo = o[i], dd = d[i];
        TraceHit hit;
        WorkCount wc;
        if (any) {
            occluded[i] = traceScene<true>(sc, V3(oo.x, oo.y, oo.z), V3(dd.x, dd.y, dd.z), oo.w, hit, errors, wc) ? 1 : 0;
        } else {
            traceScene<false>(sc, V3(oo.x, oo.y, oo.z), V3(dd.x, dd.y, dd.z), oo.w, hit, errors, wc);
            hits[2 * i] = make_float4(hit.t, __int_as_float(hit.inst), __int_as_float(hit.prim), 0.0f);
            hits[2 * i + 1] = make_float4(hit.b0, hit.b1, 0.0f, 0.0f);
        }
    }
}

void launchQuery(const SceneDev& sc, const float4* o, const float4* d, int n, int any, float4* hits, int* occluded,
                 unsigned int* errors, int grid, cudaStream_t s) {
    k_query<<<grid, kTraceBlock, 0, s>>>(sc, o, d, n, any, hits, occluded, errors);
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
    if (sc.nInstances <= kFlatInstances) {
        if (count) k_trace_flat<false, true><<<grid, kTraceBlock, 0, s>>>(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        else k_trace_flat<false, false><<<grid, kTraceBlock, 0, s>>>(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        return;
    }
    if (count) k_extend<true><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
    else k_extend<false><<<grid, kTraceBlock, 0, s>>>(sc, q, h, ctrl);
}
void launchShadow(const SceneDev& sc, const RenderParams& rp, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int grid,
                  cudaStream_t s) {
    if (sc.nInstances <= kFlatInstances) {
        k_trace_flat<true, false><<<grid, kTraceBlock, 0, s>>>(sc, rp, PathQueue{}, HitQueue{}, sq, out, ctrl);
        return;
    }
    k_shadow<<<grid, kTraceBlock, 0, s>>>(sc, rp, sq, out, ctrl);
}

}  // namespace xgb
