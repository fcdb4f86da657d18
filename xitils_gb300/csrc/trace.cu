// Extension (closest-hit) and shadow (any-hit) kernels of the wavefront.
//
// Both are persistent: a grid of (SMs x resident blocks) threads where each
// warp claims 32 queue entries at a time with one atomicAdd, so the grid drains
// queues of any length without a relaunch per batch.
#include <map>
#include <mutex>

#include "trace.cuh"
#include "xgb_kernels.h"

#include <type_traits>

namespace xgb {

__device__ __forceinline__ void filmAdd(const RenderParams& rp, int pix, V3 c) {
    if (rp.dropNonFinite && !(isfinite(c.x) && isfinite(c.y) && isfinite(c.z))) return;
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

// World-space ray for the instance-box tests of the flat kernels: origin and
// 1/d only (no watertight constants), computed once per ray.
struct BoxRay {
    float ox, oy, oz, ix, iy, iz;
};
__device__ __forceinline__ bool instBoxHit(const BoxRay& b, const float4* boxes, int inst, float tMax) {
    const float4 lo = __ldg(&boxes[2 * inst]), hi = __ldg(&boxes[2 * inst + 1]);
    float tx0 = (lo.x - b.ox) * b.ix, tx1 = (hi.x - b.ox) * b.ix;
    float ty0 = (lo.y - b.oy) * b.iy, ty1 = (hi.y - b.oy) * b.iy;
    float tz0 = (lo.z - b.oz) * b.iz, tz1 = (hi.z - b.oz) * b.iz;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tMax));
    return tn <= tf * 1.00000095367431640625f;
}

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

// Scene lookup of the flat kernels: one scene (the kernel argument) or one per
// job of a batch (the job in the high byte of the ray's pixel field).
struct OneScene {
    SceneDev sc;
    RenderParams rp;
    __device__ __forceinline__ int jobOf(unsigned int) const { return 0; }
    __device__ __forceinline__ int pixelOf(unsigned int packed) const { return (int)packed; }
    __device__ __forceinline__ const SceneDev& scene(int) const { return sc; }
    __device__ __forceinline__ const RenderParams& params(int) const { return rp; }
};
struct BatchScenes {
    BatchView b;
    __device__ __forceinline__ int jobOf(unsigned int packed) const { return (int)(packed >> 24); }
    __device__ __forceinline__ int pixelOf(unsigned int packed) const { return (int)(packed & 0xFFFFFFu); }
    __device__ __forceinline__ const SceneDev& scene(int j) const { return b.scenes[j]; }
    __device__ __forceinline__ const RenderParams& params(int j) const { return b.params[j]; }
};

// ---- scenes of a few instances: 8-wide mesh BVHs ------------------------------
// With at most kFlatInstances instances the top level is a short list: a lane
// walks the instances in order (those whose world box the ray still reaches
// within tMax) and traverses each mesh's 8-wide BVH as a persistent per-lane
// state machine in the style of Aila & Laine ("Understanding the Efficiency of
// Ray Traversal on GPUs", HPG 2009): the lanes of a warp test nodes together
// until each holds a leaf child (postponing it) or has no nodes left, then test
// their leaves' triangles together; a lane whose ray is finished fetches the
// next one at once (one atomicAdd per group of lanes), so the warp never waits
// for its slowest ray. Results are those of traceScene: the same watertight
// tests and the same closest-hit acceptance (tMax shrinks across instances).
constexpr int kFlatInstances = 16;

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_trace_wide(SceneDev sc, RenderParams rp, PathQueue q, HitQueue h,
                                                            ShadowQueue s, PathQueue out, Ctrl* ctrl) {
    const unsigned int n = ANY ? ctrl->nShadow : ctrl->nActive;
    unsigned int* head = ANY ? &ctrl->shadowHead : &ctrl->extendHead;
    const int nInst = sc.nInstances;
    const int lane = threadIdx.x & 31;
    const unsigned int ltMask = (1u << lane) - 1u;
    unsigned int stack[kWideStack];
    int sp = 0;
    int inst = nInst;  // instance being traversed
    unsigned int ray = 0;
    V3 wo(0.f, 0.f, 0.f), wd(0.f, 0.f, 1.f);
    BoxRay br{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    WRay r;
    int oct = 0;
    const WNode* nodes = nullptr;
    const TriV* tris = nullptr;
    WideHdr hd;
    hd.imask = 0; hd.childBase = 0; hd.triBase = 0; hd.meta0 = 0; hd.meta1 = 0;
    int node = 0;
    unsigned int mask = 0;
    bool inMesh = false;  // a mesh traversal is under way
    int leafFirst = 0, leafCnt = 0;  // postponed leaf child
    float tMax = 0.0f;
    TraceHit hit;
    hit.prim = -1;
    hit.inst = -1;
    hit.t = 0.0f;
    hit.b0 = hit.b1 = 0.0f;
    bool occluded = false;
    bool fetch = true;
    int steps = 0;  // traversal steps of the current ray
    WorkCount wc;
    for (;;) {
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
            // queue records: streaming loads / stores, as in k_shade
            if (ANY) { o4 = __ldcs(&s.o[ray]); d4 = __ldcs(&s.d[ray]); tMax = o4.w; }
            else { o4 = __ldcs(&q.o[ray]); d4 = __ldcs(&q.d[ray]); tMax = __int_as_float(0x7f800000); }
            wo = V3(o4.x, o4.y, o4.z);
            wd = V3(d4.x, d4.y, d4.z);
            br = BoxRay{wo.x, wo.y, wo.z, 1.0f / wd.x, 1.0f / wd.y, 1.0f / wd.z};
            hit.prim = -1;
            hit.inst = -1;
            hit.t = tMax;
            occluded = false;
            inst = -1;
            inMesh = false;
            leafCnt = 0;
            steps = 0;
            fetch = false;
        }
        if (!inMesh) {
            // next instance whose world box the ray still reaches, or the end of the ray
            if (!(ANY && occluded))
                for (++inst; inst < nInst; ++inst)
                    if (instBoxHit(br, sc.instBox, inst, tMax)) break;
            if ((ANY && occluded) || inst >= nInst) {
                if (ANY) {
                    if (!occluded) {
                        float4 cc = s.c[ray];
                        filmAdd(rp, __float_as_int(s.d[ray].w), V3(cc.x, cc.y, cc.z));
                        int target = __float_as_int(cc.w);
                        if (target >= 0) out.rng[target] = s.rng[ray];
                        if (rp.train) creditPath(rp, s.pid[ray], cc);
                    }
                } else {
                    __stcs(&h.h[ray], make_float4(hit.prim >= 0 ? hit.t : tMax, hit.b0, hit.b1, __int_as_float(hit.prim)));
                    __stcs(&h.inst[ray], hit.inst);
                }
                fetch = true;
            } else {
                const Instance& in = sc.instances[inst];
                const MeshDev& m = sc.meshes[in.mesh];
                nodes = m.nodes;
                tris = m.tris;
                if (in.identity) r = makeWRay(wo, wd);
                else r = makeWRay(xformPointRn(in.matInv, wo), xformVectorRn(in.matInv, wd));
                if (m.rootIsLeaf) {  // the whole mesh is one leaf: test it below, then the next instance
                    leafFirst = 0;
                    leafCnt = m.nTris;
                } else {
                    oct = rayOctant(r);
                    sp = 0;
                    node = 0;
                    mask = wideEval(nodes, r, oct, tMax, hd);
                    if (COUNT) wc.nodes++;
                    inMesh = true;
                }
            }
        }
        // node phase: the warp steps through nodes until every lane holds a leaf child or has none left
        for (;;) {
            const bool active = inMesh && leafCnt == 0;
            if (!__any_sync(__activemask(), active)) break;
            if (!active) continue;
            if (++steps > sc.maxSteps) {
                atomicOr(&ctrl->errors, 4u);
                inMesh = false;
                inst = nInst;
                continue;
            }
            if (mask == 0u) {
                if (sp == 0) {
                    inMesh = false;  // this mesh is done
                } else {
                    const unsigned int e = stack[--sp];
                    node = (int)(e >> 8);
                    mask = e & 0xFFu;
                    wideHeader(nodes + node, hd);
                }
                continue;
            }
            const int slot = (__ffs(mask) - 1) ^ oct;
            mask &= mask - 1u;
            const unsigned int mb = byteOf(slot >> 2 ? hd.meta1 : hd.meta0, slot);
            if ((hd.imask >> slot) & 1u) {
                if (mask) {
                    if (sp >= kWideStack || sp >= sc.stackLimit) {
                        atomicOr(&ctrl->errors, 1u);
                        inMesh = false;
                        inst = nInst;
                        continue;
                    }
                    stack[sp++] = ((unsigned int)node << 8) | mask;
                }
                node = hd.childBase + (int)mb;
                mask = wideEval(nodes + node, r, oct, tMax, hd);
                if (COUNT) wc.nodes++;
            } else {
                leafFirst = hd.triBase + (int)(mb & 31u);
                leafCnt = (int)(mb >> 5);
            }
        }
        // leaf phase: the postponed leaf children's triangles, together
        if (leafCnt) {
            if (COUNT) wc.tris += leafCnt;
            if (testTris<ANY>(tris, leafFirst, leafCnt, r, tMax, hit, inst) && ANY) {
                occluded = true;
                inMesh = false;
            }
            leafCnt = 0;
        }
    }
    if (COUNT) {
        __syncwarp();  // every lane of the warp has left the loop
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
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(ANY ? &ctrl->shadowRays : &ctrl->extensionRays, (unsigned long long)n);
}

// ---- scenes of a few instances: binary mesh BVHs ------------------------------------------------
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

// SHELL: the scene has shell-mapped meshes, whose accepted hits go through the
// discard test (shellDiscard, trace.cuh) before tMax shrinks.
template <bool ANY, bool COUNT, class S, bool SHELL = false>
__global__ void __launch_bounds__(kTraceBlock) k_trace_flat2(S scenes, PathQueue q, HitQueue h, ShadowQueue s,
                                                            PathQueue out, Ctrl* ctrl) {
    const unsigned int n = ANY ? ctrl->nShadow : ctrl->nActive;
    unsigned int* head = ANY ? &ctrl->shadowHead : &ctrl->extendHead;
    constexpr bool kBatch = !std::is_same<S, OneScene>::value;
    int rayMaxSteps = 0, rayStack = 0;  // a batch: the current ray's job's bounds
    int job = 0;
    int nInst = 0;
    const int lane = threadIdx.x & 31;
    const unsigned int ltMask = (1u << lane) - 1u;
    int stack[kStackDepth];
    int sp = 0;
    int nodeAddr = kSentinel, leafAddr = 0;
    int inst = nInst;  // instance being traversed; nInst = ray finished
    unsigned int ray = 0;
    V3 wo(0.f, 0.f, 0.f), wd(0.f, 0.f, 1.f);
    BoxRay br{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    WRay r;
    const Node2* nodes = nullptr;
    const TriV* tris = nullptr;
    const MeshDev* mesh = nullptr;
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
            if (ANY) { o4 = __ldcs(&s.o[ray]); d4 = __ldcs(&s.d[ray]); tMax = o4.w; }
            else { o4 = __ldcs(&q.o[ray]); d4 = __ldcs(&q.d[ray]); tMax = __int_as_float(0x7f800000); }
            wo = V3(o4.x, o4.y, o4.z);
            wd = V3(d4.x, d4.y, d4.z);
            br = BoxRay{wo.x, wo.y, wo.z, 1.0f / wd.x, 1.0f / wd.y, 1.0f / wd.z};
            job = scenes.jobOf(ANY ? __float_as_uint(d4.w) : __float_as_uint(q.thr[ray].w));
            nInst = scenes.scene(job).nInstances;
            if (kBatch) {  // the job's traversal bounds, read once per ray
                rayMaxSteps = scenes.scene(job).maxSteps;
                rayStack = min(kStackDepth, scenes.scene(job).stackLimit);
            }
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
            for (++inst; inst < nInst; ++inst)
                if (instBoxHit(br, scenes.scene(job).instBox, inst, tMax)) break;
            if (ANY && occluded) inst = nInst;
            if (inst >= nInst) {  // ray finished
                if (ANY) {
                    if (!occluded) {
                        float4 cc = s.c[ray];
                        const RenderParams& rp = scenes.params(job);
                        filmAdd(rp, scenes.pixelOf(__float_as_uint(s.d[ray].w)), V3(cc.x, cc.y, cc.z));
                        int target = __float_as_int(cc.w);
                        if (target >= 0) out.rng[target] = s.rng[ray];
                        if (rp.train) creditPath(rp, s.pid[ray], cc);
                    }
                } else {
                    __stcs(&h.h[ray], make_float4(hit.prim >= 0 ? hit.t : tMax, hit.b0, hit.b1, __int_as_float(hit.prim)));
                    __stcs(&h.inst[ray], hit.inst);
                }
                fetch = true;
                continue;
            }
            const SceneDev& sc = scenes.scene(job);
            const Instance& in = sc.instances[inst];
            const MeshDev& m = sc.meshes[in.mesh];
            nodes = m.nodes2;
            tris = m.tris;
            mesh = &m;
            if (in.identity) r = makeWRay(wo, wd);
            else r = makeWRay(xformPointRn(in.matInv, wo), xformVectorRn(in.matInv, wd));
            sp = 0;
            if (m.rootIsLeaf) { leafAddr = m.rootLeaf; nodeAddr = kSentinel; }
            else { leafAddr = 0; nodeAddr = 0; }
        }
        if (guard > (kBatch ? rayMaxSteps : scenes.scene(0).maxSteps)) {
            atomicOr(&ctrl->errors, 4u);
            nodeAddr = kSentinel;
            leafAddr = 0;
            inst = nInst;
        }
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
                if (sp >= (kBatch ? rayStack : min(kStackDepth, scenes.scene(0).stackLimit))) {
                    atomicOr(&ctrl->errors, 1u);
                    sp = 0;
                    nodeAddr = kSentinel;
                    break;
                }
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
                    if (SHELL && mesh->shellLayers && shellDiscard(*mesh, __float_as_int(p0.w), b0, b1)) continue;
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
        __syncwarp();  // every lane of the warp has left the loop
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
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(ANY ? &ctrl->shadowRays : &ctrl->extensionRays, (unsigned long long)n);
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

// Ten blocks per SM (48 registers, no spills) rather than the nine that 55 registers
// allow: the terrain's traversal ran 2.5 % faster; twelve (40 registers) spill and
// ran 7 % slower.
//
// S = OneScene: the mesh, its instance transform and the bounds are the kernel's
// constants. S = BatchScenes: every job of the batch is a one-instance scene with
// a binary mesh BVH; a lane loads its ray's mesh when it fetches the ray (the job
// in the high bits of the pixel field), at eight blocks per SM for the registers
// that takes.
template <class S>
struct SingleTraits {
    static constexpr int kMinBlocks = 10;
};
template <>
struct SingleTraits<BatchScenes> {
    static constexpr int kMinBlocks = 8;
};

template <bool ANY, bool COUNT, class S>
__global__ void __launch_bounds__(kTraceBlock, SingleTraits<S>::kMinBlocks)
    k_trace_single(S scenes, PathQueue q, HitQueue h, ShadowQueue s, PathQueue out, Ctrl* ctrl) {
    constexpr bool kBatch = !std::is_same<S, OneScene>::value;
    const unsigned int n = ANY ? ctrl->nShadow : ctrl->nActive;
    unsigned int* head = ANY ? &ctrl->shadowHead : &ctrl->extendHead;
    // one scene: its only mesh for every ray; a batch: the current ray's
    const Instance* in0 = kBatch ? nullptr : &scenes.scene(0).instances[0];
    const bool identity0 = kBatch ? true : in0->identity != 0;
    const MeshDev m0 = kBatch ? MeshDev{} : scenes.scene(0).meshes[in0->mesh];
    const Node2* nodes = m0.nodes2;
    const TriV* tris = m0.tris;
    int job = 0;
    int rayMaxSteps = 0, rayStack = 0;  // a batch: the current ray's job's bounds
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
            if (ANY) { o4 = __ldcs(&s.o[ray]); d4 = __ldcs(&s.d[ray]); tMax = o4.w; }
            else { o4 = __ldcs(&q.o[ray]); d4 = __ldcs(&q.d[ray]); tMax = __int_as_float(0x7f800000); }
            V3 o(o4.x, o4.y, o4.z), d(d4.x, d4.y, d4.z);
            const Instance* in = in0;
            bool identity = identity0;
            if (kBatch) {
                job = scenes.jobOf(ANY ? __float_as_uint(d4.w) : __float_as_uint(__ldg(&q.thr[ray].w)));
                in = &scenes.scene(job).instances[0];
                identity = in->identity != 0;
                rayMaxSteps = scenes.scene(job).maxSteps;
                rayStack = scenes.scene(job).stackLimit;
            }
            if (!identity) {
                o = xformPointRn(in->matInv, o);
                d = xformVectorRn(in->matInv, d);
            }
            r = makeWRay(o, d);
            hit.prim = -1;
            hit.t = tMax;
            occluded = false;
            sp = 0;
            guard = 0;
            int rootIsLeaf = m0.rootIsLeaf, rootLeaf = m0.rootLeaf;
            if (kBatch) {
                const MeshDev& m = scenes.scene(job).meshes[in->mesh];
                nodes = m.nodes2;
                tris = m.tris;
                rootIsLeaf = m.rootIsLeaf;
                rootLeaf = m.rootLeaf;
            }
            if (rootIsLeaf) { leafAddr = rootLeaf; nodeAddr = kSentinel; }
            else { leafAddr = 0; nodeAddr = 0; }
        }
        if (guard > (kBatch ? rayMaxSteps : scenes.scene(0).maxSteps)) {
            atomicOr(&ctrl->errors, 4u);
            nodeAddr = kSentinel;
            leafAddr = 0;
        }
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
                if (sp >= (kBatch ? rayStack : scenes.scene(0).stackLimit)) {
                    atomicOr(&ctrl->errors, 1u);
                    sp = 0;
                    nodeAddr = kSentinel;
                    break;
                }
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
                    const RenderParams& rp = scenes.params(job);
                    filmAdd(rp, scenes.pixelOf(__float_as_uint(s.d[ray].w)), V3(cc.x, cc.y, cc.z));
                    int target = __float_as_int(cc.w);
                    if (target >= 0) out.rng[target] = s.rng[ray];
                    if (rp.train) creditPath(rp, s.pid[ray], cc);
                }
            } else {
                __stcs(&h.h[ray], make_float4(hit.prim >= 0 ? hit.t : tMax, hit.b0, hit.b1, __int_as_float(hit.prim)));
                __stcs(&h.inst[ray], hit.prim >= 0 ? 0 : -1);
            }
        }
    }
    if (COUNT) {
        __syncwarp();  // every lane of the warp has left the loop
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
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(ANY ? &ctrl->shadowRays : &ctrl->extensionRays, (unsigned long long)n);
}

// ---- batches of scenes (xgb_render_batch) -----------------------------------------
// Each ray finds its job (and so its scene) in the high bits of its pixel field
// and is traced by the general two-level traversal.
__global__ void __launch_bounds__(kTraceBlock) k_extend_batch(BatchView b, PathQueue q, HitQueue h, Ctrl* ctrl) {
    const unsigned int n = ctrl->nActive;
    const int lane = threadIdx.x & 31;
    WorkCount wc;
    for (;;) {
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&ctrl->extendHead, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const unsigned int i = base + lane;
        if (i < n) {
            const float4 o = q.o[i], d = q.d[i];
            const int job = (int)(__float_as_uint(q.thr[i].w) >> 24);
            TraceHit hit;
            traceScene<false>(b.scenes[job], V3(o.x, o.y, o.z), V3(d.x, d.y, d.z), __int_as_float(0x7f800000), hit,
                              &ctrl->errors, wc);
            h.h[i] = make_float4(hit.t, hit.b0, hit.b1, __int_as_float(hit.prim));
            h.inst[i] = hit.inst;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctrl->extensionRays, (unsigned long long)n);
}

__global__ void __launch_bounds__(kTraceBlock) k_shadow_batch(BatchView b, ShadowQueue s, PathQueue out, Ctrl* ctrl) {
    const unsigned int n = ctrl->nShadow;
    const int lane = threadIdx.x & 31;
    WorkCount wc;
    for (;;) {
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&ctrl->shadowHead, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const unsigned int i = base + lane;
        if (i < n) {
            const float4 o = s.o[i], d = s.d[i];
            const unsigned int packed = __float_as_uint(d.w);
            const int job = (int)(packed >> 24), pix = (int)(packed & 0xFFFFFFu);
            TraceHit hit;
            if (!traceScene<true>(b.scenes[job], V3(o.x, o.y, o.z), V3(d.x, d.y, d.z), o.w, hit, &ctrl->errors, wc)) {
                const float4 c = s.c[i];
                filmAdd(b.params[job], pix, V3(c.x, c.y, c.z));
                const int target = __float_as_int(c.w);
                if (target >= 0) out.rng[target] = s.rng[i];
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctrl->shadowRays, (unsigned long long)n);
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


// Persistent grids: SMs x resident blocks of the kernel actually launched
// (looked up once per kernel; all kernels here use kTraceBlock threads).
template <class K>
static int persistentGrid(K kernel, int numSMs) {
    static std::mutex mu;
    static std::map<const void*, int> blocks;
    std::lock_guard<std::mutex> lock(mu);
    auto it = blocks.find((const void*)kernel);
    if (it == blocks.end()) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kTraceBlock, 0);
        it = blocks.emplace((const void*)kernel, b > 0 ? b : 1).first;
    }
    return numSMs * it->second;
}

// Of the specialised kernels only the flat binary one carries the shell-mapping
// discard (its SHELL variant, which also takes one-instance shell scenes); a scene
// with a shell-mapped mesh otherwise takes the generic pair.
void launchExtend(const SceneDev& sc, PathQueue q, HitQueue h, Ctrl* ctrl, int numSMs, bool count, cudaStream_t s) {
    RenderParams none{};
    const bool flat = sc.nInstances <= kFlatInstances;
#define XGB_LAUNCH(K) K<<<persistentGrid(K, numSMs), kTraceBlock, 0, s>>>
    if (sc.shell) {
        if (flat && sc.blasLayout == 0) {
            if (count) XGB_LAUNCH((k_trace_flat2<false, true, OneScene, true>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
            else XGB_LAUNCH((k_trace_flat2<false, false, OneScene, true>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        } else if (count) {
            XGB_LAUNCH((k_extend<true>))(sc, q, h, ctrl);
        } else {
            XGB_LAUNCH((k_extend<false>))(sc, q, h, ctrl);
        }
        return;
    }
    if (flat && sc.blasLayout == 1) {
        if (count) XGB_LAUNCH((k_trace_wide<false, true>))(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        else XGB_LAUNCH((k_trace_wide<false, false>))(sc, none, q, h, ShadowQueue{}, PathQueue{}, ctrl);
    } else if (sc.nInstances == 1 && sc.blasLayout == 0) {
        if (count) XGB_LAUNCH((k_trace_single<false, true, OneScene>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        else XGB_LAUNCH((k_trace_single<false, false, OneScene>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
    } else if (flat && sc.blasLayout == 0) {
        if (count) XGB_LAUNCH((k_trace_flat2<false, true, OneScene>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
        else XGB_LAUNCH((k_trace_flat2<false, false, OneScene>))(OneScene{sc, none}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
    } else if (count) {
        XGB_LAUNCH((k_extend<true>))(sc, q, h, ctrl);
    } else {
        XGB_LAUNCH((k_extend<false>))(sc, q, h, ctrl);
    }
}
void launchExtendBatch(const BatchView& b, PathQueue q, HitQueue h, Ctrl* ctrl, int numSMs, cudaStream_t s) {
    if (b.flat == kBatchSingle)
        XGB_LAUNCH((k_trace_single<false, false, BatchScenes>))(BatchScenes{b}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
    else if (b.flat) XGB_LAUNCH((k_trace_flat2<false, false, BatchScenes>))(BatchScenes{b}, q, h, ShadowQueue{}, PathQueue{}, ctrl);
    else XGB_LAUNCH(k_extend_batch)(b, q, h, ctrl);
}
void launchShadowBatch(const BatchView& b, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int numSMs, cudaStream_t s) {
    if (b.flat == kBatchSingle)
        XGB_LAUNCH((k_trace_single<true, false, BatchScenes>))(BatchScenes{b}, PathQueue{}, HitQueue{}, sq, out, ctrl);
    else if (b.flat) XGB_LAUNCH((k_trace_flat2<true, false, BatchScenes>))(BatchScenes{b}, PathQueue{}, HitQueue{}, sq, out, ctrl);
    else XGB_LAUNCH(k_shadow_batch)(b, sq, out, ctrl);
}

void launchShadow(const SceneDev& sc, const RenderParams& rp, ShadowQueue sq, PathQueue out, Ctrl* ctrl, int numSMs,
                  cudaStream_t s) {
    const bool flat = sc.nInstances <= kFlatInstances;
    if (sc.shell) {
        if (flat && sc.blasLayout == 0)
            XGB_LAUNCH((k_trace_flat2<true, false, OneScene, true>))(OneScene{sc, rp}, PathQueue{}, HitQueue{}, sq, out, ctrl);
        else XGB_LAUNCH(k_shadow)(sc, rp, sq, out, ctrl);
        return;
    }
    if (flat && sc.blasLayout == 1) XGB_LAUNCH((k_trace_wide<true, false>))(sc, rp, PathQueue{}, HitQueue{}, sq, out, ctrl);
    else if (sc.nInstances == 1 && sc.blasLayout == 0)
        XGB_LAUNCH((k_trace_single<true, false, OneScene>))(OneScene{sc, rp}, PathQueue{}, HitQueue{}, sq, out, ctrl);
    else if (flat && sc.blasLayout == 0)
        XGB_LAUNCH((k_trace_flat2<true, false, OneScene>))(OneScene{sc, rp}, PathQueue{}, HitQueue{}, sq, out, ctrl);
    else XGB_LAUNCH(k_shadow)(sc, rp, sq, out, ctrl);
#undef XGB_LAUNCH
}

}  // namespace xgb
