// Shade kernel of the wavefront integrator and what it shares with the camera
// kernel: the job policies (one scene, or the jobs of a batch), film and AOV
// accumulation, light sampling and the k_shade template. Included by
// integrator.cu and by the units that instantiate the shade kernel's variants
// (shade_nested.cu), each compiled with -fmad=false.
#pragma once
#include "guide.cuh"
#include "materials.cuh"
#include "xgb_kernels.h"

namespace xgb {

constexpr int kShadeBlock = 256;
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ void filmAddS(const RenderParams& rp, int pix, V3 c) {
    if (rp.dropNonFinite && !(isfinite(c.x) && isfinite(c.y) && isfinite(c.z))) return;
    if (rp.filmFp64) {
        double* f = (double*)rp.film + 4 * (size_t)pix;
        atomicAdd(f, (double)c.x);
        atomicAdd(f + 1, (double)c.y);
        atomicAdd(f + 2, (double)c.z);
    } else {
        atomicAdd((float4*)rp.film + pix, make_float4(c.x, c.y, c.z, 0.0f));
    }
}

// DenoisableRenderTarget planes: first-hit albedo, then first-hit normal.
__device__ __forceinline__ void aovAdd(const RenderParams& rp, int pix, V3 albedo, V3 normal) {
    const size_t plane = (size_t)rp.width * (size_t)rp.height;
    if (rp.filmFp64) {
        double* a = (double*)rp.aov + 4 * (size_t)pix;
        double* n = (double*)rp.aov + 4 * (plane + (size_t)pix);
        atomicAdd(a, (double)albedo.x); atomicAdd(a + 1, (double)albedo.y); atomicAdd(a + 2, (double)albedo.z);
        atomicAdd(n, (double)normal.x); atomicAdd(n + 1, (double)normal.y); atomicAdd(n + 2, (double)normal.z);
    } else {
        atomicAdd((float4*)rp.aov + pix, make_float4(albedo.x, albedo.y, albedo.z, 0.0f));
        atomicAdd((float4*)rp.aov + plane + pix, make_float4(normal.x, normal.y, normal.z, 0.0f));
    }
}

// Job policies: which scene and render parameters a path belongs to.
// One scene (xgb_render): the queue's pixel field is the pixel index itself.
struct OneJob {
    SceneDev sc;
    RenderParams rp;
    __device__ __forceinline__ int locate(unsigned long long g, unsigned long long& local) const {
        local = g;
        return 0;
    }
    __device__ __forceinline__ const SceneDev& scene(int) const { return sc; }
    __device__ __forceinline__ const RenderParams& params(int) const { return rp; }
    __device__ __forceinline__ void decode(int packed, int& job, int& pix) const { job = 0; pix = packed; }
    __device__ __forceinline__ int encode(int, int pix) const { return pix; }
};
// Many scenes in one wavefront (xgb_render_batch): job j owns the global path
// ids [start[j], start[j+1]); the pixel field carries job << 24 | pixel.
struct ManyJobs {
    const SceneDev* sc;
    const RenderParams* rp;
    const unsigned long long* start;  // nJobs + 1 prefix sums of W * H * spp
    int nJobs;
    __device__ __forceinline__ int locate(unsigned long long g, unsigned long long& local) const {
        int lo = 0, hi = nJobs - 1;
        while (lo < hi) {  // last job whose start is <= g
            const int mid = (lo + hi + 1) >> 1;
            if (start[mid] <= g) lo = mid;
            else hi = mid - 1;
        }
        local = g - start[lo];
        return lo;
    }
    __device__ __forceinline__ const SceneDev& scene(int j) const { return sc[j]; }
    __device__ __forceinline__ const RenderParams& params(int j) const { return rp[j]; }
    __device__ __forceinline__ void decode(int packed, int& job, int& pix) const {
        job = (int)((unsigned int)packed >> 24);
        pix = packed & 0xFFFFFF;
    }
    __device__ __forceinline__ int encode(int job, int pix) const { return (job << 24) | pix; }
};

struct LightSampleD {
    V3 p, n, sn;
    float pdf;
    int material;
};

// Scene::sampleSurface chain (Scene.h:40-47, Object.h:91-105,
// TriangleMesh.h:216-230, TriangleIndexed.h:179-209).
__device__ __forceinline__ LightSampleD sampleLight(const SceneDev& sc, Pcg& rng) {
    const LightDev L = sc.lights[rng.randi(sc.nLights)];
    const MeshDev& m = sc.meshes[L.mesh];
    const Instance& in = sc.instances[L.instance];
    int tri = rng.randi(L.nTris);
    float t0, t1, t2, sum;
    int tries = 0;
    do {  // the reference retries without bound; three zero draws in a row never happen in practice
        t0 = rng.randf(); t1 = rng.randf(); t2 = rng.randf();
        sum = t0 + t1 + t2;
    } while (sum == 0.0f && ++tries < 64);
    float inv = 1.0f / sum;
    t0 = t0 * inv;
    t1 = t1 * inv;
    int i0 = m.idx[3 * tri], i1 = m.idx[3 * tri + 1], i2 = m.idx[3 * tri + 2];
    LightSampleD ls;
    ls.p = lerp3(v3(m.pos[i0]), v3(m.pos[i1]), v3(m.pos[i2]), t0, t1);
    if (!in.identity) ls.p = xformPoint(in.mat, ls.p);
    ls.n = v3(sc.lightNormal[L.triOffset + tri]);
    if (m.nrm) {
        V3 sn = normalize(lerp3(v3(m.nrm[i0]), v3(m.nrm[i1]), v3(m.nrm[i2]), t0, t1));
        ls.sn = in.identity ? normalize(sn) : xformNormal(in.mat, sn);
    } else {
        ls.sn = ls.n;
    }
    ls.pdf = sc.lightPdf[L.triOffset + tri];
    ls.material = in.material;
    return ls;
}

__device__ __forceinline__ V3 emission(const Material& m, V3 wo, V3 n) {  // Material.h:408-410
    return dot(wo, n) > 0.0f ? V3(m.albedo.x, m.albedo.y, m.albedo.z) : V3();
}

constexpr float kRayOffset = 0.00001f;    // PathTracer.h:254
constexpr float kShadowMargin = 0.0001f;  // PathTracer.h:257

struct ShadeOut {
    // continuing path
    float4 o, d, thr;
    uint2 rng;
    int grec;
    // shadow ray
    float4 so, sd, sc;
    uint2 srng;
    bool stochastic;
};

// Whether a guided vertex becomes a training record: a hash of (path, depth),
// so that the decision draws nothing from the path's own random stream.
__device__ __forceinline__ bool keepRecord(unsigned int pid, int len, float prob) {
    if (prob >= 1.0f) return true;
    uint64_t z = splitmix64(((uint64_t)pid << 8) ^ (uint64_t)(len & 0xFF) ^ 0x9E3779B97F4A7C15ull);
    return (float)(z >> 40) * (1.0f / 16777216.0f) < prob;
}

__device__ __forceinline__ float luminance(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Materials the learned proposal may sample: non-delta BSDFs whose bsdfCos and
// getPDF are deterministic.
__device__ __forceinline__ bool guidableBasic(int kind) {
    return kind == MAT_DIFFUSE || kind == MAT_METAL || kind == MAT_GLOSSY || kind == MAT_GLOSSY_CLAMPED ||
           kind == MAT_GLOSSY_HIGHLIGHT;
}
// Materials the learned proposal is mixed into: those whose sampling density is
// known in closed form. Microfacet normal mapping is left to its own sampler:
// its random walk's density is only approximated (getPDF,
// MicrofacetBasedNormalMapping/Main.cpp:254-321), and although one-sample MIS
// with that approximation stays unbiased (the two techniques' weights still sum
// to one), a guide-sampled direction is weighted by f / (c p~ + (1 - c) p_vmf)
// with a stochastic f that p~ does not bound: measured on the normal-mapping
// scenes, rare samples 5-10x brighter than the plain path's worst, and a much
// higher error at equal time.
__device__ __forceinline__ bool guidable(const SceneDev& sc, const Material& m) {
    (void)sc;
    return guidableBasic(m.kind);
}

__device__ __forceinline__ void loadMixture(const float4* m, VmfMixture& mx) {
    for (int j = 0; j < kGuideLobes; ++j) {
        float4 a = m[j];
        mx.lobe[j].mu = V3(a.x, a.y, a.z);
        mx.lobe[j].kappa = a.w;
    }
    float4 a0 = m[8], a1 = m[9];
    mx.lobe[0].alpha = a0.x; mx.lobe[1].alpha = a0.y; mx.lobe[2].alpha = a0.z; mx.lobe[3].alpha = a0.w;
    mx.lobe[4].alpha = a1.x; mx.lobe[5].alpha = a1.y; mx.lobe[6].alpha = a1.z; mx.lobe[7].alpha = a1.w;
}

// EXTRAS: the learned proposal (guided sampling, training records), AOV planes;
// plain renders run the variant without that code (fewer registers, a smaller
// instruction footprint). Occupancy bounds, measured on GB300: without nested
// materials three blocks per SM (80 registers, ~80 bytes of spills) -- terrain
// shading 12.6 instead of 15.0 ms per render at two blocks, the guided room 82.5
// instead of 79.9 Mpaths/s, the Cornell box 2.03 instead of 1.98 ms; with nested
// materials two blocks (128 registers, 60-90 bytes of spills) -- the
// normal-mapping scene 101 instead of 88 Mpaths/s at one block (140 registers);
// the GGX-metal-only variant four blocks (64 registers, ~200 bytes of spills) --
// terrain shading 10.1 instead of 11.6 ms per render at three, 1834 instead of 1762
// Mpaths/s -- while the Lambert-only variant stays at three (the Cornell box
// 9.5 against 9.9 ms of shading over five renders at four, the room 40.8
// against 42.2). Without emitters (no emission, no NEE code) and with the
// standard integrator only, the metal variant shades the terrain in 9.2 ms per
// render at four blocks (1878 Mpaths/s) and 9.1 ms at five (51 registers, 1884).
template <class J, int NESTED, bool EXTRAS>
__global__ void __launch_bounds__(kShadeBlock, (NESTED & 3) ? 2 : (NESTED & kNoEmitters) ? 5 : (NESTED & kOnlyMetal) ? 4 : 3) k_shade(J jobs, PathQueue in, HitQueue hq, PathQueue out,
                                                       ShadowQueue sq, Ctrl* ctrl) {
    const unsigned int n = ctrl->nActive;
    const int lane = threadIdx.x & 31;
    const unsigned int warpId = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned int nWarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned int base = warpId * 32u; base < n; base += nWarps * 32u) {
        const unsigned int i = base + lane;
        bool cont = false, shadow = false, done = false;
        ShadeOut r;
        r.stochastic = false;
        r.grec = -1;
        if (i < n) {
            // Queue records are read once and written once per iteration and far
            // exceed L2 at 2^23 paths in flight: streaming (evict-first) loads and
            // stores keep L2 for BVH nodes, triangles and textures (terrain shading
            // 12.7 -> 11.6 ms per render, 1495 -> 1533 Mpaths/s on GB300).
            float4 o4 = __ldcs(&in.o[i]), d4 = __ldcs(&in.d[i]), t4 = __ldcs(&in.thr[i]);
            uint2 rs = __ldcs(&in.rng[i]);
            float4 h = __ldcs(&hq.h[i]);
            const int instId = __ldcs(&hq.inst[i]);
            const int prim = __float_as_int(h.w);
            const int meta = __float_as_int(d4.w);
            int len = meta & 0xFFFF;
            const int flags = meta >> 16;
            const int packed = __float_as_int(t4.w);
            int job, pix;
            jobs.decode(packed, job, pix);
            const SceneDev& sc = jobs.scene(job);
            const RenderParams& rp = jobs.params(job);
            // the one-kind variants run the standard integrator only
            const bool naive = !(NESTED & (kOnlyMetal | kOnlyDiffuse)) && rp.integrator == 1;
            const float pdfPrev = o4.w;
            V3 dir(d4.x, d4.y, d4.z);
            V3 thr(t4.x, t4.y, t4.z);
            // guide training: the record of the vertex this ray left takes the
            // path's accumulated contribution now, before this vertex adds any
            const unsigned int pid = (EXTRAS && rp.train) ? in.pid[i] : 0u;
            if (EXTRAS && rp.train) {
                const int prevRec = in.grec[i];
                if (prevRec >= 0) {
                    float4 a = rp.pathAcc[pid];
                    rp.arena[prevRec].snap = make_float3(a.x, a.y, a.z);
                }
            }
            V3 acc(0.0f);  // this vertex's contributions (training accumulator)
            auto contribute = [&](V3 c) {
                filmAddS(rp, pix, c);
                if (EXTRAS && rp.train) acc = acc + c;
            };
            Pcg rng;
            rng.state = ((uint64_t)rs.y << 32) | rs.x;
            rng.inc = ((uint64_t)(unsigned int)pix << 1) | 1u;
            if (prim < 0) {
                // Miss: the sky, with no MIS (PathTracer.h:133-136, 192-197).
                if (sc.skyKind != SKY_NONE) {
                    V3 Ls = skyRadiance(sc, dir);
                    V3 L = thr * Ls;
                    if (naive) L = clampPositive(L);  // PathTracer.h:96
                    contribute(L);
                }
                done = true;
            } else {
                const Instance& inst = sc.instances[instId];
                const Material& mat = sc.materials[inst.material];
                Surface s = makeSurface(sc, inst, prim, h.y, h.z, dir);
                // a scene without emitters (kNoEmitters) carries no emission or NEE code
                const bool emissive = !(NESTED & kNoEmitters) && mat.kind == MAT_EMISSION;
                if (EXTRAS && rp.aov && (flags & FLAG_PRIMARY)) aovAdd(rp, pix, albedoOf(sc, mat, s), s.n);
                if (naive) {
                    // NaivePathTracer::eval (PathTracer.h:75-100): emission, BSDF sample,
                    // then the next loop top (depth limit, Russian roulette) before tracing.
                    if (emissive) filmAddS(rp, pix, thr * emission(mat, -dir, s.n));
                    V3 wi;
                    float pdf = pdfPrev;
                    thr = thr * evalAndSampleT<NESTED>(sc, mat, s, rng, &wi, &pdf);
                    bool alive = !isZero(thr);
                    len += 1;
                    if (alive && rp.maxDepth > 0 && len > rp.maxDepth) alive = false;
                    if (alive && len > rp.rrStart) {
                        if (rng.randf() >= rp.rrProb) alive = false;
                        else thr = thr / rp.rrProb;
                    }
                    if (alive) {
                        V3 no = s.p + kRayOffset * wi;
                        r.o = make_float4(no.x, no.y, no.z, pdf);
                        r.d = make_float4(wi.x, wi.y, wi.z, __int_as_float(len));
                        r.thr = make_float4(thr.x, thr.y, thr.z, __int_as_float(packed));
                        r.rng = make_uint2((unsigned int)rng.state, (unsigned int)(rng.state >> 32));
                        cont = true;
                    } else {
                        done = true;
                    }
                } else if (flags & FLAG_PRIMARY) {
                    if (emissive) contribute(thr * emission(mat, -dir, s.n));  // PathTracer.h:143-145
                } else if (emissive) {
                    // BSDF-sampled hit on an emitter (PathTracer.h:171-190).
                    float mis;
                    if (pdfPrev >= 0.0f && sc.nLights > 0) {
                        float pl = sc.lightPdf[sc.lights[inst.lightIndex].triOffset + prim];
                        float cosLight = fabsf(dot(dir, s.sn));
                        float distSq = h.x * h.x;
                        pl *= distSq / cosLight;
                        mis = (pdfPrev * pdfPrev) / ((pdfPrev * pdfPrev) + (pl * pl));
                    } else {
                        mis = 1.0f;
                    }
                    if (mis > 0.0f) contribute(thr * mis * emission(mat, -dir, s.n));
                }
                // An emitter's evalAndSample is zero: the path ends there (its NEE
                // contribution is multiplied by Emission::bsdfCos() == 0).
                if (naive) {
                    // handled above
                } else if (emissive) {
                    done = true;
                } else if (rp.maxDepth > 0 && len > rp.maxDepth) {
                    done = true;
                } else {
                    bool alive = true;
                    if (len > rp.rrStart) {  // PathTracer.h:149-155
                        if (rng.randf() >= rp.rrProb) alive = false;
                        else thr = thr / rp.rrProb;
                    }
                    if (!alive) {
                        done = true;
                    } else {
                        V3 wi;
                        float pdf = pdfPrev;  // left untouched by materials that do not set it
                        V3 f;
                        const bool guidedHere = EXTRAS && rp.guided && guidable(sc, mat);
                        VmfMixture mx;
                        float fcos = 0.0f;  // luminance of bsdfCos(wi) at a guided vertex
                        if (!guidedHere) {
                            f = evalAndSampleT<NESTED>(sc, mat, s, rng, &wi, &pdf);
                        } else {
                            // One-sample MIS of the BSDF and the learned vMF mixture (balance
                            // heuristic): pdf = frac p_bsdf + (1 - frac) p_vmf; unbiased at any
                            // network state because the BSDF keeps support everywhere.
                            loadMixture(rp.mix + (size_t)i * 10, mx);
                            const float frac = rp.bsdfFrac;
                            if (rng.randf() < frac) {
                                float pb = 0.0f;
                                V3 e = evalAndSampleT<NESTED>(sc, mat, s, rng, &wi, &pb);
                                float pm = frac * pb + (1.0f - frac) * mixturePdf(mx, wi);
                                f = (pb > 0.0f && pm > 0.0f) ? e * (pb / pm) : V3(0.0f);
                                fcos = luminance(e) * pb;
                                pdf = pm;
                            } else {
                                wi = mixtureSample(mx, rng);
                                float pb = getPDFT<NESTED>(sc, mat, s, wi);
                                float pm = frac * pb + (1.0f - frac) * mixturePdf(mx, wi);
                                V3 bc = bsdfCosT<NESTED>(sc, mat, s, rng, wi);
                                f = pm > 0.0f ? bc / pm : V3(0.0f);
                                fcos = luminance(bc);
                                pdf = pm;
                            }
                        }
                        if (!(NESTED & kNoEmitters) && !naive && sc.nLights > 0) {  // PathTracer.h:202-233
                            LightSampleD ls = sampleLight(sc, rng);
                            V3 toL = ls.p - s.p;
                            float dist = length(toL);
                            V3 sd = toL / dist;
                            V3 so = s.p + kRayOffset * sd;
                            float stMax = dist - kShadowMargin;
                            if (dot(sd, ls.n) < 0) {
                                float distSq = dist * dist;
                                float mis;
                                if (pdf >= 0.0f) {
                                    float pb = getPDFT<NESTED>(sc, mat, s, sd);
                                    if (guidedHere) pb = rp.bsdfFrac * pb + (1.0f - rp.bsdfFrac) * mixturePdf(mx, sd);
                                    float cosLight = fabsf(dot(-sd, ls.sn));
                                    pb *= cosLight / distSq;
                                    mis = (ls.pdf * ls.pdf) / ((pb * pb) + (ls.pdf * ls.pdf));
                                } else {
                                    mis = 0.0f;
                                }
                                if (mis > 0.0f) {
                                    float G = fabsf(dot(-sd, ls.sn)) / distSq;
                                    Pcg spec = rng;  // bsdfCos draws only if the light is visible
                                    V3 bc = bsdfCosT<NESTED>(sc, mat, s, spec, sd);
                                    V3 Le = emission(sc.materials[ls.material], -sd, ls.n);
                                    V3 c = thr * mis * bc * Le * G / ls.pdf;
                                    r.so = make_float4(so.x, so.y, so.z, stMax);
                                    r.sd = make_float4(sd.x, sd.y, sd.z, __int_as_float(packed));
                                    r.sc = make_float4(c.x, c.y, c.z, 0.0f);
                                    r.stochastic = spec.state != rng.state;
                                    r.srng = make_uint2((unsigned int)spec.state, (unsigned int)(spec.state >> 32));
                                    shadow = true;
                                }
                            }
                        }
                        V3 thrNext = thr * f;
                        if (!isZero(f) && !isZero(thrNext)) {
                            V3 no = s.p + kRayOffset * wi;
                            r.o = make_float4(no.x, no.y, no.z, pdf);
                            r.d = make_float4(wi.x, wi.y, wi.z, __int_as_float(len + 1));
                            r.thr = make_float4(thrNext.x, thrNext.y, thrNext.z, __int_as_float(packed));
                            r.rng = make_uint2((unsigned int)rng.state, (unsigned int)(rng.state >> 32));
                            cont = true;
                            if (EXTRAS && rp.train && guidedHere && pdf > 0.0f && keepRecord(pid, len, rp.recordProb)) {
                                unsigned int slot = atomicAdd(rp.arenaCount, 1u);
                                if (slot < (unsigned int)rp.arenaCap) {
                                    GuideRecord g;
                                    g.p = make_float3(s.p.x, s.p.y, s.p.z);
                                    g.pdf = pdf;
                                    g.n = make_float3(s.sn.x, s.sn.y, s.sn.z);
                                    g.fcos = fcos;
                                    g.wo = make_float3(s.wo.x, s.wo.y, s.wo.z);
                                    g.pid = pid;
                                    g.wi = make_float3(wi.x, wi.y, wi.z);
                                    g.radiance = 0.0f;
                                    g.snap = make_float3(__int_as_float(0x7fc00000), 0.0f, 0.0f);
                                    g.pad0 = 0.0f;
                                    g.thr = make_float3(thrNext.x, thrNext.y, thrNext.z);
                                    g.pad1 = 0.0f;
                                    rp.arena[slot] = g;
                                    r.grec = (int)slot;
                                }
                            }
                        } else {
                            done = true;
                        }
                    }
                }
            }
            if (EXTRAS && rp.train && !isZero(acc)) {
                float4 a = rp.pathAcc[pid];
                rp.pathAcc[pid] = make_float4(a.x + acc.x, a.y + acc.y, a.z + acc.z, a.w);
            }
        }
        // compacted writes: continuing paths, then shadow rays (which may point at them)
        unsigned int mc = __ballot_sync(kFull, cont);
        unsigned int oc = 0;
        if (lane == 0 && mc) oc = atomicAdd(&ctrl->nOut, (unsigned int)__popc(mc));
        oc = __shfl_sync(kFull, oc, 0);
        unsigned int slot = oc + __popc(mc & ((1u << lane) - 1u));
        const bool train = EXTRAS && jobs.params(0).train;  // guide training runs with one job only
        if (cont) {
            __stcs(&out.o[slot], r.o);
            __stcs(&out.d[slot], r.d);
            __stcs(&out.thr[slot], r.thr);
            __stcs(&out.rng[slot], r.rng);
            if (train) {
                out.grec[slot] = r.grec;
                out.pid[slot] = in.pid[i];
            }
        }
        unsigned int ms = __ballot_sync(kFull, shadow);
        unsigned int os = 0;
        if (lane == 0 && ms) os = atomicAdd(&ctrl->nShadow, (unsigned int)__popc(ms));
        os = __shfl_sync(kFull, os, 0);
        if (shadow) {
            unsigned int ss = os + __popc(ms & ((1u << lane) - 1u));
            __stcs(&sq.o[ss], r.so);
            __stcs(&sq.d[ss], r.sd);
            r.sc.w = __int_as_float((r.stochastic && cont) ? (int)slot : -1);
            __stcs(&sq.c[ss], r.sc);
            __stcs(&sq.rng[ss], r.srng);
            if (train) sq.pid[ss] = in.pid[i];
        }
        unsigned int md = __ballot_sync(kFull, done);
        if (lane == 0 && md) atomicAdd(&ctrl->pathsDone, (unsigned long long)__popc(md));
    }
}

// Grid of a shade launch: kShadeWaves full waves of the variant's resident
// blocks (SMs x blocks per SM at its register bound). Whole waves leave no
// partial last wave idling SMs (eight blocks per SM at three resident ran as
// 2.67 waves); many small blocks let SMs whose blocks finish early take more,
// which the uneven per-path cost of nested materials needs. Measured on GB300,
// shading time per render against the earlier eight blocks per SM: one wave --
// terrain 12.1 instead of 12.6 ms, normal mapping 5.96 instead of 4.4; four
// waves -- 12.7 / 4.4; eight waves -- terrain 12.6, shell mapping 7.6 instead
// of 8.6, normal mapping 3.6.
constexpr int kShadeWaves = 8;
template <class J, int NESTED, bool EXTRAS>
inline int shadeGrid(int numSMs) {
    // looked up once per variant (a thread-safe static initialisation)
    static const int perSM = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade<J, NESTED, EXTRAS>, kShadeBlock, 0) != cudaSuccess ||
            b < 1)
            b = 1;
        return b;
    }();
    return numSMs * perSM * kShadeWaves;
}

template <class J, int NESTED, bool EXTRAS>
inline void launchShadeVariant(const J& jobs, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl,
                               int numSMs, cudaStream_t s) {
    k_shade<J, NESTED, EXTRAS><<<shadeGrid<J, NESTED, EXTRAS>(numSMs), kShadeBlock, 0, s>>>(jobs, in, h, out, sq, ctrl);
}

// Launches of the shade variants for scenes with materials that evaluate another
// (the mask: 1 microfacet normal mapping, 2 MultiLobeSVBRDF, 3 both), compiled in
// their own translation units so that the build compiles them in parallel:
// shade_layered.cu (masks 1 and 2), shade_nested.cu (mask 3, one scene),
// shade_batch_nested.cu (mask 3, a batch).
void launchShadeMask1(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int numSMs,
                      cudaStream_t s);
void launchShadeMask2(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int numSMs,
                      cudaStream_t s);
void launchShadeMask3(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int numSMs,
                      cudaStream_t s);
void launchShadeMask3Batch(const ManyJobs& jobs, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl,
                           int numSMs, cudaStream_t s);

}  // namespace xgb
