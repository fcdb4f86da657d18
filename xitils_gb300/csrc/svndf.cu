// SVNDF of a displacement map on the GPU: the precomputation of the displacement
// prefiltering sandbox (downsampleDisplacementTexture,
// Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/Main.cpp:391-470) with
// the reference's EM fit of a 4-lobe vMF mixture (approximateBySEM,
// Include/Xitils/VonMisesFisherDistribution.h:68-160), one warp per low texel.
//
// The reference runs this on OpenMP threads with one sampler per thread, so the
// stream a texel's initial lobes come from depends on scheduling; here low texel t
// draws them from the PCG stream (t, 0, seed). Everything else follows the
// reference's arithmetic in its order, unfused (this unit is compiled with
// -fmad=false): the block's normals in row-major order, the mean height as a
// sequential sum, the E-step over samples (responsibilities without the lobe
// weights, as the reference computes them), the M-step sums per lobe in sample
// order, the signed convergence difference. The EM stops on a threshold, so the
// fit is chaotic at the last ulp: exp, pow, asin, sin and cos are the correctly
// rounded ones of crmath.cuh, which round as the C library does for all but a
// small fraction of arguments.
#include <algorithm>

#include "xgb_kernels.h"
#include "materials.cuh"

namespace xgb {
namespace {

constexpr int kSvMaxRate = 16;
constexpr int kSvMaxSamples = kSvMaxRate * kSvMaxRate;
constexpr int kSvWarps = 4;
constexpr int kSvStepMax = 100000;    // StepMax
constexpr float kSvKappaLimit = 1000;  // KappaLimit
constexpr float kSvDiffThreshold = 1e-6f;

struct SvWarp {
    float sx[kSvMaxSamples], sy[kSvMaxSamples], sz[kSvMaxSamples];
    float h[kSvMaxSamples];
    float z[kSvMaxSamples * kSvndfLobes];
    float mu[kSvndfLobes][3], kappa[kSvndfLobes], alpha[kSvndfLobes];
    float lastMu[kSvndfLobes][3], lastKappa[kSvndfLobes];
    int done;
};

// vMF() (VonMisesFisherDistribution.h:205-211)
__device__ __forceinline__ float vmfLobe(V3 mu, float kappa, V3 omega) {
    if (kappa == 0.0f) return 1.0f / (4 * kPi);
    return kappa / (2 * kPi * (1.0f - crExpf(-2 * kappa))) * crExpf(kappa * (dot(omega, mu) - 1.0f));
}

__global__ void __launch_bounds__(32 * kSvWarps) k_svndfFit(TextureDev src, float scale, int rate, uint32_t seed,
                                                             int resU, int resV, float4* lobes, float4* low) {
    __shared__ SvWarp smem[kSvWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kSvWarps + warp;
    if (t >= resU * resV) return;  // the whole warp leaves; only warp-level barriers below
    SvWarp& S = smem[warp];
    const int px = t % resU, py = t / resU;
    const int x0 = px * rate, y0 = py * rate;
    const int wc = min(rate, src.w - x0), hc = min(rate, src.h - y0);
    const int n = wc * hc;
    // the block's normals (Main.cpp:418-431), row-major over the texels inside the map
    for (int k = lane; k < n; k += 32) {
        const int x = x0 + k % wc, y = y0 + k / wc;
        const float su = texDiffUAt(src, x, y), sv = texDiffVAt(src, x, y);
        const V3 nn = normalize(V3(-su * scale, -sv * scale, 1.0f));
        S.sx[k] = nn.x; S.sy[k] = nn.y; S.sz[k] = nn.z;
        S.h[k] = texAt(src, x, y).x;
    }
    __syncwarp();
    if (lane == 0) {
        float r = 0.0f;
        for (int k = 0; k < n; ++k) r += S.h[k];
        low[t] = make_float4(r / (float)n, 0.0f, 0.0f, 0.0f);
    }
    float4* out = lobes + (size_t)t * 5;
    if (n == 1) {  // VonMisesFisherDistribution.h:79-86
        if (lane < kSvndfLobes) out[lane] = make_float4(S.sx[0], S.sy[0], S.sz[0], kSvKappaLimit);
        if (lane == 0) out[4] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    if (lane == 0) {  // initial lobes (:89-98)
        Pcg rng;
        rng.seed((uint32_t)t, 0u, seed);
        for (int j = 0; j < kSvndfLobes; ++j) {
            const float u = rng.randf();
            const float v = rng.randf();
            const float theta = crAsinf(u);
            const float phi = (float)((double)(2.0f * kPi * v) - kPiD);
            float st, ct, sp, cp;
            crSinCosf(theta, &st, &ct);
            crSinCosf(phi, &sp, &cp);
            S.mu[j][0] = ct * cp;
            S.mu[j][1] = ct * sp;
            S.mu[j][2] = st;
            S.kappa[j] = 0.5f;
            S.alpha[j] = 1.0f / kSvndfLobes;
        }
        S.done = 0;
    }
    __syncwarp();
    for (int step = 0; step < kSvStepMax; ++step) {
        // E-step (:106-119)
        for (int i = lane; i < n; i += 32) {
            const V3 s(S.sx[i], S.sy[i], S.sz[i]);
            float v[kSvndfLobes];
            float gamma = 0.0f;
#pragma unroll
            for (int j = 0; j < kSvndfLobes; ++j) {
                v[j] = vmfLobe(V3(S.mu[j][0], S.mu[j][1], S.mu[j][2]), S.kappa[j], s);
                gamma += v[j];
            }
#pragma unroll
            for (int j = 0; j < kSvndfLobes; ++j) S.z[i * kSvndfLobes + j] = gamma > 0.0f ? v[j] / gamma : 0.0f;
        }
        __syncwarp();
        // M-step (:121-138), lobe j on lane j, sums in sample order
        if (lane < kSvndfLobes) {
            const int j = lane;
            float a = 0.0f;
            V3 r(0.0f, 0.0f, 0.0f);
            for (int i = 0; i < n; ++i) {
                const float zz = S.z[i * kSvndfLobes + j];
                a += zz;
                r = r + zz * V3(S.sx[i], S.sy[i], S.sz[i]);
            }
            r = r / a;
            a /= (float)n;
            const float len = length(r);
            float kappa = (3 * len - crPowf(len, 3.0f)) / (1.0f - dot(r, r));
            const V3 mu = normalize(r);
            if (kappa > kSvKappaLimit) kappa = kSvKappaLimit;
            if (kappa < 0.0f) kappa = 0.0f;
            S.mu[j][0] = mu.x; S.mu[j][1] = mu.y; S.mu[j][2] = mu.z;
            S.kappa[j] = kappa;
            S.alpha[j] = a;
        }
        __syncwarp();
        if (lane == 0) {  // convergence (:140-147): a signed sum, as in the reference
            if (step > 0) {
                float diff = 0.0f;
                for (int j = 0; j < kSvndfLobes; ++j) {
                    const V3 d(S.mu[j][0] - S.lastMu[j][0], S.mu[j][1] - S.lastMu[j][1], S.mu[j][2] - S.lastMu[j][2]);
                    diff += dot(d, d);
                    diff += (S.kappa[j] - S.lastKappa[j]) * 0.1f;
                }
                if (diff < kSvDiffThreshold) S.done = 1;
            }
            for (int j = 0; j < kSvndfLobes; ++j) {
                S.lastMu[j][0] = S.mu[j][0]; S.lastMu[j][1] = S.mu[j][1]; S.lastMu[j][2] = S.mu[j][2];
                S.lastKappa[j] = S.kappa[j];
            }
        }
        __syncwarp();
        if (S.done) break;
    }
    if (lane < kSvndfLobes) out[lane] = make_float4(S.mu[lane][0], S.mu[lane][1], S.mu[lane][2], S.kappa[lane]);
    if (lane == 0) out[4] = make_float4(S.alpha[0], S.alpha[1], S.alpha[2], S.alpha[3]);
}

}  // namespace

cudaError_t svndfFit(const TextureDev& src, float scale, int rate, uint32_t seed, int resU, int resV, float4* lobes,
                     float4* low, cudaStream_t s) {
    if (rate < 1 || rate > kSvMaxRate) return cudaErrorInvalidValue;
    const int texels = resU * resV;
    k_svndfFit<<<(texels + kSvWarps - 1) / kSvWarps, 32 * kSvWarps, 0, s>>>(src, scale, rate, seed, resU, resV, lobes,
                                                                            low);
    return cudaGetLastError();
}

}  // namespace xgb
