// Learned directional proposal: a 64-64-64-64-40 MLP maps a shading point
// (frequency-encoded position, normal, outgoing direction) to an 8-lobe von
// Mises-Fisher mixture, sampled by one-sample MIS with the BSDF.
//
// The mixture is the reference's VonMisesFisherDistribution<8>
// (Include/Xitils/VonMisesFisherDistribution.h): lobe pdf
// kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa (mu . w - 1)) (:205-211), kappa == 0
// gives 1/(4 pi); sampling follows sample() (:162-201): lobe by the cumulative
// weights (randiAlongNormalizedWeights, Sampler.h:38-49), then
// W = 1 + log(u + (1 - u) exp(-2 kappa)) / kappa along mu in the lobe's BasisVectors
// frame. One deliberate difference: the reference draws the tangential part V
// uniformly in the unit disk (r = sqrt(u), VonMisesFisherDistribution.h:172-177),
// which does not produce the density its eval() returns (it concentrates the
// samples); guided MIS needs sampling and pdf to agree, so V is a unit vector
// (Jakob, "Numerically stable sampling of the von Mises Fisher distribution on S^2").
// The log-normaliser is evaluated in FP64 for kappa < 1e-2 (kappa -> 0).
#pragma once
#include <cuda_bf16.h>

#include "xgb_math.cuh"

namespace xgb {

constexpr int kGuideIn = 64;
constexpr int kGuideHidden = 64;
constexpr int kGuideLobes = 8;
constexpr int kGuideOut = 5 * kGuideLobes;   // per lobe: m.xyz (direction, unnormalised), k (log kappa), l (weight logit)
constexpr int kGuideOutPad = 48;             // padded to whole 16-wide k-steps
constexpr int kGuideBands = 6;
constexpr float kKappaLogMin = -6.0f, kKappaLogMax = 8.0f;
// Parameter offsets (fp32 master copy): W0 b0 W1 b1 W2 b2 W3 b3, W row-major [out][in].
constexpr int kGuideW0 = 0;
constexpr int kGuideB0 = kGuideW0 + kGuideHidden * kGuideIn;
constexpr int kGuideW1 = kGuideB0 + kGuideHidden;
constexpr int kGuideB1 = kGuideW1 + kGuideHidden * kGuideHidden;
constexpr int kGuideW2 = kGuideB1 + kGuideHidden;
constexpr int kGuideB2 = kGuideW2 + kGuideHidden * kGuideHidden;
constexpr int kGuideW3 = kGuideB2 + kGuideHidden;
constexpr int kGuideB3 = kGuideW3 + kGuideOut * kGuideHidden;
constexpr int kGuideParams = kGuideB3 + kGuideOut;  // 15,080

struct GuideBounds {
    float lo[3];
    float invExtent[3];
};

// 64 features: sin / cos of 2^b * pi * p for 6 bands and 3 axes (36), p (3), n (3), wo (3), zeros;
// feature 6 b + 2 axis is the sine of band b, the next one its cosine. One sincos per
// axis, the higher bands by the double-angle recurrence (sin 2a = 2 sin a cos a,
// cos 2a = 1 - 2 sin^2 a): at band 5 it stays within 2e-5 of evaluating the band
// directly, far inside the bf16 rounding of the network's inputs.
__device__ __forceinline__ void guideFeatures(const float* p, const float* n, const float* wo, float* f) {
#pragma unroll
    for (int axis = 0; axis < 3; ++axis) {
        float s, c;
        __sincosf(p[axis] * kPi, &s, &c);
#pragma unroll
        for (int band = 0; band < kGuideBands; ++band) {
            f[band * 6 + axis * 2] = s;
            f[band * 6 + axis * 2 + 1] = c;
            const float s2 = 2.0f * s * c, c2 = 1.0f - 2.0f * s * s;
            s = s2;
            c = c2;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f[36 + k] = p[k];
        f[39 + k] = n[k];
        f[42 + k] = wo[k];
    }
#pragma unroll
    for (int k = 45; k < 64; ++k) f[k] = 0.0f;
}

struct VmfLobe {
    V3 mu;
    float kappa;
    float alpha;
};

struct VmfMixture {
    VmfLobe lobe[kGuideLobes];
};

__device__ __forceinline__ float clampLogKappa(float k) {
    return fminf(fmaxf(k, kKappaLogMin), kKappaLogMax);
}

// Network output row (40 floats) -> mixture (softmax weights, exp kappa, unit mu).
__device__ __forceinline__ void decodeMixture(const float* y, VmfMixture& mx) {
    float mxl = -1e30f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) mxl = fmaxf(mxl, y[5 * j + 4]);
    float sum = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        float e = __expf(y[5 * j + 4] - mxl);
        mx.lobe[j].alpha = e;
        sum += e;
    }
    float inv = 1.0f / sum;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        V3 m(y[5 * j], y[5 * j + 1], y[5 * j + 2]);
        float l2 = dot(m, m);
        mx.lobe[j].mu = l2 > 1e-30f ? m * rsqrtf(l2) : V3(0.0f, 0.0f, 1.0f);
        mx.lobe[j].kappa = __expf(clampLogKappa(y[5 * j + 3]));
        mx.lobe[j].alpha *= inv;
    }
}

// log of the vMF normaliser kappa / (2 pi (1 - exp(-2 kappa))); FP64 near kappa -> 0.
__device__ __forceinline__ float vmfLogNorm(float kappa) {
    if (kappa < 1e-2f) {
        double k = kappa;
        return (float)(log(k) - log(2.0 * kPiD) - log1p(-exp(-2.0 * k)));
    }
    return __logf(kappa) - 1.8378770664093453f - log1pf(-__expf(-2.0f * kappa));
}

__device__ __forceinline__ float vmfPdf(const VmfLobe& l, V3 w) {
    return __expf(vmfLogNorm(l.kappa) + l.kappa * (dot(l.mu, w) - 1.0f));
}

__device__ __forceinline__ float mixturePdf(const VmfMixture& mx, V3 w) {
    float p = 0.0f;
    for (int j = 0; j < kGuideLobes; ++j) p += mx.lobe[j].alpha * vmfPdf(mx.lobe[j], w);
    return p;
}

// VonMisesFisherDistribution::sample (VonMisesFisherDistribution.h:162-201).
__device__ __forceinline__ V3 mixtureSample(const VmfMixture& mx, Pcg& rng) {
    float u = rng.randf();
    float acc = 0.0f;
    int n = 0;
    for (; n < kGuideLobes - 1; ++n) {  // randiAlongNormalizedWeights (Sampler.h:38-49)
        acc += mx.lobe[n].alpha;
        if (u <= acc) break;
    }
    const VmfLobe& l = mx.lobe[n];
    float v1 = rng.randf();
    float th = 2.0f * kPi * v1 - kPi;
    float vx = cosf(th), vy = sinf(th);
    float u2 = rng.randf();
    float W = l.kappa > 0.0f ? 1.0f + logf(u2 + (1.0f - u2) * expf(-2.0f * l.kappa)) / l.kappa : 1.0f;
    float sq = safeSqrt(1.0f - W * W);
    Basis basis(normalize(l.mu));
    return normalize(basis.toGlobal(W, sq * vx, sq * vy));
}

// d log C / d kappa for C = kappa / (2 pi (1 - exp(-2 kappa))).
__device__ __forceinline__ float vmfDLogNorm(float kappa) {
    if (kappa < 1e-2f) {
        double k = kappa;
        return (float)(1.0 / k - 2.0 / expm1(2.0 * k));
    }
    return 1.0f / kappa - 2.0f / expm1f(2.0f * kappa);
}

// Gradient of  -w * log q(w_dir)  with respect to the 40 network outputs.
// Returns the loss term; writes dy[40].
__device__ __forceinline__ float mixtureNllGrad(const float* y, V3 wdir, float weight, float* dy) {
    VmfMixture mx;
    decodeMixture(y, mx);
    float v[kGuideLobes];
    float q = 0.0f;
    for (int j = 0; j < kGuideLobes; ++j) {
        v[j] = vmfPdf(mx.lobe[j], wdir);
        q += mx.lobe[j].alpha * v[j];
    }
    q = fmaxf(q, 1e-20f);
    const float g = -weight / q;  // d loss / d q
    for (int j = 0; j < kGuideLobes; ++j) {
        const VmfLobe& l = mx.lobe[j];
        V3 m(y[5 * j], y[5 * j + 1], y[5 * j + 2]);
        float mlen = sqrtf(fmaxf(dot(m, m), 1e-30f));
        float cosw = dot(l.mu, wdir);
        float av = l.alpha * v[j];
        // direction: d log v / d m = kappa (w - (mu.w) mu) / |m|
        float s = g * av * l.kappa / mlen;
        dy[5 * j + 0] = s * (wdir.x - cosw * l.mu.x);
        dy[5 * j + 1] = s * (wdir.y - cosw * l.mu.y);
        dy[5 * j + 2] = s * (wdir.z - cosw * l.mu.z);
        // concentration: kappa = exp(k), zero gradient outside the clamp
        float k = y[5 * j + 3];
        bool inside = k > kKappaLogMin && k < kKappaLogMax;
        dy[5 * j + 3] = inside ? g * av * (vmfDLogNorm(l.kappa) + cosw - 1.0f) * l.kappa : 0.0f;
        // weight logit (softmax)
        dy[5 * j + 4] = g * l.alpha * (v[j] - q);
    }
    return -weight * __logf(q);
}

}  // namespace xgb
