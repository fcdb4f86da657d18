// Correctly rounded float sin / cos / pow / exp / log for the sampling code.
//
// Why: a sampled direction decides which triangle the next ray hits and, inside
// microfacet normal mapping's random walk (Sandbox/MicrofacetBasedNormalMapping/
// Main.cpp:127-168), when the walk stops; a one-ulp difference in a sine or
// cosine there sends a path elsewhere. The reference calls the C library's float
// functions, which round correctly for all but about 1 % of the azimuths the
// samplers draw (counted against long double); CUDA's
// own sinf / cosf / powf are accurate to a few ulp but round differently far more
// often. An oracle whose float functions all round correctly renders the
// normal-mapping scenes within relMSE 3e-6 of the plain oracle, and the GPU
// renders within 1e-9 of that correctly rounded oracle; only on the longest
// diffuse paths (the occluded room, no depth limit) do the C library's own
// misroundings move an image by more (1.3e-4 at 128 x 128 x 4). So the samplers
// call the functions below, and the evaluation code (values, not decisions)
// keeps CUDA's faster ones.
//
// crSinCosf: double-float arithmetic (pairs of floats, Dekker 1971, "A
// floating-point technique for extending the available precision"; exact
// products with FMA), Cody-Waite argument reduction by pi/2 split into three
// floats, Taylor series of sin and cos on [-pi/4, pi/4] with the leading terms in
// double-float (relative error near 2^-43), and one final rounding of hi + lo to
// float. Results equal the correctly rounded float except when the exact value
// lies within about 2^-43 relative of a rounding boundary. Arguments beyond
// |x| = 8 (never passed by the samplers) take the double-precision path.
// crPowf / crExpf / crLogf / crAsinf: the double-precision function (error below 2 ulp of
// a double) rounded once to float -- the correctly rounded float unless the
// exact value lies within a few double ulp of a float rounding boundary.
//
// Everything here is __host__ __device__ so that a host build can test it
// exhaustively against long double; device code uses explicitly rounded
// intrinsics so that no compiler contraction changes the error-free steps.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#if defined(__CUDA_ARCH__)
#define XGB_FADD(a, b) __fadd_rn(a, b)
#define XGB_FSUB(a, b) __fsub_rn(a, b)
#define XGB_FMUL(a, b) __fmul_rn(a, b)
#define XGB_FFMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define XGB_FADD(a, b) ((a) + (b))
#define XGB_FSUB(a, b) ((a) - (b))
#define XGB_FMUL(a, b) ((a) * (b))
#define XGB_FFMA(a, b, c) fmaf(a, b, c)
#endif

namespace xgb {
namespace cr {

struct Df {
    float hi, lo;
};

// a + b = s + e exactly (Knuth's TwoSum).
__host__ __device__ __forceinline__ Df twoSum(float a, float b) {
    const float s = XGB_FADD(a, b);
    const float bb = XGB_FSUB(s, a);
    const float e = XGB_FADD(XGB_FSUB(a, XGB_FSUB(s, bb)), XGB_FSUB(b, bb));
    return Df{s, e};
}
// a + b = s + e exactly when |a| >= |b| (Dekker's FastTwoSum).
__host__ __device__ __forceinline__ Df fastTwoSum(float a, float b) {
    const float s = XGB_FADD(a, b);
    return Df{s, XGB_FSUB(b, XGB_FSUB(s, a))};
}
// a * b = p + e exactly (FMA).
__host__ __device__ __forceinline__ Df twoProd(float a, float b) {
    const float p = XGB_FMUL(a, b);
    return Df{p, XGB_FFMA(a, b, -p)};
}
// Double-float sum, relatively accurate even under cancellation.
__host__ __device__ __forceinline__ Df add(Df a, Df b) {
    Df s = twoSum(a.hi, b.hi);
    const Df t = twoSum(a.lo, b.lo);
    s = fastTwoSum(s.hi, XGB_FADD(s.lo, t.hi));
    return fastTwoSum(s.hi, XGB_FADD(s.lo, t.lo));
}
// Double-float product.
__host__ __device__ __forceinline__ Df mul(Df a, Df b) {
    Df p = twoProd(a.hi, b.hi);
    p.lo = XGB_FFMA(a.hi, b.lo, p.lo);
    p.lo = XGB_FFMA(a.lo, b.hi, p.lo);
    return fastTwoSum(p.hi, p.lo);
}
// c + z * u for a constant c larger in magnitude than z * u (Horner step of a
// series whose terms decrease).
__host__ __device__ __forceinline__ Df horner(Df c, Df z, Df u) {
    const Df p = mul(z, u);
    Df s = fastTwoSum(c.hi, p.hi);
    s.lo = XGB_FADD(s.lo, XGB_FADD(c.lo, p.lo));
    return fastTwoSum(s.hi, s.lo);
}

// pi / 2 = kC1 + kC2 + kC3 - 9.5e-23, kC1 with 21 significant bits so that k kC1
// is exact for |k| <= 7.
constexpr float kC1 = 0x1.921fb0p+0f;
constexpr float kC2 = 0x1.5110b4p-22f;
constexpr float kC3 = 0x1.84698ap-48f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
// 1/n! as double-float (hi, lo) where the series needs it, float beyond
constexpr float kF3h = 0x1.555556p-3f, kF3l = -0x1.555556p-28f;
constexpr float kF4h = 0x1.555556p-5f, kF4l = -0x1.555556p-30f;
constexpr float kF5h = 0x1.111112p-7f, kF5l = -0x1.ddddde0p-32f;
constexpr float kF6h = 0x1.6c16c2p-10f, kF6l = -0x1.27d27ep-35f;
constexpr float kF7h = 0x1.a01a02p-13f, kF7l = -0x1.7f97fap-39f;
constexpr float kF8h = 0x1.a01a02p-16f, kF8l = -0x1.7f97fap-42f;
constexpr float kF9 = 0x1.71de3ap-19f, kF10 = 0x1.27e4fcp-22f, kF11 = 0x1.ae6456p-26f;
constexpr float kF12 = 0x1.1eed8ep-29f, kF13 = 0x1.612462p-33f, kF14 = 0x1.93974ap-37f;
constexpr float kF15 = 0x1.ae7f3ep-41f, kF16 = 0x1.ae7f3ep-45f;

// sin and cos of x, |x| <= 8, as unrounded double-floats; the quadrant in *q.
// Reduction: k = nearest integer to x 2/pi; t = x - k kC1 is exact (k kC1 is, and
// Sterbenz's lemma covers the subtraction); then k kC2 exactly as a double-float
// and k kC3 as a float. Series in z = r^2: the terms above 2^-40 of the leading
// one in double-float, the rest in float.
__host__ __device__ __forceinline__ void sinCosReduced(float x, Df* s, Df* c, int* q) {
    const float k = rintf(XGB_FMUL(x, kTwoOverPi));
    const float t = XGB_FFMA(-k, kC1, x);  // exact
    const Df p = twoProd(k, kC2);
    Df r = twoSum(t, -p.hi);
    r.lo = XGB_FSUB(XGB_FSUB(r.lo, p.lo), XGB_FMUL(k, kC3));
    r = fastTwoSum(r.hi, r.lo);
    *q = ((int)k) & 3;
    const Df z = mul(r, r);
    // sin r = r + r z (-1/3! + z (1/5! - z (1/7! - z (1/9! - z (1/11! - z (1/13! - z/15!))))))
    float ts = XGB_FFMA(z.hi, -kF15, kF13);
    ts = XGB_FFMA(z.hi, ts, -kF11);
    ts = XGB_FFMA(z.hi, ts, kF9);
    Df u = horner(Df{-kF7h, -kF7l}, z, Df{ts, 0.0f});
    u = horner(Df{kF5h, kF5l}, z, u);
    u = horner(Df{-kF3h, -kF3l}, z, u);
    const Df w = mul(mul(r, z), u);
    Df sr = fastTwoSum(r.hi, w.hi);
    sr.lo = XGB_FADD(sr.lo, XGB_FADD(r.lo, w.lo));
    *s = sr;
    // cos r = 1 + z (-1/2 + z (1/4! - z (1/6! - z (1/8! - z (1/10! - z (1/12! - z (1/14! - z/16!)))))))
    float tc = XGB_FFMA(z.hi, kF16, -kF14);
    tc = XGB_FFMA(z.hi, tc, kF12);
    tc = XGB_FFMA(z.hi, tc, -kF10);
    Df v = horner(Df{kF8h, kF8l}, z, Df{tc, 0.0f});
    v = horner(Df{-kF6h, -kF6l}, z, v);
    v = horner(Df{kF4h, kF4l}, z, v);
    v = horner(Df{-0.5f, 0.0f}, z, v);
    const Df y = mul(z, v);
    Df cr = fastTwoSum(1.0f, y.hi);
    cr.lo = XGB_FADD(cr.lo, y.lo);
    *c = cr;
}

}  // namespace cr

// Correctly rounded (sinf(x), cosf(x)) (see the header of this file). Inlined:
// a call (measured) costs the terrain's shading more than the extra registers.
static __host__ __device__ __forceinline__ float2 crSinCos(float x) {
    const float ax = fabsf(x);
    if (!(ax <= 8.0f)) return make_float2((float)sin((double)x), (float)cos((double)x));  // or NaN / inf
    // |x^3 / 6| and x^2 / 2 below half an ulp: sin x rounds to x, cos x to 1
    if (ax < 0x1p-12f) return make_float2(x, 1.0f);
    cr::Df s, c;
    int q;
    cr::sinCosReduced(x, &s, &c, &q);
    const float sr = XGB_FADD(s.hi, s.lo), cr_ = XGB_FADD(c.hi, c.lo);  // one rounding of hi + lo
    return q == 0 ? make_float2(sr, cr_) : (q == 1 ? make_float2(cr_, -sr) : (q == 2 ? make_float2(-sr, -cr_)
                                                                                   : make_float2(-cr_, sr)));
}
__host__ __device__ __forceinline__ void crSinCosf(float x, float* sOut, float* cOut) {
    const float2 sc = crSinCos(x);
    *sOut = sc.x;
    *cOut = sc.y;
}

__host__ __device__ __forceinline__ float crPowf(float x, float y) { return (float)pow((double)x, (double)y); }
__host__ __device__ __forceinline__ float crExpf(float x) { return (float)exp((double)x); }
__host__ __device__ __forceinline__ float crLogf(float x) { return (float)log((double)x); }
__host__ __device__ __forceinline__ float crAsinf(float x) { return (float)asin((double)x); }

}  // namespace xgb
