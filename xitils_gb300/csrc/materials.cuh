// Materials, textures and skies on the device (Include/Xitils/Material.h,
// Texture.h, SkySphere.h; Sandbox/MicrofacetBasedNormalMapping/Main.cpp:34-340).
//
// Expression order follows the reference; this header is compiled with
// -fmad=false so float arithmetic is unfused as in the reference. Where the
// reference promotes an intermediate to double (M_PI literals, pow(float, int)),
// the device evaluates in float (values differ by at most a few ulp), except in
// the arguments of sampled directions, which the reference rounds from double
// (2 * M_PI * u): those are evaluated as the reference does. The samplers call
// the correctly rounded functions of crmath.cuh, as the C library rounds; value
// computations (BSDF values, densities, sky lookups) use CUDA's own functions.
#pragma once
#include "crmath.cuh"
#include "xgb_math.cuh"
#include "xgb_types.h"

namespace xgb {

struct Surface {  // SurfaceIntersection (Interaction.h:16-32), world space
    // stan / sbit: the shading tangent frame in object space while makeSurface
    // applies a normal map; afterwards they are only read by MultiLobeSVBRDF, for
    // which makeSurface leaves isect.tangent / bitangent there in world space.
    V3 p, wo, n, sn, stan, sbit;
    float2 uv;
};

// ---------------------------------------------------------------- textures --
__device__ __forceinline__ V3 texAt(const TextureDev& t, int x, int y) {  // Texture.h:77-81, :161-171
    if (t.clamp) {
        x = x < 0 ? 0 : (x > t.w - 1 ? t.w - 1 : x);
        y = y < 0 ? 0 : (y > t.h - 1 ? t.h - 1 : y);
    } else {
        x %= t.w; y %= t.h;
        if (x < 0) x += t.w;
        if (y < 0) y += t.h;
    }
    float4 v = __ldg(&t.texels[(size_t)x + (size_t)y * t.w]);
    return V3(v.x, v.y, v.z);
}
__device__ __forceinline__ V3 texLookup(const TextureDev& t, float u, float v) {  // Texture.h:83-103
    if (t.filter) {
        float fx = u * (float)t.w - 0.5f, fy = v * (float)t.h - 0.5f;
        int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
        int x1 = x0 + 1, y1 = y0 + 1;
        float wx1 = fx - (float)x0, wy1 = fy - (float)y0;
        float wx0 = 1.0f - wx1, wy0 = 1.0f - wy1;
        return (wx0 * wy0) * texAt(t, x0, y0) + (wx0 * wy1) * texAt(t, x0, y1) + (wx1 * wy0) * texAt(t, x1, y0) +
               (wx1 * wy1) * texAt(t, x1, y1);
    }
    return texAt(t, (int)(u * (float)t.w), (int)(v * (float)t.h));
}

// Texture::rgbDifferentialU / V (Texture.h:105-155): central differences of a
// texel, ((rgb(x + 1, y) - rgb(x - 1, y)) / 2) * width, bilinearly weighted like
// rgb(uv). The U derivative addresses rows from 1 - v, the V derivative from v,
// as the reference does (only the red channel is returned).
__device__ __forceinline__ float texDiffUAt(const TextureDev& t, int x, int y) {
    return ((texAt(t, x + 1, y).x - texAt(t, x - 1, y).x) * 0.5f) * (float)t.w;
}
__device__ __forceinline__ float texDiffVAt(const TextureDev& t, int x, int y) {
    return ((texAt(t, x, y + 1).x - texAt(t, x, y - 1).x) * 0.5f) * (float)t.h;
}
template <bool U>
__device__ __forceinline__ float texDiff(const TextureDev& t, float u, float v) {
    const float vv = U ? 1.0f - v : v;
    auto at = [&](int x, int y) { return U ? texDiffUAt(t, x, y) : texDiffVAt(t, x, y); };
    if (t.filter) {
        float fx = u * (float)t.w - 0.5f, fy = vv * (float)t.h - 0.5f;
        int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
        float wx1 = fx - (float)x0, wy1 = fy - (float)y0;
        float wx0 = 1.0f - wx1, wy0 = 1.0f - wy1;
        return (wx0 * wy0) * at(x0, y0) + (wx0 * wy1) * at(x0, y0 + 1) + (wx1 * wy0) * at(x0 + 1, y0) +
               (wx1 * wy1) * at(x0 + 1, y0 + 1);
    }
    return at((int)(u * (float)t.w), (int)(vv * (float)t.h));
}

// ------------------------------------------------------------------- SVNDF --
// VonMisesFisherDistribution<4>::sample (VonMisesFisherDistribution.h:162-201) as
// the reference draws it: lobe by the cumulative weights, tangential part in the
// unit disk (r = sqrt(u)), W from the inverse CDF; L = 5 float4 (lobes, weights).
__device__ __forceinline__ V3 vmf4SampleRef(const float4* L, Pcg& rng) {
    const float4 al = __ldg(&L[4]);
    const float u0 = rng.randf();
    int k = 0;
    float acc = al.x;
    if (!(u0 <= acc)) { k = 1; acc += al.y; if (!(u0 <= acc)) { k = 2; acc += al.z; if (!(u0 <= acc)) k = 3; } }
    const float4 l = __ldg(&L[k]);
    const V3 mu(l.x, l.y, l.z);
    const float kappa = l.w;
    if (mu.x == 0.0f && mu.y == 0.0f && mu.z == 0.0f) return V3(0.0f, 0.0f, 0.0f);
    const float u = rng.randf();
    const float v = rng.randf();
    const float r = sqrtf(u);
    const float theta = (float)((double)(2.0f * kPi * v) - kPiD);
    float st, ct;
    crSinCosf(theta, &st, &ct);
    const float vx = r * ct, vy = r * st;
    const float u2 = rng.randf();
    const float W =
        kappa > 0.0f ? 1.0f + crPowf(kappa, -1.0f) * crLogf(u2 + (1.0f - u2) * crExpf(-2.0f * kappa)) : 1.0f;
    const float sq = safeSqrt(1.0f - W * W);  // powf(W, 2) rounds W^2 once, as the product does
    Basis basis(normalize(mu));
    return normalize(basis.toGlobal(W, sq * vx, sq * vy));
}
// SVNDF::sampleNormal (Prefiltering sandbox Main.cpp:366-388): a stochastic
// bilinear choice of the texel (indices truncated, the y1 wrap compared with
// resolutionU as in the reference, then kept inside the rows that exist).
__device__ __forceinline__ V3 svndfSampleNormal(const SvndfDev& d, float2 uv, Pcg& rng) {
    const float nu = uv.x - floorf(uv.x), nv = uv.y - floorf(uv.y);
    int x0 = (int)(nu * (float)d.resU - 0.5f);
    int y0 = (int)(nv * (float)d.resV - 0.5f);
    int x1 = x0 + 1, y1 = y0 + 1;
    const float wx1 = (nu * (float)d.resU - 0.5f) - (float)x0;
    const float wy1 = (nv * (float)d.resV - 0.5f) - (float)y0;
    if (x0 < 0) x0 = d.resU - 1;
    if (y0 < 0) y0 = d.resV - 1;
    if (x1 >= d.resU) x1 = 0;
    if (y1 >= d.resU) y1 = 0;
    if (y1 >= d.resV) y1 = 0;
    x0 = min(max(x0, 0), d.resU - 1);
    y0 = min(max(y0, 0), d.resV - 1);
    const int x = (rng.randf() <= wx1) ? x1 : x0;
    const int y = (rng.randf() <= wy1) ? y1 : y0;
    return vmf4SampleRef(d.lobes + ((size_t)y * d.resU + x) * 5, rng);
}

// ------------------------------------------------------------------- skies --
__device__ __forceinline__ V3 skyRadiance(const SceneDev& sc, V3 wi) {
    switch (sc.skyKind) {
    case SKY_UNIFORM: return V3(sc.skyColor.x, sc.skyColor.y, sc.skyColor.z);  // SkySphere.h:36-45
    case SKY_PROBE: {  // SkySphereFromImage (SkySphere.h:14-34)
        V3 d = normalize(-wi);
        float sq = sqrtf(d.x * d.x + d.y * d.y);
        if (sq == 0.0f) return V3();
        float r = (1.0f / kPi) * acosf(d.z) / sq;
        float u = (d.x * r + 1.0f) / 2.0f;
        float v = (d.y * r + 1.0f) / 2.0f;
        return texLookup(sc.textures[sc.skyTex], u, v);
    }
    case SKY_LATLONG: {
        float u = atan2f(wi.x, -wi.z) * (0.5f / kPi) + 0.5f;
        float cy = wi.y < -1.0f ? -1.0f : (wi.y > 1.0f ? 1.0f : wi.y);
        float v = acosf(cy) * (1.0f / kPi);
        return texLookup(sc.textures[sc.skyTex], u, v);
    }
    default: return V3();
    }
}

// ------------------------------------------------------------------- Metal --
// horizon = the below-horizon fix (XGB_FIX_METAL_HORIZON; not the reference's
// behaviour): no reflection when wo or wi lies below the shading normal and no
// sample for wo below it (the reference divides by a clamped zero there, which
// microfacet normal mapping's random walk reaches and turns into NaN).
struct MetalD {  // Material.h:275-384
    float alpha;
    V3 f0;
    bool horizon = false;
    __device__ V3 F(V3 eye, V3 h) const { return f0 + (V3(1.0f) - f0) * powf(1 - dot(eye, h), 5.0f); }
    __device__ float D(V3 x, V3 n) const {
        float alpha2 = alpha * alpha;
        float dn = dot(n, x);
        float c2 = dn * dn;
        float c4 = c2 * c2;
        float tan2 = 1 / c2 - 1;
        float s = alpha2 + tan2;
        return alpha2 * (dn > 0 ? 1.0f : 0.0f) / (kPi * c4 * (s * s));
    }
    __device__ float G1(V3 x, V3 n) const {
        float alpha2 = alpha * alpha;
        float dn = dot(n, x);
        float c2 = dn * dn;
        float tan2 = 1 / c2 - 1;
        float lambda = (-1 + safeSqrt(1 + alpha2 * tan2)) / 2;
        return 1 / (1 + lambda);
    }
    __device__ float DV(V3 x, V3 n, V3 eye) const { return G1(eye, n) * clampPositive(dot(eye, x)) * D(x, n) / dot(eye, n); }
    __device__ V3 sampleVNDF(V3 eye, V3 n, Pcg& rng) const {  // [Heitz 2018]
        Basis basis(n);
        V3 Ve = basis.fromGlobal(eye);
        V3 Vh = normalize(V3(Ve.x, alpha * Ve.y, alpha * Ve.z));
        float lensq = Vh.y * Vh.y + Vh.z * Vh.z;
        V3 T1 = lensq > 0 ? V3(0, -Vh.z, Vh.y) / safeSqrt(lensq) : V3(0, 0, 1);
        V3 T2 = cross(Vh, T1);
        float U1 = rng.randf();
        float U2 = rng.randf();
        float r = sqrtf(U1);
        float phi = (float)(2.0 * kPiD * (double)U2);  // 2.0f * M_PI * U2 in double, as the reference
        float sp, cp;
        crSinCosf(phi, &sp, &cp);
        float t1 = r * cp;
        float t2 = r * sp;
        float s = 0.5f * (1.0f + Vh.x);
        t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
        V3 Nh = t1 * T1 + t2 * T2 + safeSqrt(1.0f - t1 * t1 - t2 * t2) * Vh;
        V3 Ne = normalize(V3(clampPositive(Nh.x), alpha * Nh.y, alpha * Nh.z));
        return basis.toGlobal(Ne);
    }
    __device__ V3 bsdfCos(const Surface& s, V3 wi) const {
        if (horizon && (dot(s.wo, s.sn) <= 0.0f || dot(wi, s.sn) <= 0.0f)) return V3(0.0f);
        V3 h = normalize(wi + s.wo);
        V3 Fr = F(s.wo, h);
        float Dv = D(h, s.sn);
        float G = G1(wi, s.sn) * G1(s.wo, s.sn);
        return Fr * Dv * G / clampPositive(4 * dot(s.wo, s.sn));
    }
    __device__ float pdf(const Surface& s, V3 wi) const {
        if (horizon && (dot(s.wo, s.sn) <= 0.0f || dot(wi, s.sn) <= 0.0f)) return 0.0f;
        V3 h = normalize(wi + s.wo);
        if (horizon && !(dot(s.sn, h) > 0.0f && dot(s.wo, h) > 0.0f)) return 0.0f;
        return DV(h, s.sn, s.wo) / (4 * dot(s.wo, h));
    }
    __device__ V3 evalAndSample(const Surface& s, Pcg& rng, V3* wi, float* p) const {
        if (horizon && dot(s.wo, s.sn) <= 0.0f) {
            *wi = s.sn;
            *p = 0.0f;
            return V3(0.0f);
        }
        V3 h = sampleVNDF(s.wo, s.sn, rng);
        *wi = (2.0f * dot(s.wo, h)) * h - s.wo;
        *p = pdf(s, *wi);
        if (horizon && !(*p > 0.0f)) return V3(0.0f);
        return bsdfCos(s, *wi) / *p;
    }
};

// -------------------------------------------------------------- Glossy family --
struct GlossyD {  // Material.h:88-132; clamped: Main.cpp:34-84
    V3 albedo;
    float sh;
    bool clamped;
    __device__ V3 bsdfCos(const Surface& s, V3 wi) const {
        float N = 2 * kPi / (sh + 2);
        if (clamped && !(dot(s.wo, s.sn) > 0.0f && dot(wi, s.sn) > 0.0f)) return V3(0.0f);
        return albedo * powf(dot(normalize(s.wo + wi), s.sn), sh) / N;
    }
    __device__ float pdf(const Surface& s, V3 wi) const {
        if (clamped && !(dot(s.wo, s.sn) > 0.0f && dot(wi, s.sn) > 0.0f)) return 0.0f;
        return (sh + 1) / (2 * kPi) * powf(clampPositive(dot(normalize(s.wo + wi), s.sn)), sh);
    }
    __device__ V3 evalAndSample(const Surface& s, Pcg& rng, V3* wi, float* p) const {
        float r1 = rng.randf();
        float r2 = rng.randf();
        Basis basis(s.sn);
        float sq = safeSqrt(1 - crPowf(r2, 2 / (sh + 1.0f)));
        float sp, cp;
        crSinCosf((float)(2.0 * kPiD * (double)r1), &sp, &cp);  // cosf(2 * M_PI * r1): the argument in double
        V3 h = normalize(basis.toGlobal(crPowf(r2, 1 / (sh + 1.0f)), cp * sq, sp * sq));
        *wi = -normalize(s.wo - (2.0f * dot(s.wo, h)) * h);
        *p = pdf(s, *wi);
        if (*p == 0.0f) return V3(0.0f);
        return bsdfCos(s, *wi) / *p;
    }
};

__device__ __forceinline__ float fresnelDielectric(V3 wo, V3 n, float eta_o, float eta_i) {  // Material.h:265-271
    const float c = fabsf(dot(wo, n));
    float r = eta_o / eta_i;
    float g_sq = r * r - 1.0f + c * c;
    if (g_sq <= 0.0f) return 1.0f;
    float g = sqrtf(g_sq);
    float a = (g - c) / (g + c);
    float b = (c * (g + c) - 1.0f) / (c * (g - c) + 1.0f);
    return 0.5f * (a * a) * (1.0f + b * b);
}

// ------------------------------------------------------- material dispatch --
__device__ __forceinline__ float metalRoughness(const SceneDev& sc, const Material& m, const Surface& s) {
    if (m.tex < 0) return m.roughness;
    return texLookup(sc.textures[m.tex], s.uv.x, s.uv.y).x;
}

// Shade-kernel variants for scenes whose non-emissive materials are all of one
// kind carry only that kind's code: VARIANT bits 8 and 9 (kOnlyDiffuse,
// kOnlyMetal) restrict the basic material switch, bits 0 and 1 are the nested
// materials (see bsdfCosT below). kindOn<V>(k): the code of kind k is compiled in.
constexpr int kOnlyDiffuse = 0x100, kOnlyMetal = 0x200;
// VARIANT bit 10: the scene has no emissive material (and so no lights): the
// shade kernel leaves out emission and next-event estimation.
constexpr int kNoEmitters = 0x400;
template <int V>
__device__ __forceinline__ constexpr bool kindOn(int k) {
    return (V & kOnlyDiffuse) ? k == MAT_DIFFUSE : (V & kOnlyMetal) ? k == MAT_METAL : true;
}

template <int V = 0>
__device__ __forceinline__ V3 bsdfCosBasic(const SceneDev& sc, const Material& m, const Surface& s, V3 wi) {
    if (V & kOnlyDiffuse) {
        V3 a = V3(m.albedo.x, m.albedo.y, m.albedo.z) / kPi;
        if (m.tex >= 0) a = a * texLookup(sc.textures[m.tex], s.uv.x, s.uv.y);
        return m.kind == MAT_DIFFUSE ? a * clampPositive(dot(s.sn, wi)) : V3();
    }
    if (V & kOnlyMetal) {
        if (m.kind != MAT_METAL) return V3();
        float r = metalRoughness(sc, m, s);
        return MetalD{r * r, V3(m.albedo.x, m.albedo.y, m.albedo.z), (m.flags & 1) != 0}.bsdfCos(s, wi);
    }
    switch (m.kind) {
    case MAT_DIFFUSE: {  // Material.h:59-65
        V3 a = V3(m.albedo.x, m.albedo.y, m.albedo.z) / kPi;
        if (m.tex >= 0) a = a * texLookup(sc.textures[m.tex], s.uv.x, s.uv.y);
        return a * clampPositive(dot(s.sn, wi));
    }
    case MAT_METAL: {
        float r = metalRoughness(sc, m, s);
        return MetalD{r * r, V3(m.albedo.x, m.albedo.y, m.albedo.z), (m.flags & 1) != 0}.bsdfCos(s, wi);
    }
    case MAT_GLOSSY: return GlossyD{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, false}.bsdfCos(s, wi);
    case MAT_GLOSSY_CLAMPED: return GlossyD{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, true}.bsdfCos(s, wi);
    case MAT_GLOSSY_HIGHLIGHT:
        return (1.0f - m.rate) * GlossyD{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, false}.bsdfCos(s, wi) +
               m.rate * GlossyD{V3(m.highlight.x, m.highlight.y, m.highlight.z), m.sharpnessHL, false}.bsdfCos(s, wi);
    default: return V3();  // emission and delta BSDFs
    }
}

template <int V = 0>
__device__ __forceinline__ float pdfBasic(const SceneDev& sc, const Material& m, const Surface& s, V3 wi) {
    if (V & kOnlyDiffuse) return m.kind == MAT_DIFFUSE ? clampPositive(dot(wi, s.sn)) / kPi : 0.0f;
    if (V & kOnlyMetal) {
        if (m.kind != MAT_METAL) return 0.0f;
        float r = metalRoughness(sc, m, s);
        return MetalD{r * r, V3(m.albedo.x, m.albedo.y, m.albedo.z), (m.flags & 1) != 0}.pdf(s, wi);
    }
    switch (m.kind) {
    case MAT_DIFFUSE: return clampPositive(dot(wi, s.sn)) / kPi;  // Material.h:78-81
    case MAT_METAL: {
        float r = metalRoughness(sc, m, s);
        return MetalD{r * r, V3(m.albedo.x, m.albedo.y, m.albedo.z), (m.flags & 1) != 0}.pdf(s, wi);
    }
    case MAT_GLOSSY: return GlossyD{V3(), m.sharpness, false}.pdf(s, wi);
    case MAT_GLOSSY_CLAMPED: return GlossyD{V3(), m.sharpness, true}.pdf(s, wi);
    case MAT_GLOSSY_HIGHLIGHT:
        return (1.0f - m.rate) * GlossyD{V3(), m.sharpness, false}.pdf(s, wi) +
               m.rate * GlossyD{V3(), m.sharpnessHL, false}.pdf(s, wi);
    default: return 0.0f;
    }
}

template <int V = 0>
__device__ __forceinline__ V3 sampleBasic(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng, V3* wi,
                                          float* pdf) {
    if ((V & (kOnlyDiffuse | kOnlyMetal)) && !kindOn<V>(m.kind)) {  // not in the scene: never reached
        *wi = s.sn;
        *pdf = 0.0f;
        return V3();
    }
    switch ((V & kOnlyDiffuse) ? (int)MAT_DIFFUSE : (V & kOnlyMetal) ? (int)MAT_METAL : m.kind) {
    case MAT_DIFFUSE: {  // Material.h:67-76, Vector.h:817-824
        Basis basis(s.sn);
        float u = rng.randf() * 1.0f;
        float r = sqrtf(u);
        float phi = rng.randf() * (2.0f * kPi);
        float sp, cp;
        crSinCosf(phi, &sp, &cp);
        *wi = basis.toGlobal(safeSqrt(1.0f - u), r * cp, r * sp);
        *pdf = dot(*wi, s.sn) / kPi;
        V3 a(m.albedo.x, m.albedo.y, m.albedo.z);
        if (m.tex >= 0) a = a * texLookup(sc.textures[m.tex], s.uv.x, s.uv.y);
        return a;
    }
    case MAT_METAL: {
        float r = metalRoughness(sc, m, s);
        return MetalD{r * r, V3(m.albedo.x, m.albedo.y, m.albedo.z), (m.flags & 1) != 0}.evalAndSample(s, rng, wi, pdf);
    }
    case MAT_GLOSSY:
        return GlossyD{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, false}.evalAndSample(s, rng, wi, pdf);
    case MAT_GLOSSY_CLAMPED:
        return GlossyD{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, true}.evalAndSample(s, rng, wi, pdf);
    case MAT_GLOSSY_HIGHLIGHT: {  // Material.h:148-162
        GlossyD base{V3(m.albedo.x, m.albedo.y, m.albedo.z), m.sharpness, false};
        GlossyD hl{V3(m.highlight.x, m.highlight.y, m.highlight.z), m.sharpnessHL, false};
        V3 eval;
        float tmp;
        if (rng.randf() <= m.rate) {
            V3 te = hl.evalAndSample(s, rng, wi, &tmp);
            eval = (1.0f - m.rate) * base.bsdfCos(s, *wi) + m.rate * te;
            *pdf = (1.0f - m.rate) * base.pdf(s, *wi) + m.rate * tmp;
        } else {
            V3 te = base.evalAndSample(s, rng, wi, &tmp);
            eval = (1.0f - m.rate) * te + m.rate * hl.bsdfCos(s, *wi);
            *pdf = (1.0f - m.rate) * tmp + m.rate * hl.pdf(s, *wi);
        }
        return eval;
    }
    case MAT_SPECULAR_REFLECTION:  // Material.h:180-187
        *wi = -normalize(s.wo - (2.0f * dot(s.sn, s.wo)) * s.sn);
        *pdf = -1.0f;
        return V3(1.0f);
    case MAT_SPECULAR_REFRACTION:
    case MAT_SPECULAR_FRESNEL: {  // Material.h:196-250
        float eta_i, eta_o;
        if (dot(s.n, s.wo) > 0.0f) { eta_o = 1.0f; eta_i = m.index; }
        else { eta_o = m.index; eta_i = 1.0f; }
        bool reflect = false;
        if (m.kind == MAT_SPECULAR_FRESNEL) reflect = fresnelDielectric(s.wo, s.sn, eta_o, eta_i) >= rng.randf();
        if (reflect) {
            *wi = -normalize(s.wo - (2.0f * dot(s.sn, s.wo)) * s.sn);
        } else {
            float rindex = eta_o / eta_i;
            float c = dot(-s.wo, s.sn);
            *wi = rindex * (-s.wo - c * s.sn) - safeSqrt(1 - (rindex * rindex) * (1 - c * c)) * s.sn;
        }
        *pdf = -1.0f;
        return V3(1.0f);
    }
    default: return V3();  // Emission: zero, pdf untouched (Material.h:400-402)
    }
}

// ---- MicrofacetNormalMapping, TangentFacetMode = SameMaterialExplicit ------
struct MfnmFrame {
    V3 wg, wp, wt;
    int kind;  // 0: wg == wp (plain base), 1: wt is NaN, 2: full model
};
__device__ __forceinline__ MfnmFrame mfnmFrame(const Surface& s) {  // Main.cpp:97-115
    MfnmFrame f;
    f.wg = s.n;
    f.wp = s.sn;
    if (dot(s.wo, f.wg) < 0.0f) f.wg = f.wg * -1.0f;
    if (dot(f.wg, f.wp) < 0.0f) f.wp = f.wp * -1.0f;
    if (eq(f.wg, f.wp)) { f.kind = 0; return f; }
    f.wt = normalize(cross(normalize(cross(f.wg, f.wp)), f.wg));
    if (hasNan(f.wt)) { f.kind = 1; return f; }
    if (dot(f.wp, f.wt) > 0) f.wt = f.wt * -1.0f;
    f.kind = 2;
    return f;
}
__device__ __forceinline__ float a_p(V3 w, V3 wp, V3 wg) { return clampPositive(dot(w, wp)) / fabsf(dot(wp, wg)); }
__device__ __forceinline__ float a_t(V3 w, V3 wp, V3 wt, V3 wg) {
    float d = dot(wp, wg);
    return clampPositive(dot(w, wt)) * safeSqrt(1 - d * d) / fabsf(d);
}
__device__ __forceinline__ float lambda_p(V3 w, V3 wp, V3 wt, V3 wg) {
    return a_p(w, wp, wg) / (a_p(w, wp, wg) + a_t(w, wp, wt, wg));
}
__device__ __forceinline__ float G1m(V3 w, V3 wm, V3 wp, V3 wt, V3 wg) {
    return dot(w, wm) > 0.0f ? minf_ref(1.0f, clampPositive(dot(w, wg)) / (a_p(w, wp, wg) + a_t(w, wp, wt, wg))) : 0.0f;
}

// MultiLobeSVBRDF::perturbInteraction (Prefiltering sandbox Main.cpp:502-515).
__device__ __forceinline__ Surface svbrdfPerturb(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng) {
    Surface p = s;
    const V3 n = svndfSampleNormal(sc.svndfs[m.tex], s.uv, rng);
    p.sn = normalize(n.z * s.n + n.x * s.stan + n.y * s.sbit);
    return p;
}

// MicrofacetNormalMapping (m.kind == MAT_MF_NORMALMAP) bsdfCos / getPDF / evalAndSample.
__device__ __forceinline__ V3 bsdfCosMfnm(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng, V3 wi) {
    const Material& b = sc.materials[m.base];
    MfnmFrame f = mfnmFrame(s);  // Main.cpp:94-171
    if (f.kind == 0) return bsdfCosBasic(sc, b, s, wi);
    if (f.kind == 1) return V3(0.0f);
    V3 result(0.0f), weight(1.0f);
    bool d = rng.randf() < lambda_p(s.wo, f.wp, f.wt, f.wg);
    V3 wr = -s.wo;
    Surface facet = s;
    int i = 0;
    float pdf;
    while (true) {
        V3 wm = d ? f.wp : f.wt;
        facet.n = wm; facet.sn = wm; facet.wo = -wr;
        result = result + weight * G1m(wi, wm, f.wp, f.wt, f.wg) * bsdfCosBasic(sc, b, facet, wi);
        weight = weight * sampleBasic(sc, b, facet, rng, &wr, &pdf);
        float g = G1m(wr, wm, f.wp, f.wt, f.wg);
        if (rng.randf() < g) break;
        d = !d;
        if (isZero(weight)) break;
        ++i;
        if (i > 100) break;
    }
    return result;
}

__device__ __forceinline__ float getPDFMfnm(const SceneDev& sc, const Material& m, const Surface& s, V3 wi) {
    const Material& b = sc.materials[m.base];
    MfnmFrame f = mfnmFrame(s);  // Main.cpp:254-321
    if (f.kind == 0) return pdfBasic(sc, b, s, wi);
    if (f.kind == 1) return 1.0f;
    float prob = lambda_p(s.wo, f.wp, f.wt, f.wg);
    Surface facet = s;
    float pdf = 0, diff = 0.0f;
    float g_wi_wp = G1m(wi, f.wp, f.wp, f.wt, f.wg);
    if (prob > 0.0f) {
        facet.n = f.wp; facet.sn = f.wp;
        pdf += prob * g_wi_wp * pdfBasic(sc, b, facet, wi);
        diff += prob * (1.0f - g_wi_wp);
    }
    if (prob < 1.0f) {
        facet.n = f.wt; facet.sn = f.wt;
        float g_wi_wt = G1m(wi, f.wt, f.wp, f.wt, f.wg);
        pdf += prob * g_wi_wt * pdfBasic(sc, b, facet, wi);
        diff += prob * g_wi_wt;
    }
    return pdf + diff * clampPositive(dot(wi, f.wg)) / kPi;
}

__device__ __forceinline__ V3 evalAndSampleMfnm(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng,
                                                V3* wi, float* pdf) {
    const Material& b = sc.materials[m.base];
    MfnmFrame f = mfnmFrame(s);  // Main.cpp:173-252
    if (f.kind == 0) return sampleBasic(sc, b, s, rng, wi, pdf);
    if (f.kind == 1) return V3(0.0f);
    V3 weight(1.0f);
    bool d = rng.randf() < lambda_p(s.wo, f.wp, f.wt, f.wg);
    V3 wr = -s.wo;
    Surface facet = s;
    int i = 0;
    float tmppdf = 0.0f;
    bool specular = true;
    while (true) {
        ++i;
        V3 wm = d ? f.wp : f.wt;
        facet.n = wm; facet.sn = wm; facet.wo = -wr;
        weight = weight * sampleBasic(sc, b, facet, rng, &wr, &tmppdf);
        if (tmppdf >= 0.0f) specular = false;
        float g = G1m(wr, wm, f.wp, f.wt, f.wg);
        if (rng.randf() < g) break;
        d = !d;
        if (isZero(weight)) break;
        if (i > 100) { weight = weight * V3(0.0f); break; }
    }
    *wi = wr;
    *pdf = !specular ? getPDFMfnm(sc, m, s, *wi) : -1.0f;
    return V3(0.0f) + weight;
}

__device__ __forceinline__ V3 albedoOf(const SceneDev& sc, const Material& m, const Surface& s) {  // getAlbedo
    switch (m.kind) {
    case MAT_DIFFUSE: {
        V3 a(m.albedo.x, m.albedo.y, m.albedo.z);
        if (m.tex >= 0) a = a * texLookup(sc.textures[m.tex], s.uv.x, s.uv.y);
        return a;
    }
    case MAT_METAL:
    case MAT_GLOSSY:
    case MAT_GLOSSY_HIGHLIGHT: return V3(m.albedo.x, m.albedo.y, m.albedo.z);
    default: return V3();
    }
}

// Material dispatch (Material.h:9-48). NESTED is a mask of the materials that
// evaluate another material which the code is compiled for: 1 microfacet normal
// mapping, 2 MultiLobeSVBRDF; with kOnlyDiffuse or kOnlyMetal (and no nested
// material) the basic switch holds that one kind. The shade kernel is
// instantiated per mask so that a scene only carries the code (and registers)
// of the materials it has.
template <int NESTED>
__device__ __forceinline__ V3 bsdfCosT(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng, V3 wi) {
    if ((NESTED & 2) && m.kind == MAT_MULTILOBE_SVBRDF)  // Main.cpp:489-491
        return bsdfCosBasic(sc, sc.materials[m.base], svbrdfPerturb(sc, m, s, rng), wi);
    if ((NESTED & 1) && m.kind == MAT_MF_NORMALMAP) return bsdfCosMfnm(sc, m, s, rng, wi);
    return bsdfCosBasic<NESTED>(sc, m, s, wi);
}
template <int NESTED>
__device__ __forceinline__ float getPDFT(const SceneDev& sc, const Material& m, const Surface& s, V3 wi) {
    if ((NESTED & 2) && m.kind == MAT_MULTILOBE_SVBRDF)  // Main.cpp:497-499, divided by the double M_PI
        return (float)((double)clampPositive(dot(s.sn, wi)) / kPiD);
    if ((NESTED & 1) && m.kind == MAT_MF_NORMALMAP) return getPDFMfnm(sc, m, s, wi);
    return pdfBasic<NESTED>(sc, m, s, wi);
}
// Returns material_eval = f * cos / pdf and samples wi (Material.h:22-28).
// *pdf is left untouched where the reference leaves it untouched.
template <int NESTED>
__device__ __forceinline__ V3 evalAndSampleT(const SceneDev& sc, const Material& m, const Surface& s, Pcg& rng, V3* wi,
                                             float* pdf) {
    if ((NESTED & 2) && m.kind == MAT_MULTILOBE_SVBRDF)  // Main.cpp:493-495
        return sampleBasic(sc, sc.materials[m.base], svbrdfPerturb(sc, m, s, rng), rng, wi, pdf);
    if ((NESTED & 1) && m.kind == MAT_MF_NORMALMAP) return evalAndSampleMfnm(sc, m, s, rng, wi, pdf);
    return sampleBasic<NESTED>(sc, m, s, rng, wi, pdf);
}

// SurfaceIntersection of a hit (TriangleIndexed.h:128-171 + Object.h:44-85).
__device__ __forceinline__ Surface makeSurface(const SceneDev& sc, const Instance& in, int prim, float b0, float b1,
                                               V3 dWorld) {
    const MeshDev& m = sc.meshes[in.mesh];
    int i0 = m.idx[3 * prim], i1 = m.idx[3 * prim + 1], i2 = m.idx[3 * prim + 2];
    V3 p0 = v3(m.pos[i0]), p1 = v3(m.pos[i1]), p2 = v3(m.pos[i2]);
    V3 dObj = in.identity ? dWorld : xformVector(in.matInv, dWorld);
    Surface s;
    s.uv = m.uv ? lerp3(m.uv[i0], m.uv[i1], m.uv[i2], b0, b1) : make_float2(0.0f, 0.0f);
    s.p = lerp3(p0, p1, p2, b0, b1);
    s.wo = normalize(-dObj);
    s.n = m.nrm ? normalize(lerp3(v3(m.nrm[i0]), v3(m.nrm[i1]), v3(m.nrm[i2]), b0, b1)) : v3(m.gnrm[prim]);
    s.sn = s.n;
    if (m.tan) {
        s.stan = normalize(lerp3(v3(m.tan[i0]), v3(m.tan[i1]), v3(m.tan[i2]), b0, b1));
        s.sbit = normalize(lerp3(v3(m.bit[i0]), v3(m.bit[i1]), v3(m.bit[i2]), b0, b1));
    } else {
        s.stan = V3();
        s.sbit = V3();
    }
    const V3 tanObj = s.stan, bitObj = s.sbit;  // isect.tangent / bitangent before any shading change
    s.sn = faceForward(s.sn, s.wo);
    if (m.shellLayers) {  // TriangleIndexedWithShellMapping::perturbIntersection (TriangleIndexed.h:237-254)
        const TextureDev d{m.shellTexels, m.shellW, m.shellH, m.shellClamp, m.shellFilter};
        V3 a(-texDiff<true>(d, s.uv.x, s.uv.y) * m.shellScale, -texDiff<false>(d, s.uv.x, s.uv.y) * m.shellScale, 1.0f);
        a = normalize(a);
        s.sn = normalize(a.x * s.stan + a.y * s.sbit + a.z * s.sn);
        s.stan = V3();
        s.sbit = V3();
    }
    // object -> world (an identity matrix product is exact, its normalize is not skipped)
    if (!in.identity) s.p = xformPoint(in.mat, s.p);
    s.n = in.identity ? normalize(s.n) : xformNormal(in.mat, s.n);
    s.wo = in.identity ? normalize(s.wo) : xformNormal(in.mat, s.wo);
    const Material& mat = sc.materials[in.material];
    if (mat.normalmap >= 0) {
        V3 nm = texLookup(sc.textures[mat.normalmap], s.uv.x, s.uv.y) * 2.0f - V3(1.0f);
        s.sn = normalize(nm.z * s.sn + nm.x * s.stan + nm.y * s.sbit);
    }
    if (mat.kind == MAT_MULTILOBE_SVBRDF) {  // isect.tangent / bitangent to world space (Object.h:52-57)
        s.stan = isZero(tanObj) ? tanObj : (in.identity ? normalize(tanObj) : xformNormal(in.mat, tanObj));
        s.sbit = isZero(bitObj) ? bitObj : (in.identity ? normalize(bitObj) : xformNormal(in.mat, bitObj));
    }
    s.sn = in.identity ? normalize(s.sn) : xformNormal(in.mat, s.sn);
    return s;
}

}  // namespace xgb
