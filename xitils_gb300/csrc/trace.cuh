// Ray traversal: top-level BVH over instances, per-mesh BVH over triangles.
//
// Semantics follow the reference's Scene::intersect / intersectAny
// (AccelerationStructure.h:94-156, Object.h:44-85, TriangleMesh.h:202-214):
// the ray is moved into object space with the instance's inverse matrix
// (Transform::inverse(Ray), Transform.h:151-153, direction not renormalised, so
// t is shared), triangles are tested with the PBRT watertight test in FP32
// (TriangleIndexed.h:75-177), and a hit is accepted while t <= tMax, tMax
// shrinking to each accepted hit. The triangle test and the ray transform use
// explicitly unfused IEEE operations (__fadd_rn / __fmul_rn), so their results
// are bit-identical to the reference's float arithmetic; only the visiting
// order differs (nearest child first), which changes nothing but ties.
#pragma once
#include "xgb_math.cuh"
#include "xgb_types.h"

namespace xgb {

constexpr int kStackDepth = kMaxStackLimit;  // binary mesh traversal
constexpr int kTlasStack = 16;                // top level over instances
// Loop iterations of one traversal are bounded by SceneDev::maxSteps (a
// well-formed BVH never comes close to the default, 2^22); exceeding it sets
// error bit 4 and ends the traversal. Stack pushes are bounded by
// SceneDev::stackLimit (at most the stacks' size); exceeding it sets error
// bit 1 and ends the traversal.
struct Limits {
    int steps, stack;
};
__device__ __forceinline__ Limits limitsOf(const SceneDev& sc) { return Limits{sc.maxSteps, sc.stackLimit}; }

struct TraceHit {
    float t, b0, b1;
    int prim;  // original triangle index, -1 on a miss
    int inst;
};

struct WorkCount {
    unsigned int nodes = 0;
    unsigned int tris = 0;
};

__device__ __forceinline__ float pick(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

// Per-ray constants of the watertight test (TriangleIndexed.h:83-95).
struct WRay {
    float ox, oy, oz;
    int kx, ky, kz;
    float sx, sy, sz;
    float ix, iy, iz;  // 1 / d for the slab test
};

__device__ __forceinline__ WRay makeWRay(V3 o, V3 d) {
    WRay r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay && ax > az) ? 0 : ((ay > az) ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    r.kx = kx; r.ky = ky; r.kz = kz;
    float dx = pick(d.x, d.y, d.z, kx), dy = pick(d.x, d.y, d.z, ky), dz = pick(d.x, d.y, d.z, kz);
    r.sx = __fdiv_rn(-dx, dz);
    r.sy = __fdiv_rn(-dy, dz);
    r.sz = __fdiv_rn(1.0f, dz);
    r.ix = 1.0f / d.x; r.iy = 1.0f / d.y; r.iz = 1.0f / d.z;
    return r;
}

// TriangleIndexed::intersect, decision and barycentric part.
__device__ __forceinline__ bool watertight(const WRay& r, float4 P0, float4 P1, float4 P2, float tMax, float& t,
                                           float& b0, float& b1) {
    float ax = __fsub_rn(P0.x, r.ox), ay = __fsub_rn(P0.y, r.oy), az = __fsub_rn(P0.z, r.oz);
    float bx = __fsub_rn(P1.x, r.ox), by = __fsub_rn(P1.y, r.oy), bz = __fsub_rn(P1.z, r.oz);
    float cx = __fsub_rn(P2.x, r.ox), cy = __fsub_rn(P2.y, r.oy), cz = __fsub_rn(P2.z, r.oz);
    float p0x = pick(ax, ay, az, r.kx), p0y = pick(ax, ay, az, r.ky), p0z = pick(ax, ay, az, r.kz);
    float p1x = pick(bx, by, bz, r.kx), p1y = pick(bx, by, bz, r.ky), p1z = pick(bx, by, bz, r.kz);
    float p2x = pick(cx, cy, cz, r.kx), p2y = pick(cx, cy, cz, r.ky), p2z = pick(cx, cy, cz, r.kz);
    p0x = __fadd_rn(p0x, __fmul_rn(r.sx, p0z)); p0y = __fadd_rn(p0y, __fmul_rn(r.sy, p0z));
    p1x = __fadd_rn(p1x, __fmul_rn(r.sx, p1z)); p1y = __fadd_rn(p1y, __fmul_rn(r.sy, p1z));
    p2x = __fadd_rn(p2x, __fmul_rn(r.sx, p2z)); p2y = __fadd_rn(p2y, __fmul_rn(r.sy, p2z));
    float e0 = __fsub_rn(__fmul_rn(p1x, p2y), __fmul_rn(p1y, p2x));
    float e1 = __fsub_rn(__fmul_rn(p2x, p0y), __fmul_rn(p2y, p0x));
    float e2 = __fsub_rn(__fmul_rn(p0x, p1y), __fmul_rn(p0y, p1x));
    if ((e0 < 0 || e1 < 0 || e2 < 0) && (e0 > 0 || e1 > 0 || e2 > 0)) return false;
    float det = __fadd_rn(__fadd_rn(e0, e1), e2);
    if (det == 0) return false;
    p0z = __fmul_rn(p0z, r.sz); p1z = __fmul_rn(p1z, r.sz); p2z = __fmul_rn(p2z, r.sz);
    float ts = __fadd_rn(__fadd_rn(__fmul_rn(e0, p0z), __fmul_rn(e1, p1z)), __fmul_rn(e2, p2z));
    float lim = __fmul_rn(tMax, det);
    if (det < 0 && (ts >= 0 || ts < lim)) return false;
    if (det > 0 && (ts <= 0 || ts > lim)) return false;
    float inv = __fdiv_rn(1.0f, det);
    b0 = __fmul_rn(e0, inv);
    b1 = __fmul_rn(e1, inv);
    t = __fmul_rn(ts, inv);
    return true;
}

// Slab test against [lo, hi] for t in [0, tMax]; NaN planes (0 * inf) are
// ignored like the reference's comparisons ignore them (Bounds.h:176-191).
// The far distance is widened by 2^-20 relative so that a box never culls a
// triangle the watertight test would accept.
__device__ __forceinline__ bool slab(const WRay& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                     float tMax, float& tNear) {
    float tx0 = (lx - r.ox) * r.ix, tx1 = (hx - r.ox) * r.ix;
    float ty0 = (ly - r.oy) * r.iy, ty1 = (hy - r.oy) * r.iy;
    float tz0 = (lz - r.oz) * r.iz, tz1 = (hz - r.oz) * r.iz;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tMax));
    tNear = tn;
    return tn <= tf * 1.00000095367431640625f;
}

__device__ __forceinline__ V3 xformPointRn(const float* m, V3 v) {
    float xp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[1], v.y)), __fmul_rn(m[2], v.z)), m[3]);
    float yp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[6], v.z)), m[7]);
    float zp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], v.x), __fmul_rn(m[9], v.y)), __fmul_rn(m[10], v.z)), m[11]);
    float wp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[12], v.x), __fmul_rn(m[13], v.y)), __fmul_rn(m[14], v.z)), m[15]);
    if (wp == 1.0f) return V3(xp, yp, zp);
    float inv = __fdiv_rn(1.0f, wp);
    return V3(__fmul_rn(xp, inv), __fmul_rn(yp, inv), __fmul_rn(zp, inv));
}
__device__ __forceinline__ V3 xformVectorRn(const float* m, V3 v) {
    return V3(__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[1], v.y)), __fmul_rn(m[2], v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[4], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[6], v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[8], v.x), __fmul_rn(m[9], v.y)), __fmul_rn(m[10], v.z)));
}

// ---- 8-wide compressed mesh BVH (WNode, xgb_types.h) ---------------------------
constexpr int kWideStack = 32;  // (node << 8 | remaining hit mask) entries

struct WideHdr {
    unsigned int imask;
    int childBase, triBase;
    unsigned int meta0, meta1;
};

__device__ __forceinline__ int rayOctant(const WRay& r) {
    return (__float_as_uint(r.ix) >> 31) | ((__float_as_uint(r.iy) >> 31) << 1) | ((__float_as_uint(r.iz) >> 31) << 2);
}

__device__ __forceinline__ unsigned int byteOf(unsigned int w, int s) { return (w >> (8 * (s & 3))) & 0xFFu; }

__device__ __forceinline__ void wideHeader(const WNode* nd, WideHdr& h) {
    const float4 a = __ldg(&nd->a), b = __ldg(&nd->b);
    h.imask = __float_as_uint(a.w) >> 24;
    h.childBase = __float_as_int(b.x);
    h.triBase = __float_as_int(b.y);
    h.meta0 = __float_as_uint(b.z);
    h.meta1 = __float_as_uint(b.w);
}

// Tests the eight child boxes of a node; returns the hit children as bits at
// position slot ^ oct (lowest bit first = roughly nearest first).
// Per axis the plane distance is t = q * (2^e / d) + (p - o) / d. The byte q is
// turned into the float Q = 2^23 + q by a byte permute (0x4B0000qq), and the
// 2^23 is folded into the per-node offset, b' = (p - o) / d - 2^23 (2^e / d), so
// that each plane costs one permute and one FMA: t = Q (2^e / d) + b'. Rounding
// b' moves a plane by at most half a quantisation step (or an ulp of the offset
// when that is larger); every plane is moved one more step outwards (near planes
// by -|2^e / d|, far planes by +|2^e / d|, folded into b') and the far distance
// is widened by 2^-20 relative as in slab(), so the test stays conservative. The near plane of each axis is the
// low one for a positive direction component and the high one for a negative
// one. Empty slots hold inverted boxes (low 255, high 0), which no ray accepts,
// so every slot is tested without a branch.
__device__ __forceinline__ unsigned int wideEval(const WNode* nd, const WRay& r, int oct, float tMax, WideHdr& h) {
    const float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c), d = __ldg(&nd->d), e = __ldg(&nd->e);
    const unsigned int bits = __float_as_uint(a.w);
    h.imask = bits >> 24;
    h.childBase = __float_as_int(b.x);
    h.triBase = __float_as_int(b.y);
    h.meta0 = __float_as_uint(b.z);
    h.meta1 = __float_as_uint(b.w);
    const float scx = __uint_as_float((bits & 0xFFu) << 23) * r.ix;
    const float scy = __uint_as_float(((bits >> 8) & 0xFFu) << 23) * r.iy;
    const float scz = __uint_as_float(((bits >> 16) & 0xFFu) << 23) * r.iz;
    const float bx = fmaf(-8388608.0f, scx, (a.x - r.ox) * r.ix);
    const float by = fmaf(-8388608.0f, scy, (a.y - r.oy) * r.iy);
    const float bz = fmaf(-8388608.0f, scz, (a.z - r.oz) * r.iz);
    // one quantisation step of slack outwards on every plane (near planes earlier,
    // far planes later): children that touch the node's own box have no padding
    // step on that side (the byte is clamped at 0 or 255)
    const float nbx = bx - fabsf(scx), fbx = bx + fabsf(scx);
    const float nby = by - fabsf(scy), fby = by + fabsf(scy);
    const float nbz = bz - fabsf(scz), fbz = bz + fabsf(scz);
    const unsigned int lx0 = __float_as_uint(c.x), lx1 = __float_as_uint(c.y);
    const unsigned int ly0 = __float_as_uint(c.z), ly1 = __float_as_uint(c.w);
    const unsigned int lz0 = __float_as_uint(d.x), lz1 = __float_as_uint(d.y);
    const unsigned int hx0 = __float_as_uint(d.z), hx1 = __float_as_uint(d.w);
    const unsigned int hy0 = __float_as_uint(e.x), hy1 = __float_as_uint(e.y);
    const unsigned int hz0 = __float_as_uint(e.z), hz1 = __float_as_uint(e.w);
    const bool fx = oct & 1, fy = oct & 2, fz = oct & 4;
    const unsigned int nx[2] = {fx ? hx0 : lx0, fx ? hx1 : lx1}, xx[2] = {fx ? lx0 : hx0, fx ? lx1 : hx1};
    const unsigned int ny[2] = {fy ? hy0 : ly0, fy ? hy1 : ly1}, xy[2] = {fy ? ly0 : hy0, fy ? ly1 : hy1};
    const unsigned int nz[2] = {fz ? hz0 : lz0, fz ? hz1 : lz1}, xz[2] = {fz ? lz0 : hz0, fz ? lz1 : hz1};
    const float tLim = tMax;
    unsigned int mask = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int w = s >> 2;
        const unsigned int sel = 0x7540u | (unsigned int)(s & 3);
        const float tnx = fmaf(__uint_as_float(__byte_perm(nx[w], 0x4B000000u, sel)), scx, nbx);
        const float tny = fmaf(__uint_as_float(__byte_perm(ny[w], 0x4B000000u, sel)), scy, nby);
        const float tnz = fmaf(__uint_as_float(__byte_perm(nz[w], 0x4B000000u, sel)), scz, nbz);
        const float tfx = fmaf(__uint_as_float(__byte_perm(xx[w], 0x4B000000u, sel)), scx, fbx);
        const float tfy = fmaf(__uint_as_float(__byte_perm(xy[w], 0x4B000000u, sel)), scy, fby);
        const float tfz = fmaf(__uint_as_float(__byte_perm(xz[w], 0x4B000000u, sel)), scz, fbz);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tLim));
        if (tn <= tf * 1.00000095367431640625f) mask |= 1u << (s ^ oct);
    }
    return mask;
}

// ---- shell mapping ---------------------------------------------------------------
// Red channel of the displacement texture at (u, v): Texture::rgb(uv) with its
// clamp / wrap addressing and bilinear or nearest filter (Texture.h:83-103,
// :161-171), in explicitly unfused float operations.
__device__ __forceinline__ float shellTexel(const MeshDev& m, int x, int y) {
    if (m.shellClamp) {
        x = x < 0 ? 0 : (x > m.shellW - 1 ? m.shellW - 1 : x);
        y = y < 0 ? 0 : (y > m.shellH - 1 ? m.shellH - 1 : y);
    } else {
        x %= m.shellW; y %= m.shellH;
        if (x < 0) x += m.shellW;
        if (y < 0) y += m.shellH;
    }
    return __ldg(&m.shellTexels[(size_t)x + (size_t)y * m.shellW]).x;
}
__device__ __forceinline__ float shellRed(const MeshDev& m, float u, float v) {
    const float W = (float)m.shellW, H = (float)m.shellH;
    if (!m.shellFilter) return shellTexel(m, (int)__fmul_rn(u, W), (int)__fmul_rn(v, H));
    const float fx = __fsub_rn(__fmul_rn(u, W), 0.5f), fy = __fsub_rn(__fmul_rn(v, H), 0.5f);
    const int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    const float wx1 = __fsub_rn(fx, (float)x0), wy1 = __fsub_rn(fy, (float)y0);
    const float wx0 = __fsub_rn(1.0f, wx1), wy0 = __fsub_rn(1.0f, wy1);
    float r = __fmul_rn(__fmul_rn(wx0, wy0), shellTexel(m, x0, y0));
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(wx0, wy1), shellTexel(m, x0, y0 + 1)));
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(wx1, wy0), shellTexel(m, x0 + 1, y0)));
    return __fadd_rn(r, __fmul_rn(__fmul_rn(wx1, wy1), shellTexel(m, x0 + 1, y0 + 1)));
}
// TriangleIndexedWithShellMapping::discardByAlpha (TriangleIndexed.h:233-235),
// asked by TriangleIndexed::intersect once the hit is inside [0, tMax]
// (:132-141): the texcoord lerp(uv0, uv1, uv2, b0, b1) (Utils.h:81-83), then
// red < height with height = layer / (layers - 1) (TriangleMesh.h:305-318).
__device__ __noinline__ bool shellDiscard(const MeshDev& m, int prim, float b0, float b1) {
    const int i0 = __ldg(&m.idx[3 * prim]), i1 = __ldg(&m.idx[3 * prim + 1]), i2 = __ldg(&m.idx[3 * prim + 2]);
    const float2 a = __ldg(&m.uv[i0]), b = __ldg(&m.uv[i1]), c = __ldg(&m.uv[i2]);
    const float w = __fsub_rn(__fsub_rn(1.0f, b0), b1);
    const float u = __fadd_rn(__fadd_rn(__fmul_rn(a.x, b0), __fmul_rn(b.x, b1)), __fmul_rn(c.x, w));
    const float v = __fadd_rn(__fadd_rn(__fmul_rn(a.y, b0), __fmul_rn(b.y, b1)), __fmul_rn(c.y, w));
    const float height = __fdiv_rn((float)(prim / m.shellFaces), (float)(m.shellLayers - 1));
    return shellRed(m, u, v) < height;
}

// Watertight tests of `cnt` triangles from `first`; ANY: stops at the first hit.
template <bool ANY>
__device__ __forceinline__ bool testTris(const TriV* tris, int first, int cnt, const WRay& r, float& tMax, TraceHit& hit,
                                         int inst) {
    bool found = false;
    for (int k = 0; k < cnt; ++k) {
        const TriV* tv = tris + first + k;
        const float4 p0 = __ldg(&tv->p0), p1 = __ldg(&tv->p1), p2 = __ldg(&tv->p2);
        float t, b0, b1;
        if (watertight(r, p0, p1, p2, tMax, t, b0, b1)) {
            tMax = t;
            found = true;
            if (ANY) return true;
            hit.t = t; hit.b0 = b0; hit.b1 = b1;
            hit.prim = __float_as_int(p0.w);
            hit.inst = inst;
        }
    }
    return found;
}

// testTris for a mesh that may be shell-mapped (generic traversal path).
template <bool ANY>
__device__ __forceinline__ bool testTrisMesh(const MeshDev& m, int first, int cnt, const WRay& r, float& tMax,
                                             TraceHit& hit, int inst) {
    if (!m.shellLayers) return testTris<ANY>(m.tris, first, cnt, r, tMax, hit, inst);
    bool found = false;
    for (int k = 0; k < cnt; ++k) {
        const TriV* tv = m.tris + first + k;
        const float4 p0 = __ldg(&tv->p0), p1 = __ldg(&tv->p1), p2 = __ldg(&tv->p2);
        float t, b0, b1;
        if (watertight(r, p0, p1, p2, tMax, t, b0, b1) && !shellDiscard(m, __float_as_int(p0.w), b0, b1)) {
            tMax = t;
            found = true;
            if (ANY) return true;
            hit.t = t; hit.b0 = b0; hit.b1 = b1;
            hit.prim = __float_as_int(p0.w);
            hit.inst = inst;
        }
    }
    return found;
}

// Traverses one binary mesh BVH (Node2). ANY: returns at the first accepted hit.
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool traverseBlas2(const MeshDev& m, const WRay& r, float& tMax, TraceHit& hit, int inst,
                                             unsigned int* errors, WorkCount& wc, Limits lim) {
    int stack[kStackDepth];
    int sp = 0;
    int node = m.rootIsLeaf ? m.rootLeaf : 0;
    bool found = false;
    for (int guard = 0;; ++guard) {
        if (guard > lim.steps) { atomicOr(errors, 4u); return found; }
        if (node >= 0) {
            if (COUNT) wc.nodes++;
            const Node2* nd = m.nodes2 + node;
            float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
            int4 d = __ldg(&nd->d);
            float t0, t1;
            bool h0 = slab(r, a.x, a.y, a.z, a.w, b.x, b.y, tMax, t0);
            bool h1 = slab(r, b.z, b.w, c.x, c.y, c.z, c.w, tMax, t1);
            if (h0 && h1) {
                int near = d.x, far = d.y;
                if (t1 < t0) { near = d.y; far = d.x; }
                if (sp >= lim.stack) { atomicOr(errors, 1u); return found; }
                stack[sp++] = far;
                node = near;
            } else if (h0) {
                node = d.x;
            } else if (h1) {
                node = d.y;
            } else {
                if (sp == 0) break;
                node = stack[--sp];
            }
        } else {
            int first = leafFirst(node), cnt = leafCount(node);
            if (COUNT) wc.tris += cnt;
            for (int k = 0; k < cnt; ++k) {
                const TriV* tv = m.tris + first + k;
                float4 p0 = __ldg(&tv->p0), p1 = __ldg(&tv->p1), p2 = __ldg(&tv->p2);
                float t, b0, b1;
                if (watertight(r, p0, p1, p2, tMax, t, b0, b1)) {
                    if (m.shellLayers && shellDiscard(m, __float_as_int(p0.w), b0, b1)) continue;
                    tMax = t;
                    found = true;
                    if (ANY) return true;
                    hit.t = t; hit.b0 = b0; hit.b1 = b1;
                    hit.prim = __float_as_int(p0.w);
                    hit.inst = inst;
                }
            }
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return found;
}

// Traverses one 8-wide mesh BVH (WNode). ANY: returns at the first accepted hit.
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool traverseBlasWide(const MeshDev& m, const WRay& r, float& tMax, TraceHit& hit, int inst,
                                                 unsigned int* errors, WorkCount& wc, Limits lim) {
    if (m.rootIsLeaf) {
        if (COUNT) wc.tris += m.nTris;
        return testTrisMesh<ANY>(m, 0, m.nTris, r, tMax, hit, inst);
    }
    const int oct = rayOctant(r);
    unsigned int stack[kWideStack];
    int sp = 0;
    WideHdr h;
    int node = 0;
    unsigned int mask = wideEval(m.nodes, r, oct, tMax, h);
    if (COUNT) wc.nodes++;
    bool found = false;
    const int stackCap = lim.stack < kWideStack ? lim.stack : kWideStack;
    for (int guard = 0;; ++guard) {
        if (guard > lim.steps) { atomicOr(errors, 4u); return found; }
        if (mask == 0u) {
            if (sp == 0) break;
            const unsigned int e = stack[--sp];
            node = (int)(e >> 8);
            mask = e & 0xFFu;
            wideHeader(m.nodes + node, h);
            continue;
        }
        const int slot = (__ffs(mask) - 1) ^ oct;
        mask &= mask - 1u;
        const unsigned int mb = byteOf(slot >> 2 ? h.meta1 : h.meta0, slot);
        if ((h.imask >> slot) & 1u) {
            if (mask) {
                if (sp >= stackCap) { atomicOr(errors, 1u); return found; }
                stack[sp++] = ((unsigned int)node << 8) | mask;
            }
            node = h.childBase + (int)mb;
            mask = wideEval(m.nodes + node, r, oct, tMax, h);
            if (COUNT) wc.nodes++;
        } else {
            const int cnt = (int)(mb >> 5);
            if (COUNT) wc.tris += cnt;
            if (testTrisMesh<ANY>(m, h.triBase + (int)(mb & 31u), cnt, r, tMax, hit, inst)) {
                found = true;
                if (ANY) return true;
            }
        }
    }
    return found;
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool traverseBlas(const MeshDev& m, const WRay& r, float& tMax, TraceHit& hit, int inst,
                                             unsigned int* errors, WorkCount& wc, Limits lim) {
    return m.wide ? traverseBlasWide<ANY, COUNT>(m, r, tMax, hit, inst, errors, wc, lim)
                  : traverseBlas2<ANY, COUNT>(m, r, tMax, hit, inst, errors, wc, lim);
}

// Scene::intersect (ANY = false) / Scene::intersectAny (ANY = true).
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ bool traceScene(const SceneDev& sc, V3 o, V3 d, float tMax, TraceHit& hit,
                                           unsigned int* errors, WorkCount& wc) {
    hit.prim = -1;
    hit.inst = -1;
    hit.t = tMax;
    WRay wr = makeWRay(o, d);
    const Limits lim = limitsOf(sc);
    const int stackCap = lim.stack < kTlasStack ? lim.stack : kTlasStack;
    int stack[kTlasStack];
    int sp = 0;
    int node = sc.tlasRootIsLeaf ? leafEncode(0, 1) : 0;
    bool found = false;
    for (int guard = 0;; ++guard) {
        if (guard > lim.steps) { atomicOr(errors, 4u); return found; }
        if (node >= 0) {
            if (COUNT) wc.nodes++;
            const Node2* nd = sc.tlas + node;
            float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
            int4 dd = __ldg(&nd->d);
            float t0, t1;
            bool h0 = slab(wr, a.x, a.y, a.z, a.w, b.x, b.y, tMax, t0);
            bool h1 = slab(wr, b.z, b.w, c.x, c.y, c.z, c.w, tMax, t1);
            if (h0 && h1) {
                int near = dd.x, far = dd.y;
                if (t1 < t0) { near = dd.y; far = dd.x; }
                if (sp >= stackCap) { atomicOr(errors, 1u); return found; }
                stack[sp++] = far;
                node = near;
            } else if (h0) {
                node = dd.x;
            } else if (h1) {
                node = dd.y;
            } else {
                if (sp == 0) break;
                node = stack[--sp];
            }
        } else {
            int inst = leafFirst(node);
            const Instance& in = sc.instances[inst];
            const MeshDev& m = sc.meshes[in.mesh];
            bool h;
            if (in.identity) {
                h = traverseBlas<ANY, COUNT>(m, wr, tMax, hit, inst, errors, wc, lim);
            } else {
                V3 oo = xformPointRn(in.matInv, o);
                V3 od = xformVectorRn(in.matInv, d);
                WRay orr = makeWRay(oo, od);
                h = traverseBlas<ANY, COUNT>(m, orr, tMax, hit, inst, errors, wc, lim);
            }
            if (h) {
                found = true;
                if (ANY) return true;
            }
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return found;
}

}  // namespace xgb
