// xgb_cpu — CPU restatement of Xitils' StandardPathTracer and everything on
// its path (BVH, triangles, instancing, materials, lights, camera, sky, film).
//
// TEST INFRASTRUCTURE ONLY (the oracle). It is never linked into, loaded by,
// or called from the product library; only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load it, and only as the checker.
//
// Parity status: pinned. tests/test_oracle_vs_ref.py checks this file against
// the reference's own headers (oracle/_ref, built by oracle/build_ref.py) on the
// same scenes and the same per-(pixel, sample) PCG streams.
//
// Every function restates reference code; each cites the file:line it follows
// (paths relative to the reference repository). Floating-point expressions keep
// the reference's evaluation order and mixed float/double promotions, and the
// file is compiled with -ffp-contract=off so that no FMA contraction happens.
// Vector semantics follow Vector.h: 16-byte lanes with a zero padding lane,
// dot = (x*x' + y*y') + (z*z' + 0) (libsimdpp SSE3 horizontal adds), division by
// a scalar multiplies by its reciprocal (Vector.h:356-361), cross in FP64
// (Vector.h:637-654).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "scene_api.h"

namespace {

#ifdef XGB_ORACLE_ULP_PERTURB
// Sensitivity probe (tests only): every nonzero cosf / sinf / powf / expf / logf /
// asinf result moves one ulp toward zero, the size of the difference between two
// libm implementations (toward zero so that |cos| and |sin| never exceed 1).
inline float towardZero(float r) { return r == 0.0f ? r : std::nextafter(r, 0.0f); }
inline float perturbedCos(float x) { return towardZero(std::cos(x)); }
inline float perturbedSin(float x) { return towardZero(std::sin(x)); }
inline float perturbedPow(float x, float y) { return towardZero(std::pow(x, y)); }
inline float perturbedExp(float x) { return towardZero(std::exp(x)); }
inline float perturbedLog(float x) { return towardZero(std::log(x)); }
inline float perturbedAsin(float x) { return towardZero(std::asin(x)); }
#define cosf perturbedCos
#define sinf perturbedSin
#define powf perturbedPow
#define expf perturbedExp
#define logf perturbedLog
#define asinf perturbedAsin
#endif

#ifdef XGB_ORACLE_CR
// Diagnostic variant (tests only): the float functions selected by the bit mask
// XGB_ORACLE_CR (1 sinf, 2 cosf, 4 powf, 8 expf, 16 logf, 32 asinf, 64 acosf,
// 128 atan2f) return the correctly rounded result, computed in long double and
// rounded once to float, instead of the C library's. Comparing this build with
// the plain one measures how much each library function's misrounded results
// move an image.
inline float crSin(float x) { return (XGB_ORACLE_CR & 1) ? (float)sinl((long double)x) : std::sin(x); }
inline float crCos(float x) { return (XGB_ORACLE_CR & 2) ? (float)cosl((long double)x) : std::cos(x); }
inline float crPow(float x, float y) {
    return (XGB_ORACLE_CR & 4) ? (float)powl((long double)x, (long double)y) : std::pow(x, y);
}
inline float crExp(float x) { return (XGB_ORACLE_CR & 8) ? (float)expl((long double)x) : std::exp(x); }
inline float crLog(float x) { return (XGB_ORACLE_CR & 16) ? (float)logl((long double)x) : std::log(x); }
inline float crAsin(float x) { return (XGB_ORACLE_CR & 32) ? (float)asinl((long double)x) : std::asin(x); }
inline float crAcos(float x) { return (XGB_ORACLE_CR & 64) ? (float)acosl((long double)x) : std::acos(x); }
inline float crAtan2(float y, float x) {
    return (XGB_ORACLE_CR & 128) ? (float)atan2l((long double)y, (long double)x) : std::atan2(y, x);
}
#define sinf crSin
#define cosf crCos
#define powf crPow
#define expf crExp
#define logf crLog
#define asinf crAsin
#define acosf crAcos
#define atan2f crAtan2
#endif

const float kPi = (float)M_PI;  // Utils.h:32
const float kInf = std::numeric_limits<float>::infinity();

// ---------------------------------------------------------------- vectors --
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit V3(float s) : x(s), y(s), z(s) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct V2 {
    float x = 0, y = 0;
    V2() = default;
    V2(float a, float b) : x(a), y(b) {}
};

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return a * s; }  // Vector.h:611-613 (v * val)
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
// Vector.h:356-361: v / s == v * (1 / s)
inline V3 operator/(V3 a, float s) { float inv = (float)1 / s; return a * inv; }
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator*(V2 a, float s) { return {a.x * s, a.y * s}; }
inline V2 operator*(float s, V2 a) { return a * s; }

// Vector.h:628-631 + libsimdpp reduce_add: (l0 + l1) + (l2 + l3), l3 = 0 * 0.
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + 0.0f * 0.0f); }
inline float lengthSq(V3 a) { return dot(a, a); }
inline float length(V3 a) { return sqrtf(dot(a, a)); }    // Vector.h:349-352
inline V3 normalize(V3 a) { return a / length(a); }        // Vector.h:615
inline bool isZero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }  // Vector.h:382-387
inline bool hasNan(V3 a) { return std::isnan(a.x) || std::isnan(a.y) || std::isnan(a.z); }
inline bool eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline int maxDimension(V3 a) { return (a.x > a.y && a.x > a.z) ? 0 : ((a.y > a.z) ? 1 : 2); }  // Vector.h:379
inline V3 permute(V3 a, int x, int y, int z) { return {a[x], a[y], a[z]}; }
inline V3 faceForward(V3 n, V3 v) { return (dot(n, v) < 0.0f) ? -n : n; }  // Vector.h:771
// Vector.h:637-654: both operands widened to double, result rounded to float.
inline V3 cross(V3 a, V3 b) {
    double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return {(float)(ay * bz - az * by), (float)(az * bx - ax * bz), (float)(ax * by - ay * bx)};
}
template <class T> inline T maxT(T a, T b) { return a > b ? a : b; }  // Utils.h:38
template <class T> inline T minT(T a, T b) { return a < b ? a : b; }  // Utils.h:37
inline float clampPositive(float x) { return maxT(x, 0.0f); }  // Utils.h:44
inline V3 clampPositive(V3 v) { return {maxT(v.x, 0.0f), maxT(v.y, 0.0f), maxT(v.z, 0.0f)}; }
inline float safeSqrt(float x) { return sqrtf(clampPositive(x)); }  // Utils.h:89
inline float heaviside(float x) { return x > 0 ? 1.0f : 0.0f; }    // Utils.h:45
// Utils.h:81-83 (lerp of three values with barycentrics t1, t2)
inline V3 lerp3(V3 a, V3 b, V3 c, float t1, float t2) { return t1 * a + t2 * b + (1.0f - t1 - t2) * c; }
inline V2 lerp3(V2 a, V2 b, V2 c, float t1, float t2) { return t1 * a + t2 * b + (1.0f - t1 - t2) * c; }

// Vector.h:781-795
struct Basis {
    V3 e1, e2, e3;
    explicit Basis(V3 v) {
        e1 = normalize(v);
        e2 = normalize(cross(v, std::fabs(v.x) < 0.5f ? V3(1, 0, 0) : (std::fabs(v.y) < 0.5f ? V3(0, 1, 0) : V3(0, 0, 1))));
        e3 = normalize(cross(e1, e2));
    }
    V3 fromGlobal(V3 v) const { return {dot(v, e1), dot(v, e2), dot(v, e3)}; }
    V3 toGlobal(float x, float y, float z) const { return e1 * x + e2 * y + e3 * z; }
    V3 toGlobal(V3 v) const { return e1 * v.x + e2 * v.y + e3 * v.z; }
};

// ------------------------------------------------------------------- RNG --
// Per-(pixel, sample) PCG32 stream. The draw helpers restate Sampler.h:17-32.
inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
struct Rng {
    uint64_t state = 0, inc = 1;
    void seed(uint32_t pixel, uint32_t sample, uint32_t seed) {
        uint64_t initstate = splitmix64(((uint64_t)seed << 32) ^ (uint64_t)sample);
        state = 0;
        inc = ((uint64_t)pixel << 1) | 1u;
        next();
        state += initstate;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((-rot) & 31));
    }
    float randf() { return (float)next() / 0xFFFFFFFF; }   // Sampler.h:17-19
    int randi(int max) { return (int)(next() % (unsigned)max); }  // Sampler.h:30-32
};

// --------------------------------------------------------------- texture --
// Texture.h:11-219 (RGB float, clamp or wrap, bilinear or nearest)
struct Texture {
    int w = 0, h = 0;
    bool clamp = true, filter = true;
    std::vector<float> rgb;
    void warp(int& x, int& y) const {  // Texture.h:161-171
        if (clamp) {
            x = maxT(0, minT(w - 1, x));
            y = maxT(0, minT(h - 1, y));
        } else {
            x %= w; y %= h;
            if (x < 0) x += w;
            if (y < 0) y += h;
        }
    }
    V3 at(int x, int y) const {  // Texture.h:77-81
        warp(x, y);
        size_t i = ((size_t)x + (size_t)y * w) * 3;
        return {rgb[i], rgb[i + 1], rgb[i + 2]};
    }
    V3 lookup(V2 uv) const {  // Texture.h:83-103
        if (filter) {
            int x0 = (int)floorf(uv.x * w - 0.5f);
            int y0 = (int)floorf(uv.y * h - 0.5f);
            int x1 = x0 + 1, y1 = y0 + 1;
            float wx1 = (uv.x * w - 0.5f) - x0;
            float wy1 = (uv.y * h - 0.5f) - y0;
            float wx0 = 1.0f - wx1, wy0 = 1.0f - wy1;
            return wx0 * wy0 * at(x0, y0) + wx0 * wy1 * at(x0, y1) + wx1 * wy0 * at(x1, y0) + wx1 * wy1 * at(x1, y1);
        }
        int x = (int)(uv.x * w);
        int y = (int)(uv.y * h);
        return at(x, y);
    }
    // Texture.h:105-111: central differences scaled by the size
    V3 diffUAt(int x, int y) const { return (at(x + 1, y) - at(x - 1, y)) / 2.0f * (float)w; }
    V3 diffVAt(int x, int y) const { return (at(x, y + 1) - at(x, y - 1)) / 2.0f * (float)h; }
    // Texture.h:113-132: rows addressed from 1 - v
    V3 diffU(V2 uv) const {
        if (filter) {
            int x0 = (int)floorf(uv.x * w - 0.5f);
            int y0 = (int)floorf((1 - uv.y) * h - 0.5f);
            int x1 = x0 + 1, y1 = y0 + 1;
            float wx1 = (uv.x * w - 0.5f) - x0;
            float wy1 = ((1 - uv.y) * h - 0.5f) - y0;
            float wx0 = 1.0f - wx1, wy0 = 1.0f - wy1;
            return wx0 * wy0 * diffUAt(x0, y0) + wx0 * wy1 * diffUAt(x0, y1) + wx1 * wy0 * diffUAt(x1, y0) +
                   wx1 * wy1 * diffUAt(x1, y1);
        }
        return diffUAt((int)(uv.x * w), (int)((1 - uv.y) * h));
    }
    // Texture.h:135-155: rows addressed from v
    V3 diffV(V2 uv) const {
        if (filter) {
            int x0 = (int)floorf(uv.x * w - 0.5f);
            int y0 = (int)floorf(uv.y * h - 0.5f);
            int x1 = x0 + 1, y1 = y0 + 1;
            float wx1 = (uv.x * w - 0.5f) - x0;
            float wy1 = (uv.y * h - 0.5f) - y0;
            float wx0 = 1.0f - wx1, wy0 = 1.0f - wy1;
            return wx0 * wy0 * diffVAt(x0, y0) + wx0 * wy1 * diffVAt(x0, y1) + wx1 * wy0 * diffVAt(x1, y0) +
                   wx1 * wy1 * diffVAt(x1, y1);
        }
        return diffVAt((int)(uv.x * w), (int)(uv.y * h));
    }
};

// --------------------------------------------------------------- geometry --
struct Ray {
    V3 o, d;
    float tMax = kInf;
};

struct Mat4 {
    float m[4][4];
    // Transform.h:61-72 (point), :105-111 (vector), :121-127 (normal)
    V3 point(V3 v) const {
        float xp = m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z + m[0][3];
        float yp = m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z + m[1][3];
        float zp = m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z + m[2][3];
        float wp = m[3][0] * v.x + m[3][1] * v.y + m[3][2] * v.z + m[3][3];
        if (wp == 1) return {xp, yp, zp};
        return V3(xp, yp, zp) / wp;
    }
    V3 vector(V3 v) const {
        return {m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z,
                m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
                m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z};
    }
    V3 normal(V3 v) const { return normalize(vector(v)); }
};

struct Bounds {  // Bounds.h:466-570
    V3 lo{std::numeric_limits<float>::max(), std::numeric_limits<float>::max(), std::numeric_limits<float>::max()};
    V3 hi{std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest()};
    V3 size() const { return hi - lo; }
    V3 center() const { return (hi + lo) / 2; }
    float surfaceArea() const { V3 s = size(); return 2 * s.x * s.y * s.z; }  // Bounds.h:144-147 (sic)
    // Bounds.h:176-191
    bool intersect(const Ray& r) const {
        float t1 = 0, t2 = r.tMax;
        for (int i = 0; i < 3; ++i) {
            float invD = 1.0f / r.d[i];
            float tNear = ((i == 0 ? lo.x : i == 1 ? lo.y : lo.z) - r.o[i]) * invD;
            float tFar = ((i == 0 ? hi.x : i == 1 ? hi.y : hi.z) - r.o[i]) * invD;
            if (tNear > tFar) std::swap(tNear, tFar);
            t1 = tNear > t1 ? tNear : t1;
            t2 = tFar < t2 ? tFar : t2;
            if (t1 > t2) return false;
        }
        return true;
    }
};
inline V3 vmin(V3 a, V3 b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
inline V3 vmax(V3 a, V3 b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }
inline Bounds merge(const Bounds& a, const Bounds& b) { Bounds r; r.lo = vmin(a.lo, b.lo); r.hi = vmax(a.hi, b.hi); return r; }
inline Bounds merge(const Bounds& a, V3 p) { Bounds r; r.lo = vmin(a.lo, p); r.hi = vmax(a.hi, p); return r; }
inline Bounds bounds3(V3 a, V3 b, V3 c) { Bounds r; r.lo = vmin(a, vmin(b, c)); r.hi = vmax(a, vmax(b, c)); return r; }

// Transform.h:155-178: bounds of a transformed box through its 8 corners.
Bounds transformBounds(const Mat4& m, const Bounds& b) {
    V3 size = b.size();
    V3 tmin = m.point(b.lo);
    V3 bx(m.m[0][0], m.m[1][0], m.m[2][0]), by(m.m[0][1], m.m[1][1], m.m[2][1]), bz(m.m[0][2], m.m[1][2], m.m[2][2]);
    V3 vx = bx * size.x, vy = by * size.y, vz = bz * size.z;
    Bounds r; r.lo = tmin; r.hi = tmin;
    r = merge(r, tmin + vx);
    r = merge(r, tmin + vy);
    r = merge(r, tmin + vy + vx);
    r = merge(r, tmin + vz);
    r = merge(r, tmin + vz + vx);
    r = merge(r, tmin + vz + vy);
    r = merge(r, tmin + vz + vy + vx);
    return r;
}

// AccelerationStructure.h:65-293: binary BVH, leaves of one primitive,
// longest-axis centroid sort, median split for <= 8 primitives, else 8
// equal-count buckets scored by SA(b1)*n1 + SA(b2)*n2.
struct BvhNode {
    Bounds aabb;
    int axis = 0;
    int prim = -1;  // leaf primitive, -1 for inner nodes
    int child[2] = {-1, -1};
};
struct Bvh {
    std::vector<BvhNode> nodes;
    struct GeoBounds { int prim; Bounds bound; V3 center; };

    void build(const std::vector<Bounds>& primBounds) {
        int n = (int)primBounds.size();
        std::vector<GeoBounds> gb;
        gb.reserve(n);
        for (int i = 0; i < n; ++i) gb.push_back({i, primBounds[i], primBounds[i].center()});
        nodes.clear();
        nodes.reserve(2 * (size_t)n);
        nodes.push_back(BvhNode());
        Bounds root;
        for (auto& g : gb) root = merge(root, g.bound);
        nodes[0].aabb = root;
        sub(gb.begin(), gb.end(), 0, 0, Bounds());
    }

    void sub(std::vector<GeoBounds>::iterator begin, std::vector<GeoBounds>::iterator end, int node, int depth, Bounds aabb) {
        if (end - begin == 1) {
            nodes[node].prim = begin->prim;
            nodes[node].aabb = begin->bound;
            return;
        }
        if (depth != 0) nodes[node].aabb = aabb;
        int axis = maxDimension(nodes[node].aabb.size());
        nodes[node].axis = axis;
        std::sort(begin, end, [axis](const GeoBounds& a, const GeoBounds& b) { return a.center[axis] < b.center[axis]; });
        int splitIndex = 0;
        Bounds s1, s2;
        int primNum = (int)(end - begin);
        if (primNum <= 8) {
            splitIndex = primNum / 2;
            for (int i = 0; i < splitIndex; ++i) s1 = merge(s1, (begin + i)->bound);
            for (int i = splitIndex; i < primNum; ++i) s2 = merge(s2, (begin + i)->bound);
        } else {
            const int bucketNum = minT(8, primNum);
            std::vector<Bounds> bb, b1, b2;
            std::vector<int> bs, n1, n2;
            int bucketBegin = 0;
            for (int i = 0; i < bucketNum; ++i) {
                Bounds bound;
                int bucketEnd = primNum * (i + 1) / bucketNum;
                for (int k = bucketBegin; k < bucketEnd; ++k) bound = merge(bound, (begin + k)->bound);
                bb.push_back(bound);
                bs.push_back(bucketEnd - bucketBegin);
                bucketBegin = bucketEnd;
            }
            for (int i = 0; i < bucketNum - 1; ++i) {
                b1.push_back(bb[i]); n1.push_back(bs[i]);
                if (i > 0) { b1[i] = merge(b1[i], b1[i - 1]); n1[i] += n1[i - 1]; }
            }
            for (int i = 0; i < bucketNum - 1; ++i) {
                b2.push_back(bb[bucketNum - 1 - i]); n2.push_back(bs[bucketNum - 1 - i]);
                if (i > 0) { b2[i] = merge(b2[i], b2[i - 1]); n2[i] += n2[i - 1]; }
            }
            float best = kInf;
            int bucketIndex = 0;
            for (int i = 0; i < bucketNum - 1; ++i) {
                float sah = b1[i].surfaceArea() * n1[i] + b2[bucketNum - 2 - i].surfaceArea() * n2[bucketNum - 2 - i];
                if (sah < best) { splitIndex = n1[i]; bucketIndex = i; best = sah; }
            }
            s1 = b1[bucketIndex];
            s2 = b2[bucketNum - 2 - bucketIndex];
        }
        int c0 = (int)nodes.size();
        nodes.push_back(BvhNode());
        nodes.push_back(BvhNode());
        nodes[node].child[0] = c0;
        nodes[node].child[1] = c0 + 1;
        sub(begin, begin + splitIndex, c0, depth + 1, s1);
        sub(begin + splitIndex, end, c0 + 1, depth + 1, s2);
    }
};

// ---------------------------------------------------------------- meshes --
struct Mesh {
    std::vector<V3> pos, nrm, tan, bit;
    std::vector<V2> uv;
    std::vector<int32_t> idx;
    int nTris = 0;
    std::vector<float> triArea;  // TriangleIndexed::surfaceArea, TriangleIndexed.h:56-62
    float area = 0;               // TriangleMesh::calcSurfaceArea, TriangleMesh.h:253-258
    Bvh bvh;
    // shell mapping (TriangleMesh.h:279-324): triangle t is face t % shellFaces on layer t / shellFaces
    int shellLayers = 0, shellFaces = 0;
    float shellScale = 0;
    Texture shellTex;

    V3 p(int t, int k) const { return pos[idx[t * 3 + k]]; }

    void build() {
        nTris = (int)idx.size() / 3;
        triArea.resize(nTris);
        std::vector<Bounds> bounds(nTris);
        area = 0.0f;
        for (int t = 0; t < nTris; ++t) {
            V3 p0 = p(t, 0), p1 = p(t, 1), p2 = p(t, 2);
            triArea[t] = length(cross(p1 - p0, p2 - p0)) / 2.0f;
            bounds[t] = bounds3(p0, p1, p2);
            area += triArea[t];
        }
        bvh.build(bounds);
    }
    // TriangleMesh.h:181-187
    Bounds bound() const {
        Bounds r;
        for (auto& q : pos) r = merge(r, q);
        return r;
    }
    // TriangleMesh.h:193-200 and TriangleIndexed.h:64-72
    float areaScaling(const Mat4& t) const {
        float scaled = 0.0f;
        for (int i = 0; i < nTris; ++i) {
            V3 p0 = t.point(p(i, 0)), p1 = t.point(p(i, 1)), p2 = t.point(p(i, 2));
            float s = length(cross(p1 - p0, p2 - p0)) / 2.0f / triArea[i];
            scaled += triArea[i] * s;
        }
        return scaled / area;
    }
};

// ------------------------------------------------------------ intersection --
struct Isect {  // Interaction.h:16-32
    V3 p, wo, n, tangent, bitangent;
    V2 uv;
    V3 sn, stangent, sbitangent;  // shading frame
    int object = -1, tri = -1;
};

// TriangleIndexed.h:75-177 (PBRT watertight test, FP32, no FP64 fallback).
bool intersectTriangle(const Mesh& m, int tri, const Ray& ray, float* tHit, Isect* is) {
    V3 p0 = m.p(tri, 0), p1 = m.p(tri, 1), p2 = m.p(tri, 2);
    V3 p0t = p0 - ray.o, p1t = p1 - ray.o, p2t = p2 - ray.o;
    int kz = maxDimension(vabs(ray.d));
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    V3 d = permute(ray.d, kx, ky, kz);
    p0t = permute(p0t, kx, ky, kz);
    p1t = permute(p1t, kx, ky, kz);
    p2t = permute(p2t, kx, ky, kz);
    float sx = -d.x / d.z, sy = -d.y / d.z, sz = 1.0f / d.z;
    p0t.x += sx * p0t.z; p0t.y += sy * p0t.z;
    p1t.x += sx * p1t.z; p1t.y += sy * p1t.z;
    p2t.x += sx * p2t.z; p2t.y += sy * p2t.z;
    float e0 = p1t.x * p2t.y - p1t.y * p2t.x;
    float e1 = p2t.x * p0t.y - p2t.y * p0t.x;
    float e2 = p0t.x * p1t.y - p0t.y * p1t.x;
    if ((e0 < 0 || e1 < 0 || e2 < 0) && (e0 > 0 || e1 > 0 || e2 > 0)) return false;
    float det = e0 + e1 + e2;
    if (det == 0) return false;
    p0t.z *= sz; p1t.z *= sz; p2t.z *= sz;
    float tScaled = e0 * p0t.z + e1 * p1t.z + e2 * p2t.z;
    if (det < 0 && (tScaled >= 0 || tScaled < ray.tMax * det)) return false;
    if (det > 0 && (tScaled <= 0 || tScaled > ray.tMax * det)) return false;
    float invDet = 1 / det;
    float b0 = e0 * invDet, b1 = e1 * invDet;
    float t = tScaled * invDet;
    int i0 = m.idx[tri * 3], i1 = m.idx[tri * 3 + 1], i2 = m.idx[tri * 3 + 2];
    V2 uv = m.uv.empty() ? V2() : lerp3(m.uv[i0], m.uv[i1], m.uv[i2], b0, b1);
    // TriangleIndexedWithShellMapping::discardByAlpha (TriangleIndexed.h:233-235) with
    // height = layer / (layerNum - 1) (TriangleMesh.h:316); any-hit queries too
    // (Geometry::intersectAny calls intersect, Geometry.h:16-20).
    if (m.shellLayers) {
        float height = (float)(tri / m.shellFaces) / (m.shellLayers - 1);
        if (m.shellTex.lookup(uv).x < height) return false;
    }
    if (!is) { *tHit = t; return true; }
    is->uv = uv;
    *tHit = t;
    is->p = lerp3(p0, p1, p2, b0, b1);
    is->wo = normalize(-ray.d);
    if (!m.nrm.empty()) is->n = normalize(lerp3(m.nrm[i0], m.nrm[i1], m.nrm[i2], b0, b1));
    else is->n = normalize(cross(p1 - p0, p2 - p0));
    is->sn = is->n;
    if (!m.tan.empty()) {
        is->tangent = normalize(lerp3(m.tan[i0], m.tan[i1], m.tan[i2], b0, b1));
        is->bitangent = normalize(lerp3(m.bit[i0], m.bit[i1], m.bit[i2], b0, b1));
    } else {
        is->tangent = V3(); is->bitangent = V3();
    }
    is->stangent = is->tangent;
    is->sbitangent = is->bitangent;
    is->sn = faceForward(is->sn, is->wo);
    is->tri = tri;
    if (m.shellLayers) {  // TriangleIndexedWithShellMapping::perturbIntersection (TriangleIndexed.h:237-254)
        V3 a;
        a.x = -m.shellTex.diffU(is->uv).x * m.shellScale;
        a.y = -m.shellTex.diffV(is->uv).x * m.shellScale;
        a.z = 1;
        a = normalize(a);
        is->sn = normalize(a.x * is->stangent + a.y * is->sbitangent + a.z * is->sn);
        is->stangent = V3();
        is->sbitangent = V3();
    }
    return true;
}

// AccelerationStructure.h:119-137 over a mesh BVH (leaves = triangles)
bool meshIntersect(const Mesh& m, int node, Ray& ray, Isect* is) {
    const BvhNode& n = m.bvh.nodes[node];
    if (!n.aabb.intersect(ray)) return false;
    if (n.prim >= 0) return intersectTriangle(m, n.prim, ray, &ray.tMax, is);
    bool h0, h1;
    if (ray.d[n.axis] > 0) { h0 = meshIntersect(m, n.child[0], ray, is); h1 = meshIntersect(m, n.child[1], ray, is); }
    else { h1 = meshIntersect(m, n.child[1], ray, is); h0 = meshIntersect(m, n.child[0], ray, is); }
    return h0 || h1;
}
// AccelerationStructure.h:139-156; TriangleIndexed uses Geometry::intersectAny (Geometry.h:16-20)
bool meshIntersectAny(const Mesh& m, int node, const Ray& ray) {
    const BvhNode& n = m.bvh.nodes[node];
    if (!n.aabb.intersect(ray)) return false;
    if (n.prim >= 0) { float t; return intersectTriangle(m, n.prim, ray, &t, nullptr); }
    if (ray.d[n.axis] > 0) return meshIntersectAny(m, n.child[0], ray) || meshIntersectAny(m, n.child[1], ray);
    return meshIntersectAny(m, n.child[1], ray) || meshIntersectAny(m, n.child[0], ray);
}

// --------------------------------------------------------------- materials --
struct Material {
    int type = ORC_MAT_DIFFUSE;
    V3 albedo, f0, highlight, power;
    float roughness = 0, sharpness = 0, sharpnessHL = 0, rate = 0, index = 1;
    int tex = -1, normalmap = -1, base = -1;
    int fixes = 0;  // bit 0: Metal below-horizon fix
    bool emissive() const { return type == ORC_MAT_EMISSION; }
};

struct Object {
    int mesh, material;
    Mat4 mat, matInv;
    float areaScaling = 1;
};

struct Scene;

struct Shading {
    const Scene* sc;
    // material dispatch (Material.h:9-48)
    V3 bsdfCos(int mi, const Isect& is, Rng& rng, V3 wi) const;
    V3 evalAndSample(int mi, const Isect& is, Rng& rng, V3* wi, float* pdf) const;
    float getPDF(int mi, const Isect& is, V3 wi) const;
};

// ---- vMF mixture with 4 lobes and the SVNDF of the displacement sandbox ------
// VonMisesFisherDistribution<4> (VonMisesFisherDistribution.h): vMF() (:205-211),
// approximateBySEM (:68-160, E-step without the lobe weights, convergence test on a
// signed difference, both as in the reference) and sample() (:162-201, the
// tangential part drawn in the unit disk, as in the reference).
constexpr int kSvLobes = 4;
struct Vmf4 {
    V3 mu[kSvLobes];
    float kappa[kSvLobes];
    float alpha[kSvLobes];
    Vmf4() {  // VonMisesFisherDistribution() (:21-34)
        for (int i = 0; i < kSvLobes; ++i) { mu[i] = V3(1, 0, 0); kappa[i] = 0.0f; alpha[i] = 0.0f; }
        alpha[0] = 1.0f;
    }
};
inline float vmfLobe(V3 mu, float kappa, V3 omega) {
    if (kappa == 0.0f) return 1.0f / (4 * (float)M_PI);
    return kappa / (2 * (float)M_PI * (1.0f - expf(-2 * kappa))) * expf(kappa * (dot(omega, mu) - 1.0f));
}
Vmf4 vmf4Fit(const std::vector<V3>& samples, Rng& rng) {
    const float KappaLimit = 1000;
    const int StepMax = 100000;
    const float DiffThreshold = 1e-6;
    Vmf4 vmf;
    const int n = (int)samples.size();
    if (n == 1) {
        for (int i = 0; i < kSvLobes; ++i) {
            vmf.mu[i] = samples[0]; vmf.kappa[i] = KappaLimit; vmf.alpha[i] = i == 0 ? 1.0f : 0.0f;
        }
        return vmf;
    }
    for (int j = 0; j < kSvLobes; j++) {
        float u = rng.randf();
        float v = rng.randf();
        float theta = asinf(u);
        float phi = 2.0f * (float)M_PI * v - M_PI;
        vmf.mu[j] = V3(cosf(theta) * cosf(phi), cosf(theta) * sinf(phi), sinf(theta));
        vmf.kappa[j] = 0.5f;
        vmf.alpha[j] = 1.0f / kSvLobes;
    }
    std::vector<float> z((size_t)n * kSvLobes);
    Vmf4 last;
    for (int step = 0; step < StepMax; ++step) {
        for (int i = 0; i < n; i++) {
            float gamma = 0.0f;
            for (int j = 0; j < kSvLobes; j++) gamma += vmfLobe(vmf.mu[j], vmf.kappa[j], samples[i]);
            for (int j = 0; j < kSvLobes; j++)
                z[(size_t)i * kSvLobes + j] = gamma > 0.0f ? vmfLobe(vmf.mu[j], vmf.kappa[j], samples[i]) / gamma : 0.0f;
        }
        for (int j = 0; j < kSvLobes; j++) {
            float a = 0.0f;
            V3 r(0.0f, 0.0f, 0.0f);
            for (int i = 0; i < n; i++) {
                a += z[(size_t)i * kSvLobes + j];
                r = r + z[(size_t)i * kSvLobes + j] * samples[i];
            }
            r = r / a;
            a /= n;
            vmf.alpha[j] = a;
            vmf.kappa[j] = (3 * length(r) - powf(length(r), 3.0f)) / (1.0f - lengthSq(r));
            vmf.mu[j] = normalize(r);
            if (vmf.kappa[j] > KappaLimit) vmf.kappa[j] = KappaLimit;
            if (vmf.kappa[j] < 0.0f) vmf.kappa[j] = 0.0f;
        }
        if (step > 0) {
            float diff = 0.0f;
            for (int j = 0; j < kSvLobes; ++j) {
                diff += lengthSq(vmf.mu[j] - last.mu[j]);
                diff += (vmf.kappa[j] - last.kappa[j]) * 0.1f;
            }
            if (diff < DiffThreshold) break;
        }
        last = vmf;
    }
    return vmf;
}
V3 vmf4Sample(const Vmf4& vmf, Rng& rng) {
    // randiAlongNormalizedWeights (Sampler.h:52-61)
    float uw = rng.randf();
    float accum = 0.0f;
    int k = 0;
    for (; k < kSvLobes - 1; ++k) {
        accum += vmf.alpha[k];
        if (uw <= accum) break;
    }
    const V3 mu = vmf.mu[k];
    const float kappa = vmf.kappa[k];
    if (eq(mu, V3(0, 0, 0))) return V3(0, 0, 0);
    float Vx, Vy, W;
    {
        float u = rng.randf();
        float v = rng.randf();
        float r = sqrtf(u);
        float theta = 2.0f * (float)M_PI * v - M_PI;
        Vx = r * cosf(theta);
        Vy = r * sinf(theta);
    }
    {
        float u = rng.randf();
        if (kappa > 0.0f) W = 1.0f + powf(kappa, -1.0f) * logf(u + (1.0f - u) * std::exp(-2.0f * kappa));
        else W = 1.0f;
    }
    float sq = safeSqrt(1.0f - powf(W, 2.0f));
    Basis basis(normalize(mu));
    return normalize(basis.toGlobal(W, sq * Vx, sq * Vy));
}

// SVNDF of a displacement map (Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/
// Main.cpp:361-389) and its construction by downsampleDisplacementTexture (:391-470):
// low texel (px, py) averages the red channel of its rate x rate source texels and
// fits a 4-lobe mixture to their normals normalize(-dh/du * scale, -dh/dv * scale, 1)
// from Texture::rgbDifferentialU / V at the texel. The reference draws the fit's
// initial lobes from one sampler per OpenMP thread (so which stream a texel gets
// depends on scheduling); here texel t uses the stream seeded (t, 0, seed).
struct Svndf {
    int resU = 0, resV = 0;
    std::vector<Vmf4> vmfs;
    // SVNDF::sampleNormal (:366-388): stochastic bilinear choice of the texel; the
    // y1 wrap compares with resolutionU as the reference does (then clamped to the
    // rows that exist, which only matters for non-square maps).
    V3 sampleNormal(V2 uv, Rng& rng) const {
        float nu = uv.x - floorf(uv.x), nv = uv.y - floorf(uv.y);
        int x0 = (int)(nu * resU - 0.5f);
        int y0 = (int)(nv * resV - 0.5f);
        int x1 = x0 + 1, y1 = y0 + 1;
        float wx1 = (nu * resU - 0.5f) - x0;
        float wy1 = (nv * resV - 0.5f) - y0;
        if (x0 < 0) x0 = resU - 1;
        if (y0 < 0) y0 = resV - 1;
        if (x1 >= resU) x1 = 0;
        if (y1 >= resU) y1 = 0;
        if (y1 >= resV) y1 = 0;
        int x = (rng.randf() <= wx1) ? x1 : x0;
        int y = (rng.randf() <= wy1) ? y1 : y0;
        return vmf4Sample(vmfs[(size_t)y * resU + x], rng);
    }
};
// Returns the low-resolution height texture (red channel; green and blue zero).
Texture svndfFit(const Texture& orig, float scale, int rate, uint32_t seed, Svndf& out) {
    Texture low;
    low.w = (orig.w + rate - 1) / rate;
    low.h = (orig.h + rate - 1) / rate;
    low.clamp = orig.clamp;
    low.filter = true;
    low.rgb.assign((size_t)low.w * low.h * 3, 0.0f);
    out.resU = low.w;
    out.resV = low.h;
    out.vmfs.assign((size_t)low.w * low.h, Vmf4());
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < low.w * low.h; ++t) {
        const int px = t % low.w, py = t / low.w;
        int count = 0;
        float r = 0.0f;
        std::vector<V3> normals;
        for (int ly = 0; ly < rate; ++ly) {
            int y = py * rate + ly;
            if (y >= orig.h) continue;
            for (int lx = 0; lx < rate; ++lx) {
                int x = px * rate + lx;
                if (x >= orig.w) continue;
                float su = orig.diffUAt(x, y).x, sv = orig.diffVAt(x, y).x;
                normals.push_back(normalize(V3(-su * scale, -sv * scale, 1)));
                r += orig.at(x, y).x;
                ++count;
            }
        }
        low.rgb[3 * (size_t)t] = r / count;
        Rng rng;
        rng.seed((uint32_t)t, 0, seed);
        out.vmfs[t] = vmf4Fit(normals, rng);
    }
    return low;
}

struct Scene {
    std::vector<Texture> textures;
    std::vector<Mesh> meshes;
    std::vector<Material> materials;
    std::vector<Object> objects;
    std::vector<int> lights;  // Scene.h:17-22
    Bvh top;
    Mat4 c2w, c2wInv;
    float fov = 1, aspect = 1;
    int skyType = ORC_SKY_NONE;
    V3 skyColor;
    int skyTex = -1;
    int fixes = 0;  // opt-in quirk fixes of the render (xcpu_set_fixes)
    std::vector<Svndf> svndfs;
    bool built = false;
};

// ---- Metal (Material.h:275-384); alpha = roughness^2, roughness from the
// constant or from a roughness texture (nearest lookup of the red channel).
// horizon = the below-horizon fix (not the reference's behaviour, which has
// none): no reflection when wo or wi lies below the shading normal, and no
// sample for wo below it. Inside microfacet normal mapping's random walk the
// reference's Metal otherwise divides by a clamped zero and yields NaN.
struct MetalEval {
    float alpha;
    V3 f0;
    bool horizon = false;
    V3 F(V3 eye, V3 h) const { return f0 + (V3(1.0f) - f0) * powf(1 - dot(eye, h), 5.0f); }
    float D(V3 x, V3 n) const {
        float alpha2 = alpha * alpha;
        float c2 = (float)std::pow(dot(n, x), 2);
        float c4 = c2 * c2;
        float tan2 = 1 / c2 - 1;
        return alpha2 * heaviside(dot(n, x)) / (M_PI * c4 * std::pow(alpha2 + tan2, 2));
    }
    float G1(V3 x, V3 n) const {
        float alpha2 = alpha * alpha;
        float c2 = (float)std::pow(dot(n, x), 2);
        float tan2 = 1 / c2 - 1;
        float lambda = (-1 + safeSqrt(1 + alpha2 * tan2)) / 2;
        return 1 / (1 + lambda);
    }
    float DV(V3 x, V3 n, V3 eye) const { return G1(eye, n) * clampPositive(dot(eye, x)) * D(x, n) / dot(eye, n); }
    V3 sampleVNDF(V3 eye, V3 n, Rng& rng) const {
        Basis basis(n);
        V3 Ve = basis.fromGlobal(eye);
        V3 Vh = normalize(V3(Ve.x, alpha * Ve.y, alpha * Ve.z));
        float lensq = Vh.y * Vh.y + Vh.z * Vh.z;
        V3 T1 = lensq > 0 ? V3(0, -Vh.z, Vh.y) / safeSqrt(lensq) : V3(0, 0, 1);
        V3 T2 = cross(Vh, T1);
        float U1 = rng.randf();
        float U2 = rng.randf();
        float r = sqrtf(U1);
        float phi = 2.0f * M_PI * U2;
        float t1 = r * cosf(phi);
        float t2 = r * sinf(phi);
        float s = 0.5f * (1.0f + Vh.x);
        t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
        V3 Nh = t1 * T1 + t2 * T2 + safeSqrt(1.0f - t1 * t1 - t2 * t2) * Vh;
        V3 Ne = normalize(V3(clampPositive(Nh.x), alpha * Nh.y, alpha * Nh.z));
        return basis.toGlobal(Ne);
    }
    V3 bsdfCos(const Isect& is, V3 wi) const {
        V3 wo = is.wo, n = is.sn;
        if (horizon && (dot(wo, n) <= 0.0f || dot(wi, n) <= 0.0f)) return V3(0.0f);
        V3 h = normalize(wi + wo);
        V3 Fr = F(wo, h);
        float Dv = D(h, n);
        float G = G1(wi, n) * G1(wo, n);
        return Fr * Dv * G / clampPositive(4 * dot(wo, n));
    }
    float pdf(const Isect& is, V3 wi) const {
        V3 wo = is.wo, n = is.sn;
        if (horizon && (dot(wo, n) <= 0.0f || dot(wi, n) <= 0.0f)) return 0.0f;
        V3 h = normalize(wi + wo);
        if (horizon && !(dot(n, h) > 0.0f && dot(wo, h) > 0.0f)) return 0.0f;
        return DV(h, n, wo) / (4 * dot(wo, h));
    }
    V3 evalAndSample(const Isect& is, Rng& rng, V3* wi, float* pdfOut) const {
        V3 wo = is.wo, n = is.sn;
        if (horizon && dot(wo, n) <= 0.0f) {
            *wi = n;
            *pdfOut = 0.0f;
            return V3(0.0f);
        }
        V3 h = sampleVNDF(wo, n, rng);
        *wi = 2 * dot(wo, h) * h - wo;
        *pdfOut = pdf(is, *wi);
        if (horizon && !(*pdfOut > 0.0f)) return V3(0.0f);
        return bsdfCos(is, *wi) / *pdfOut;
    }
};

// ---- Glossy (Material.h:88-132) and GlossyClamped (MicrofacetBasedNormalMapping/Main.cpp:34-84)
struct GlossyEval {
    V3 albedo;
    float s;
    bool clamped;
    V3 bsdfCos(const Isect& is, V3 wi) const {
        V3 n = is.sn;
        float N = 2 * M_PI / (s + 2);
        if (clamped && !(dot(is.wo, n) > 0.0f && dot(wi, n) > 0.0f)) return V3(0.0f);
        return albedo * powf(dot(normalize(is.wo + wi), n), s) / N;
    }
    float pdf(const Isect& is, V3 wi) const {
        V3 n = is.sn;
        if (clamped && !(dot(is.wo, n) > 0.0f && dot(wi, n) > 0.0f)) return 0.0f;
        return (s + 1) / (2 * M_PI) * powf(clampPositive(dot(normalize(is.wo + wi), n)), s);
    }
    V3 evalAndSample(const Isect& is, Rng& rng, V3* wi, float* pdfOut) const {
        float r1 = rng.randf();
        float r2 = rng.randf();
        V3 n = is.sn;
        Basis basis(n);
        float sq = safeSqrt(1 - powf(r2, 2 / (s + 1.0f)));
        V3 h = normalize(basis.toGlobal(powf(r2, 1 / (s + 1.0f)), cosf(2 * M_PI * r1) * sq, sinf(2 * M_PI * r1) * sq));
        *wi = -normalize(is.wo - 2.0f * dot(is.wo, h) * h);
        *pdfOut = pdf(is, *wi);
        if (*pdfOut == 0.0f) return V3(0.0f);
        return bsdfCos(is, *wi) / *pdfOut;
    }
};

float metalRoughness(const Scene& sc, const Material& m, const Isect& is) {
    if (m.tex < 0) return m.roughness;
    return sc.textures[m.tex].lookup(is.uv).x;
}

// Specular Fresnel term (Material.h:265-271)
float fresnelDielectric(V3 wo, V3 n, float eta_o, float eta_i) {
    const float c = fabsf(dot(wo, n));
    float g_sq = powf(eta_o / eta_i, 2.0f) - 1.0f + c * c;
    if (g_sq <= 0.0f) return 1.0f;
    float g = sqrtf(g_sq);
    return 0.5f * powf((g - c) / (g + c), 2.0f) * (1.0f + powf((c * (g + c) - 1.0f) / (c * (g - c) + 1.0f), 2.0f));
}

// ---- MicrofacetNormalMapping (MicrofacetBasedNormalMapping/Main.cpp:86-340),
// TangentFacetMode = SameMaterialExplicit (Main.cpp:24).
struct MfnmFrame {
    V3 wg, wp, wt;
    int kind;  // 0 = plain (wg == wp), 1 = numerical error (wt NaN), 2 = full model
};
MfnmFrame mfnmFrame(const Isect& is) {
    MfnmFrame f;
    V3 wo = is.wo;
    f.wg = is.n;
    f.wp = is.sn;
    if (dot(wo, f.wg) < 0.0f) f.wg = f.wg * -1.0f;
    if (dot(f.wg, f.wp) < 0.0f) f.wp = f.wp * -1.0f;
    if (eq(f.wg, f.wp)) { f.kind = 0; return f; }
    f.wt = normalize(cross(normalize(cross(f.wg, f.wp)), f.wg));
    if (hasNan(f.wt)) { f.kind = 1; return f; }
    if (dot(f.wp, f.wt) > 0) f.wt = f.wt * -1.0f;
    f.kind = 2;
    return f;
}
inline float a_p(V3 w, V3 wp, V3 wg) { return clampPositive(dot(w, wp)) / fabsf(dot(wp, wg)); }
inline float a_t(V3 w, V3 wp, V3 wt, V3 wg) {
    float d = dot(wp, wg);
    return clampPositive(dot(w, wt)) * safeSqrt(1 - powf(d, 2)) / fabsf(d);
}
inline float lambda_p(V3 w, V3 wp, V3 wt, V3 wg) { return a_p(w, wp, wg) / (a_p(w, wp, wg) + a_t(w, wp, wt, wg)); }
inline float G1m(V3 w, V3 wm, V3 wp, V3 wt, V3 wg) {
    return dot(w, wm) > 0.0f ? minT(1.0f, clampPositive(dot(w, wg)) / (a_p(w, wp, wg) + a_t(w, wp, wt, wg))) : 0.0f;
}

// MultiLobeSVBRDF::perturbInteraction (Prefiltering sandbox Main.cpp:502-515): the shading
// normal replaced by a normal drawn from the SVNDF at the texcoord, expressed in the
// frame of the (non-shading) normal, tangent and bitangent.
Isect svbrdfPerturb(const Scene& sc, const Material& m, const Isect& is, Rng& rng) {
    Isect p = is;
    V3 n = sc.svndfs[m.tex].sampleNormal(is.uv, rng);
    p.sn = normalize(n.z * is.n + n.x * is.tangent + n.y * is.bitangent);
    return p;
}

V3 Shading::bsdfCos(int mi, const Isect& is, Rng& rng, V3 wi) const {
    const Material& m = sc->materials[mi];
    switch (m.type) {
    case ORC_MAT_MULTILOBE_SVBRDF:  // Main.cpp:489-491
        return bsdfCos(m.base, svbrdfPerturb(*sc, m, is, rng), rng, wi);
    case ORC_MAT_DIFFUSE:  // Material.h:59-65
        if (m.tex < 0) return m.albedo / M_PI * clampPositive(dot(is.sn, wi));
        return m.albedo / M_PI * sc->textures[m.tex].lookup(is.uv) * clampPositive(dot(is.sn, wi));
    case ORC_MAT_METAL: {
        float r = metalRoughness(*sc, m, is);
        return MetalEval{r * r, m.f0, (m.fixes & 1) != 0}.bsdfCos(is, wi);
    }
    case ORC_MAT_GLOSSY: return GlossyEval{m.albedo, m.sharpness, false}.bsdfCos(is, wi);
    case ORC_MAT_GLOSSY_CLAMPED: return GlossyEval{m.albedo, m.sharpness, true}.bsdfCos(is, wi);
    case ORC_MAT_GLOSSY_HIGHLIGHT:  // Material.h:144-146
        return (1.0f - m.rate) * GlossyEval{m.albedo, m.sharpness, false}.bsdfCos(is, wi) +
               m.rate * GlossyEval{m.highlight, m.sharpnessHL, false}.bsdfCos(is, wi);
    case ORC_MAT_EMISSION: return V3();  // Material.h:396-398
    case ORC_MAT_MF_NORMALMAP: {  // Main.cpp:94-171
        MfnmFrame f = mfnmFrame(is);
        if (f.kind == 0) return bsdfCos(m.base, is, rng, wi);
        if (f.kind == 1) return V3(0.0f);
        V3 result(0.0f), weight(1.0f);
        bool d = rng.randf() < lambda_p(is.wo, f.wp, f.wt, f.wg);
        V3 wr = -is.wo;
        Isect facet = is;
        int i = 0;
        float pdf;
        while (true) {
            V3 wm = d ? f.wp : f.wt;
            facet.n = wm; facet.sn = wm; facet.wo = -wr;
            result = result + weight * G1m(wi, wm, f.wp, f.wt, f.wg) * bsdfCos(m.base, facet, rng, wi);
            weight = weight * evalAndSample(m.base, facet, rng, &wr, &pdf);
            float g = G1m(wr, wm, f.wp, f.wt, f.wg);
            if (rng.randf() < g) break;
            d = !d;
            if (isZero(weight)) break;
            ++i;
            if (i > 100) break;
        }
        return result;
    }
    default: return V3();  // specular materials: delta BSDF (Material.h:15-20)
    }
}

float Shading::getPDF(int mi, const Isect& is, V3 wi) const {
    const Material& m = sc->materials[mi];
    switch (m.type) {
    case ORC_MAT_MULTILOBE_SVBRDF: return clampPositive(dot(is.sn, wi)) / M_PI;  // Main.cpp:497-499
    case ORC_MAT_DIFFUSE: return clampPositive(dot(wi, is.sn)) / M_PI;  // Material.h:78-81
    case ORC_MAT_METAL: {
        float r = metalRoughness(*sc, m, is);
        return MetalEval{r * r, m.f0, (m.fixes & 1) != 0}.pdf(is, wi);
    }
    case ORC_MAT_GLOSSY: return GlossyEval{m.albedo, m.sharpness, false}.pdf(is, wi);
    case ORC_MAT_GLOSSY_CLAMPED: return GlossyEval{m.albedo, m.sharpness, true}.pdf(is, wi);
    case ORC_MAT_GLOSSY_HIGHLIGHT:
        return (1.0f - m.rate) * GlossyEval{m.albedo, m.sharpness, false}.pdf(is, wi) +
               m.rate * GlossyEval{m.highlight, m.sharpnessHL, false}.pdf(is, wi);
    case ORC_MAT_EMISSION: return 0.0f;
    case ORC_MAT_MF_NORMALMAP: {  // Main.cpp:254-321
        MfnmFrame f = mfnmFrame(is);
        if (f.kind == 0) return getPDF(m.base, is, wi);
        if (f.kind == 1) return 1.0f;
        float prob = lambda_p(is.wo, f.wp, f.wt, f.wg);
        Isect facet = is;
        float pdf = 0, diff = 0.0f;
        float g_wi_wp = G1m(wi, f.wp, f.wp, f.wt, f.wg);
        if (prob > 0.0f) {
            facet.n = f.wp; facet.sn = f.wp;
            pdf += prob * g_wi_wp * getPDF(m.base, facet, wi);
            diff += prob * (1.0f - g_wi_wp);
        }
        if (prob < 1.0f) {
            facet.n = f.wt; facet.sn = f.wt;
            float g_wi_wt = G1m(wi, f.wt, f.wp, f.wt, f.wg);
            pdf += prob * g_wi_wt * getPDF(m.base, facet, wi);
            diff += prob * g_wi_wt;
        }
        return pdf + diff * clampPositive(dot(wi, f.wg)) / M_PI;
    }
    default: return 0.0f;
    }
}

V3 Shading::evalAndSample(int mi, const Isect& is, Rng& rng, V3* wi, float* pdf) const {
    const Material& m = sc->materials[mi];
    switch (m.type) {
    case ORC_MAT_MULTILOBE_SVBRDF:  // Main.cpp:493-495
        return evalAndSample(m.base, svbrdfPerturb(*sc, m, is, rng), rng, wi, pdf);
    case ORC_MAT_DIFFUSE: {  // Material.h:67-76, Vector.h:817-824
        V3 n = is.sn;
        Basis basis(n);
        float u = rng.randf() * 1.0f;
        float r = sqrtf(u);
        float phi = rng.randf() * (2.0f * kPi);
        *wi = basis.toGlobal(safeSqrt(1.0f - u), r * cosf(phi), r * sinf(phi));
        *pdf = dot(*wi, n) / M_PI;
        if (m.tex < 0) return m.albedo;
        return m.albedo * sc->textures[m.tex].lookup(is.uv);
    }
    case ORC_MAT_METAL: {
        float r = metalRoughness(*sc, m, is);
        return MetalEval{r * r, m.f0, (m.fixes & 1) != 0}.evalAndSample(is, rng, wi, pdf);
    }
    case ORC_MAT_GLOSSY: return GlossyEval{m.albedo, m.sharpness, false}.evalAndSample(is, rng, wi, pdf);
    case ORC_MAT_GLOSSY_CLAMPED: return GlossyEval{m.albedo, m.sharpness, true}.evalAndSample(is, rng, wi, pdf);
    case ORC_MAT_GLOSSY_HIGHLIGHT: {  // Material.h:148-162
        GlossyEval base{m.albedo, m.sharpness, false}, hl{m.highlight, m.sharpnessHL, false};
        V3 eval;
        if (rng.randf() <= m.rate) {
            float tmp;
            V3 te = hl.evalAndSample(is, rng, wi, &tmp);
            eval = (1.0f - m.rate) * base.bsdfCos(is, *wi) + m.rate * te;
            *pdf = (1.0f - m.rate) * base.pdf(is, *wi) + m.rate * tmp;
        } else {
            float tmp;
            V3 te = base.evalAndSample(is, rng, wi, &tmp);
            eval = (1.0f - m.rate) * te + m.rate * hl.bsdfCos(is, *wi);
            *pdf = (1.0f - m.rate) * tmp + m.rate * hl.pdf(is, *wi);
        }
        return eval;
    }
    case ORC_MAT_SPECULAR_REFLECTION: {  // Material.h:180-187
        V3 wo = is.wo, n = is.sn;
        *wi = -normalize(wo - 2 * dot(n, wo) * n);
        *pdf = -1.0f;
        return V3(1.0f);
    }
    case ORC_MAT_SPECULAR_REFRACTION:  // Material.h:196-216
    case ORC_MAT_SPECULAR_FRESNEL: {   // Material.h:225-250
        V3 wo = is.wo, n = is.sn;
        float eta_i, eta_o;
        if (dot(is.n, wo) > 0.0f) { eta_o = 1.0f; eta_i = m.index; }
        else { eta_o = m.index; eta_i = 1.0f; }
        bool reflect = false;
        if (m.type == ORC_MAT_SPECULAR_FRESNEL) reflect = fresnelDielectric(wo, n, eta_o, eta_i) >= rng.randf();
        if (reflect) {
            *wi = -normalize(wo - 2 * dot(n, wo) * n);
        } else {
            float rindex = eta_o / eta_i;
            float c = dot(-wo, n);
            *wi = rindex * (-wo - c * n) - safeSqrt(1 - powf(rindex, 2) * (1 - powf(c, 2))) * n;
        }
        *pdf = -1.0f;
        return V3(1.0f);
    }
    case ORC_MAT_MF_NORMALMAP: {  // Main.cpp:173-252
        MfnmFrame f = mfnmFrame(is);
        if (f.kind == 0) return evalAndSample(m.base, is, rng, wi, pdf);
        if (f.kind == 1) return V3(0.0f);  // *pdf is left untouched, as in the reference
        V3 result(0.0f), weight(1.0f);
        bool d = rng.randf() < lambda_p(is.wo, f.wp, f.wt, f.wg);
        V3 wr = -is.wo;
        Isect facet = is;
        int i = 0;
        float tmppdf;
        bool specular = true;
        while (true) {
            ++i;
            V3 wm = d ? f.wp : f.wt;
            facet.n = wm; facet.sn = wm; facet.wo = -wr;
            weight = weight * evalAndSample(m.base, facet, rng, &wr, &tmppdf);
            if (tmppdf >= 0.0f) specular = false;
            float g = G1m(wr, wm, f.wp, f.wt, f.wg);
            if (rng.randf() < g) break;
            d = !d;
            if (isZero(weight)) break;
            if (i > 100) { weight = weight * V3(0.0f); break; }
        }
        result = result + weight;
        *wi = wr;
        *pdf = !specular ? getPDF(mi, is, *wi) : -1.0f;
        return result;
    }
    default: return V3();  // Emission (Material.h:400-402): pdf untouched
    }
}

// Emission::getEmission (Material.h:408-410)
V3 emission(const Material& m, V3 wo, V3 n) { return dot(wo, n) > 0.0f ? m.power : V3(); }

// ------------------------------------------------------------------ scene --
// Object::intersect (Object.h:44-85) for the object at a top-level leaf.
bool objectIntersect(const Scene& sc, int oi, Ray& ray, Isect* is) {
    const Object& ob = sc.objects[oi];
    const Mesh& m = sc.meshes[ob.mesh];
    Ray r;  // Transform::inverse(Ray), Transform.h:151-153
    r.o = ob.matInv.point(ray.o);
    r.d = ob.matInv.vector(ray.d);
    r.tMax = ray.tMax;
    Ray rt = r;  // TriangleMesh::intersect copies the ray (TriangleMesh.h:202-210)
    if (!meshIntersect(m, 0, rt, is)) return false;
    ray.tMax = rt.tMax;
    const Mat4& M = ob.mat;
    is->p = M.point(is->p);
    is->n = M.normal(is->n);
    if (!isZero(is->tangent)) is->tangent = M.normal(is->tangent);
    if (!isZero(is->bitangent)) is->bitangent = M.normal(is->bitangent);
    is->wo = M.normal(is->wo);
    const Material& mat = sc.materials[ob.material];
    if (mat.normalmap >= 0) {
        V3 nm = sc.textures[mat.normalmap].lookup(is->uv) * 2 - V3(1.0f);
        is->sn = normalize(nm.z * is->sn + nm.x * is->stangent + nm.y * is->sbitangent);
    }
    is->sn = M.normal(is->sn);
    if (!isZero(is->stangent)) is->stangent = M.normal(is->stangent);
    if (!isZero(is->sbitangent)) is->sbitangent = M.normal(is->sbitangent);
    is->object = oi;
    return true;
}
bool sceneIntersectSub(const Scene& sc, int node, Ray& ray, Isect* is) {
    const BvhNode& n = sc.top.nodes[node];
    if (!n.aabb.intersect(ray)) return false;
    if (n.prim >= 0) return objectIntersect(sc, n.prim, ray, is);
    bool h0, h1;
    if (ray.d[n.axis] > 0) { h0 = sceneIntersectSub(sc, n.child[0], ray, is); h1 = sceneIntersectSub(sc, n.child[1], ray, is); }
    else { h1 = sceneIntersectSub(sc, n.child[1], ray, is); h0 = sceneIntersectSub(sc, n.child[0], ray, is); }
    return h0 || h1;
}
bool sceneIntersect(const Scene& sc, Ray& ray, Isect* is) { return sceneIntersectSub(sc, 0, ray, is); }
bool sceneAnySub(const Scene& sc, int node, const Ray& ray) {
    const BvhNode& n = sc.top.nodes[node];
    if (!n.aabb.intersect(ray)) return false;
    if (n.prim >= 0) {
        const Object& ob = sc.objects[n.prim];
        Ray r;
        r.o = ob.matInv.point(ray.o);
        r.d = ob.matInv.vector(ray.d);
        r.tMax = ray.tMax;
        return meshIntersectAny(sc.meshes[ob.mesh], 0, r);
    }
    if (ray.d[n.axis] > 0) return sceneAnySub(sc, n.child[0], ray) || sceneAnySub(sc, n.child[1], ray);
    return sceneAnySub(sc, n.child[1], ray) || sceneAnySub(sc, n.child[0], ray);
}
bool sceneIntersectAny(const Scene& sc, const Ray& ray) { return sceneAnySub(sc, 0, ray); }

struct LightSample { V3 p, n, sn; int object; };

// Scene::sampleSurface (Scene.h:40-47) -> Object::sampleSurface (Object.h:91-105)
// -> TriangleMesh::sampleSurface (TriangleMesh.h:216-230) -> TriangleIndexed::sampleSurface
// (TriangleIndexed.h:179-209)
LightSample sampleLight(const Scene& sc, Rng& rng, float* pdf) {
    int oi = sc.lights[rng.randi((int)sc.lights.size())];
    const Object& ob = sc.objects[oi];
    const Mesh& m = sc.meshes[ob.mesh];
    int tri = rng.randi(m.nTris);
    float t0, t1, t2, s;
    do {
        t0 = rng.randf(); t1 = rng.randf(); t2 = rng.randf();
        s = t0 + t1 + t2;
    } while (s == 0.0f);
    float inv = 1.0f / s;
    t0 *= inv; t1 *= inv;
    *pdf = 1.0f / m.triArea[tri];
    V3 p0 = m.p(tri, 0), p1 = m.p(tri, 1), p2 = m.p(tri, 2);
    LightSample ls;
    ls.p = lerp3(p0, p1, p2, t0, t1);
    ls.n = normalize(cross(p1 - p0, p2 - p0));
    if (m.nrm.empty()) ls.sn = ls.n;
    else {
        int i0 = m.idx[tri * 3], i1 = m.idx[tri * 3 + 1], i2 = m.idx[tri * 3 + 2];
        ls.sn = normalize(lerp3(m.nrm[i0], m.nrm[i1], m.nrm[i2], t0, t1));
    }
    *pdf /= m.nTris;
    *pdf /= ob.areaScaling;
    ls.p = ob.mat.point(ls.p);
    ls.n = ob.mat.normal(ls.n);
    ls.sn = ob.mat.normal(ls.sn);
    ls.object = oi;
    *pdf /= sc.lights.size();
    return ls;
}
// Scene::surfacePDF (Scene.h:49-55) -> Object::surfacePDF (Object.h:107-110)
// -> TriangleMesh::surfacePDF (TriangleMesh.h:232-235)
float surfacePDF(const Scene& sc, const Isect& is) {
    if (sc.lights.empty()) return 0.0f;
    const Object& ob = sc.objects[is.object];
    const Mesh& m = sc.meshes[ob.mesh];
    float p = 1.0f / m.triArea[is.tri] / m.nTris;
    return p / ob.areaScaling / sc.lights.size();
}

// SkySphere.h:20-45, plus a lat-long map (the reference's SkySphere is a
// virtual interface, SkySphere.h:9-12; the lat-long subclass is this project's).
V3 skyRadiance(const Scene& sc, V3 wi) {
    switch (sc.skyType) {
    case ORC_SKY_UNIFORM: return sc.skyColor;
    case ORC_SKY_PROBE: {
        V3 d = normalize(-wi);
        float sq = sqrtf(d.x * d.x + d.y * d.y);
        if (sq == 0.0f) return V3();
        float r = (1.0f / M_PI) * acosf(d.z) / sq;
        float u = (d.x * r + 1.0f) / 2.0f;
        float v = (d.y * r + 1.0f) / 2.0f;
        return sc.textures[sc.skyTex].lookup(V2(u, v));
    }
    case ORC_SKY_LATLONG: {
        float u = atan2f(wi.x, -wi.z) * (0.5f / kPi) + 0.5f;
        float cy = wi.y < -1.0f ? -1.0f : (wi.y > 1.0f ? 1.0f : wi.y);
        float v = acosf(cy) * (1.0f / kPi);
        return sc.textures[sc.skyTex].lookup(V2(u, v));
    }
    default: return V3();
    }
}

struct Params {
    int integrator, maxDepth, rrStart;
    float rrProb;
};
const float kRayOffset = 0.00001f;     // PathTracer.h:254
const float kShadowMargin = 0.0001f;   // PathTracer.h:257

// radiance + c, or radiance alone when the drop-non-finite fix is on and c has
// a non-finite component (the reference adds it, and the pixel becomes NaN).
V3 addContribution(const Scene& sc, V3 radiance, V3 c) {
    if ((sc.fixes & 2) && !(std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z))) return radiance;
    return radiance + c;
}

// Material::getAlbedo (Material.h:44-47, 83-85, 129-131, 168-170, 380-382):
// Diffuse albedo (times its texture), Glossy albedo, GlossyWithHighLight its
// base's albedo, Metal f0; every other material (the sandbox's GlossyClamped
// and MicrofacetNormalMapping included) keeps the zero default.
V3 albedoOf(const Scene& sc, const Material& m, const Isect& is) {
    switch (m.type) {
    case ORC_MAT_DIFFUSE: return m.tex < 0 ? m.albedo : m.albedo * sc.textures[m.tex].lookup(is.uv);
    case ORC_MAT_GLOSSY:
    case ORC_MAT_GLOSSY_HIGHLIGHT: return m.albedo;
    case ORC_MAT_METAL: return m.f0;
    default: return V3(0.0f);
    }
}

// StandardPathTracer::eval (PathTracer.h:117-251) with two additions that the
// reference hard-codes: rrStart / rrProb (its russianRouletteLengthMin = 5,
// russianRouletteProb = 0.9) and maxDepth (0 = unlimited, as in the reference:
// the loop stops before vertex pathLength when pathLength > maxDepth).
// aov (optional): albedo and normal of the first hit (PathTracer.h:138-139).
V3 evalStandard(const Scene& sc, const Params& P, Rng& rng, Ray ray, V3* aov = nullptr) {
    Shading sh{&sc};
    V3 radiance(0.0f), weight(1.0f);
    Isect isect, next;
    int pathLength = 1;
    bool canSampleLight = !sc.lights.empty();
    if (!sceneIntersect(sc, ray, &isect)) {
        if (sc.skyType != ORC_SKY_NONE) radiance = addContribution(sc, radiance, weight * skyRadiance(sc, ray.d));
        return radiance;
    }
    ++pathLength;
    const Material* mat = &sc.materials[sc.objects[isect.object].material];
    if (aov) {
        aov[0] = albedoOf(sc, *mat, isect);
        aov[1] = isect.n;
    }
    if (mat->emissive()) radiance = addContribution(sc, radiance, weight * emission(*mat, -ray.d, isect.n));
    while (true) {
        // An emitter's evalAndSample returns zero (Material.h:400-402): the
        // reference ends the path after an NEE step whose contribution is
        // multiplied by Emission::bsdfCos() == 0. Ending here is equivalent.
        if (mat->emissive()) break;
        if (P.maxDepth > 0 && pathLength > P.maxDepth) break;
        if (pathLength > P.rrStart) {
            if (rng.randf() >= P.rrProb) break;
            weight = weight / P.rrProb;
        }
        bool nextSampled = true;
        float pdfBsdf = 0;
        int mi = sc.objects[isect.object].material;
        V3 f = sh.evalAndSample(mi, isect, rng, &ray.d, &pdfBsdf);
        if (!isZero(f)) {
            ray.o = isect.p + kRayOffset * ray.d;
            ray.tMax = kInf;
            if (sceneIntersect(sc, ray, &next)) {
                const Material& nm = sc.materials[sc.objects[next.object].material];
                if (nm.emissive()) {
                    float mis;
                    if (pdfBsdf >= 0.0f && canSampleLight) {
                        float pl = surfacePDF(sc, next);
                        float cosLight = fabsf(dot(ray.d, next.sn));
                        float distSq = powf(ray.tMax, 2.0f);
                        pl *= distSq / cosLight;
                        mis = powf(pdfBsdf, 2.0f) / (powf(pdfBsdf, 2.0f) + powf(pl, 2.0f));
                    } else {
                        mis = 1.0f;
                    }
                    if (mis > 0.0f) radiance = addContribution(sc, radiance, weight * mis * f * emission(nm, -ray.d, next.n));
                }
            } else {
                if (sc.skyType != ORC_SKY_NONE) radiance = addContribution(sc, radiance, weight * f * skyRadiance(sc, ray.d));
                nextSampled = false;
            }
        }
        if (canSampleLight) {  // PathTracer.h:202-233
            float pl;
            LightSample ls = sampleLight(sc, rng, &pl);
            float dist = length(ls.p - isect.p);
            Ray sray;
            sray.d = (ls.p - isect.p) / dist;
            sray.o = isect.p + kRayOffset * sray.d;
            sray.tMax = dist - kShadowMargin;
            if (dot(sray.d, ls.n) < 0 && !sceneIntersectAny(sc, sray)) {
                float mis;
                float distSq = powf(dist, 2.0f);
                if (pdfBsdf >= 0.0f) {
                    float pb = sh.getPDF(mi, isect, sray.d);
                    float cosLight = fabsf(dot(-sray.d, ls.sn));
                    pb *= cosLight / distSq;
                    mis = powf(pl, 2.0f) / (powf(pb, 2.0f) + powf(pl, 2.0f));
                } else {
                    mis = 0.0f;
                }
                if (mis > 0.0f) {
                    float G = fabsf(dot(-sray.d, ls.sn)) / distSq;
                    const Material& lm = sc.materials[sc.objects[ls.object].material];
                    radiance = addContribution(sc, radiance, weight * mis * sh.bsdfCos(mi, isect, rng, sray.d) * emission(lm, -sray.d, ls.n) * G / pl);
                }
            }
        }
        if (!nextSampled) break;
        isect = next;
        weight = weight * f;
        ++pathLength;
        if (isZero(weight)) break;
        mat = &sc.materials[sc.objects[isect.object].material];
    }
    return radiance;
}

// NaivePathTracer::eval (PathTracer.h:50-104), same parameter additions.
// aov (optional): albedo and normal of the first hit (PathTracer.h:76-80).
V3 evalNaive(const Scene& sc, const Params& P, Rng& rng, Ray ray, V3* aov = nullptr) {
    Shading sh{&sc};
    V3 radiance(0.0f), weight(1.0f);
    Isect isect;
    int pathLength = 1;
    V3 wi;
    while (true) {
        if (P.maxDepth > 0 && pathLength > P.maxDepth) break;
        if (pathLength > P.rrStart) {
            if (rng.randf() >= P.rrProb) break;
            weight = weight / P.rrProb;
        }
        if (sceneIntersect(sc, ray, &isect)) {
            const Material& m = sc.materials[sc.objects[isect.object].material];
            if (aov && pathLength == 1) {
                aov[0] = albedoOf(sc, m, isect);
                aov[1] = isect.n;
            }
            if (m.emissive()) radiance = addContribution(sc, radiance, weight * emission(m, -ray.d, isect.n));
            float pdf;
            weight = weight * sh.evalAndSample(sc.objects[isect.object].material, isect, rng, &wi, &pdf);
            if (isZero(weight)) break;
            ray.d = wi;
            ray.o = isect.p + kRayOffset * ray.d;
            ray.tMax = kInf;
        } else if (sc.skyType != ORC_SKY_NONE) {
            radiance = addContribution(sc, radiance, clampPositive(weight * skyRadiance(sc, ray.d)));
            break;
        } else {
            // The reference loops forever here (no sky, miss); a miss ends the path.
            break;
        }
        ++pathLength;
    }
    return radiance;
}

// PinholeCamera::generateRay (Camera.h:45-55) with Transform::operator()(Ray).
Ray cameraRay(const Scene& sc, float fx, float fy) {
    Ray r;
    V3 d = normalize(V3(tanf(sc.fov / 2) * (fx - 0.5f) * 2, tanf(sc.fov / 2 * sc.aspect) * (fy - 0.5f) * 2, 1));
    r.o = sc.c2w.point(V3(0, 0, 0));
    r.d = sc.c2w.vector(d);
    r.tMax = kInf;
    return r;
}

}  // namespace

#if defined(XGB_ORACLE_ULP_PERTURB) || defined(XGB_ORACLE_CR)
#undef cosf
#undef sinf
#undef powf
#undef expf
#undef logf
#undef asinf
#endif
#ifdef XGB_ORACLE_CR
#undef acosf
#undef atan2f
#endif

// ------------------------------------------------------------------ C API --
extern "C" {
ORC_DECLARE_SCENE_API(xcpu_)

void* xcpu_scene_new(void) { return new Scene(); }
void xcpu_scene_free(void* s) { delete (Scene*)s; }

int xcpu_add_texture(void* s, int w, int h, const float* rgb, int wrap_clamp, int filter) {
    Scene* sc = (Scene*)s;
    if (w <= 0 || h <= 0 || !rgb) return -1;
    Texture t;
    t.w = w; t.h = h; t.clamp = wrap_clamp != 0; t.filter = filter != 0;
    t.rgb.assign(rgb, rgb + (size_t)w * h * 3);
    sc->textures.push_back(std::move(t));
    return (int)sc->textures.size() - 1;
}

int xcpu_add_mesh(void* s, int nV, const float* pos, const float* uv, const float* nrm, const float* tan,
                  const float* bit, int nIdx, const int32_t* idx) {
    Scene* sc = (Scene*)s;
    if (nV <= 0 || !pos || nIdx <= 0 || nIdx % 3 || !idx) return -1;
    for (int i = 0; i < nIdx; ++i) if (idx[i] < 0 || idx[i] >= nV) return -1;
    Mesh m;
    auto v3 = [&](const float* a, std::vector<V3>& out) {
        if (!a) return;
        out.resize(nV);
        for (int i = 0; i < nV; ++i) out[i] = V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    };
    v3(pos, m.pos); v3(nrm, m.nrm); v3(tan, m.tan); v3(bit, m.bit);
    if (uv) { m.uv.resize(nV); for (int i = 0; i < nV; ++i) m.uv[i] = V2(uv[2 * i], uv[2 * i + 1]); }
    if (!m.tan.empty() && m.bit.empty()) return -1;
    m.idx.assign(idx, idx + nIdx);
    m.build();
    sc->meshes.push_back(std::move(m));
    return (int)sc->meshes.size() - 1;
}

// TriangleMesh::setGeometryWithShellMapping (TriangleMesh.h:163-177) and
// buildTrianglesWithShellMapping (:279-324).
int xcpu_add_mesh_shell(void* s, int nV, const float* pos, const float* uv, const float* nrm, const float* tan,
                        const float* bit, int nIdx, const int32_t* idx, int tex, float scale, int layers) {
    Scene* sc = (Scene*)s;
    if (nV <= 0 || !pos || !uv || !nrm || !tan || !bit || nIdx <= 0 || nIdx % 3 || !idx || layers < 1) return -1;
    if (tex < 0 || tex >= (int)sc->textures.size()) return -1;
    for (int i = 0; i < nIdx; ++i) if (idx[i] < 0 || idx[i] >= nV) return -1;
    Mesh m;
    const size_t V = (size_t)nV;
    m.pos.resize(V * layers); m.nrm.resize(V * layers); m.tan.resize(V * layers); m.bit.resize(V * layers);
    m.uv.resize(V * layers);
    for (size_t i = 0; i < V; ++i) {
        m.pos[i] = V3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        m.nrm[i] = V3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        m.tan[i] = V3(tan[3 * i], tan[3 * i + 1], tan[3 * i + 2]);
        m.bit[i] = V3(bit[3 * i], bit[3 * i + 1], bit[3 * i + 2]);
        m.uv[i] = V2(uv[2 * i], uv[2 * i + 1]);
    }
    m.idx.resize((size_t)nIdx * layers);
    for (int i = 0; i < nIdx; ++i) m.idx[i] = idx[i];
    for (int layer = 1; layer < layers; ++layer) {
        for (size_t i = 0; i < V; ++i) {
            float d = scale * layer / (layers - 1);
            m.pos[layer * V + i] = m.pos[i] + d * m.nrm[i];
            m.uv[layer * V + i] = m.uv[i];
            m.nrm[layer * V + i] = m.nrm[i];
            m.tan[layer * V + i] = m.tan[i];
            m.bit[layer * V + i] = m.bit[i];
        }
        for (int i = 0; i < nIdx; ++i) m.idx[(size_t)layer * nIdx + i] = idx[i] + layer * nV;
    }
    m.shellLayers = layers;
    m.shellFaces = nIdx / 3;
    m.shellScale = scale;
    m.shellTex = sc->textures[tex];
    m.build();
    sc->meshes.push_back(std::move(m));
    return (int)sc->meshes.size() - 1;
}

int xcpu_add_svndf(void* s, int tex, float scale, int rate, uint32_t seed, int* low_tex) {
    Scene* sc = (Scene*)s;
    if (tex < 0 || tex >= (int)sc->textures.size() || rate < 1 || !low_tex) return -1;
    Svndf sv;
    Texture low = svndfFit(sc->textures[tex], scale, rate, seed, sv);
    sc->textures.push_back(std::move(low));
    *low_tex = (int)sc->textures.size() - 1;
    sc->svndfs.push_back(std::move(sv));
    return (int)sc->svndfs.size() - 1;
}

// Stand-alone fit for tests: low red channel [ceil(h/rate)][ceil(w/rate)] and, per low
// texel, 4 lobes x (mu.xyz, kappa, alpha).
int xcpu_svndf_fit(const float* rgb, int w, int h, int wrap_clamp, float scale, int rate, uint32_t seed,
                   float* low_r, float* lobes) {
    if (!rgb || w <= 0 || h <= 0 || rate < 1) return -1;
    Texture t;
    t.w = w; t.h = h; t.clamp = wrap_clamp != 0; t.filter = true;
    t.rgb.assign(rgb, rgb + (size_t)w * h * 3);
    Svndf sv;
    Texture low = svndfFit(t, scale, rate, seed, sv);
    for (size_t i = 0; i < sv.vmfs.size(); ++i) {
        low_r[i] = low.rgb[3 * i];
        for (int j = 0; j < kSvLobes; ++j) {
            float* o = lobes + (i * kSvLobes + j) * 5;
            o[0] = sv.vmfs[i].mu[j].x; o[1] = sv.vmfs[i].mu[j].y; o[2] = sv.vmfs[i].mu[j].z;
            o[3] = sv.vmfs[i].kappa[j]; o[4] = sv.vmfs[i].alpha[j];
        }
    }
    return 0;
}

// Directions drawn from a 4-lobe mixture (lobes: 4 x (mu.xyz, kappa, alpha)), one PCG
// stream (i, 0, seed) per draw.
int xcpu_vmf4_sample_pcg(const float* lobes, int n, uint32_t seed, float* dirs) {
    Vmf4 v;
    for (int j = 0; j < kSvLobes; ++j) {
        v.mu[j] = V3(lobes[5 * j], lobes[5 * j + 1], lobes[5 * j + 2]);
        v.kappa[j] = lobes[5 * j + 3]; v.alpha[j] = lobes[5 * j + 4];
    }
    for (int i = 0; i < n; ++i) {
        Rng rng;
        rng.seed((uint32_t)i, 0, seed);
        V3 d = vmf4Sample(v, rng);
        dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    }
    return 0;
}

// Flat shading point of the per-material queries (scene_api.h).
static Isect flatIsect(const float* wo) {
    Isect is;
    is.p = V3(0, 0, 0);
    is.wo = V3(wo[0], wo[1], wo[2]);
    is.n = is.sn = V3(0, 0, 1);
    is.tangent = is.stangent = V3(1, 0, 0);
    is.bitangent = is.sbitangent = V3(0, 1, 0);
    is.uv = V2(0.5f, 0.5f);
    return is;
}

static bool specularKind(int type) {
    return type == ORC_MAT_SPECULAR_REFLECTION || type == ORC_MAT_SPECULAR_REFRACTION ||
           type == ORC_MAT_SPECULAR_FRESNEL || type == ORC_MAT_EMISSION;
}

int xcpu_bsdf_sample_pcg(void* s, int material, const float* wo, int n, uint32_t seed, float* out) {
    const Scene* sc = (const Scene*)s;
    if (!sc || !wo || !out || n < 0 || material < 0 || material >= (int)sc->materials.size()) return -1;
    const Isect is = flatIsect(wo);
    const Shading sh{sc};
    for (int k = 0; k < n; ++k) {
        Rng rng;
        rng.seed((uint32_t)k, 0, seed);
        V3 wi;
        float pdf = 0.0f;
        V3 f = sh.evalAndSample(material, is, rng, &wi, &pdf);
        float* o = out + 7 * (size_t)k;
        o[0] = wi.x; o[1] = wi.y; o[2] = wi.z; o[3] = f.x; o[4] = f.y; o[5] = f.z; o[6] = pdf;
    }
    return 0;
}

int xcpu_bsdf_eval_pcg(void* s, int material, const float* wo, int n, const float* wi, uint32_t seed, float* out) {
    const Scene* sc = (const Scene*)s;
    if (!sc || !wo || !wi || !out || n < 0 || material < 0 || material >= (int)sc->materials.size()) return -1;
    if (specularKind(sc->materials[material].type)) return -2;
    const Isect is = flatIsect(wo);
    const Shading sh{sc};
    for (int k = 0; k < n; ++k) {
        Rng rng;
        rng.seed((uint32_t)k, 1, seed);
        const V3 w(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
        float pdf = sh.getPDF(material, is, w);
        V3 f = sh.bsdfCos(material, is, rng, w);
        float* o = out + 4 * (size_t)k;
        o[0] = pdf; o[1] = f.x; o[2] = f.y; o[3] = f.z;
    }
    return 0;
}

int xcpu_light_sample_pcg(void* s, int n, uint32_t seed, float* out) {
    const Scene* sc = (const Scene*)s;
    if (!sc || !out || n < 0) return -1;
    if (!sc->built) return -3;
    if (sc->lights.empty()) return -2;
    for (int k = 0; k < n; ++k) {
        Rng rng;
        rng.seed((uint32_t)k, 2, seed);
        float pdf = 0.0f;
        LightSample ls = sampleLight(*sc, rng, &pdf);
        float* o = out + 7 * (size_t)k;
        o[0] = ls.p.x; o[1] = ls.p.y; o[2] = ls.p.z; o[3] = ls.n.x; o[4] = ls.n.y; o[5] = ls.n.z; o[6] = pdf;
    }
    return 0;
}

int xcpu_add_material(void* s, int type, const float* f, int base, int tex, int normalmap) {
    Scene* sc = (Scene*)s;
    Material m;
    m.type = type;
    m.tex = tex; m.normalmap = normalmap; m.base = base;
    switch (type) {
    case ORC_MAT_DIFFUSE: m.albedo = V3(f[0], f[1], f[2]); break;
    case ORC_MAT_METAL: m.roughness = f[0]; m.f0 = V3(f[1], f[2], f[3]); m.fixes = (int)f[4]; break;
    case ORC_MAT_GLOSSY:
    case ORC_MAT_GLOSSY_CLAMPED: m.albedo = V3(f[0], f[1], f[2]); m.sharpness = f[3]; break;
    case ORC_MAT_GLOSSY_HIGHLIGHT:
        m.albedo = V3(f[0], f[1], f[2]); m.highlight = V3(f[3], f[4], f[5]);
        m.sharpness = f[6]; m.sharpnessHL = f[7]; m.rate = f[8]; break;
    case ORC_MAT_EMISSION: m.power = V3(f[0], f[1], f[2]); break;
    case ORC_MAT_SPECULAR_REFLECTION: break;
    case ORC_MAT_SPECULAR_REFRACTION:
    case ORC_MAT_SPECULAR_FRESNEL: m.index = f[0]; break;
    case ORC_MAT_MF_NORMALMAP:
        if (base < 0 || base >= (int)sc->materials.size()) return -1;
        break;
    case ORC_MAT_MULTILOBE_SVBRDF:  // base material and SVNDF (index in tex)
        if (base < 0 || base >= (int)sc->materials.size() || tex < 0 || tex >= (int)sc->svndfs.size()) return -1;
        break;
    default: return -1;
    }
    sc->materials.push_back(m);
    return (int)sc->materials.size() - 1;
}

int xcpu_add_object(void* s, int mesh, int material, const float* mat, const float* matInv) {
    Scene* sc = (Scene*)s;
    if (mesh < 0 || mesh >= (int)sc->meshes.size() || material < 0 || material >= (int)sc->materials.size()) return -1;
    Object o;
    o.mesh = mesh; o.material = material;
    std::memcpy(o.mat.m, mat, 64);
    std::memcpy(o.matInv.m, matInv, 64);
    sc->objects.push_back(o);
    if (sc->materials[material].emissive()) sc->lights.push_back((int)sc->objects.size() - 1);
    return (int)sc->objects.size() - 1;
}

int xcpu_set_camera(void* s, const float* c2w, const float* c2wInv, float fov, float aspect) {
    Scene* sc = (Scene*)s;
    std::memcpy(sc->c2w.m, c2w, 64);
    std::memcpy(sc->c2wInv.m, c2wInv, 64);
    sc->fov = fov; sc->aspect = aspect;
    return 0;
}

// Opt-in quirk fixes of the render (not reference behaviour): bit 1 drops a
// radiance contribution with a non-finite component instead of adding it.
int xcpu_set_fixes(void* s, int fixes) {
    ((Scene*)s)->fixes = fixes;
    return 0;
}

int xcpu_set_sky(void* s, int type, const float* rgb, int tex) {
    Scene* sc = (Scene*)s;
    sc->skyType = type;
    if (rgb) sc->skyColor = V3(rgb[0], rgb[1], rgb[2]);
    sc->skyTex = tex;
    if ((type == ORC_SKY_PROBE || type == ORC_SKY_LATLONG) && (tex < 0 || tex >= (int)sc->textures.size())) return -1;
    return 0;
}

int xcpu_build(void* s) {
    Scene* sc = (Scene*)s;
    if (sc->objects.empty()) return -1;
    std::vector<Bounds> ob;
    for (auto& o : sc->objects) {
        o.areaScaling = sc->meshes[o.mesh].areaScaling(o.mat);
        ob.push_back(transformBounds(o.mat, sc->meshes[o.mesh].bound()));
    }
    sc->top.build(ob);
    sc->built = true;
    return 0;
}

// Per-(pixel, sample) PCG render over the pixel rectangle [x0,x1) x [y0,y1).
// Film position follows RenderTargetTile::GenerateFilmPosition (RenderTarget.h:68-80).
static int renderPcg(void* s, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                     int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                     float* aovFilm, int nthreads) {
    Scene* sc = (Scene*)s;
    if (!sc->built) return -1;
    Params P{integrator, max_depth, rr_start, rr_prob};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; ++y) {
        Rng rng;
        for (int x = x0; x < x1; ++x) {
            uint32_t pixel = (uint32_t)(x + y * W);
            V3 sum(0.0f), albedo(0.0f), normal(0.0f);
            for (uint32_t k = 0; k < spp_count; ++k) {
                rng.seed(pixel, spp_begin + k, seed);
                float fx = (float)x, fy = (float)y;
                fx /= W;
                fy /= H;
                fy = 1.0f - fy;
                fx += (rng.randf() - 0.5f) / W;
                fy += (rng.randf() - 0.5f) / H;
                Ray r = cameraRay(*sc, fx, fy);
                V3 aov[2] = {V3(0.0f), V3(0.0f)};
                V3* a = aovFilm ? aov : nullptr;
                V3 c = integrator == ORC_INTEGRATOR_NAIVE ? evalNaive(*sc, P, rng, r, a) : evalStandard(*sc, P, rng, r, a);
                sum = sum + c;
                albedo = albedo + aov[0];
                normal = normal + aov[1];
            }
            float* px = film + 3 * (size_t)pixel;
            px[0] += sum.x; px[1] += sum.y; px[2] += sum.z;
            if (aovFilm) {
                float* q = aovFilm + 6 * (size_t)pixel;
                q[0] += albedo.x; q[1] += albedo.y; q[2] += albedo.z;
                q[3] += normal.x; q[4] += normal.y; q[5] += normal.z;
            }
        }
    }
    return 0;
}

// Per-(pixel, sample) PCG render over the pixel rectangle [x0,x1) x [y0,y1).
// Film position follows RenderTargetTile::GenerateFilmPosition (RenderTarget.h:68-80).
int xcpu_render_pcg(void* s, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                    int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                    int nthreads) {
    return renderPcg(s, W, H, spp_begin, spp_count, seed, integrator, max_depth, rr_start, rr_prob, x0, y0, x1, y1,
                     film, nullptr, nthreads);
}

// The same render accumulating DenoisableRenderTargetPixel's albedo and normal
// (RenderTarget.h:131-145) as well: aov is float[H][W][6] (albedo rgb, normal xyz).
int xcpu_render_pcg_aov(void* s, int W, int H, uint32_t spp_begin, uint32_t spp_count, uint32_t seed, int integrator,
                        int max_depth, int rr_start, float rr_prob, int x0, int y0, int x1, int y1, float* film,
                        float* aov, int nthreads) {
    return renderPcg(s, W, H, spp_begin, spp_count, seed, integrator, max_depth, rr_start, rr_prob, x0, y0, x1, y1,
                     film, aov, nthreads);
}

// Scene::intersect / intersectAny for the checkers' known-answer tests (scene_api.h).
int xcpu_intersect(void* s, int n, const float* rays, float* out) {
    Scene* sc = (Scene*)s;
    if (!sc || !rays || !out || n < 0) return -1;
    if (!sc->built) return -3;
    for (int i = 0; i < n; ++i) {
        Ray r;
        r.o = V3(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]);
        r.d = V3(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]);
        r.tMax = rays[7 * i + 6];
        Isect is;
        float* o = out + 8 * (size_t)i;
        const bool hit = sceneIntersect(*sc, r, &is);
        o[0] = r.tMax;
        o[1] = hit ? (float)is.object : -1.0f;
        o[2] = hit ? is.p.x : 0.0f; o[3] = hit ? is.p.y : 0.0f; o[4] = hit ? is.p.z : 0.0f;
        o[5] = hit ? is.sn.x : 0.0f; o[6] = hit ? is.sn.y : 0.0f; o[7] = hit ? is.sn.z : 0.0f;
    }
    return 0;
}

int xcpu_intersect_any(void* s, int n, const float* rays, int32_t* out) {
    Scene* sc = (Scene*)s;
    if (!sc || !rays || !out || n < 0) return -1;
    if (!sc->built) return -3;
    for (int i = 0; i < n; ++i) {
        Ray r;
        r.o = V3(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]);
        r.d = V3(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]);
        r.tMax = rays[7 * i + 6];
        out[i] = sceneIntersectAny(*sc, r) ? 1 : 0;
    }
    return 0;
}

// Closest-hit query for traversal known-answer tests: rays are float[n][7]
// (o, d, tMax); hits are float[n][5] (t, object, triangle, b0, b1), object = -1
// on a miss. b0/b1 are recomputed by the watertight test on the hit triangle.
int xcpu_trace(void* s, int n, const float* rays, float* hits) {
    Scene* sc = (Scene*)s;
    if (!sc->built) return -1;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        Ray r;
        r.o = V3(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]);
        r.d = V3(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]);
        r.tMax = rays[7 * i + 6];
        Isect is;
        float* h = hits + 5 * (size_t)i;
        if (sceneIntersect(*sc, r, &is)) {
            h[0] = r.tMax; h[1] = (float)is.object; h[2] = (float)is.tri;
            h[3] = 0; h[4] = 0;
        } else {
            h[0] = r.tMax; h[1] = -1; h[2] = -1; h[3] = 0; h[4] = 0;
        }
    }
    return 0;
}

// Any-hit query: out[i] = 1 if ray i is occluded within its tMax.
int xcpu_occluded(void* s, int n, const float* rays, int32_t* out) {
    Scene* sc = (Scene*)s;
    if (!sc->built) return -1;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        Ray r;
        r.o = V3(rays[7 * i], rays[7 * i + 1], rays[7 * i + 2]);
        r.d = V3(rays[7 * i + 3], rays[7 * i + 4], rays[7 * i + 5]);
        r.tMax = rays[7 * i + 6];
        out[i] = sceneIntersectAny(*sc, r) ? 1 : 0;
    }
    return 0;
}
}  // extern "C"
