// Device vector math with the semantics of Xitils' Vector3f (Include/Xitils/Vector.h).
//
// Vector3f is four float lanes with a zero padding lane; the reference's
// operators are lane-wise IEEE float ops. The helpers below keep its rules:
//   dot(a, b)   = (a.x*b.x + a.y*b.y) + (a.z*b.z + 0)   (libsimdpp SSE3 horizontal adds)
//   v / s       = v * (1 / s)                            (Vector.h:356-361)
//   normalize   = v / length(v)                          (Vector.h:615)
//   cross       = FP64 products rounded once to float    (Vector.h:637-654)
// Translation units that include this header for shading are compiled with
// -fmad=false so that no multiply-add is contracted, matching the reference's
// unfused float arithmetic; transcendental functions are CUDA's own.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace xgb {

#ifndef XGB_CROSS64
#define XGB_CROSS64 1
#endif

constexpr float kPi = 3.14159265358979323846f;  // (float)M_PI, Utils.h:32
constexpr double kPiD = 3.14159265358979323846;

struct V3 {
    float x, y, z;
    __host__ __device__ V3() : x(0), y(0), z(0) {}
    __host__ __device__ V3(float a, float b, float c) : x(a), y(b), z(c) {}
    __host__ __device__ explicit V3(float s) : x(s), y(s), z(s) {}
    __device__ float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return a * s; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator/(V3 a, float s) { float inv = 1.0f / s; return a * inv; }

__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + 0.0f); }
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return a / length(a); }
__device__ __forceinline__ bool isZero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__device__ __forceinline__ bool hasNan(V3 a) { return isnan(a.x) || isnan(a.y) || isnan(a.z); }
__device__ __forceinline__ bool eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ V3 faceForward(V3 n, V3 v) { return dot(n, v) < 0.0f ? -n : n; }
__device__ __forceinline__ float clampPositive(float x) { return x > 0.0f ? x : 0.0f; }
__device__ __forceinline__ V3 clampPositive(V3 v) { return V3(clampPositive(v.x), clampPositive(v.y), clampPositive(v.z)); }
__device__ __forceinline__ float safeSqrt(float x) { return sqrtf(clampPositive(x)); }
__device__ __forceinline__ float minf_ref(float a, float b) { return a < b ? a : b; }

__device__ __forceinline__ V3 cross(V3 a, V3 b) {
#if XGB_CROSS64
    double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return V3((float)(ay * bz - az * by), (float)(az * bx - ax * bz), (float)(ax * by - ay * bx));
#else
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
#endif
}

// Utils.h:81-83
__device__ __forceinline__ V3 lerp3(V3 a, V3 b, V3 c, float t1, float t2) {
    return t1 * a + t2 * b + (1.0f - t1 - t2) * c;
}
__device__ __forceinline__ float2 lerp3(float2 a, float2 b, float2 c, float t1, float t2) {
    float w = 1.0f - t1 - t2;
    return make_float2((a.x * t1 + b.x * t2) + c.x * w, (a.y * t1 + b.y * t2) + c.y * w);
}

__device__ __forceinline__ V3 v3(float4 a) { return V3(a.x, a.y, a.z); }

// Vector.h:781-795. cross(v, axis) with a unit axis is exact in float.
struct Basis {
    V3 e1, e2, e3;
    __device__ explicit Basis(V3 v) {
        e1 = normalize(v);
        V3 c;
        if (fabsf(v.x) < 0.5f) c = V3(v.y * 0.0f - v.z * 0.0f, v.z * 1.0f - v.x * 0.0f, v.x * 0.0f - v.y * 1.0f);
        else if (fabsf(v.y) < 0.5f) c = V3(v.y * 0.0f - v.z * 1.0f, v.z * 0.0f - v.x * 0.0f, v.x * 1.0f - v.y * 0.0f);
        else c = V3(v.y * 1.0f - v.z * 0.0f, v.z * 0.0f - v.x * 1.0f, v.x * 0.0f - v.y * 0.0f);
        e2 = normalize(c);
        e3 = normalize(cross(e1, e2));
    }
    __device__ V3 fromGlobal(V3 v) const { return V3(dot(v, e1), dot(v, e2), dot(v, e3)); }
    __device__ V3 toGlobal(float x, float y, float z) const { return e1 * x + e2 * y + e3 * z; }
    __device__ V3 toGlobal(V3 v) const { return e1 * v.x + e2 * v.y + e3 * v.z; }
};

// Transform.h:61-72, 105-127 on a row-major float[16]
__device__ __forceinline__ V3 xformPoint(const float* m, V3 v) {
    float xp = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
    float yp = m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7];
    float zp = m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11];
    float wp = m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15];
    if (wp == 1.0f) return V3(xp, yp, zp);
    return V3(xp, yp, zp) / wp;
}
__device__ __forceinline__ V3 xformVector(const float* m, V3 v) {
    return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
__device__ __forceinline__ V3 xformNormal(const float* m, V3 v) { return normalize(xformVector(m, v)); }

// ------------------------------------------------------------------ PCG32 --
// Per-(pixel, sample) stream: pcg32 with initstate = splitmix64(seed << 32 ^ sample),
// sequence = pixel. The draw helpers restate Sampler.h:17-32.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
struct Pcg {
    uint64_t state;
    uint64_t inc;
    __device__ __forceinline__ void seed(uint32_t pixel, uint32_t sample, uint32_t seed) {
        uint64_t initstate = splitmix64(((uint64_t)seed << 32) ^ (uint64_t)sample);
        state = 0;
        inc = ((uint64_t)pixel << 1) | 1u;
        next();
        state += initstate;
        next();
    }
    __device__ __forceinline__ uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return __funnelshift_r(xorshifted, xorshifted, rot);
    }
    // (float)rand() / 0xFFFFFFFF == (float)u / 4294967296.0f (exact division by 2^32)
    __device__ __forceinline__ float randf() { return __uint2float_rn(next()) * 2.3283064365386963e-10f; }
    __device__ __forceinline__ int randi(int max) { return (int)(next() % (uint32_t)max); }
};

}  // namespace xgb
