// Scalar 4-lane stand-in for the subset of libsimdpp that the Xitils headers use.
//
// TEST INFRASTRUCTURE ONLY: this header lets the reference's own headers compile
// on gcc (x86_64 and aarch64) so that oracle/_ref can be built as a CPU checker.
// libsimdpp is an un-vendored submodule of the reference (ThirdParty/libsimdpp,
// no pinned commit is visible), so its published lane-wise semantics are
// restated here in plain C++:
//   * every arithmetic op is IEEE lane-wise (add/sub/mul/div/min/max/abs);
//   * min/max follow SSE minps/maxps: min(a,b) = a < b ? a : b;
//   * reduce_add(float32x4) follows the SSE3 path (two horizontal adds):
//     (l0 + l1) + (l2 + l3);
//   * comparisons give all-ones / all-zero lane masks; cmp_neq is unordered;
//   * blend(on, off, mask) picks `on` where the mask is set;
//   * shuffle4x2<a,b,c,d>(x, y) picks lanes 0..3 from x and 4..7 from y.
// All Xitils vector types are 16 bytes (Vector2/3 carry padding lanes), so
// load_u/store_u always move 16 bytes (32 for float64x4 is never loaded).
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

namespace simdpp {

struct float32x4 { float v[4]; };
struct int32x4 { int32_t v[4]; };
struct uint32x4 { uint32_t v[4]; };
struct mask_float32x4 { uint32_t v[4]; };
struct mask_int32x4 { uint32_t v[4]; };
struct float64x4 { double v[4]; };

struct zero_proxy {
    template <class V> operator V() const { V r; std::memset(&r, 0, sizeof r); return r; }
};
inline zero_proxy make_zero() { return {}; }

template <class V> inline V load_u(const void* p) { V r; std::memcpy(&r, p, sizeof r); return r; }
template <class V> inline void store_u(void* p, const V& v) { std::memcpy(p, &v, sizeof v); }

template <class V> struct lane_of;
template <> struct lane_of<float32x4> { using type = float; using mask = mask_float32x4; };
template <> struct lane_of<int32x4> { using type = int32_t; using mask = mask_int32x4; };
template <> struct lane_of<uint32x4> { using type = uint32_t; using mask = mask_int32x4; };
template <> struct lane_of<float64x4> { using type = double; using mask = mask_float32x4; };

template <class V> inline V load_splat(const void* p) {
    typename lane_of<V>::type s; std::memcpy(&s, p, sizeof s);
    V r; for (int i = 0; i < 4; ++i) r.v[i] = s; return r;
}
template <class V> inline V splat(typename lane_of<V>::type s) {
    V r; for (int i = 0; i < 4; ++i) r.v[i] = s; return r;
}

#define SIMDPP_SHIM_BINOP(name, expr)                                           \
    template <class V> inline V name(const V& a, const V& b) {                  \
        V r; for (int i = 0; i < 4; ++i) { auto x = a.v[i]; auto y = b.v[i]; r.v[i] = (expr); } return r; }
SIMDPP_SHIM_BINOP(add, x + y)
SIMDPP_SHIM_BINOP(sub, x - y)
SIMDPP_SHIM_BINOP(mul, x * y)
SIMDPP_SHIM_BINOP(div, x / y)
SIMDPP_SHIM_BINOP(min, x < y ? x : y)
SIMDPP_SHIM_BINOP(max, x > y ? x : y)
#undef SIMDPP_SHIM_BINOP

template <class V> inline V fmadd(const V& a, const V& b, const V& c) {
    V r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * b.v[i] + c.v[i]; return r;
}

inline float32x4 abs(const float32x4& a) {
    float32x4 r; for (int i = 0; i < 4; ++i) r.v[i] = std::fabs(a.v[i]); return r;
}
inline int32x4 abs(const int32x4& a) {
    int32x4 r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] < 0 ? -a.v[i] : a.v[i]; return r;
}

#define SIMDPP_SHIM_CMP(name, expr)                                             \
    template <class V> inline typename lane_of<V>::mask name(const V& a, const V& b) { \
        typename lane_of<V>::mask m;                                            \
        for (int i = 0; i < 4; ++i) { auto x = a.v[i]; auto y = b.v[i]; m.v[i] = (expr) ? 0xFFFFFFFFu : 0u; } \
        return m; }
SIMDPP_SHIM_CMP(cmp_eq, x == y)
SIMDPP_SHIM_CMP(cmp_neq, !(x == y))
SIMDPP_SHIM_CMP(cmp_gt, x > y)
SIMDPP_SHIM_CMP(cmp_lt, x < y)
SIMDPP_SHIM_CMP(cmp_ge, x >= y)
SIMDPP_SHIM_CMP(cmp_le, x <= y)
#undef SIMDPP_SHIM_CMP

inline mask_float32x4 isnan(const float32x4& a) {
    mask_float32x4 m; for (int i = 0; i < 4; ++i) m.v[i] = std::isnan(a.v[i]) ? 0xFFFFFFFFu : 0u; return m;
}

template <class To, class From> inline To bit_cast(const From& f) {
    static_assert(sizeof(To) == sizeof(From), "bit_cast size");
    To t; std::memcpy(&t, &f, sizeof t); return t;
}

template <class V, class M> inline V blend(const V& on, const V& off, const M& mask) {
    V r; for (int i = 0; i < 4; ++i) r.v[i] = mask.v[i] ? on.v[i] : off.v[i]; return r;
}

template <unsigned id, unsigned N, class V, class S> inline V insert(const V& a, S s) {
    V r = a; r.v[id] = (typename lane_of<V>::type)s; return r;
}

template <class V> inline typename lane_of<V>::type reduce_add(const V& a) {
    return (a.v[0] + a.v[1]) + (a.v[2] + a.v[3]);
}
template <class V> inline typename lane_of<V>::type reduce_min(const V& a) {
    auto x = a.v[0] < a.v[1] ? a.v[0] : a.v[1];
    auto y = a.v[2] < a.v[3] ? a.v[2] : a.v[3];
    return x < y ? x : y;
}
template <class V> inline typename lane_of<V>::type reduce_max(const V& a) {
    auto x = a.v[0] > a.v[1] ? a.v[0] : a.v[1];
    auto y = a.v[2] > a.v[3] ? a.v[2] : a.v[3];
    return x > y ? x : y;
}
inline uint32_t reduce_and(const uint32x4& a) { return a.v[0] & a.v[1] & a.v[2] & a.v[3]; }
inline uint32_t reduce_or(const uint32x4& a) { return a.v[0] | a.v[1] | a.v[2] | a.v[3]; }

inline float64x4 to_float64(const float32x4& a) {
    float64x4 r; for (int i = 0; i < 4; ++i) r.v[i] = (double)a.v[i]; return r;
}
inline float32x4 to_float32(const float64x4& a) {
    float32x4 r; for (int i = 0; i < 4; ++i) r.v[i] = (float)a.v[i]; return r;
}

// Named by the never-instantiated Vector.h `_inRange`; declared so that its
// qualified names resolve.
template <class V> inline V make_float(float a, float b, float c, float d) {
    V r; r.v[0] = a; r.v[1] = b; r.v[2] = c; r.v[3] = d; return r;
}
inline mask_float32x4 to_mask(const float32x4& a) {
    mask_float32x4 m; for (int i = 0; i < 4; ++i) m.v[i] = a.v[i] != 0.0f ? 0xFFFFFFFFu : 0u; return m;
}

template <unsigned s0, unsigned s1, unsigned s2, unsigned s3, class V>
inline V shuffle4x2(const V& a, const V& b) {
    const unsigned s[4] = {s0, s1, s2, s3};
    V r; for (int i = 0; i < 4; ++i) r.v[i] = s[i] < 4 ? a.v[s[i]] : b.v[s[i] - 4]; return r;
}

}  // namespace simdpp
