// Minimal glm stand-in so the Xitils headers compile for the CPU checker.
// TEST INFRASTRUCTURE ONLY. Xitils uses glm types only as conversion targets
// (Vector.h, Matrix.h) and for cinder mesh data; no glm arithmetic is on the
// path-tracing path.
#pragma once
#include <initializer_list>

namespace glm {

template <class T> struct tvec2 {
    T x{}, y{};
    tvec2() = default;
    tvec2(T a, T b) : x(a), y(b) {}
    T& operator[](int i) { return i == 0 ? x : y; }
    const T& operator[](int i) const { return i == 0 ? x : y; }
};
template <class T> struct tvec3 {
    T x{}, y{}, z{};
    tvec3() = default;
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
};
template <class T> inline tvec3<T> operator*(T s, const tvec3<T>& v) { return tvec3<T>(s * v.x, s * v.y, s * v.z); }
template <class T> struct tvec4 {
    T x{}, y{}, z{}, w{};
    tvec4() = default;
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using ivec2 = tvec2<int>;

struct mat4x4 {
    tvec4<float> c[4];
    mat4x4() = default;
    mat4x4(std::initializer_list<float> l) {
        int i = 0;
        for (float f : l) { c[i / 4][i % 4] = f; ++i; }
    }
    tvec4<float>& operator[](int i) { return c[i]; }
    const tvec4<float>& operator[](int i) const { return c[i]; }
};
using mat4 = mat4x4;

}  // namespace glm
