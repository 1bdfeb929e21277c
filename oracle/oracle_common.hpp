// oracle_common.hpp -- TEST INFRASTRUCTURE ONLY.
//
// Scalar/vector helpers for the CPU restatement of the reference's shader
// arithmetic (Snowapril/vk_voxel_cone_tracing, VFS/Shaders/*).  Only tests,
// the smoke check and bench.py's CPU-baseline leg load this code; the CUDA
// product path never links it.
//
// Every function is templated on the arithmetic type T: float gives the FP32
// mirror of the GLSL (the timed CPU baseline and the bit-level checker for
// integer / RGBA8 outputs), double gives the FP64 error reference.
// The file is compiled with -ffp-contract=off so that no multiply-add is fused
// behind our back: each GLSL expression is evaluated in its written order.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

#include "ad_tape.hpp"  // before the templates: its std:: overloads must be visible to them

namespace vcto {

template <class T> struct V2 { T x, y; };
template <class T> struct V3 {
    T x, y, z;
    V3() = default;
    constexpr V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit constexpr V3(T a) : x(a), y(a), z(a) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> struct V4 {
    T x, y, z, w;
    V4() = default;
    constexpr V4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    explicit constexpr V4(T a) : x(a), y(a), z(a), w(a) {}
    V3<T> xyz() const { return V3<T>(x, y, z); }
};

struct I3 { int32_t x, y, z; };

template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V4<T> operator+(V4<T> a, V4<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> inline V4<T> operator*(V4<T> a, T s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class T> inline V4<T> operator*(T s, V4<T> a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }

template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) {
    T inv = T(1) / std::sqrt(dot(a, a));
    return a * inv;
}
// GLSL reflect(I, N) = I - 2 * dot(N, I) * N.
template <class T> inline V3<T> reflect(V3<T> i, V3<T> n) { return i - n * (T(2) * dot(n, i)); }
template <class T> inline T clampv(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }
// GLSL mix(x, y, a) = x * (1 - a) + y * a.
template <class T> inline T mixv(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template <class T> inline T fractv(T x) { return x - std::floor(x); }

// Column-major 4x4 (glm / GLSL storage) times (x, y, z, w).
template <class T> inline V4<T> mat_mul(const float* m, V4<T> v) {
    V4<T> r;
    r.x = T(m[0]) * v.x + T(m[4]) * v.y + T(m[8]) * v.z + T(m[12]) * v.w;
    r.y = T(m[1]) * v.x + T(m[5]) * v.y + T(m[9]) * v.z + T(m[13]) * v.w;
    r.z = T(m[2]) * v.x + T(m[6]) * v.y + T(m[10]) * v.z + T(m[14]) * v.w;
    r.w = T(m[3]) * v.x + T(m[7]) * v.y + T(m[11]) * v.z + T(m[15]) * v.w;
    return r;
}

// RGBA8 UNORM <-> float.  Load: c / 255 (correctly rounded).  Store: the
// pinned rule is round-half-up of clamp(x, 0, 1) * 255 (Vulkan leaves the
// tie rule to the implementation).
inline uint32_t unorm8_store(float x) {
    float c = std::min(std::max(x, 0.0f), 1.0f);
    return (uint32_t)std::floor(c * 255.0f + 0.5f);
}
inline uint32_t unorm8_store(double x) {
    double c = std::min(std::max(x, 0.0), 1.0);
    return (uint32_t)std::floor(c * 255.0 + 0.5);
}
template <class T> inline V4<T> unpack_unorm(uint32_t v) {
    return V4<T>(T(v & 0xffu) / T(255), T((v >> 8) & 0xffu) / T(255), T((v >> 16) & 0xffu) / T(255),
                 T((v >> 24) & 0xffu) / T(255));
}
template <class T> inline uint32_t pack_unorm(V4<T> c) {
    return unorm8_store(c.x) | (unorm8_store(c.y) << 8) | (unorm8_store(c.z) << 16) | (unorm8_store(c.w) << 24);
}

// Atlas geometry: width = (R+2)*6 faces, height = (R+2)*6 levels, depth = R+2.
struct Atlas {
    int R;
    int W, H, D;
    explicit Atlas(int res) : R(res), W((res + 2) * 6), H((res + 2) * 6), D(res + 2) {}
    int64_t index(int x, int y, int z) const { return ((int64_t)z * H + y) * W + x; }
    int64_t texels() const { return (int64_t)W * H * D; }
};

inline int wrap_repeat(int i, int n) {
    int m = i % n;
    return m < 0 ? m + n : m;
}

}  // namespace vcto
