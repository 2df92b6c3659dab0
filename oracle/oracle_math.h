// oracle_math.h — TEST INFRASTRUCTURE ONLY (the oracle). Scalar/vector helpers for the CPU restatement of vkrt's
// path-tracing shaders, templated on the real type so the same restatement runs in FP32 (bit-level parity target)
// and FP64 (precision oracle). Never linked into the product library.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace oracle {

template <class R>
struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a) : x(a), y(a), z(a) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    template <class S>
    explicit V3(const V3<S>& o) : x(R(o.x)), y(R(o.y)), z(R(o.z)) {}
    R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> V3<R> operator*(R s, V3<R> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> V3<R>& operator+=(V3<R>& a, V3<R> b) { a = a + b; return a; }
template <class R> V3<R>& operator*=(V3<R>& a, V3<R> b) { a = a * b; return a; }
template <class R> V3<R>& operator*=(V3<R>& a, R s) { a = a * s; return a; }
template <class R> V3<R>& operator/=(V3<R>& a, R s) { a = a / s; return a; }
template <class R> R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> R maxc(V3<R> a) { return std::max(a.x, std::max(a.y, a.z)); }
template <class R> V3<R> vmax(V3<R> a, V3<R> b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
template <class R> R sat(R v) { return v < R(0) ? R(0) : (v > R(1) ? R(1) : v); }
template <class R> V3<R> sat(V3<R> v) { return {sat(v.x), sat(v.y), sat(v.z)}; }
template <class R> R clampr(R v, R lo, R hi) { return v < lo ? lo : (v > hi ? hi : v); }
template <class R> bool anyPositive(V3<R> v) { return v.x > R(0) || v.y > R(0) || v.z > R(0); }
template <class R> R rsqrtr(R v) { return R(1) / std::sqrt(v); }
template <class R> V3<R> normalize(V3<R> v) { return v * rsqrtr(dot(v, v)); }
template <class R> R lerpr(R a, R b, R t) { return a + (b - a) * t; }
template <class R> R fracr(R v) { return v - std::floor(v); }

template <class R>
struct V4 {
    R x, y, z, w;
    V4() : x(0), y(0), z(0), w(0) {}
    V4(R a) : x(a), y(a), z(a), w(a) {}
    V4(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
    R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
template <class R> V4<R> operator+(V4<R> a, V4<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class R> V4<R> operator*(V4<R> a, V4<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
template <class R> V4<R> operator*(V4<R> a, R s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class R> V4<R> operator*(R s, V4<R> a) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class R> V4<R> operator/(V4<R> a, R s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
template <class R> V4<R>& operator+=(V4<R>& a, V4<R> b) { a = a + b; return a; }
template <class R> V4<R>& operator*=(V4<R>& a, V4<R> b) { a = a * b; return a; }
template <class R> R sum4(V4<R> a) { return a.x + a.y + a.z + a.w; }
template <class R> R max4(V4<R> a) { return std::max(std::max(a.x, a.y), std::max(a.z, a.w)); }
template <class R> bool anyPositive(V4<R> v) { return v.x > R(0) || v.y > R(0) || v.z > R(0) || v.w > R(0); }

}  // namespace oracle
