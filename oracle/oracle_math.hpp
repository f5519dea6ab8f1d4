// TEST INFRASTRUCTURE — the oracle.  Not part of the product: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
// only as the checker.
//
// GLSL-semantics scalar/vector helpers for the CPU restatement of the
// reference shaders.  Every operation is spelled out in the order the GLSL
// source writes it, so that a float instantiation performs the same IEEE
// single-precision operations as the shader source (the oracle is compiled
// with -ffp-contract=off: no fused multiply-add).
//
// Definitions the GLSL spec leaves to the implementation, fixed here:
//   dot(a,b)        = ((a.x*b.x + a.y*b.y) + a.z*b.z)
//   length(v)       = sqrt(dot(v,v))
//   normalize(v)    = v / length(v)            (component-wise division)
//   mix(x,y,a)      = x*(1-a) + y*a            (GLSL 4.50 §8.3 formula)
//   min(x,y)        = y < x ? y : x ;  max(x,y) = x < y ? y : x
//   clamp(x,lo,hi)  = min(max(x,lo),hi)
//   smoothstep      = t*t*(3-2t), t = clamp((x-e0)/(e1-e0),0,1)
//   fract(x)        = x - floor(x) ;  mod(x,y) = x - y*floor(x/y)
//   round(x)        = half away from zero (C roundf)
//   int(x)          = truncation, saturating to the int range, NaN -> 0
#pragma once
#include <climits>
#include <cmath>
#include <cstdint>

namespace orc {

// A literal as the shader writes it: `lit<T>(0.38f, 0.38)` is the float
// literal for T = float and the double literal for T = double.
template <class T> constexpr T lit(float f, double d);
template <> constexpr float lit<float>(float f, double) { return f; }
template <> constexpr double lit<double>(float, double d) { return d; }
#define L(x) ::orc::lit<T>(x##f, x)

template <class T> inline T gmin(T a, T b) { return b < a ? b : a; }
template <class T> inline T gmax(T a, T b) { return a < b ? b : a; }
template <class T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline T gmix(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template <class T> inline T gfract(T x) { return x - std::floor(x); }
template <class T> inline T gmod(T x, T y) { return x - y * std::floor(x / y); }
template <class T> inline T gsmoothstep(T e0, T e1, T x) {
    T t = gclamp((x - e0) / (e1 - e0), T(0), T(1));
    return t * t * (T(3) - T(2) * t);
}

inline int f2i(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}

template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };
template <class T> struct V4 { T x, y, z, w; };

template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }

template <class T> inline V4<T> operator+(V4<T> a, V4<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> inline V4<T> operator-(V4<T> a, V4<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class T> inline V4<T> operator*(V4<T> a, T s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class T> inline V4<T> operator/(V4<T> a, T s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }

template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> inline V3<T> vmix(V3<T> x, V3<T> y, T a) {
    return {gmix(x.x, y.x, a), gmix(x.y, y.y, a), gmix(x.z, y.z, a)};
}
template <class T> inline V4<T> vmin(V4<T> a, V4<T> b) {
    return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z), gmin(a.w, b.w)};
}
template <class T> inline V4<T> vmax(V4<T> a, V4<T> b) {
    return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z), gmax(a.w, b.w)};
}
template <class T> inline V4<T> vclamp(V4<T> x, V4<T> lo, V4<T> hi) { return vmin(vmax(x, lo), hi); }
template <class T> inline V4<T> vmix4(V4<T> x, V4<T> y, T a) {
    return {gmix(x.x, y.x, a), gmix(x.y, y.y, a), gmix(x.z, y.z, a), gmix(x.w, y.w, a)};
}

// GLSL mat3(c0,c1,c2) * v: result[i] = c0[i]*v.x + c1[i]*v.y + c2[i]*v.z
template <class T> inline V3<T> mat3_mul(V3<T> c0, V3<T> c1, V3<T> c2, V3<T> v) {
    return {c0.x * v.x + c1.x * v.y + c2.x * v.z, c0.y * v.x + c1.y * v.y + c2.y * v.z,
            c0.z * v.x + c1.z * v.y + c2.z * v.z};
}

}  // namespace orc
