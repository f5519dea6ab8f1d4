// TEST INFRASTRUCTURE — builds the reference's own GLSL shader source as C++
// (oracle/ref_build.py), to pin the oracle's restatement against it.
//
// A minimal GLSL 4.50 environment: vector/matrix types with GLSL's implicit
// int -> float conversions, swizzles (through sw<...>() values and swref<...>()
// assignable proxies, which ref_build.py substitutes for `.xyz`-style
// members), the built-in functions the shaders call, and software samplers and
// storage images.  Implementation-defined corners are fixed exactly as the
// oracle restatement (oracle_math.hpp) fixes them; the sampler is the same
// exact-weight LINEAR filter (interpolate raw texel values, then scale).
#pragma once
#include <climits>
#include <cmath>
#include <cstdint>
#include <type_traits>

namespace glsl {

using uint = unsigned int;

inline int f2i(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}

template <class T> struct Swz2;
struct ivec2;
struct uvec2;

template <class S> struct tvec2 {
    S x{}, y{};
    tvec2() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic_v<A>>>
    explicit tvec2(A s) : x(S(s)), y(S(s)) {}
    template <class A, class B, class = std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B>>>
    tvec2(A a, B b) : x(S(a)), y(S(b)) {}
    template <class O> tvec2(const tvec2<O>& o) : x(S(o.x)), y(S(o.y)) {}
    S& operator[](int i) { return i == 0 ? x : y; }
    S operator[](int i) const { return i == 0 ? x : y; }
    template <int... I> auto sw() const;
};

template <class S> struct tvec3 {
    S x{}, y{}, z{};
    tvec3() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic_v<A>>>
    explicit tvec3(A s) : x(S(s)), y(S(s)), z(S(s)) {}
    template <class A, class B, class C>
    tvec3(A a, B b, C c) : x(S(a)), y(S(b)), z(S(c)) {}
    template <class O> tvec3(const tvec3<O>& o) : x(S(o.x)), y(S(o.y)), z(S(o.z)) {}
    S& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    S operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    template <int... I> auto sw() const;
    template <int... I> auto swref();
};

template <class S> struct tvec4 {
    S x{}, y{}, z{}, w{};
    tvec4() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic_v<A>>>
    explicit tvec4(A s) : x(S(s)), y(S(s)), z(S(s)), w(S(s)) {}
    template <class A, class B, class C, class D>
    tvec4(A a, B b, C c, D d) : x(S(a)), y(S(b)), z(S(c)), w(S(d)) {}
    template <class B> tvec4(const tvec3<S>& v, B d) : x(v.x), y(v.y), z(v.z), w(S(d)) {}
    S& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    S operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    template <int... I> auto sw() const;
};

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using uvec3 = tvec3<uint>;

struct ivec2 {
    int x{}, y{};
    ivec2() = default;
    explicit ivec2(int s) : x(s), y(s) {}
    explicit ivec2(float s) : x(f2i(s)), y(f2i(s)) {}
    explicit ivec2(double s) : x(f2i(s)), y(f2i(s)) {}
    ivec2(int a, int b) : x(a), y(b) {}
    ivec2(float a, float b) : x(f2i(a)), y(f2i(b)) {}
    ivec2(uint a, uint b) : x((int)a), y((int)b) {}
    explicit ivec2(const vec2& v) : x(f2i(v.x)), y(f2i(v.y)) {}
    operator vec2() const { return vec2((float)x, (float)y); }
};
struct uvec2 {
    uint x{}, y{};
    operator vec2() const { return vec2((float)x, (float)y); }
};

template <class S> struct vec_of;
template <> struct vec_of<float> {
    using v2 = vec2;
    using v3 = vec3;
    using v4 = vec4;
};
template <> struct vec_of<uint> {
    using v2 = uvec2;
    using v3 = uvec3;
};

template <class S> template <int... I> auto tvec2<S>::sw() const {
    const S c[2] = {x, y};
    if constexpr (sizeof...(I) == 2) return tvec2<S>(c[I]...);
    else if constexpr (sizeof...(I) == 3) return tvec3<S>(c[I]...);
    else return tvec4<S>(c[I]...);
}
template <class S> template <int... I> auto tvec3<S>::sw() const {
    const S c[3] = {x, y, z};
    if constexpr (sizeof...(I) == 2) {
        if constexpr (std::is_same_v<S, uint>) {
            uvec2 r;
            const int idx[2] = {I...};
            r.x = c[idx[0]];
            r.y = c[idx[1]];
            return r;
        } else {
            return tvec2<S>(c[I]...);
        }
    } else if constexpr (sizeof...(I) == 3) return tvec3<S>(c[I]...);
    else return tvec4<S>(c[I]...);
}
template <class S> template <int... I> auto tvec4<S>::sw() const {
    const S c[4] = {x, y, z, w};
    if constexpr (sizeof...(I) == 2) return tvec2<S>(c[I]...);
    else if constexpr (sizeof...(I) == 3) return tvec3<S>(c[I]...);
    else return tvec4<S>(c[I]...);
}

// Assignable 2-component swizzle of a vec3 (`point.xy += ...`).
template <class S> struct Swz2 {
    S* a;
    S* b;
    Swz2& operator=(const tvec2<S>& v) {
        *a = v.x;
        *b = v.y;
        return *this;
    }
    Swz2& operator+=(const tvec2<S>& v) {
        *a = *a + v.x;
        *b = *b + v.y;
        return *this;
    }
    Swz2& operator-=(const tvec2<S>& v) {
        *a = *a - v.x;
        *b = *b - v.y;
        return *this;
    }
    operator tvec2<S>() const { return tvec2<S>(*a, *b); }
};
template <class S> template <int... I> auto tvec3<S>::swref() {
    static_assert(sizeof...(I) == 2, "only 2-component assignable swizzles are used");
    S* c[3] = {&x, &y, &z};
    const int idx[2] = {I...};
    return Swz2<S>{c[idx[0]], c[idx[1]]};
}

// ---- arithmetic (component-wise, float) ----------------------------------
#define GLSL_BINOP(OP)                                                                                        \
    inline vec2 operator OP(vec2 a, vec2 b) { return vec2(a.x OP b.x, a.y OP b.y); }                          \
    inline vec2 operator OP(vec2 a, float s) { return vec2(a.x OP s, a.y OP s); }                             \
    inline vec2 operator OP(float s, vec2 a) { return vec2(s OP a.x, s OP a.y); }                             \
    inline vec2 operator OP(vec2 a, ivec2 b) { return a OP vec2(b); }                                          \
    inline vec3 operator OP(vec3 a, vec3 b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); }              \
    inline vec3 operator OP(vec3 a, float s) { return vec3(a.x OP s, a.y OP s, a.z OP s); }                   \
    inline vec3 operator OP(float s, vec3 a) { return vec3(s OP a.x, s OP a.y, s OP a.z); }                   \
    inline vec4 operator OP(vec4 a, vec4 b) { return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }  \
    inline vec4 operator OP(vec4 a, float s) { return vec4(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }         \
    inline vec4 operator OP(float s, vec4 a) { return vec4(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }
GLSL_BINOP(+)
GLSL_BINOP(-)
GLSL_BINOP(*)
GLSL_BINOP(/)
#undef GLSL_BINOP

inline ivec2 operator-(ivec2 a, ivec2 b) { return ivec2(a.x - b.x, a.y - b.y); }
inline ivec2 operator+(ivec2 a, ivec2 b) { return ivec2(a.x + b.x, a.y + b.y); }

inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator-(vec4 a) { return vec4(-a.x, -a.y, -a.z, -a.w); }

template <class V, class R> inline V& operator+=(V& a, const R& b) { return a = a + b; }
template <class V, class R> inline V& operator-=(V& a, const R& b) { return a = a - b; }
template <class V, class R> inline V& operator*=(V& a, const R& b) { return a = a * b; }
template <class V, class R> inline V& operator/=(V& a, const R& b) { return a = a / b; }

// ---- matrices (column-major, m[c] is column c) -----------------------------
struct mat3 {
    vec3 c[3];
    mat3() = default;
    mat3(vec3 a, vec3 b, vec3 d) : c{a, b, d} {}
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, vec3 v) {
    return vec3(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z, m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
                m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
inline vec4 operator*(const mat4& m, vec4 v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r[i] = m.c[0][i] * v.x + m.c[1][i] * v.y + m.c[2][i] * v.z + m.c[3][i] * v.w;
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = a * b.c[j];
    return r;
}

// ---- built-in functions ----------------------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline vec3 abs(vec3 v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline vec4 min(vec4 a, vec4 b) { return vec4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
inline vec4 max(vec4 a, vec4 b) { return vec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec4 clamp(vec4 x, vec4 lo, vec4 hi) { return min(max(x, lo), hi); }
inline vec2 clamp(vec2 x, float lo, float hi) { return vec2(clamp(x.x, lo, hi), clamp(x.y, lo, hi)); }
inline ivec2 clamp(ivec2 x, ivec2 lo, ivec2 hi) { return ivec2(min(max(x.x, lo.x), hi.x), min(max(x.y, lo.y), hi.y)); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(vec3 x, vec3 y, float a) { return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a)); }
inline vec4 mix(vec4 x, vec4 y, float a) {
    return vec4(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a), mix(x.w, y.w, a));
}
inline vec3 mix(vec3 x, vec3 y, vec3 a) { return vec3(mix(x.x, y.x, a.x), mix(x.y, y.y, a.y), mix(x.z, y.z, a.z)); }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float floor(float x) { return std::floor(x); }
inline float fract(float x) { return x - std::floor(x); }
inline vec4 fract(vec4 v) { return vec4(fract(v.x), fract(v.y), fract(v.z), fract(v.w)); }
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
inline float round(float x) { return std::round(x); }
inline vec2 round(vec2 v) { return vec2(std::round(v.x), std::round(v.y)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline vec3 pow(vec3 x, vec3 y) { return vec3(std::pow(x.x, y.x), std::pow(x.y, y.y), std::pow(x.z, y.z)); }
inline float exp(float x) { return std::exp(x); }
inline vec3 exp(vec3 v) { return vec3(std::exp(v.x), std::exp(v.y), std::exp(v.z)); }
inline float acos(float x) { return std::acos(x); }
inline float cos(float x) { return std::cos(x); }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(vec4 a, vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / length(v); }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---- samplers and storage images -------------------------------------------
enum class Address { Repeat, ClampToBorder };

// RGBA texture: uint8 texels (UNORM) or float texels.
struct Texture {
    const uint8_t* u8 = nullptr;
    const float* f32 = nullptr;
    int w = 0, h = 0, d = 1;
    Address mode = Address::Repeat;
    vec4 fetch(long long x, long long y, long long z) const {
        if (mode == Address::Repeat) {
            x = (long long)((unsigned long long)x & (unsigned long long)(w - 1));
            y = (long long)((unsigned long long)y & (unsigned long long)(h - 1));
            z = (long long)((unsigned long long)z & (unsigned long long)(d - 1));
        } else if (x < 0 || y < 0 || z < 0 || x >= w || y >= h || z >= d) {
            return vec4(0.0f, 0.0f, 0.0f, u8 ? 255.0f : 1.0f);  // opaque black
        }
        size_t i = 4 * (((size_t)z * (size_t)h + (size_t)y) * (size_t)w + (size_t)x);
        if (u8) return vec4((float)u8[i], (float)u8[i + 1], (float)u8[i + 2], (float)u8[i + 3]);
        return vec4(f32[i], f32[i + 1], f32[i + 2], f32[i + 3]);
    }
    float scale() const { return u8 ? 1.0f / 255.0f : 1.0f; }
};
struct sampler2D : Texture {};
struct sampler3D : Texture {};

inline vec4 lerp4(vec4 p, vec4 q, float t) {
    return vec4(p.x + t * (q.x - p.x), p.y + t * (q.y - p.y), p.z + t * (q.z - p.z), p.w + t * (q.w - p.w));
}

inline vec4 texture(const sampler3D& s, vec3 c) {
    float u = c.x * (float)s.w - 0.5f, v = c.y * (float)s.h - 0.5f, q = c.z * (float)s.d - 0.5f;
    float fu = std::floor(u), fv = std::floor(v), fq = std::floor(q);
    float a = u - fu, b = v - fv, g = q - fq;
    long long i = f2i(fu), j = f2i(fv), k = f2i(fq);
    vec4 c00 = lerp4(s.fetch(i, j, k), s.fetch(i + 1, j, k), a);
    vec4 c10 = lerp4(s.fetch(i, j + 1, k), s.fetch(i + 1, j + 1, k), a);
    vec4 c01 = lerp4(s.fetch(i, j, k + 1), s.fetch(i + 1, j, k + 1), a);
    vec4 c11 = lerp4(s.fetch(i, j + 1, k + 1), s.fetch(i + 1, j + 1, k + 1), a);
    return lerp4(lerp4(c00, c10, b), lerp4(c01, c11, b), g) * s.scale();
}
inline vec4 texture(const sampler2D& s, vec2 c) {
    float u = c.x * (float)s.w - 0.5f, v = c.y * (float)s.h - 0.5f;
    float fu = std::floor(u), fv = std::floor(v);
    float a = u - fu, b = v - fv;
    long long i = f2i(fu), j = f2i(fv);
    vec4 c0 = lerp4(s.fetch(i, j, 0), s.fetch(i + 1, j, 0), a);
    vec4 c1 = lerp4(s.fetch(i, j + 1, 0), s.fetch(i + 1, j + 1, 0), a);
    return lerp4(c0, c1, b) * s.scale();
}

// RGBA32F storage image.  Out-of-range loads return 0, stores do nothing
// (robust image access).  Reads come from `src`, writes go to `dst`, so an
// image the shader both reads and writes can be kept race-free.
struct image2D {
    const float* src = nullptr;
    float* dst = nullptr;
    int w = 0, h = 0;
};
inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }
inline vec4 imageLoad(const image2D& im, ivec2 p) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h || !im.src) return vec4(0.0f);
    const float* s = im.src + 4 * ((size_t)p.y * (size_t)im.w + (size_t)p.x);
    return vec4(s[0], s[1], s[2], s[3]);
}
inline void imageStore(const image2D& im, ivec2 p, vec4 v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h || !im.dst) return;
    float* d = im.dst + 4 * ((size_t)p.y * (size_t)im.w + (size_t)p.x);
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
    d[3] = v.w;
}

}  // namespace glsl
