// Device-side arithmetic of the compute stage, GLSL semantics, FP32.
//
// The translation units that include this header are compiled with
// -fmad=false and IEEE division/square root, and every expression below keeps
// the operation order of the reference shaders, so the control flow of the
// march (the `t += stepSize` recurrence, the `baseDensity > 0` branch and the
// `accumDensity >= 1` exit of cloudRayMarch.comp:627-684) is reproduced exactly.
// What differs from a host evaluation feeds colour only, never control flow:
// acos/cos/exp/pow of the sky in the last bits (CUDA's libdevice vs the host's
// libm), and the cone-light samples and light energy, evaluated with fused
// multiply-adds, reciprocal products and the special-function unit's
// exp2/log2 (a few to tens of ulp).
//
// Fixed meanings of what GLSL leaves to the implementation:
//   dot = ((a.x*b.x + a.y*b.y) + a.z*b.z); normalize(v) = v / length(v);
//   mix(x,y,a) = x*(1-a) + y*a; min(x,y) = y<x ? y : x; max(x,y) = x<y ? y : x;
//   round = half away from zero; float->int truncates and saturates (NaN -> 0).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/meteoros.h"
#include "mt_kernels.h"

#define MT_HD __device__ __forceinline__

namespace mt {

struct f3 {
    float x, y, z;
};
struct f4v {
    float x, y, z, w;
};

MT_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
MT_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
MT_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
MT_HD f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
MT_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
MT_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
MT_HD f3 operator/(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
MT_HD f3 operator/(f3 a, f3 b) { return f3{a.x / b.x, a.y / b.y, a.z / b.z}; }
MT_HD f4v operator+(f4v a, f4v b) { return f4v{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
MT_HD f4v operator-(f4v a, f4v b) { return f4v{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
MT_HD f4v operator*(f4v a, float s) { return f4v{a.x * s, a.y * s, a.z * s, a.w * s}; }
MT_HD f4v operator/(f4v a, float s) { return f4v{a.x / s, a.y / s, a.z / s, a.w / s}; }

MT_HD float gmin(float a, float b) { return b < a ? b : a; }
MT_HD float gmax(float a, float b) { return a < b ? b : a; }
MT_HD int imin(int a, int b) { return b < a ? b : a; }
MT_HD int imax(int a, int b) { return a < b ? b : a; }
MT_HD float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
MT_HD float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
MT_HD float gfract(float x) { return x - floorf(x); }
MT_HD float gmod(float x, float y) { return x - y * floorf(x / y); }
MT_HD float gsmoothstep(float e0, float e1, float x) {
    float t = gclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
// cvt.rzi.s32.f32: truncation, saturating to the int range, NaN -> 0.
MT_HD int f2i(float v) { return __float2int_rz(v); }

// ---------------------------------------------------------------------------
// Division by a reused denominator, bit-identical to IEEE a / b.
// With y = RN(1/b) and q0 = RN(a*y) (within one ulp of a/b), the residual
// r = a - q0*b is exact in one FMA and q = RN(q0 + r*y) is the correctly
// rounded quotient (Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  The
// theorem excludes overflow and underflow, so tiny, huge and non-finite
// quotients go through the IEEE division; a zero dividend takes q0, which
// carries the quotient's sign when y is finite.
// ---------------------------------------------------------------------------
// The IEEE division, out of line by default: one shared copy keeps the callers
// small in the instruction cache (the march loop is instruction-fetch bound
// otherwise).  Translation units of small kernels define MT_DIV_INLINE.
#ifdef MT_DIV_INLINE
MT_HD float div_ieee(float a, float b) { return a / b; }
#else
static __device__ __noinline__ float div_ieee(float a, float b) { return a / b; }
#endif
// The reciprocal of a denominator: __frcp_rn is the IEEE round-to-nearest-even
// reciprocal, RN(1/b) -- the value 1.0f / b gives -- inline, without the call.
MT_HD Rcp make_rcp(float b) { return Rcp{b, __frcp_rn(b)}; }
MT_HD float rdiv_core(float a, Rcp r) {
    const float q0 = __fmul_rn(a, r.y);
    return __fmaf_rn(__fmaf_rn(-q0, r.b, a), r.y, q0);
}
MT_HD bool rdiv_in_range(float q) {
    const float aq = fabsf(q);
    return aq >= 0x1p-100f && aq <= 0x1p100f;
}
MT_HD float rdiv(float a, Rcp r) {
    const float q = rdiv_core(a, r);
    if (rdiv_in_range(q)) return q;
    if (a == 0.0f && fabsf(r.y) <= 0x1.fffffep127f) return __fmul_rn(a, r.y);
    return div_ieee(a, r.b);
}
// Three quotients by one denominator with one range check; when any falls
// outside it, all three are redone one by one out of line.
static __device__ __noinline__ float2 rdiv2_exceptional(float a, float b, Rcp r) {
    return make_float2(rdiv(a, r), rdiv(b, r));
}
// Two quotients by one denominator, one range check.
MT_HD float2 rdiv2(float a, float b, Rcp r) {
    const float qa = rdiv_core(a, r), qb = rdiv_core(b, r);
    if (rdiv_in_range(qa) & rdiv_in_range(qb)) return make_float2(qa, qb);
    return rdiv2_exceptional(a, b, r);
}
static __device__ __noinline__ f3 rdiv3_exceptional(float ax, float ay, float az, Rcp r) {
    return f3{rdiv(ax, r), rdiv(ay, r), rdiv(az, r)};
}
MT_HD f3 rdiv3(f3 a, Rcp r) {
    const f3 q{rdiv_core(a.x, r), rdiv_core(a.y, r), rdiv_core(a.z, r)};
    if (rdiv_in_range(q.x) & rdiv_in_range(q.y) & rdiv_in_range(q.z)) return q;
    return rdiv3_exceptional(a.x, a.y, a.z, r);
}

MT_HD float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MT_HD float length3(f3 a) { return sqrtf(dot3(a, a)); }
MT_HD f3 normalize3(f3 a) { return a / length3(a); }
// normalize(v) = v / length(v), the three divisions sharing one reciprocal.
MT_HD f3 normalize3_r(f3 a) { return rdiv3(a, make_rcp(length3(a))); }
MT_HD f3 mix3(f3 x, f3 y, float a) { return f3{gmix(x.x, y.x, a), gmix(x.y, y.y, a), gmix(x.z, y.z, a)}; }
MT_HD f4v min4(f4v a, f4v b) { return f4v{gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z), gmin(a.w, b.w)}; }
MT_HD f4v max4(f4v a, f4v b) { return f4v{gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z), gmax(a.w, b.w)}; }
MT_HD f3 ld3(const float* p) { return f3{p[0], p[1], p[2]}; }

MT_HD float lerp1(float p, float q, float t) { return p + t * (q - p); }

// ---------------------------------------------------------------------------
// Packed FP32 pairs: the f32x2 add and multiply-add instructions of sm_100 and
// later carry two values per instruction, each half rounded exactly like the
// scalar operation.  The compiler contracts a packed multiply whose only use
// is a packed add into one fused multiply-add (one rounding instead of two),
// with contraction disabled and explicit round-to-nearest alike, so products
// are formed as fma(a, b, z) with z = -0 read from constant memory:
// fma(a, b, -0) = RN(a * b) for every a and b (signed zeros, infinities and
// NaN included), and an addend unknown to the compiler leaves nothing to
// contract.
// ---------------------------------------------------------------------------
static __constant__ float kNegZero2[2] = {-0.0f, -0.0f};
MT_HD float2 splat2(float v) { return make_float2(v, v); }
MT_HD float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as RN(-1 * b + a): the product is exact, so the one rounding is that of a - b.
MT_HD float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
MT_HD float2 mul2(float2 a, float2 b) { return __ffma2_rn(a, b, make_float2(kNegZero2[0], kNegZero2[1])); }
// p + t * (q - p), each operation rounded (lerp1 on both halves)
MT_HD float2 lerp2(float2 p, float2 q, float2 t) { return add2(p, mul2(t, sub2(q, p))); }

// Four channels as two packed pairs (x, y) and (z, w).
struct f4p {
    float2 xy, zw;
};
MT_HD f4p lerp4p(f4p p, f4p q, float2 t) { return f4p{lerp2(p.xy, q.xy, t), lerp2(p.zw, q.zw, t)}; }
MT_HD f4p pack4(f4v v) { return f4p{make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
MT_HD f4v unpack4(f4p v) { return f4v{v.xy.x, v.xy.y, v.zw.x, v.zw.y}; }
MT_HD f4p add4p(f4p a, f4p b) { return f4p{add2(a.xy, b.xy), add2(a.zw, b.zw)}; }
MT_HD f4p mul4p(f4p a, float s) { return f4p{mul2(a.xy, splat2(s)), mul2(a.zw, splat2(s))}; }
// rdiv of four values by one denominator (rdiv_core on packed pairs: fma(q0, -b, a)
// is fma(-q0, b, a) exactly), one range check; exceptional values redone one by one.
MT_HD f4p rdiv4p(f4p a, Rcp r) {
    const float2 y2 = splat2(r.y), nb2 = splat2(-r.b);
    const float2 q0a = mul2(a.xy, y2), q0b = mul2(a.zw, y2);
    const float2 qa = __ffma2_rn(__ffma2_rn(q0a, nb2, a.xy), y2, q0a);
    const float2 qb = __ffma2_rn(__ffma2_rn(q0b, nb2, a.zw), y2, q0b);
    if (rdiv_in_range(qa.x) & rdiv_in_range(qa.y) & rdiv_in_range(qb.x) & rdiv_in_range(qb.y)) return f4p{qa, qb};
    return f4p{make_float2(rdiv(a.xy.x, r), rdiv(a.xy.y, r)), make_float2(rdiv(a.zw.x, r), rdiv(a.zw.y, r))};
}
MT_HD f4v scale4p(f4p c, float s) {
    const float2 xy = mul2(c.xy, splat2(s)), zw = mul2(c.zw, splat2(s));
    return f4v{xy.x, xy.y, zw.x, zw.y};
}

// A texel byte as a float without a conversion instruction: byte_perm builds
// the word 0x4B0000bb, which is the float 2^23 + bb exactly (the byte lands in
// the low mantissa bits).  Interpolation works on these biased values:
// p = P - 2^23 and q - p = Q - P are exact, so lerp(p, q, t) = p + t*(q - p)
// is reproduced bit for bit.
MT_HD float biased_byte(uint32_t word, unsigned c) { return __int_as_float(__byte_perm(word, 0x4B000000u, 0x7540u | c)); }
constexpr float kByteBias = 8388608.0f;
MT_HD float2 biased_pair(uint32_t word, unsigned c) { return make_float2(biased_byte(word, c), biased_byte(word, c + 1u)); }

// The x interpolation of two RGBA8 texels, (P - 2^23) + t * (Q - P) per channel.
MT_HD f4p lerp_texels(uint32_t w0, uint32_t w1, float2 t) {
    const float2 bias = splat2(kByteBias);
    const float2 P0 = biased_pair(w0, 0u), Q0 = biased_pair(w1, 0u);
    const float2 P1 = biased_pair(w0, 2u), Q1 = biased_pair(w1, 2u);
    return f4p{add2(sub2(P0, bias), mul2(t, sub2(Q0, P0))), add2(sub2(P1, bias), mul2(t, sub2(Q1, P1)))};
}

// ---------------------------------------------------------------------------
// Light-sample sampler: the same trilinear filter with every lerp one fused
// multiply-add, p + t * (q - p) rounded once.  The cone-light samples reach
// colour only (through the light energy), never the accumulated density, the
// control flow or the god-ray mask, so they are held to the colour tolerance
// rather than to the shader's exact operation sequence.
// ---------------------------------------------------------------------------
MT_HD f4p lerp_texels_fused(uint32_t w0, uint32_t w1, float2 t) {
    const float2 bias = splat2(kByteBias);
    const float2 P0 = biased_pair(w0, 0u), Q0 = biased_pair(w1, 0u);
    const float2 P1 = biased_pair(w0, 2u), Q1 = biased_pair(w1, 2u);
    return f4p{__ffma2_rn(t, sub2(Q0, P0), sub2(P0, bias)), __ffma2_rn(t, sub2(Q1, P1), sub2(P1, bias))};
}
MT_HD f4p lerp4p_fused(f4p p, f4p q, float2 t) {
    return f4p{__ffma2_rn(t, sub2(q.xy, p.xy), p.xy), __ffma2_rn(t, sub2(q.zw, p.zw), p.zw)};
}

// ---------------------------------------------------------------------------
// Samplers.  Vulkan LINEAR filter with exact FP32 weights: u = s*N - 0.5,
// i0 = floor(u), alpha = u - i0, REPEAT wraps the integer texel coordinate
// (N is a power of two).  Raw texel values are interpolated x, then y, then
// z, and the result is scaled once (1/255 for UNORM8), channels in packed
// pairs.  The RGBA8 volumes are read in their plane-quad layout
// (launch_quads3): entry (x0, y0, z) holds the four texels {(x0,y0), (x1,y0),
// (x0,y1), (x1,y1)} of plane z, each an RGBA8 word of the volume (x fastest,
// then y, then z, ImageLoadingUtility.cpp:75-139), so a trilinear fetch is two
// 16-byte loads (planes z0 and z1); the images are read in bilinear cells
// (launch_cells2), one 16-byte load per fetch.
// ---------------------------------------------------------------------------
template <int N> MT_HD f4v tex3_u8(const uint4* __restrict__ quads, f3 s) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = s.x * fn - 0.5f, v = s.y * fn - 0.5f, w = s.z * fn - 0.5f;
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    float a = u - fu, b = v - fv, g = w - fw;
    const unsigned x0 = (unsigned)f2i(fu) & M, y0 = (unsigned)f2i(fv) & M, z0 = (unsigned)f2i(fw) & M;
    const uint4 q0 = __ldg(quads + (((size_t)z0 * N + y0) * N + x0));
    const uint4 q1 = __ldg(quads + (((size_t)((z0 + 1u) & M) * N + y0) * N + x0));
    const float2 a2 = splat2(a), b2 = splat2(b), g2 = splat2(g);
    const f4p c00 = lerp_texels(q0.x, q0.y, a2);
    const f4p c10 = lerp_texels(q0.z, q0.w, a2);
    const f4p c01 = lerp_texels(q1.x, q1.y, a2);
    const f4p c11 = lerp_texels(q1.z, q1.w, a2);
    const f4p c0 = lerp4p(c00, c10, b2);
    const f4p c1 = lerp4p(c01, c11, b2);
    return scale4p(lerp4p(c0, c1, g2), 1.0f / 255.0f);
}

// tex3_u8 with fused lerps (light samples).
template <int N> MT_HD f4v tex3_u8_fused(const uint4* __restrict__ quads, f3 s) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = fmaf(s.x, fn, -0.5f), v = fmaf(s.y, fn, -0.5f), w = fmaf(s.z, fn, -0.5f);
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    float a = u - fu, b = v - fv, g = w - fw;
    const unsigned x0 = (unsigned)f2i(fu) & M, y0 = (unsigned)f2i(fv) & M, z0 = (unsigned)f2i(fw) & M;
    const uint4 q0 = __ldg(quads + (((size_t)z0 * N + y0) * N + x0));
    const uint4 q1 = __ldg(quads + (((size_t)((z0 + 1u) & M) * N + y0) * N + x0));
    const float2 a2 = splat2(a), b2 = splat2(b), g2 = splat2(g);
    const f4p c00 = lerp_texels_fused(q0.x, q0.y, a2);
    const f4p c10 = lerp_texels_fused(q0.z, q0.w, a2);
    const f4p c01 = lerp_texels_fused(q1.x, q1.y, a2);
    const f4p c11 = lerp_texels_fused(q1.z, q1.w, a2);
    const f4p c0 = lerp4p_fused(c00, c10, b2);
    const f4p c1 = lerp4p_fused(c01, c11, b2);
    return scale4p(lerp4p_fused(c0, c1, g2), 1.0f / 255.0f);
}

template <int N> MT_HD f4v tex2_u8(const uint4* __restrict__ cells, float sx, float sy) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = sx * fn - 0.5f, v = sy * fn - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    const unsigned x0 = (unsigned)f2i(fu) & M, y0 = (unsigned)f2i(fv) & M;
    const uint4 q = __ldg(cells + ((size_t)y0 * N + x0));
    const float2 a2 = splat2(a);
    const f4p c0 = lerp_texels(q.x, q.y, a2);
    const f4p c1 = lerp_texels(q.z, q.w, a2);
    return scale4p(lerp4p(c0, c1, splat2(b)), 1.0f / 255.0f);
}

// ---------------------------------------------------------------------------
// Precision-form samplers: texels stored as four 16-bit values (uint2 =
// (r,g),(b,a) pairs, IEEE half or bfloat16), interpolated as packed pairs
// (half2 / bfloat16x2 fused multiply-adds), the weights rounded to the pair
// type.  The index arithmetic is the FP32 one above.  Results are returned
// in FP32; the precision form is measured against the FP64 oracle.
// ---------------------------------------------------------------------------
template <class P> struct Pair;
template <> struct Pair<__half2> {
    static MT_HD __half2 from_bits(uint32_t u) { return *reinterpret_cast<__half2*>(&u); }
    static MT_HD __half2 splat(float f) { return __float2half2_rn(f); }
    static MT_HD float2 to_float2(__half2 h) { return __half22float2(h); }
    // (a.low, b.low) and (a.high, b.high)
    static MT_HD __half2 lows(__half2 a, __half2 b) { return __lows2half2(a, b); }
    static MT_HD __half2 highs(__half2 a, __half2 b) { return __highs2half2(a, b); }
};
template <> struct Pair<__nv_bfloat162> {
    static MT_HD __nv_bfloat162 from_bits(uint32_t u) { return *reinterpret_cast<__nv_bfloat162*>(&u); }
    static MT_HD __nv_bfloat162 splat(float f) { return __float2bfloat162_rn(f); }
    static MT_HD float2 to_float2(__nv_bfloat162 h) { return __bfloat1622float2(h); }
    static MT_HD __nv_bfloat162 lows(__nv_bfloat162 a, __nv_bfloat162 b) { return __lows2bfloat162(a, b); }
    static MT_HD __nv_bfloat162 highs(__nv_bfloat162 a, __nv_bfloat162 b) { return __highs2bfloat162(a, b); }
};

template <class P> struct PairTexel {
    P rg, ba;
};
template <class P> MT_HD PairTexel<P> ld_pair(const uint2* __restrict__ p) {
    const uint2 v = __ldg(p);
    return PairTexel<P>{Pair<P>::from_bits(v.x), Pair<P>::from_bits(v.y)};
}
template <class P> MT_HD PairTexel<P> lerp_pair(PairTexel<P> p, PairTexel<P> q, P t) {
    return PairTexel<P>{__hfma2(t, __hsub2(q.rg, p.rg), p.rg), __hfma2(t, __hsub2(q.ba, p.ba), p.ba)};
}
template <class P> MT_HD f4v pair_to_f4(PairTexel<P> c) {
    const float2 rg = Pair<P>::to_float2(c.rg), ba = Pair<P>::to_float2(c.ba);
    return f4v{rg.x, rg.y, ba.x, ba.y};
}

// The 16-bit volumes in their plane-quad layout (launch_quads16): entry
// (x0, y0, z) holds {(x0,y0), (x1,y0)} and {(x0,y1), (x1,y1)} of plane z, so a
// trilinear fetch is two 32-byte entries (planes z0 and z1), four 16-byte
// loads; the lerps run in the pair type (weights rounded to it).
template <class P> MT_HD PairTexel<P> pair_lo(uint4 q) {
    return PairTexel<P>{Pair<P>::from_bits(q.x), Pair<P>::from_bits(q.y)};
}
template <class P> MT_HD PairTexel<P> pair_hi(uint4 q) {
    return PairTexel<P>{Pair<P>::from_bits(q.z), Pair<P>::from_bits(q.w)};
}
template <int N, class P> MT_HD PairTexel<P> tex3_p16q_pairs(const uint4* __restrict__ quads, f3 s);
template <int N, class P> MT_HD f4v tex3_p16q(const uint4* __restrict__ quads, f3 s) {
    return pair_to_f4(tex3_p16q_pairs<N, P>(quads, s));
}
// The filtered texel as its two pairs, (r, g) and (b, a), in the pair type.
template <int N, class P> MT_HD PairTexel<P> tex3_p16q_pairs(const uint4* __restrict__ quads, f3 s) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = s.x * fn - 0.5f, v = s.y * fn - 0.5f, w = s.z * fn - 0.5f;
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const P a = Pair<P>::splat(u - fu), b = Pair<P>::splat(v - fv), g = Pair<P>::splat(w - fw);
    const unsigned x0 = (unsigned)f2i(fu) & M, y0 = (unsigned)f2i(fv) & M, z0 = (unsigned)f2i(fw) & M;
    const unsigned z1 = (z0 + 1u) & M;
    const uint4* q0 = quads + 2 * (((size_t)z0 * N + y0) * N + x0);
    const uint4* q1 = quads + 2 * (((size_t)z1 * N + y0) * N + x0);
    const uint4 e00 = __ldg(q0), e01 = __ldg(q0 + 1), e10 = __ldg(q1), e11 = __ldg(q1 + 1);
    PairTexel<P> c00 = lerp_pair(pair_lo<P>(e00), pair_hi<P>(e00), a);
    PairTexel<P> c10 = lerp_pair(pair_lo<P>(e01), pair_hi<P>(e01), a);
    PairTexel<P> c01 = lerp_pair(pair_lo<P>(e10), pair_hi<P>(e10), a);
    PairTexel<P> c11 = lerp_pair(pair_lo<P>(e11), pair_hi<P>(e11), a);
    return lerp_pair(lerp_pair(c00, c10, b), lerp_pair(c01, c11, b), g);
}

// The same fetch with FP32 weights and FP32 lerps of the 16-bit texel values
// (each pair widened to float2, then the packed FP32 pairs of the RGBA8 path).
template <class P> MT_HD f4p widen(uint32_t rg, uint32_t ba) {
    return f4p{Pair<P>::to_float2(Pair<P>::from_bits(rg)), Pair<P>::to_float2(Pair<P>::from_bits(ba))};
}
template <int N, class P> MT_HD f4v tex3_p16q_f32(const uint4* __restrict__ quads, f3 s) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = s.x * fn - 0.5f, v = s.y * fn - 0.5f, w = s.z * fn - 0.5f;
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const float2 a2 = splat2(u - fu), b2 = splat2(v - fv), g2 = splat2(w - fw);
    const unsigned x0 = (unsigned)f2i(fu) & M, y0 = (unsigned)f2i(fv) & M, z0 = (unsigned)f2i(fw) & M;
    const unsigned z1 = (z0 + 1u) & M;
    const uint4* q0 = quads + 2 * (((size_t)z0 * N + y0) * N + x0);
    const uint4* q1 = quads + 2 * (((size_t)z1 * N + y0) * N + x0);
    const uint4 e00 = __ldg(q0), e01 = __ldg(q0 + 1), e10 = __ldg(q1), e11 = __ldg(q1 + 1);
    const f4p c00 = lerp4p_fused(widen<P>(e00.x, e00.y), widen<P>(e00.z, e00.w), a2);
    const f4p c10 = lerp4p_fused(widen<P>(e01.x, e01.y), widen<P>(e01.z, e01.w), a2);
    const f4p c01 = lerp4p_fused(widen<P>(e10.x, e10.y), widen<P>(e10.z, e10.w), a2);
    const f4p c11 = lerp4p_fused(widen<P>(e11.x, e11.y), widen<P>(e11.z, e11.w), a2);
    return unpack4(lerp4p_fused(lerp4p_fused(c00, c10, b2), lerp4p_fused(c01, c11, b2), g2));
}
template <int N, class P> MT_HD f4v tex2_p16_f32(const uint2* __restrict__ img, float sx, float sy) {
    constexpr unsigned M = (unsigned)N - 1u;
    const float fn = (float)N;
    float u = sx * fn - 0.5f, v = sy * fn - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    const float2 a2 = splat2(u - fu), b2 = splat2(v - fv);
    unsigned iu = (unsigned)f2i(fu), iv = (unsigned)f2i(fv);
    unsigned x0 = iu & M, x1 = (iu + 1u) & M, y0 = iv & M, y1 = (iv + 1u) & M;
    const uint2 t00 = __ldg(img + y0 * N + x0), t10 = __ldg(img + y0 * N + x1);
    const uint2 t01 = __ldg(img + y1 * N + x0), t11 = __ldg(img + y1 * N + x1);
    const f4p c0 = lerp4p_fused(widen<P>(t00.x, t00.y), widen<P>(t10.x, t10.y), a2);
    const f4p c1 = lerp4p_fused(widen<P>(t01.x, t01.y), widen<P>(t11.x, t11.y), a2);
    return unpack4(lerp4p_fused(c0, c1, b2));
}

// Bilinear sample of an RGBA32F frame with CLAMP_TO_BORDER, opaque black
// border (Texture2D.cpp:75 with Image.cpp:324).
MT_HD f4v tex2_border(const float4* __restrict__ img, int W, int H, float sx, float sy) {
    float u = sx * (float)W - 0.5f, v = sy * (float)H - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    int i0 = f2i(fu), j0 = f2i(fv);
    long long i1 = (long long)i0 + 1, j1 = (long long)j0 + 1;
    auto at = [&](long long i, long long j) -> f4p {
        if (i < 0 || j < 0 || i >= W || j >= H) return f4p{make_float2(0.0f, 0.0f), make_float2(0.0f, 1.0f)};
        float4 q = __ldg(img + (size_t)j * (size_t)W + (size_t)i);
        return f4p{make_float2(q.x, q.y), make_float2(q.z, q.w)};
    };
    const float2 a2 = splat2(a);
    const f4p c0 = lerp4p(at(i0, j0), at(i1, j0), a2);
    const f4p c1 = lerp4p(at(i0, j1), at(i1, j1), a2);
    return unpack4(lerp4p(c0, c1, splat2(b)));
}

}  // namespace mt
