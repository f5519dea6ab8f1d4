// The raymarch kernel (cloudRayMarch.comp:565-826), templated on the lanes
// per ray and on the storage of the noise volumes:
//   MT_STORAGE_U8    RGBA8 volumes, exact FP32 filtering (the plain form)
//   MT_STORAGE_F16   IEEE half volumes (precision form): the primary fetches
//                    filtered in FP32; the cone-light samples' filtering and
//                    density math (FBM, remaps, coverage) in half2, two
//                    samples per pair
//   MT_STORAGE_BF16  bfloat16 volumes, filtered in FP32 (a storage form)
// Apart from the FP16 form's cone-light density math, everything after the
// filtered texel (FBM, remaps, erosion, lighting, transmittance, radiance,
// accumulation) is FP32.  Each storage is instantiated by its own translation
// unit (mt_march_u8.cu, mt_march_f16.cu, mt_march_bf16.cu).
#pragma once
#include "mt_shared.cuh"

namespace mt {

// Storage-specific volume access.
template <int S> struct Vol;
// T3: the element of the 3D volumes (base, detail), T2: of the 2D images
// (curl, weather), as build_march_args points at them.
template <> struct Vol<MT_STORAGE_U8> {
    using T3 = uint4;  // plane quads (launch_quads3)
    using T2 = uint4;  // bilinear cells (launch_cells2)
    template <int N> static MT_HD f4v tex3(const T3* v, f3 s) { return tex3_u8<N>(v, s); }
    template <int N> static MT_HD f4v tex3_light(const T3* v, f3 s) { return tex3_u8_fused<N>(v, s); }
    template <int N> static MT_HD f4v tex2(const T2* v, float x, float y) { return tex2_u8<N>(v, x, y); }
};
// The 16-bit storages (P the packed pair type): every fetch filters the
// 16-bit texels in FP32, except the FP16 form's six cone-light samples per
// in-cloud step, which reach colour only and run in half2 (lerps and density
// math, sample_light_pair).
template <class P> struct Vol16 {
    using T3 = uint4;  // plane quads (launch_quads16)
    using T2 = uint2;
    template <int N> static MT_HD f4v tex3(const T3* v, f3 s) { return tex3_p16q_f32<N, P>(v, s); }
    // bfloat16 (an 8-bit mantissa) filters its cone-light samples in FP32 too
    template <int N> static MT_HD f4v tex3_light(const T3* v, f3 s) { return tex3_p16q_f32<N, P>(v, s); }
    template <int N> static MT_HD f4v tex2(const T2* v, float x, float y) { return tex2_p16_f32<N, P>(v, x, y); }
};
template <> struct Vol<MT_STORAGE_F16> : Vol16<__half2> {};
template <> struct Vol<MT_STORAGE_BF16> : Vol16<__nv_bfloat162> {};

struct Weather {
    float lo, mul, type;
    float hgrad;  // height gradient at the primary sample, shared by its light samples
    Rcp r_lo;     // {1 - lo, ~1/(1 - lo)}: the coverage remap's width (b, exact division)
                  // and an approximate reciprocal for the light samples (y)
};

template <int S> struct Tex {
    const typename Vol<S>::T3* base;
    const typename Vol<S>::T3* detail;
    const typename Vol<S>::T2* curl;
    const typename Vol<S>::T2* weather;
};
template <int S> MT_HD Tex<S> make_tex(const MarchArgs& a) {
    return Tex<S>{(const typename Vol<S>::T3*)a.vol[0], (const typename Vol<S>::T3*)a.vol[1],
                  (const typename Vol<S>::T2*)a.vol[2], (const typename Vol<S>::T2*)a.vol[3]};
}

template <int S> MT_HD Weather weather_at(const mt_params& p, const Frame& F, const Tex<S>& tx, f3 pos, f3 ec) {
    Weather w;
    w.hgrad = 1.0f;
    if (p.coverage_mode == 0) {
        w.lo = p.coverage;
        w.mul = p.coverage;
        w.type = 0.0f;
    } else {
        const float2 wuv = rdiv2(pos.x - ec.x, pos.z - ec.z, F.r_weather);
        f4v wd = Vol<S>::template tex2<MT_WEATHER_N>(tx.weather, wuv.x, wuv.y);
        w.lo = 1.0f - wd.x;
        w.mul = wd.x;
        w.type = wd.z;
    }
    w.r_lo = Rcp{1.0f - w.lo, __fdividef(1.0f, 1.0f - w.lo)};
    return w;
}

// cloudRayMarch.comp:499-540
template <int S>
MT_HD float sample_low_frequency(const mt_params& p, const Tex<S>& tx, f3 point, float relH, const Weather& wt) {
    f4v n = Vol<S>::template tex3<MT_BASE_N>(tx.base, point);
    float fbm = (n.y * 0.625f) + (n.z * 0.25f) + (n.w * 0.125f);
    fbm = gclamp(fbm, 0.0f, 1.0f);
    float baseCloud = remap_clamped(n.x, (fbm - 0.9f), 1.0f, 0.0f, 1.0f);
    // getDensityHeightGradientForPoint(relH, type): every call of a step passes
    // the primary sample's height and weather, so it is evaluated once per step
    // (Weather::hgrad).
    if (p.height_gradient) baseCloud = baseCloud * wt.hgrad;
    // remapClampedBeforeAndAfter(baseCloud, lo, 1, 0, 1), its width 1 - lo
    // computed once per step
    float v = gclamp(baseCloud, wt.lo, 1.0f);
    float bc = gclamp(0.0f + (((v - wt.lo) / wt.r_lo.b) * (1.0f - 0.0f)), 0.0f, 1.0f);
    return bc * wt.mul;
}

// sample_low_frequency for a cone-light sample (cloudRayMarch.comp:659-666).
// Light samples reach colour only: fused lerps, the quotients as products with
// the reciprocal (the remap's varying one by the fast division) and min/max
// clamps, a few ulp from the exact sequence above.
template <int S>
MT_HD float sample_light(const mt_params& p, const Tex<S>& tx, f3 point, const Weather& wt) {
    const f4v n = Vol<S>::template tex3_light<MT_BASE_N>(tx.base, point);
    float fbm = fmaf(n.w, 0.125f, fmaf(n.z, 0.25f, n.y * 0.625f));
    fbm = fminf(fmaxf(fbm, 0.0f), 1.0f);
    const float lo = fbm - 0.9f;
    float baseCloud = fminf(fmaxf(__fdividef(n.x - lo, 1.0f - lo), 0.0f), 1.0f);
    if (p.height_gradient) baseCloud = baseCloud * wt.hgrad;
    const float v = fminf(fmaxf(baseCloud, wt.lo), 1.0f);
    const float bc = fminf(fmaxf((v - wt.lo) * wt.r_lo.y, 0.0f), 1.0f);
    return bc * wt.mul;
}

// Two cone-light samples at once in the pair type (FP16 storage): sample i in
// the low half, sample i + 1 in the high half.  Each sample's filtered texel,
// FBM, base-shape remap, height gradient and coverage remap --
// sample_light's steps, with the division by a reciprocal -- run as half2
// arithmetic; the results return to FP32 for the erosion and the accumulation
// of the light density.  (bfloat16's 8-bit mantissa is too coarse for this:
// the bfloat16 form does its cone-light samples in FP32.)
template <class P>
MT_HD float2 sample_light_pair(const mt_params& p, const uint4* base, f3 s0, f3 s1, const Weather& wt) {
    using Q = Pair<P>;
    const PairTexel<P> n0 = tex3_p16q_pairs<MT_BASE_N, P>(base, s0);
    const PairTexel<P> n1 = tex3_p16q_pairs<MT_BASE_N, P>(base, s1);
    const P x = Q::lows(n0.rg, n1.rg), y = Q::highs(n0.rg, n1.rg);
    const P z = Q::lows(n0.ba, n1.ba), w = Q::highs(n0.ba, n1.ba);
    const P zero = Q::splat(0.0f), one = Q::splat(1.0f);
    P fbm = __hfma2(w, Q::splat(0.125f), __hfma2(z, Q::splat(0.25f), __hmul2(y, Q::splat(0.625f))));
    fbm = __hmin2(__hmax2(fbm, zero), one);
    const P lo = __hsub2(fbm, Q::splat(0.9f));
    P bc = __hmin2(__hmax2(__hmul2(__hsub2(x, lo), h2rcp(__hsub2(one, lo))), zero), one);
    if (p.height_gradient) bc = __hmul2(bc, Q::splat(wt.hgrad));
    const P wlo = Q::splat(wt.lo);
    const P v = __hmin2(__hmax2(bc, wlo), one);
    bc = __hmin2(__hmax2(__hmul2(__hsub2(v, wlo), Q::splat(wt.r_lo.y)), zero), one);
    return Q::to_float2(__hmul2(bc, Q::splat(wt.mul)));
}

// cloudRayMarch.comp:542-563.  The texture part is the same for the primary
// erosion (:645) and the six cone-light erosions (:665): all are evaluated at
// the primary sample point with the primary height, so it is computed once.
template <int S> MT_HD float erosion_modifier(const Tex<S>& tx, f3 point, float h) {
    f4v curl = Vol<S>::template tex2<MT_CURL_N>(tx.curl, point.x, point.y);
    point.x = point.x + (curl.x * (1.0f - h)) * 0.5f;
    point.y = point.y + (curl.y * (1.0f - h)) * 0.5f;
    f4v hf = Vol<S>::template tex3<MT_DETAIL_N>(tx.detail, point);
    float hfbm = (hf.x * 0.625f) + (hf.y * 0.25f) + (hf.z * 0.125f);
    return gclamp(gmix(hfbm, 1.0f - hfbm, gclamp(h * 2.0f, 0.0f, 1.0f)), 0.0f, 1.0f);
}
// Per-ray constants of cloudRayMarch.comp:565-624, shared by every step (the
// per-frame ones are in Frame).
struct RayConsts {
    f3 dir, startPos;
    f3 koff[6];  // cone-light offsets ((stepSize * kernel[i]) * i) / thickness
    float stepSize, cos_angle, cos_q, HG_light, lenInner;
};

MT_HD void ray_consts(const mt_params& p, const Frame& F, f3 dir, f3 startPos, float stepSize, RayConsts& rc) {
    rc.dir = dir;
    rc.startPos = startPos;
    rc.stepSize = stepSize;
    // the sun direction and the cone-light kernel are the frame's (Frame::light_dir, cone)
    const f3 lightDir = ld3(F.light_dir);
    rc.cos_angle = dot3(normalize3_r(dir), lightDir);
    rc.cos_q = rdiv(rc.cos_angle - 0.7f, MT_RCP(0.7f, 1.0f));
    rc.HG_light = gmax(henyey_greenstein(rc.cos_angle, 0.6f), 0.7f * henyey_greenstein(rc.cos_angle, 0.99f - 0.1f));
    // the step-independent part of the light sample position
    // pos + ((stepSize * kernel[i]) * i) (cloudRayMarch.comp:656)
    // in units of the layer thickness, as the light samples' positions are used
    for (int i = 0; i < 6; ++i) rc.koff[i] = ((stepSize * ld3(F.cone[i])) * (float)i) * F.r_thick.y;
    rc.lenInner = length3(startPos - ld3(F.eye));
}

struct StepOut {
    // bit 4: baseDensity > 0 (cloudRayMarch.comp:642).  Traced marches (TR)
    // also carry the step's jitter index in bits 0-3 and its light samples'
    // cbl > 0 in bits 5-10: the step's part of the control-flow signature.
    int code;
    float hfd;  // eroded density (:645)
    float E;    // light energy (:673)
};
constexpr int kInCloud = 16;

// One iteration of the march loop body (cloudRayMarch.comp:629-678) at
// parameter t, up to the accumulation: everything that does not depend on the
// running accumDensity / transmittance.
template <int S, bool TR>
MT_HD StepOut eval_step(const mt_params& p, const Frame& F, const Tex<S>& tx, const mt_time_ubo& tm,
                        const float (*jitter)[3], const RayConsts& rc, float t) {
    StepOut o{0, 0.0f, 0.0f};
    const int _index = f2i(gmod((float)(tm.frame_count_mod16 + f2i(t)), 16.0f));
    if (TR) o.code = _index & 15;
    const float* j = jitter[_index & 15];  // _index is in 0..15 for every finite t
    f3 jd = rc.dir + f3{j[0], j[1], j[2]};
    f3 pos = ld3(F.eye) + t * jd;
    f3 sp = relative_position(F, pos, ld3(F.ec));
    sp = rdiv3(sp, F.r_period);
    float relH = relative_height(F, pos, ld3(F.ec), rc.lenInner, rc.dir, ld3(F.eye));
    sp = sp + ((relH * ld3(F.skew)) * p.cloud_top_offset) * 0.009f;
    sp = sp + ld3(F.wind_t);
    Weather wt = weather_at<S>(p, F, tx, pos, ld3(F.ec));
    if (p.height_gradient) wt.hgrad = height_gradient(relH, wt.type);
    // A zero height gradient or zero coverage makes the density 0 (or NaN
    // when the coverage is 0), never > 0: the step is empty whatever the base
    // volume holds, so its texture fetch is skipped (results unchanged).
    if ((p.height_gradient && wt.hgrad == 0.0f) || wt.mul == 0.0f) return o;
    float baseDensity = sample_low_frequency<S>(p, tx, sp, relH, wt) * 0.380f;
    if (baseDensity > 0.0f) {
        const Erosion ero = make_erosion(erosion_modifier<S>(tx, sp, relH));
        o.code |= kInCloud;
        o.hfd = erode(baseDensity * 1.4f, ero);
        float dl = 0.0f;
        // The six cone-light samples (colour only: see sample_light).  Kept
        // rolled: six inlined copies of the sampler overflow the instruction
        // cache.
        // relative_position(pos + offset) = (pos - base) / thickness + offset / thickness.
        // Explicit roundings and fmas: the same bits in every kernel that
        // inlines this, whatever the compiler's contraction setting.
        const f3 pb = pos - f3{F.ec[0], F.inner_alt, F.ec[2]};
        const f3 prel{__fmul_rn(pb.x, F.r_thick.y), __fmul_rn(pb.y, F.r_thick.y), __fmul_rn(pb.z, F.r_thick.y)};
        auto light_point = [&](int i) {
            const f3 k = rc.koff[i];
            return f3{__fadd_rn(prel.x, k.x), __fadd_rn(prel.y, k.y), __fadd_rn(prel.z, k.z)};
        };
        if constexpr (S != MT_STORAGE_F16) {
#pragma unroll 1
            for (int i = 0; i < 6; ++i) {
                const float cbl = sample_light<S>(p, tx, light_point(i), wt);
                if (cbl > 0.0f) {
                    dl = fmaf(fmaf(1.5f, cbl, -ero.lo), ero.r.y, dl);  // erode(1.5 * cbl)
                    if (TR) o.code |= 32 << i;
                }
            }
        } else {
            // FP16 storage: two samples at a time, density math in half2
#pragma unroll 1
            for (int i = 0; i < 6; i += 2) {
                const float2 cbl = sample_light_pair<__half2>(p, tx.base, light_point(i), light_point(i + 1), wt);
                if (cbl.x > 0.0f) {
                    dl = fmaf(fmaf(1.5f, cbl.x, -ero.lo), ero.r.y, dl);
                    if (TR) o.code |= 32 << i;
                }
                if (cbl.y > 0.0f) {
                    dl = fmaf(fmaf(1.5f, cbl.y, -ero.lo), ero.r.y, dl);
                    if (TR) o.code |= 32 << (i + 1);
                }
            }
        }
        o.E = light_energy(relH, dl, baseDensity, rc.HG_light, rc.cos_q, 5.0f);
    }
    return o;
}

// cloudRayMarch.comp:565-688, step-parallel.  A group of G lanes marches one
// ray: lane j evaluates step c*G + j of chunk c, with t rebuilt by the same
// serial `t += stepSize` additions as the reference's loop, so every lane sees
// bit-identical t.  The loop-carried part (accumDensity, transmittance,
// colour, the early exit) is then applied in step order by an in-group scan;
// steps past the exit are discarded.  Result, counters and control flow equal
// the sequential loop's.
template <int G, int S, bool TR>
MT_HD f3 ray_march_group(const mt_params& p, const Frame& F, const Tex<S>& tx, const mt_time_ubo& tm,
                         const float (*jitter)[3], f3 dir, f3 startPos, float start_t, float end_t, float& accum,
                         Counts& cnt, unsigned gmask, int lane) {
    float _dot = dot3(dir, f3{0.0f, 1.0f, 0.0f});
    float maxSteps;
    if (p.steps_min == p.steps_max)
        maxSteps = (float)p.steps_min;
    else
        maxSteps = floorf(gmix((float)p.steps_min, (float)p.steps_max, 1.0f - _dot));
    const float thick = end_t - start_t;
    const float stepSize = thick / maxSteps;
    RayConsts rc;
    ray_consts(p, F, dir, startPos, stepSize, rc);
    float transmittance = 1.0f;
    f3 color{0.0f, 0.0f, 0.0f};
    // Iteration guard (not in the reference): a step below the ulp of t would
    // never advance.  A valid ray runs steps or steps+1 iterations.
    const int cap = 2 * f2i(maxSteps) + 8;
    if (lane == 0) cnt.rays++;
    float t_base = start_t;
    int s_base = 0;
    bool done = false;
    while (!done) {
        float t = t_base;
        for (int k = 0; k < lane; ++k) t += stepSize;
        const int valid = (t < end_t) && (s_base + lane < cap);
        StepOut o{0, 0.0f, 0.0f};
        if (valid) o = eval_step<S, TR>(p, F, tx, tm, jitter, rc, t);
#pragma unroll
        for (int k = 0; k < G; ++k) {
            if (!__shfl_sync(gmask, valid, k, G)) {
                done = true;
                break;
            }
            const int code = __shfl_sync(gmask, o.code, k, G);
            const float hfd = __shfl_sync(gmask, o.hfd, k, G);
            const float E = __shfl_sync(gmask, o.E, k, G);
            if (lane == 0) cnt.primary++;
            if (TR && lane == 0) cnt.sig = (cnt.sig ^ (unsigned)code) * 16777619u;  // FNV-1a step
            if (code & kInCloud) {
                accum = accum + hfd * 0.5f;
                transmittance = gmix(transmittance, E, (1.0f - accum));
                color = color + f3{transmittance, transmittance, transmittance};
                if (lane == 0) cnt.light += 6;
            }
            if (accum >= p.accum_limit) {
                accum = 1.0f;
                done = true;
                break;
            }
        }
        if (!done) {
            t_base = __shfl_sync(gmask, t, G - 1, G) + stepSize;
            s_base += G;
        }
    }
    return color;
}

// cloudRayMarch.comp:690-826 for one pixel, marched by a group of G lanes;
// lane 0 stores.  `jitter`: the view's per-step jitter table (a.jitter, or a
// copy of it in shared memory).
template <int G, int S, bool TR = false>
MT_HD void march_pixel(const MarchArgs& a, const Frame& F, const Tex<S>& tx, int px, int py, Counts& cnt,
                       unsigned gmask, int lane, const float (*jitter)[3]) {
    const mt_params& p = a.params;
    const int W = a.width;
    // this frame's camera basis and cloudRayMarch.comp's jitter: the TXAA
    // geometry constants (the same camera, slot and image size)
    const ViewConsts& vc = a.vc_txaa;
    float ux = rdiv((float)px, Rcp{vc.r_w[0], vc.r_w[1]}), uy = rdiv((float)py, Rcp{vc.r_h[0], vc.r_h[1]});
    uy = 1.0f - uy;
    const Ray ray = cast_ray(vc, ld3(F.eye), ux, uy);
    float _dot = dot3(f3{0.0f, 1.0f, 0.0f}, ray.direction);
    const float bgMul = gmax(0.620f, _dot);
    const float fade = 0.06f;
    const size_t o = (size_t)py * (size_t)W + (size_t)px;
    f3 bg;
    if (_dot < 0.0f) {
        f3 cNear = f3{0.0f, 0.16f, 0.51f} * 0.4f;
        f3 c2 = f3{0.0f, 0.73f, 0.95f} * 0.5f;
        bg = mix3(cNear, c2, -ray.direction.y * 5.5f);
        if (lane == 0) {
            a.cur[o] = make_float4(bg.x, bg.y, bg.z, 1.0f);
            if (a.mask) a.mask[o] = 0.0f;
            if (TR) a.trace[o] = make_uint4(0u, 0u, 0u, 0u);
        }
        return;
    }
    bg = atmosphere_color(F, ray.direction);  // sunIntensity 0.780 is in F.sky_sunE
    bg = bg * bgMul;
    if (_dot < fade) {
        if (lane == 0) {
            a.cur[o] = make_float4(bg.x, bg.y, bg.z, 1.0f);
            if (a.mask) a.mask[o] = 0.0f;
            if (TR) a.trace[o] = make_uint4(0u, 0u, 0u, 0u);
        }
        return;
    }
    const f3 ec = ld3(F.ec);
    Isect in, out;
    if (p.fp64_shells) {
        // ray.origin is the eye: the origin terms are the frame's
        in = ray_sphere_fp64(F.sh_o[0], F.sh_c[0], ray.direction, ec, F.Rin);
        out = ray_sphere_fp64(F.sh_o[1], F.sh_c[1], ray.direction, ec, F.Rout);
    } else {
        in = ray_sphere(F.sh32_o[0], F.sh32_c[0], ray.direction, ec, F.Rin);
        out = ray_sphere(F.sh32_o[1], F.sh32_c[1], ray.direction, ec, F.Rout);
    }
    float accum = 0.0f;
    if (TR) cnt.sig = 2166136261u;
    f3 res = ray_march_group<G, S, TR>(p, F, tx, a.time, jitter, ray.direction, in.point, in.t, out.t, accum, cnt,
                                       gmask, lane);
    if (lane != 0) return;
    float godAccum = accum;
    accum = accum * gsmoothstep(0.0f, 1.0f, gmin(1.0f, remap(ray.direction.y, fade, 0.2f, 0.0f, 1.0f)));
    f3 fc = mix3(bg, res, accum);
    a.cur[o] = make_float4(fc.x, fc.y, fc.z, 1.0f);
    if (a.mask) a.mask[o] = godray_value(25.0f * gmin(0.05f, 1.0f - godAccum), ray.direction.y);
    // one ray per thread in march_kernel: lane 0's counters are this ray's
    if (TR) a.trace[o] = make_uint4(cnt.primary, cnt.light / 6u, cnt.primary ? cnt.sig : 0u, 0u);
}

// Ray -> marched pixel.  Checkerboard: the reference's group grid covers
// groups_x x groups_y blocks of 4x4 (Renderer.cpp:713-716); each ray is one
// block's slot pixel.  Full: one ray per pixel.  G consecutive lanes (an
// aligned segment of a warp) march one ray.  BS threads per CTA (256 by
// default, 128 or 32 selectable).  Resident threads per SM: 1024 (64
// registers a thread) when G lanes share a ray; 1280 (48 registers, a few
// spills) for one lane per ray, whose full-frame launches run 2-3 % faster
// for the extra warps while the 4-lane checkerboard launches gain nothing.
// Every step reads its jitter vector at an index taken from int(t), which
// differs from lane to lane: from the parameter space a warp's reads at up to
// 16 different words are served one word at a time, from shared memory in one
// pass (48 words, 3 apart: distinct banks), so the table is copied there.
constexpr int march_min_blocks(int G, int BS) {
    return ((G == 1 ? 1280 : 1024) / BS) < 32 ? ((G == 1 ? 1280 : 1024) / BS) : 32;  // at most 32 CTAs an SM
}
template <int G, int S, int BS, bool TR = false>
__global__ void __launch_bounds__(BS, march_min_blocks(G, BS)) march_kernel(const __grid_constant__ MarchArgs a) {
    static_assert(G >= 1 && G <= 32 && (32 % G) == 0, "G must divide the warp");
    const Frame& F = a.frame;
    const Tex<S> tx = make_tex<S>(a);
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned idx = (unsigned)(tid / G);  // rays < 2^31 (images are at most 16384^2)
    const int lane = (int)(threadIdx.x % G);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    __shared__ float s_jitter[16][3];
    for (int i = threadIdx.x; i < 48; i += BS) (&s_jitter[0][0])[i] = (&a.jitter[0][0])[i];
    __syncthreads();
    Counts cnt{0u, 0u, 0u};
    unsigned pixels = 0;
    int px = 0, py = 0;
    bool active;
    if (a.flags & MT_RENDER_FULL) {
        active = (long long)idx < (long long)a.width * a.height;
        if (active) {
            px = (int)(idx % (unsigned)a.width);
            py = march_row((int)(idx / (unsigned)a.width), a.height, a.bottom_up);
        }
    } else {
        active = (long long)idx < (long long)a.groups_x * a.groups_y;
        if (active) {
            const int id = a.time.frame_count_mod16;
            px = (int)(idx % (unsigned)a.groups_x) * 4 + a.params.slot_x[id];
            py = march_row((int)(idx / (unsigned)a.groups_x), a.groups_y, a.bottom_up) * 4 + a.params.slot_y[id];
            active = px < a.width && py < a.height;
        }
    }
    if (active) {
        march_pixel<G, S, TR>(a, F, tx, px, py, cnt, gmask, lane, s_jitter);
        pixels = lane == 0 ? 1u : 0u;
    }
    if (a.stats) flush_counts(a.stats, cnt, pixels);
}


// Batched form (config 3): one persistent launch over many views of uneven
// size.  Each CTA repeatedly takes the next tile from the batch's counter and
// marches its rays, 128/G rays per pass; per-view arguments come from the
// view table in global memory.  Per-pixel results equal those of separate
// march_kernel launches (the same march_pixel runs on the same inputs).
template <int G, int S>
__global__ void __launch_bounds__(128, 8) march_batch_kernel(const __grid_constant__ BatchArgs b) {
    __shared__ int s_tile;
    const int lane = (int)(threadIdx.x % G);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    constexpr int kRaysPerPass = 128 / G;
    Counts cnt{0u, 0u, 0u};
    unsigned pixels = 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(b.counter, 1u);
        __syncthreads();
        const int t = s_tile;
        __syncthreads();
        if (t >= b.n_tiles) break;
        const BatchTile tile = b.tiles[t];
        const MarchArgs& a = b.views[tile.view];
        const Frame& F = a.frame;
        const Tex<S> tx = make_tex<S>(a);
        const bool full = (a.flags & MT_RENDER_FULL) != 0;
        const int id = a.time.frame_count_mod16;
        const int sx = full ? 0 : a.params.slot_x[id], sy = full ? 0 : a.params.slot_y[id];
        const int step = full ? 1 : 4;
        const int tile_rays = b.tile_w * b.tile_h;
        for (int r0 = 0; r0 < tile_rays; r0 += kRaysPerPass) {
            const int r = r0 + (int)(threadIdx.x / G);
            const int rx = tile.rx0 + r % b.tile_w, ry = tile.ry0 + r / b.tile_w;
            const int px = rx * step + sx, py = ry * step + sy;
            const bool active = r < tile_rays && rx < tile.nrx && ry < tile.nry && px < a.width && py < a.height;
            if (active) {
                march_pixel<G, S>(a, F, tx, px, py, cnt, gmask, lane, a.jitter);
                pixels += lane == 0 ? 1u : 0u;
            }
        }
    }
    if (b.stats) flush_counts(b.stats, cnt, pixels);
}

template <int S> cudaError_t launch_batch_storage(const BatchArgs& b, int lanes, int blocks, cudaStream_t s) {
    switch (lanes) {
        case 1: march_batch_kernel<1, S><<<blocks, 128, 0, s>>>(b); break;
        case 4: march_batch_kernel<4, S><<<blocks, 128, 0, s>>>(b); break;
        case 16: march_batch_kernel<16, S><<<blocks, 128, 0, s>>>(b); break;
        default: march_batch_kernel<8, S><<<blocks, 128, 0, s>>>(b); break;
    }
    return cudaGetLastError();
}

template <int S> int batch_blocks_storage(int device, int lanes) {
    int per_sm = 0, sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    switch (lanes) {
        case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_batch_kernel<1, S>, 128, 0); break;
        case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_batch_kernel<4, S>, 128, 0); break;
        case 16: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_batch_kernel<16, S>, 128, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_batch_kernel<8, S>, 128, 0); break;
    }
    return (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
}

template <int S, int BS> void launch_march_bs(const MarchArgs& a, cudaStream_t s, long long rays) {
    const int G = a.lanes;
    const unsigned blocks = (unsigned)((rays * G + BS - 1) / BS);
    switch (G) {
        case 1: march_kernel<1, S, BS><<<blocks, BS, 0, s>>>(a); break;
        case 4: march_kernel<4, S, BS><<<blocks, BS, 0, s>>>(a); break;
        case 16: march_kernel<16, S, BS><<<blocks, BS, 0, s>>>(a); break;
        default: march_kernel<8, S, BS><<<blocks, BS, 0, s>>>(a); break;
    }
}

template <int S> cudaError_t launch_march_storage(const MarchArgs& a, cudaStream_t s, long long rays) {
    if (a.trace) {  // traced march (mt_set_sample_trace): 256-thread CTAs, 1 or 4 lanes
        const int G = a.lanes == 1 ? 1 : 4;
        const unsigned blocks = (unsigned)((rays * G + 255) / 256);
        if (G == 1)
            march_kernel<1, S, 256, true><<<blocks, 256, 0, s>>>(a);
        else
            march_kernel<4, S, 256, true><<<blocks, 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (a.block == 256)
        launch_march_bs<S, 256>(a, s, rays);
    else if (a.block == 128)
        launch_march_bs<S, 128>(a, s, rays);
    else
        launch_march_bs<S, 32>(a, s, rays);
    return cudaGetLastError();
}

}  // namespace mt
