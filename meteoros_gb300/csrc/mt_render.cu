// Raymarch, reprojection and TXAA kernels of the compute stage (FP32 form).
//
//   march_kernel        <- shaders/cloudRayMarch.comp:690-826 (one thread per
//                          marched pixel)
//   reproject_kernel    <- shaders/reprojection.comp:193-244 (one thread per
//                          pixel not marched this frame)
//   txaa_kernel         <- shaders/postProcess_TXAA.frag:223-269 (one thread
//                          per pixel)
//
// The reference runs reprojection over every pixel and then the raymarch over
// one pixel per 4x4 block with no barrier between the two dispatches
// (Renderer.cpp:688-716); the marched pixel is meant to win.  Here the two
// kernels write disjoint pixel sets, so the outcome is defined and the two
// launches can overlap.
//
// Compiled with -fmad=false: see mt_device.cuh.
#include <cuda_runtime.h>

#include "mt_device.cuh"
#include "mt_kernels.h"

namespace mt {

struct Frame {
    float R, Rin, Rout, thickness, inner_alt;
    Rcp r_thick, r_period, r_weather;  // per-frame denominators (see rdiv)
};

MT_HD Frame make_frame(const mt_params& p) {
    Frame F;
    F.R = p.earth_radius;
    F.Rin = p.shell_inner_radius;
    F.Rout = p.shell_outer_radius;
    F.thickness = F.Rout - F.Rin;
    F.inner_alt = F.Rin - F.R;
    F.r_thick = make_rcp(F.thickness);
    F.r_period = make_rcp(p.noise_period);
    F.r_weather = make_rcp(p.weather_scale);
    return F;
}

// remap() whose range width omax - omin is known ahead: the quotient through
// the correctly rounded reciprocal of that width (rdiv).
MT_HD float remap_r(float v, float omin, Rcp width, float nmin, float nmax) {
    return nmin + ((rdiv(v - omin, width)) * (nmax - nmin));
}
// The reciprocal of a compile-time width, rounded once by the compiler.
#define MT_RCP(omin, omax) (Rcp{(omax) - (omin), 1.0f / ((omax) - (omin))})

struct Ray {
    f3 origin, direction;
};
struct Isect {
    f3 point;
    bool valid;
    float t;
};

// cloudRayMarch.comp:114-132; reprojection.comp:72-90 reads halton 1/2 again
// for index >= 4 (`repro`).
MT_HD void jitter_offset(const mt_time_ubo& tm, int index, float dimx, float dimy, bool repro, float& jx,
                         float& jy) {
    index = index / 2;
    float x, y;
    if (index < 4) {
        x = tm.halton_seq1[index];
        y = tm.halton_seq2[index];
    } else {
        index -= 4;
        if (repro) {
            x = tm.halton_seq1[index];
            y = tm.halton_seq2[index];
        } else {
            x = tm.halton_seq3[index];
            y = tm.halton_seq4[index];
        }
    }
    jx = x / dimx;
    jy = y / dimy;
}

// cloudRayMarch.comp:194-226
MT_HD Ray cast_ray(float sx, float sy, f3 eye, const mt_camera_ubo& cam, const mt_time_ubo& tm, int pixelID, int W,
                   int H, bool repro) {
    const float* v = cam.view;
    f3 camRight = normalize3(f3{v[0], v[4], v[8]});
    f3 camUp = normalize3(f3{v[1], v[5], v[9]});
    f3 camLook = -normalize3(f3{v[2], v[6], v[10]});
    float nx = sx * 2.0f - 1.0f, ny = sy * 2.0f - 1.0f;
    float jx, jy;
    jitter_offset(tm, pixelID, (float)W, (float)H, repro, jx, jy);
    nx = nx + jx;
    ny = ny + jy;
    f3 cam_x = (nx * cam.tan_fov_by_2[0]) * camRight;
    f3 cam_y = (ny * cam.tan_fov_by_2[1]) * camUp;
    f3 ref = eye + camLook;
    f3 pp = ref + cam_x + cam_y;
    return Ray{eye, normalize3(pp - eye)};
}

// cloudRayMarch.comp:229-273 (t = length(p - rO) with the normalised rO, as
// the reference defines it).
MT_HD Isect ray_sphere(f3 rO, f3 rD, f3 c, float radius) {
    Isect is;
    is.valid = false;
    is.point = f3{0.0f, 0.0f, 0.0f};
    is.t = 0.0f;
    rO = rO - c;
    rO = rO / radius;
    float A = dot3(rD, rD);
    float B = 2.0f * dot3(rD, rO);
    float C = dot3(rO, rO) - 1.0f;
    float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return is;
    float t = (-B - sqrtf(disc)) / (2.0f * A);
    if (t < 0.0f) t = (-B + sqrtf(disc)) / (2.0f * A);
    if (t >= 0.0f) {
        f3 pnt = rO + t * rD;
        is.valid = true;
        pnt = pnt * radius;
        pnt = pnt + c;
        is.point = pnt;
        is.t = length3(pnt - rO);
    }
    return is;
}

// The same intersection in FP64 (precision form): the normalised-sphere
// quadratic cancels badly in FP32 (C = |rO|^2 - 1 with |rO| ~ 1).
MT_HD Isect ray_sphere_fp64(f3 rOf, f3 rDf, f3 cf, float radiusf) {
    double ox = (double)rOf.x - (double)cf.x, oy = (double)rOf.y - (double)cf.y, oz = (double)rOf.z - (double)cf.z;
    const double r = (double)radiusf;
    ox = ox / r;
    oy = oy / r;
    oz = oz / r;
    const double dx = rDf.x, dy = rDf.y, dz = rDf.z;
    double A = dx * dx + dy * dy + dz * dz;
    double B = 2.0 * (dx * ox + dy * oy + dz * oz);
    double C = (ox * ox + oy * oy + oz * oz) - 1.0;
    double disc = B * B - 4.0 * A * C;
    Isect is;
    is.valid = false;
    is.point = f3{0.0f, 0.0f, 0.0f};
    is.t = 0.0f;
    if (disc < 0.0) return is;
    double t = (-B - sqrt(disc)) / (2.0 * A);
    if (t < 0.0) t = (-B + sqrt(disc)) / (2.0 * A);
    if (t >= 0.0) {
        double px = (ox + t * dx) * r + (double)cf.x;
        double py = (oy + t * dy) * r + (double)cf.y;
        double pz = (oz + t * dz) * r + (double)cf.z;
        is.valid = true;
        is.point = f3{(float)px, (float)py, (float)pz};
        double qx = px - ox, qy = py - oy, qz = pz - oz;
        is.t = (float)sqrt(qx * qx + qy * qy + qz * qz);
    }
    return is;
}

// cloudRayMarch.comp:153-169
MT_HD float remap(float v, float omin, float omax, float nmin, float nmax) {
    return nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
}
MT_HD float remap_clamped(float v, float omin, float omax, float nmin, float nmax) {
    float t = nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
    return gclamp(t, nmin, nmax);
}
MT_HD float remap_clamped_ba(float v, float omin, float omax, float nmin, float nmax) {
    v = gclamp(v, omin, omax);
    float t = nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
    return gclamp(t, nmin, nmax);
}

// cloudRayMarch.comp:171-186
MT_HD float relative_height(const Frame& F, f3 point, f3 ec, f3 startPos, f3 rayDir, f3 eye) {
    float lenCam = length3(point - eye);
    float lenInner = length3(startPos - eye);
    f3 p2e = normalize3_r(point - ec);
    float cosTheta = dot3(rayDir, p2e);
    float num = fabsf(cosTheta * (lenCam - lenInner));
    return rdiv(num, F.r_thick);
}

// cloudRayMarch.comp:188-191
MT_HD f3 relative_position(const Frame& F, f3 pos, f3 ec) {
    const f3 d = pos - f3{ec.x, F.inner_alt, ec.z};
    return f3{rdiv(d.x, F.r_thick), rdiv(d.y, F.r_thick), rdiv(d.z, F.r_thick)};
}

// cloudRayMarch.comp:475-487
MT_HD float height_gradient(float h, float type) {
    h = gclamp(h, 0.0f, 1.0f);
    float stratocumulus = gmax(0.0f, remap_r(h, 0.0f, MT_RCP(0.0f, 0.25f), 0.0f, 1.0f) *
                                         remap_r(h, 0.3f, MT_RCP(0.3f, 0.65f), 1.0f, 0.0f));
    float stratus = gmax(0.0f, remap_r(h, 0.0f, MT_RCP(0.0f, 0.1f), 0.0f, 1.0f) *
                                   remap_r(h, 0.2f, MT_RCP(0.2f, 0.3f), 1.0f, 0.0f));
    float a = gmix(stratus, stratocumulus, gclamp(type * 2.0f, 0.0f, 1.0f));
    float b = gmix(stratocumulus, stratus, gclamp((type - 0.5f) * 2.0f, 0.0f, 1.0f));
    return gmix(a, b, type);
}

struct Weather {
    float lo, mul, type;
    float hgrad;  // height gradient at the primary sample, shared by its light samples
    Rcp r_lo;     // 1 - lo, the coverage remap's width, shared by the step's samples
};

struct Tex {
    const uint32_t* base;
    const uint32_t* detail;
    const uint32_t* curl;
    const uint32_t* weather;
};

MT_HD Weather weather_at(const mt_params& p, const Frame& F, const Tex& tx, f3 pos, f3 ec) {
    Weather w;
    w.hgrad = 1.0f;
    if (p.coverage_mode == 0) {
        w.lo = p.coverage;
        w.mul = p.coverage;
        w.type = 0.0f;
    } else {
        f4v wd = tex2_u8<MT_WEATHER_N>(tx.weather, rdiv(pos.x - ec.x, F.r_weather), rdiv(pos.z - ec.z, F.r_weather));
        w.lo = 1.0f - wd.x;
        w.mul = wd.x;
        w.type = wd.z;
    }
    w.r_lo = make_rcp(1.0f - w.lo);
    return w;
}

// cloudRayMarch.comp:499-540
MT_HD float sample_low_frequency(const mt_params& p, const Tex& tx, f3 point, float relH, const Weather& wt) {
    f4v n = tex3_u8<MT_BASE_N>(tx.base, point);
    float fbm = (n.y * 0.625f) + (n.z * 0.25f) + (n.w * 0.125f);
    fbm = gclamp(fbm, 0.0f, 1.0f);
    float baseCloud = remap_clamped(n.x, (fbm - 0.9f), 1.0f, 0.0f, 1.0f);
    // getDensityHeightGradientForPoint(relH, type): every call of a step passes
    // the primary sample's height and weather, so it is evaluated once per step
    // (Weather::hgrad).
    if (p.height_gradient) baseCloud = baseCloud * wt.hgrad;
    // remapClampedBeforeAndAfter(baseCloud, lo, 1, 0, 1) with its width 1 - lo
    // shared by the step's samples
    float v = gclamp(baseCloud, wt.lo, 1.0f);
    float bc = gclamp(0.0f + ((rdiv(v - wt.lo, wt.r_lo)) * (1.0f - 0.0f)), 0.0f, 1.0f);
    return bc * wt.mul;
}

// cloudRayMarch.comp:542-563.  The texture part is the same for the primary
// erosion (:645) and the six cone-light erosions (:665): all are evaluated at
// the primary sample point with the primary height, so it is computed once.
MT_HD float erosion_modifier(const Tex& tx, f3 point, float h) {
    f4v curl = tex2_u8<MT_CURL_N>(tx.curl, point.x, point.y);
    point.x = point.x + (curl.x * (1.0f - h)) * 0.5f;
    point.y = point.y + (curl.y * (1.0f - h)) * 0.5f;
    f4v hf = tex3_u8<MT_DETAIL_N>(tx.detail, point);
    float hfbm = (hf.x * 0.625f) + (hf.y * 0.25f) + (hf.z * 0.125f);
    return gclamp(gmix(hfbm, 1.0f - hfbm, gclamp(h * 2.0f, 0.0f, 1.0f)), 0.0f, 1.0f);
}
struct Erosion {
    float lo;  // high_freq_modifier * 0.005
    Rcp r;     // 1 - lo, shared by the step's seven erosions
};
MT_HD Erosion make_erosion(float modifier) {
    Erosion e;
    e.lo = modifier * 0.005f;
    e.r = make_rcp(1.0f - e.lo);
    return e;
}
MT_HD float erode(float baseCloud, const Erosion& e) { return remap_r(baseCloud, e.lo, e.r, 0.0f, 1.0f); }

// cloudRayMarch.comp:295-306
MT_HD float henyey_greenstein(float c, float e) {
    float num = 1.0f - e * e;
    float den = powf((1.0f + e * e - 2.0f * e * c), 1.5f);
    return (num / den) * 0.07957747154594767f;
}

// cloudRayMarch.comp:331-388.  cos_q = (cos_angle - 0.7) / (1.0 - 0.7), the
// ray-constant quotient of the attenuation remap (:341-343).
MT_HD float light_energy(float h, float dl, float ds, float phase, float cos_q, float brightness) {
    const float primary = expf(-dl);
    const float secondary = primary;  // exp(-dl) twice in the reference (:334, :340)
    float att = gmax(secondary + (cos_q * (secondary * 0.25f - secondary)), primary);
    float depth = 0.05f + pow_nl(ds, gclamp(remap_r(h * 0.125f, 0.3f, MT_RCP(0.3f, 0.85f), 0.5f, 2.0f), 0.5f, 2.0f));
    float vert = pow_nl(gclamp(remap_r(h * 1.5f, 0.07f, MT_RCP(0.07f, 0.34f), 0.1f, 1.0f), 0.1f, 1.0f), 0.8f);
    float in_scatter = depth * vert;
    return att * primary * in_scatter * phase * brightness;
}

// cloudRayMarch.comp:401-467 (Preetham).  Once per ray: kept out of line so
// the march loop stays small in the instruction cache.
__device__ __noinline__ f3 atmosphere_color(const mt_params& p, f3 dir, f3 sunDir, float sunIntensity) {
    const f3 skySun = ld3(p.sky_sun_pos);
    const float PI = 3.14159265f;
    sunDir = normalize3(sunDir);
    float zenithAngleCos = gclamp(normalize3(skySun).y, -1.0f, 1.0f);
    float sunI = 1000.0f * gmax(0.0f, 1.0f - powf(2.718281828459f, -((1.6110731557f - acosf(zenithAngleCos)) / 1.5f)));
    float sunE = sunIntensity * sunI;
    float sunFade = 1.0f - gclamp(1.0f - expf(skySun.y / 450000.0f), 0.0f, 1.0f);
    const f3 RT{5.804542996261093E-6f, 1.3562911419845635E-5f, 3.0265902468824876E-5f};
    f3 BetaR = RT * (2.0f - 1.0f + sunFade);
    float c = (0.2f * 10.0f) * 10E-18f;
    const f3 MIE{1.839991851443397f, 2.779802391966052f, 4.079047954386109f};
    f3 BetaM = ((0.434f * c) * MIE) * 0.005f;
    float zenith = acosf(gmax(0.0f, dir.y));
    float inverse = 1.0f / (cosf(zenith) + 0.15f * powf(93.885f - ((zenith * 180.0f) / PI), -1.253f));
    float sR = 8.4E3f * inverse;
    float sM = 1.25E3f * inverse;
    f3 ex = (-BetaR) * sR + BetaM * sM;
    f3 fex{expf(ex.x), expf(ex.y), expf(ex.z)};
    float cosTheta = dot3(sunDir, dir);
    float rp = cosTheta * 0.5f + 0.5f;
    float rPhase = 0.05968310365946075f * (1.0f + rp * rp);
    f3 betaRTheta = BetaR * rPhase;
    float mPhase = henyey_greenstein(cosTheta, 0.8f);
    f3 betaMTheta = BetaM * mPhase;
    float yDot = 1.0f - sunDir.y;
    yDot = yDot * (yDot * yDot * yDot * yDot);
    f3 betas = (betaRTheta + betaMTheta) / (BetaR + BetaM);
    f3 a = (sunE * betas) * (f3{1.0f, 1.0f, 1.0f} - fex);
    f3 Lin{powf(a.x, 1.5f), powf(a.y, 1.5f), powf(a.z, 1.5f)};
    f3 b = (sunE * betas) * fex;
    f3 pb{powf(b.x, 0.5f), powf(b.y, 0.5f), powf(b.z, 0.5f)};
    Lin = Lin * mix3(f3{1.0f, 1.0f, 1.0f}, pb, gclamp(yDot, 0.0f, 1.0f));
    f3 L0 = 0.1f * fex;
    const float SAC = 0.999956676946448443553574619906976478926848692873900859324f;
    float sunDisk = gsmoothstep(SAC, SAC + 0.00002f, cosTheta);
    L0 = L0 + ((sunE * 15000.0f) * fex) * sunDisk;
    return (Lin + L0) * 0.04f + f3{0.0f, 0.0003f, 0.00075f};
}

struct Counts {
    unsigned primary, light, rays;
};

// Per-ray constants of cloudRayMarch.comp:565-624, shared by every step.
struct RayConsts {
    Ray ray;
    f3 ec, startPos;
    f3 kernel[6];
    f3 wind, skew;
    float stepSize, cos_angle, cos_q, HG_light, total_time;
    int pixelID;
};

__device__ __noinline__ void ray_consts(const mt_params& p, const mt_time_ubo& tm, const Ray& ray, f3 ec,
                                        f3 startPos, float stepSize, int pixelID, RayConsts& rc) {
    rc.ray = ray;
    rc.ec = ec;
    rc.startPos = startPos;
    rc.stepSize = stepSize;
    rc.pixelID = pixelID;
    const f3 lightDir = normalize3(ld3(p.sun_light_pos) - ray.origin);
    rc.cos_angle = dot3(normalize3(ray.direction), lightDir);
    rc.cos_q = (rc.cos_angle - 0.7f) / (1.0f - 0.7f);
    rc.HG_light = gmax(henyey_greenstein(rc.cos_angle, 0.6f), 0.7f * henyey_greenstein(rc.cos_angle, 0.99f - 0.1f));
    float ax = fabsf(lightDir.x), ay = fabsf(lightDir.y), az = fabsf(lightDir.z);
    f3 maxComp;
    if (ax > ay && ax > az)
        maxComp = f3{ax, 0.0f, 0.0f};
    else if (ay > ax && ay > az)
        maxComp = f3{0.0f, ay, 0.0f};
    else
        maxComp = f3{0.0f, 0.0f, az};
    f3 zC = cross3(lightDir, maxComp);
    f3 xC = cross3(zC, lightDir);
    rc.kernel[0] = mat3mul(xC, lightDir, zC, f3{0.1f, 0.25f, -0.15f});
    rc.kernel[1] = mat3mul(xC, lightDir, zC, f3{0.2f, 0.5f, 0.2f});
    rc.kernel[2] = mat3mul(xC, lightDir, zC, f3{-0.2f, 0.1f, -0.1f});
    rc.kernel[3] = mat3mul(xC, lightDir, zC, f3{-0.05f, 0.75f, 0.05f});
    rc.kernel[4] = mat3mul(xC, lightDir, zC, f3{-0.1f, 1.0f, 0.0f});
    rc.kernel[5] = mat3mul(xC, lightDir, zC, f3{0.0f, 3.0f, 0.0f});
    rc.wind = ld3(p.wind_dir) * p.wind_speed;
    rc.skew = ld3(p.skew_dir);
    rc.total_time = tm.time[1];
}

struct StepOut {
    int in_cloud;  // baseDensity > 0 (cloudRayMarch.comp:642)
    float hfd;     // eroded density (:645)
    float E;       // light energy (:673)
};

// One iteration of the march loop body (cloudRayMarch.comp:629-678) at
// parameter t, up to the accumulation: everything that does not depend on the
// running accumDensity / transmittance.
MT_HD StepOut eval_step(const mt_params& p, const Frame& F, const Tex& tx, const mt_time_ubo& tm,
                        const RayConsts& rc, float t) {
    StepOut o{0, 0.0f, 0.0f};
    int _index = f2i(gmod((float)(rc.pixelID + f2i(t)), 16.0f));
    float jx, jy;
    jitter_offset(tm, _index, 1.0f, 1.0f, false, jx, jy);  // halton values; / 75 below
    jx = rdiv(jx, MT_RCP(0.0f, 75.0f));
    jy = rdiv(jy, MT_RCP(0.0f, 75.0f));
    f3 jd = rc.ray.direction + f3{jx, (jx + jy) * 1.180f, jy};
    f3 pos = rc.ray.origin + t * jd;
    f3 sp = relative_position(F, pos, rc.ec);
    sp = f3{rdiv(sp.x, F.r_period), rdiv(sp.y, F.r_period), rdiv(sp.z, F.r_period)};
    float relH = relative_height(F, pos, rc.ec, rc.startPos, rc.ray.direction, rc.ray.origin);
    sp = sp + ((relH * rc.skew) * p.cloud_top_offset) * 0.009f;
    sp = sp + rc.wind * rc.total_time;
    Weather wt = weather_at(p, F, tx, pos, rc.ec);
    if (p.height_gradient) wt.hgrad = height_gradient(relH, wt.type);
    float baseDensity = sample_low_frequency(p, tx, sp, relH, wt) * 0.380f;
    if (baseDensity > 0.0f) {
        const Erosion ero = make_erosion(erosion_modifier(tx, sp, relH));
        o.in_cloud = 1;
        o.hfd = erode(baseDensity * 1.4f, ero);
        float dl = 0.0f;
        // Kept rolled: six inlined copies of the sampler overflow the
        // instruction cache (the dominant stall when unrolled).
#pragma unroll 1
        for (int i = 0; i < 6; ++i) {
            f3 lightPos = pos + ((rc.stepSize * rc.kernel[i]) * (float)i);
            f3 slp = relative_position(F, lightPos, rc.ec);
            float cbl = sample_low_frequency(p, tx, slp, relH, wt);
            if (cbl > 0.0f) dl = dl + erode(1.5f * cbl, ero);
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
template <int G>
MT_HD f3 ray_march_group(const mt_params& p, const Frame& F, const Tex& tx, const mt_time_ubo& tm, const Ray& ray,
                         f3 ec, f3 startPos, float start_t, float end_t, int pixelID, float& accum, Counts& cnt,
                         unsigned gmask, int lane) {
    float _dot = dot3(ray.direction, f3{0.0f, 1.0f, 0.0f});
    float maxSteps;
    if (p.steps_min == p.steps_max)
        maxSteps = (float)p.steps_min;
    else
        maxSteps = floorf(gmix((float)p.steps_min, (float)p.steps_max, 1.0f - _dot));
    const float thick = end_t - start_t;
    const float stepSize = thick / maxSteps;
    RayConsts rc;
    ray_consts(p, tm, ray, ec, startPos, stepSize, pixelID, rc);
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
        if (valid) o = eval_step(p, F, tx, tm, rc, t);
#pragma unroll
        for (int k = 0; k < G; ++k) {
            if (!__shfl_sync(gmask, valid, k, G)) {
                done = true;
                break;
            }
            const int in_cloud = __shfl_sync(gmask, o.in_cloud, k, G);
            const float hfd = __shfl_sync(gmask, o.hfd, k, G);
            const float E = __shfl_sync(gmask, o.E, k, G);
            if (lane == 0) cnt.primary++;
            if (in_cloud) {
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

// cloudRayMarch.comp:106-112 + postProcess_GodRays.frag:36-43
MT_HD float godray_value(float v, float dir_y) {
    f4v enc{1.0f * v, 255.0f * v, 65025.0f * v, 16581375.0f * v};
    enc = f4v{gfract(enc.x), gfract(enc.y), gfract(enc.z), gfract(enc.w)};
    const float k = 1.0f / 255.0f;
    enc = f4v{enc.x - enc.y * k, enc.y - enc.z * k, enc.z - enc.w * k, enc.w - enc.w * 0.0f};
    if (dir_y < 0.05f) enc = enc * gmax(5.0f, dir_y);
    return enc.x * (1.0f / 1.0f) + enc.y * (1.0f / 255.0f) + enc.z * (1.0f / 65025.0f) + enc.w * (1.0f / 16581375.0f);
}

// cloudRayMarch.comp:690-826 for one pixel, marched by a group of G lanes;
// lane 0 stores.
template <int G>
MT_HD void march_pixel(const MarchArgs& a, const Frame& F, const Tex& tx, int px, int py, Counts& cnt,
                       unsigned gmask, int lane) {
    const mt_params& p = a.params;
    const int W = a.width, H = a.height;
    const int pixelID = a.time.frame_count_mod16;
    float ux = (float)px / (float)W, uy = (float)py / (float)H;
    uy = 1.0f - uy;
    f3 eyePos = p.eye_sign * ld3(a.camera.eye);
    Ray ray = cast_ray(ux, uy, eyePos, a.camera, a.time, pixelID, W, H, false);
    const float sunIntensity = 0.780f;
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
        }
        return;
    }
    bg = atmosphere_color(p, ray.direction, ld3(p.sky_sun_pos) - ray.origin, sunIntensity);
    bg = bg * bgMul;
    if (_dot < fade) {
        if (lane == 0) {
            a.cur[o] = make_float4(bg.x, bg.y, bg.z, 1.0f);
            if (a.mask) a.mask[o] = 0.0f;
        }
        return;
    }
    f3 ec = eyePos;
    ec.y = -F.R;
    Isect in, out;
    if (p.fp64_shells) {
        in = ray_sphere_fp64(ray.origin, ray.direction, ec, F.Rin);
        out = ray_sphere_fp64(ray.origin, ray.direction, ec, F.Rout);
    } else {
        in = ray_sphere(ray.origin, ray.direction, ec, F.Rin);
        out = ray_sphere(ray.origin, ray.direction, ec, F.Rout);
    }
    float accum = 0.0f;
    f3 res = ray_march_group<G>(p, F, tx, a.time, ray, ec, in.point, in.t, out.t, pixelID, accum, cnt, gmask, lane);
    if (lane != 0) return;
    float godAccum = accum;
    accum = accum * gsmoothstep(0.0f, 1.0f, gmin(1.0f, remap(ray.direction.y, fade, 0.2f, 0.0f, 1.0f)));
    f3 fc = mix3(bg, res, accum);
    a.cur[o] = make_float4(fc.x, fc.y, fc.z, 1.0f);
    if (a.mask) a.mask[o] = godray_value(25.0f * gmin(0.05f, 1.0f - godAccum), ray.direction.y);
}

__device__ __forceinline__ void flush_counts(unsigned long long* stats, const Counts& c, unsigned pixels) {
    unsigned prim = __reduce_add_sync(0xffffffffu, c.primary);
    unsigned light = __reduce_add_sync(0xffffffffu, c.light);
    unsigned rays = __reduce_add_sync(0xffffffffu, c.rays);
    unsigned pix = __reduce_add_sync(0xffffffffu, pixels);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(stats + 0, (unsigned long long)prim);
        atomicAdd(stats + 1, (unsigned long long)light);
        atomicAdd(stats + 2, (unsigned long long)rays);
        atomicAdd(stats + 3, (unsigned long long)pix);
    }
}

// Ray -> marched pixel.  Checkerboard: the reference's group grid covers
// groups_x x groups_y blocks of 4x4 (Renderer.cpp:713-716); each ray is one
// block's slot pixel.  Full: one ray per pixel.  G consecutive lanes (an
// aligned segment of a warp) march one ray.
template <int G>
__global__ void __launch_bounds__(128, 8) march_kernel(const __grid_constant__ MarchArgs a) {
    static_assert(G >= 1 && G <= 32 && (32 % G) == 0, "G must divide the warp");
    const Frame F = make_frame(a.params);
    const Tex tx{a.base, a.detail, a.curl, a.weather};
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long idx = tid / G;
    const int lane = (int)(threadIdx.x % G);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    Counts cnt{0u, 0u, 0u};
    unsigned pixels = 0;
    int px = 0, py = 0;
    bool active;
    if (a.flags & MT_RENDER_FULL) {
        active = idx < (long long)a.width * a.height;
        if (active) {
            px = (int)(idx % a.width);
            py = (int)(idx / a.width);
        }
    } else {
        active = idx < (long long)a.groups_x * a.groups_y;
        if (active) {
            const int id = a.time.frame_count_mod16;
            px = (int)(idx % a.groups_x) * 4 + a.params.slot_x[id];
            py = (int)(idx / a.groups_x) * 4 + a.params.slot_y[id];
            active = px < a.width && py < a.height;
        }
    }
    if (active) {
        march_pixel<G>(a, F, tx, px, py, cnt, gmask, lane);
        pixels = lane == 0 ? 1u : 0u;
    }
    if (a.stats) flush_counts(a.stats, cnt, pixels);
}

// Pixels the checkerboard raymarch writes this frame (cloudRayMarch.comp:695-701
// under the dispatch of Renderer.cpp:713-716).
MT_HD bool is_marched(const MarchArgs& a, int x, int y) {
    const int id = a.time.frame_count_mod16;
    const int dx = x - a.params.slot_x[id], dy = y - a.params.slot_y[id];
    return dx >= 0 && dy >= 0 && (dx & 3) == 0 && (dy & 3) == 0 && (dx >> 2) < a.groups_x && (dy >> 2) < a.groups_y;
}

// The previous camera's uv of the inner-shell hit of a ray
// (reprojection.comp:205-222, postProcess_TXAA.frag:230-247).
MT_HD void old_uv(const mt_params& p, const Frame& F, const mt_camera_ubo& cam, const mt_camera_ubo& cam_old,
                  const mt_time_ubo& tm, float sx, float sy, int W, int H, bool repro, float& old_u, float& old_v) {
    f3 eyePos = p.eye_sign * ld3(cam.eye);
    Ray ray = cast_ray(sx, sy, eyePos, cam, tm, tm.frame_count_mod16, W, H, repro);
    f3 ec = eyePos;
    ec.y = -F.R;
    Isect in = ray_sphere(ray.origin, ray.direction, ec, F.Rin);
    const float* ov = cam_old.view;
    f3 q = in.point;
    f3 od{ov[0] * q.x + ov[4] * q.y + ov[8] * q.z + ov[12] * 1.0f, ov[1] * q.x + ov[5] * q.y + ov[9] * q.z + ov[13] * 1.0f,
          ov[2] * q.x + ov[6] * q.y + ov[10] * q.z + ov[14] * 1.0f};
    od = normalize3(od);
    od = od / (-od.z);
    old_u = (od.x / cam.tan_fov_by_2[0]) * 0.5f + 0.5f;
    old_v = (od.y / cam.tan_fov_by_2[1]) * 0.5f + 0.5f;
}

// reprojection.comp:193-244 for pixel (x, y).
MT_HD f4v reproject_pixel(const MarchArgs& a, const Frame& F, int x, int y) {
    const int W = a.width, H = a.height;
    const float ux = (float)x / (float)W, uy = (float)y / (float)H;
    float old_u, old_v;
    old_uv(a.params, F, a.camera, a.camera_old, a.time, ux, uy, W, H, true, old_u, old_v);
    const float mx = old_u - ux, my = old_v - uy;
    f4v blur{0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const float f = (float)i / 10.0f;
        const float iu = roundf((old_u - mx * f) * (float)W);
        const float iv = roundf((old_v - my * f) * (float)H);
        const int ix = imin(imax(f2i(iu), 0), W - 1);
        const int iy = imin(imax(f2i(iv), 0), H - 1);
        const float4 s = __ldg(a.prev + (size_t)iy * (size_t)W + (size_t)ix);
        blur = blur + f4v{s.x, s.y, s.z, s.w};
    }
    return blur / 10.0f;
}

// The centre pixel of fragment (x, y)'s neighbourhood: pixelPos of
// postProcess_TXAA.frag:227 with in_uv at the fragment centre.
MT_HD void txaa_centre(int x, int y, int W, int H, float& iux, float& iuy, int& ppx, int& ppy) {
    iux = ((float)x + 0.5f) / (float)W;
    iuy = ((float)y + 0.5f) / (float)H;
    ppx = imin(imax(f2i(roundf((float)W * iux)), 0), W - 1);
    ppy = imin(imax(f2i(roundf((float)H * iuy)), 0), H - 1);
}

// postProcess_TXAA.frag:223-269 for fragment (x, y); `load(i, j)` reads the
// current frame (0 outside the image, as imageLoad does).
template <class Load>
MT_HD f4v txaa_pixel(const mt_params& p, const Frame& F, const mt_camera_ubo& cam, const mt_camera_ubo& cam_old,
                     const mt_time_ubo& tm, const float4* __restrict__ history, int x, int y, int W, int H,
                     Load load) {
    float iux, iuy;
    int ppx, ppy;
    txaa_centre(x, y, W, H, iux, iuy, ppx, ppy);
    float old_u, old_v;
    old_uv(p, F, cam, cam_old, tm, iux, iuy, W, H, false, old_u, old_v);
    f4v ctl = load(ppx - 1, ppy - 1), ctc = load(ppx, ppy - 1), ctr = load(ppx + 1, ppy - 1);
    f4v cml = load(ppx - 1, ppy), cmc = load(ppx, ppy), cmr = load(ppx + 1, ppy);
    f4v cbl = load(ppx - 1, ppy + 1), cbc = load(ppx, ppy + 1), cbr = load(ppx + 1, ppy + 1);
    f4v cmin = min4(ctl, min4(ctc, min4(ctr, min4(cml, min4(cmc, min4(cmr, min4(cbl, min4(cbc, cbr))))))));
    f4v cmax = max4(ctl, max4(ctc, max4(ctr, max4(cml, max4(cmc, max4(cmr, max4(cbl, max4(cbc, cbr))))))));
    f4v cavg = (ctl + ctc + ctr + cml + cmc + cmr + cbl + cbc + cbr) / 9.0f;
    f4v cmin5 = min4(ctc, min4(cml, min4(cmc, min4(cmr, cbc))));
    f4v cmax5 = max4(ctc, max4(cml, max4(cmc, max4(cmr, cbc))));
    f4v cavg5 = (ctc + cml + cmc + cmr + cbc) / 5.0f;
    cmin = f4v{0.5f * (cmin.x + cmin5.x), 0.5f * (cmin.y + cmin5.y), 0.5f * (cmin.z + cmin5.z), 0.5f * (cmin.w + cmin5.w)};
    cmax = f4v{0.5f * (cmax.x + cmax5.x), 0.5f * (cmax.y + cmax5.y), 0.5f * (cmax.z + cmax5.z), 0.5f * (cmax.w + cmax5.w)};
    cavg = f4v{0.5f * (cavg.x + cavg5.x), 0.5f * (cavg.y + cavg5.y), 0.5f * (cavg.z + cavg5.z), 0.5f * (cavg.w + cavg5.w)};
    f4v curr = cmc;
    f4v prev = tex2_border(history, W, H, old_u, old_v);
    // clip_aabb (:171-191)
    f4v pc = min4(max4(cavg, cmin), cmax);
    f3 p_clip{0.5f * (cmax.x + cmin.x), 0.5f * (cmax.y + cmin.y), 0.5f * (cmax.z + cmin.z)};
    const float EPS = 0.0000000001f;
    f3 e_clip{0.5f * (cmax.x - cmin.x) + EPS, 0.5f * (cmax.y - cmin.y) + EPS, 0.5f * (cmax.z - cmin.z) + EPS};
    f4v v_clip = prev - f4v{p_clip.x, p_clip.y, p_clip.z, pc.w};
    float vux = fabsf(v_clip.x / e_clip.x), vuy = fabsf(v_clip.y / e_clip.y), vuz = fabsf(v_clip.z / e_clip.z);
    float ma = gmax(vux, gmax(vuy, vuz));
    if (ma > 1.0f) prev = f4v{p_clip.x, p_clip.y, p_clip.z, pc.w} + v_clip / ma;
    const f3 lw{0.2125f, 0.7154f, 0.0721f};
    float lum0 = dot3(f3{curr.x, curr.y, curr.z}, lw);
    float lum1 = dot3(f3{prev.x, prev.y, prev.z}, lw);
    float ud = fabsf(lum0 - lum1) / gmax(lum0, gmax(lum1, 0.2f));
    float uw = 1.0f - ud;
    float k = gmix(p.feedback_min, p.feedback_max, uw * uw);
    return mix4(prev, curr, k);
}

// reprojection.comp:193-244 for every pixel the march does not write.
__global__ void __launch_bounds__(256) reproject_kernel(const __grid_constant__ MarchArgs a) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int W = a.width, H = a.height;
    bool active = idx < (long long)W * H;
    int x = 0, y = 0;
    if (active) {
        x = (int)(idx % W);
        y = (int)(idx / W);
        active = !is_marched(a, x, y);
    }
    if (active) {
        const Frame F = make_frame(a.params);
        const f4v b = reproject_pixel(a, F, x, y);
        a.cur[(size_t)y * (size_t)W + (size_t)x] = make_float4(b.x, b.y, b.z, b.w);
    }
    if (a.stats) {
        Counts none{0u, 0u, 0u};
        flush_counts(a.stats, none, active ? 1u : 0u);
    }
}

// postProcess_TXAA.frag:223-269, one thread per output pixel (fragment).
__global__ void __launch_bounds__(256) txaa_kernel(const __grid_constant__ TxaaArgs a) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int W = a.width, H = a.height;
    if (idx >= (long long)W * H) return;
    const int x = (int)(idx % W), y = (int)(idx / W);
    const Frame F = make_frame(a.params);
    auto load = [&](int i, int j) -> f4v {
        if (i < 0 || j < 0 || i >= W || j >= H) return f4v{0.0f, 0.0f, 0.0f, 0.0f};
        float4 s = __ldg(a.current + (size_t)j * (size_t)W + (size_t)i);
        return f4v{s.x, s.y, s.z, s.w};
    };
    const f4v r = txaa_pixel(a.params, F, a.camera, a.camera_old, a.time, a.history, x, y, W, H, load);
    a.out[(size_t)y * (size_t)W + (size_t)x] = make_float4(r.x, r.y, r.z, r.w);
}

// Reprojection fused with the TXAA resolve, after the raymarch of the frame.
// A block owns a TW x TH tile of output pixels.  It first builds the current
// frame over the tile plus the halo its TXAA neighbourhoods reach (one pixel
// left/up, two right/down: the neighbourhood centre is the fragment's pixel or
// the next one): marched pixels come from the march's output, the others are
// reprojected here.  It stores the reprojected pixels it owns (the raw frame
// the next frame reprojects from), then resolves every owned pixel's TXAA
// from shared memory.  Values equal those of reproject_kernel + txaa_kernel.
template <int TW, int TH>
__global__ void __launch_bounds__(TW * TH) resolve_kernel(const __grid_constant__ MarchArgs a) {
    constexpr int SW = TW + 3, SH = TH + 3;
    __shared__ float4 tile[SH][SW];
    const int W = a.width, H = a.height;
    const int x0 = blockIdx.x * TW - 1, y0 = blockIdx.y * TH - 1;
    const Frame F = make_frame(a.params);
    const bool full = (a.flags & MT_RENDER_FULL) != 0;
    unsigned reprojected = 0;
    for (int i = threadIdx.x; i < SW * SH; i += TW * TH) {
        const int sx = i % SW, sy = i / SW;
        const int x = x0 + sx, y = y0 + sy;
        f4v v{0.0f, 0.0f, 0.0f, 0.0f};
        if (x >= 0 && y >= 0 && x < W && y < H) {
            const size_t o = (size_t)y * (size_t)W + (size_t)x;
            if (full || is_marched(a, x, y)) {
                const float4 c = a.cur[o];
                v = f4v{c.x, c.y, c.z, c.w};
            } else {
                v = reproject_pixel(a, F, x, y);
                const bool owned = sx >= 1 && sy >= 1 && sx <= TW && sy <= TH;
                if (owned) {
                    a.cur[o] = make_float4(v.x, v.y, v.z, v.w);
                    ++reprojected;
                }
            }
        }
        tile[sy][sx] = make_float4(v.x, v.y, v.z, v.w);
    }
    __syncthreads();
    const int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
    const int x = x0 + 1 + tx, y = y0 + 1 + ty;
    if (x < W && y < H) {
        auto load = [&](int i, int j) -> f4v {
            if (i < 0 || j < 0 || i >= W || j >= H) return f4v{0.0f, 0.0f, 0.0f, 0.0f};
            const float4 s = tile[j - y0][i - x0];
            return f4v{s.x, s.y, s.z, s.w};
        };
        const f4v r = txaa_pixel(a.params, F, a.camera, a.camera_old, a.time, a.history, x, y, W, H, load);
        a.out[(size_t)y * (size_t)W + (size_t)x] = make_float4(r.x, r.y, r.z, r.w);
    }
    if (a.stats) {
        Counts none{0u, 0u, 0u};
        flush_counts(a.stats, none, reprojected);
    }
}

// rdiv(a, 1/b) against the device's IEEE division, element by element.
__global__ void selftest_division_kernel(const float* __restrict__ a, const float* __restrict__ b, float* out_rdiv,
                                         float* out_ieee, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out_rdiv[i] = rdiv(a[i], make_rcp(b[i]));
    out_ieee[i] = a[i] / b[i];
}

}  // namespace mt

// ---------------------------------------------------------------------------
// Launchers (called from the C ABI in mt_capi.cu)
// ---------------------------------------------------------------------------
namespace mt {

static cudaError_t launch_march(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev) {
    const bool timed = ev && ev->on;
    const long long m = (a.flags & MT_RENDER_FULL) ? (long long)a.width * a.height
                                                   : (long long)a.groups_x * a.groups_y;
    // Images narrower or shorter than 4 pixels give the reference an empty
    // raymarch dispatch (Renderer.cpp:713-716): nothing is marched.
    if (timed) cudaEventRecord(ev->march[0], s);
    if (m > 0) {
        const int G = a.lanes;
        const unsigned blocks = (unsigned)((m * G + 127) / 128);
        switch (G) {
            case 1: march_kernel<1><<<blocks, 128, 0, s>>>(a); break;
            case 4: march_kernel<4><<<blocks, 128, 0, s>>>(a); break;
            case 16: march_kernel<16><<<blocks, 128, 0, s>>>(a); break;
            default: march_kernel<8><<<blocks, 128, 0, s>>>(a); break;
        }
    }
    if (timed) cudaEventRecord(ev->march[1], s);
    return cudaGetLastError();
}

cudaError_t launch_render(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev) {
    const bool timed = ev && ev->on;
    if (!(a.flags & MT_RENDER_FULL)) {
        const long long n = (long long)a.width * a.height;
        if (timed) cudaEventRecord(ev->reproject[0], s);
        reproject_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
        if (timed) cudaEventRecord(ev->reproject[1], s);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_march(a, s, ev);
}

constexpr int kResolveTW = 32, kResolveTH = 8;

cudaError_t launch_frame(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev) {
    const bool timed = ev && ev->on;
    if (!a.fused_resolve) {
        // reprojection, raymarch, TXAA as three launches
        cudaError_t e = launch_render(a, s, ev);
        if (e != cudaSuccess) return e;
        TxaaArgs t;
        t.camera = a.camera;
        t.camera_old = a.camera_old;
        t.time = a.time;
        t.params = a.params;
        t.current = a.cur;
        t.history = a.history;
        t.out = a.out;
        t.width = a.width;
        t.height = a.height;
        return launch_txaa(t, s, timed ? ev->resolve : nullptr);
    }
    cudaError_t e = launch_march(a, s, ev);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((a.width + kResolveTW - 1) / kResolveTW), (unsigned)((a.height + kResolveTH - 1) / kResolveTH));
    if (timed) cudaEventRecord(ev->resolve[0], s);
    resolve_kernel<kResolveTW, kResolveTH><<<grid, kResolveTW * kResolveTH, 0, s>>>(a);
    if (timed) cudaEventRecord(ev->resolve[1], s);
    return cudaGetLastError();
}

cudaError_t launch_selftest_division(const float* a, const float* b, float* out_rdiv, float* out_ieee, int n,
                                     cudaStream_t s) {
    if (n > 0) selftest_division_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, b, out_rdiv, out_ieee, n);
    return cudaGetLastError();
}

cudaError_t launch_txaa(const TxaaArgs& a, cudaStream_t s, const cudaEvent_t* ev) {
    const long long n = (long long)a.width * a.height;
    if (ev) cudaEventRecord(ev[0], s);
    txaa_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    return cudaGetLastError();
}

}  // namespace mt
