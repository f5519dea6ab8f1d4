// Geometry, lighting and sky functions of the compute stage shared by every
// kernel translation unit (FP32, reference operation order; see
// mt_device.cuh for the arithmetic conventions).
#pragma once
#include <cuda_runtime.h>

#include "mt_device.cuh"
#include "mt_kernels.h"

namespace mt {

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

// cloudRayMarch.comp:194-226 (castRay, with getJitterOffset :114-132) for
// screen point (sx, sy).  The camera basis, the jitter of this frame's slot
// and ref = eye + look are the same for every pixel: they come in `v`, made
// on the host by make_view_consts with the same operations (mt_consts.cpp),
// and each ray computes only its own part.
MT_HD Ray cast_ray(const ViewConsts& v, f3 eye, float sx, float sy) {
    float nx = sx * 2.0f - 1.0f, ny = sy * 2.0f - 1.0f;
    nx = nx + v.jx;
    ny = ny + v.jy;
    const f3 cam_x = (nx * v.tanx) * ld3(v.right);
    const f3 cam_y = (ny * v.tany) * ld3(v.up);
    const f3 pp = ld3(v.ref) + cam_x + cam_y;
    return Ray{eye, normalize3_r(pp - eye)};
}

// cloudRayMarch.comp:229-273 (t = length(p - rO) with the normalised rO, as
// the reference defines it).
// The origin terms rO = (eye - c) / radius and C = dot(rO, rO) - 1 are the
// same for every ray of a frame (every ray leaves the eye): they come in
// precomputed (Frame::sh32_o, sh32_c).
MT_HD Isect ray_sphere(const float o[3], float C, f3 rD, f3 c, float radius) {
    Isect is;
    is.valid = false;
    is.point = f3{0.0f, 0.0f, 0.0f};
    is.t = 0.0f;
    const f3 rO = ld3(o);
    float A = dot3(rD, rD);
    float B = 2.0f * dot3(rD, rO);
    float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return is;
    // t = (-B - sqrt(disc)) / 2A, or the other root where that is negative.
    // 2A = 2|rD|^2 > 0, so the first root's sign is its numerator's and only
    // the root taken is divided (the camera inside the shell always takes the
    // second).
    const float sq = sqrtf(disc), n1 = -B - sq;
    const float t = (n1 < 0.0f ? -B + sq : n1) / (2.0f * A);
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
// quadratic cancels badly in FP32 (C = |rO|^2 - 1 with |rO| ~ 1).  The
// origin terms -- o = (rO - c) / radius and C, the same for every ray of a
// frame (Frame::sh_o, sh_c) -- come in precomputed: three FP64 divisions and
// the |o|^2 sum fewer per ray, on a GPU whose FP64 rate is a small fraction
// of its FP32 rate.
MT_HD Isect ray_sphere_fp64(const double o[3], double C, f3 rDf, f3 cf, float radiusf) {
    const double ox = o[0], oy = o[1], oz = o[2];
    const double r = (double)radiusf;
    const double dx = rDf.x, dy = rDf.y, dz = rDf.z;
    double A = dx * dx + dy * dy + dz * dz;
    double B = 2.0 * (dx * ox + dy * oy + dz * oz);
    double disc = B * B - 4.0 * A * C;
    Isect is;
    is.valid = false;
    is.point = f3{0.0f, 0.0f, 0.0f};
    is.t = 0.0f;
    if (disc < 0.0) return is;
    const double sq = sqrt(disc), n1 = -B - sq;  // as in ray_sphere: one division
    const double t = (n1 < 0.0 ? -B + sq : n1) / (2.0 * A);
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

// cloudRayMarch.comp:171-186
// lenInner = length(startPos - eye) is the same for every step of a ray; the
// raymarch passes it in precomputed.
MT_HD float relative_height(const Frame& F, f3 point, f3 ec, float lenInner, f3 rayDir, f3 eye) {
    float lenCam = length3(point - eye);
    f3 p2e = normalize3_r(point - ec);
    float cosTheta = dot3(rayDir, p2e);
    float num = fabsf(cosTheta * (lenCam - lenInner));
    return rdiv(num, F.r_thick);
}

// cloudRayMarch.comp:188-191
MT_HD f3 relative_position(const Frame& F, f3 pos, f3 ec) {
    return rdiv3(pos - f3{ec.x, F.inner_alt, ec.z}, F.r_thick);
}

// The four quotients of height_gradient's remaps, (h - omin) / (omax - omin).
struct HgQuot {
    float q1, q2, q3, q4;
};
static __device__ __noinline__ HgQuot hg_quotients_exceptional(float h) {
    return HgQuot{rdiv(h - 0.0f, MT_RCP(0.0f, 0.25f)), rdiv(h - 0.3f, MT_RCP(0.3f, 0.65f)),
                  rdiv(h - 0.0f, MT_RCP(0.0f, 0.1f)), rdiv(h - 0.2f, MT_RCP(0.2f, 0.3f))};
}

// cloudRayMarch.comp:475-487.  The remaps' four quotients share one range
// check (rdiv_core; all four redone by rdiv when any falls outside it).
MT_HD float height_gradient(float h, float type) {
    h = gclamp(h, 0.0f, 1.0f);
    HgQuot q{rdiv_core(h - 0.0f, MT_RCP(0.0f, 0.25f)), rdiv_core(h - 0.3f, MT_RCP(0.3f, 0.65f)),
             rdiv_core(h - 0.0f, MT_RCP(0.0f, 0.1f)), rdiv_core(h - 0.2f, MT_RCP(0.2f, 0.3f))};
    if (!(rdiv_in_range(q.q1) & rdiv_in_range(q.q2) & rdiv_in_range(q.q3) & rdiv_in_range(q.q4)))
        q = hg_quotients_exceptional(h);
    // remap(h, omin, omax, nmin, nmax) = nmin + q * (nmax - nmin)
    float stratocumulus = gmax(0.0f, (0.0f + (q.q1 * (1.0f - 0.0f))) * (1.0f + (q.q2 * (0.0f - 1.0f))));
    float stratus = gmax(0.0f, (0.0f + (q.q3 * (1.0f - 0.0f))) * (1.0f + (q.q4 * (0.0f - 1.0f))));
    float a = gmix(stratus, stratocumulus, gclamp(type * 2.0f, 0.0f, 1.0f));
    float b = gmix(stratocumulus, stratus, gclamp((type - 0.5f) * 2.0f, 0.0f, 1.0f));
    return gmix(a, b, type);
}

struct Erosion {
    float lo;  // high_freq_modifier * 0.005
    Rcp r;     // {1 - lo, ~1/(1 - lo)}: the width (b, exact division) and an
               // approximate reciprocal for the light samples (y)
};
MT_HD Erosion make_erosion(float modifier) {
    Erosion e;
    e.lo = modifier * 0.005f;
    e.r = Rcp{1.0f - e.lo, __fdividef(1.0f, 1.0f - e.lo)};
    return e;
}
MT_HD float erode(float baseCloud, const Erosion& e) { return 0.0f + (((baseCloud - e.lo) / e.r.b) * (1.0f - 0.0f)); }

// cloudRayMarch.comp:295-306.  The phase weights the light energy and the
// sky, colour only: pow in the special-function unit's form (see
// light_energy).
MT_HD float henyey_greenstein(float c, float e) {
    float num = 1.0f - e * e;
    float den = __powf((1.0f + e * e - 2.0f * e * c), 1.5f);
    return (num / den) * 0.07957747154594767f;
}

// cloudRayMarch.comp:331-388.  cos_q = (cos_angle - 0.7) / (1.0 - 0.7), the
// ray-constant quotient of the attenuation remap (:341-343).  exp and pow are
// the special-function unit's forms, exp2(x * log2 e) and exp2(y * log2 x),
// which is how GLSL defines pow's precision: they differ from the correctly
// rounded values by tens of ulp at most.  The light energy reaches colour
// only, never the accumulated density, the control flow or the god-ray mask.
MT_HD float light_energy(float h, float dl, float ds, float phase, float cos_q, float brightness) {
    const float primary = __expf(-dl);
    const float secondary = primary;  // exp(-dl) twice in the reference (:334, :340)
    float att = gmax(secondary + (cos_q * (secondary * 0.25f - secondary)), primary);
    float depth = 0.05f + __powf(ds, gclamp(remap_r(h * 0.125f, 0.3f, MT_RCP(0.3f, 0.85f), 0.5f, 2.0f), 0.5f, 2.0f));
    float vert = __powf(gclamp(remap_r(h * 1.5f, 0.07f, MT_RCP(0.07f, 0.34f), 0.1f, 1.0f), 0.1f, 1.0f), 0.8f);
    float in_scatter = depth * vert;
    return att * primary * in_scatter * phase * brightness;
}

// cloudRayMarch.comp:401-467 (Preetham) for ray direction `dir`.  The terms
// that depend on the sun only -- its direction from the eye, sunE, the
// Rayleigh and Mie coefficients and yDot -- are the frame's (Frame::sky_*,
// made on the host by make_march_frame with the same operations); the rest
// is per ray, its exp and pow in the special-function unit's forms as in
// light_energy (the background reaches colour only).  Once per ray: kept out
// of line so the march loop stays small in the instruction cache.
static __device__ __noinline__ f3 atmosphere_color(const Frame& F, f3 dir) {
    const float PI = 3.14159265f;
    const f3 sunDir = ld3(F.sky_sun_dir), BetaR = ld3(F.sky_betaR), BetaM = ld3(F.sky_betaM);
    const float sunE = F.sky_sunE;
    float zenith = acosf(gmax(0.0f, dir.y));
    float inverse = 1.0f / (cosf(zenith) + 0.15f * __powf(93.885f - ((zenith * 180.0f) / PI), -1.253f));
    float sR = 8.4E3f * inverse;
    float sM = 1.25E3f * inverse;
    f3 ex = (-BetaR) * sR + BetaM * sM;
    f3 fex{__expf(ex.x), __expf(ex.y), __expf(ex.z)};
    float cosTheta = dot3(sunDir, dir);
    float rp = cosTheta * 0.5f + 0.5f;
    float rPhase = 0.05968310365946075f * (1.0f + rp * rp);
    f3 betaRTheta = BetaR * rPhase;
    float mPhase = henyey_greenstein(cosTheta, 0.8f);
    f3 betaMTheta = BetaM * mPhase;
    f3 betas = (betaRTheta + betaMTheta) / ld3(F.sky_betaRM);
    f3 a = (sunE * betas) * (f3{1.0f, 1.0f, 1.0f} - fex);
    f3 Lin{__powf(a.x, 1.5f), __powf(a.y, 1.5f), __powf(a.z, 1.5f)};
    f3 b = (sunE * betas) * fex;
    f3 pb{__powf(b.x, 0.5f), __powf(b.y, 0.5f), __powf(b.z, 0.5f)};
    Lin = Lin * mix3(f3{1.0f, 1.0f, 1.0f}, pb, gclamp(F.sky_yDot, 0.0f, 1.0f));
    f3 L0 = 0.1f * fex;
    const float SAC = 0.999956676946448443553574619906976478926848692873900859324f;
    float sunDisk = gsmoothstep(SAC, SAC + 0.00002f, cosTheta);
    L0 = L0 + ((sunE * 15000.0f) * fex) * sunDisk;
    return (Lin + L0) * 0.04f + f3{0.0f, 0.0003f, 0.00075f};
}

struct Counts {
    unsigned primary, light, rays;
    unsigned sig;  // traced marches: control-flow signature of the ray being marched
};

// cloudRayMarch.comp:106-112 + postProcess_GodRays.frag:36-43
MT_HD float godray_value(float v, float dir_y) {
    f4v enc{1.0f * v, 255.0f * v, 65025.0f * v, 16581375.0f * v};
    enc = f4v{gfract(enc.x), gfract(enc.y), gfract(enc.z), gfract(enc.w)};
    const float k = 1.0f / 255.0f;
    enc = f4v{enc.x - enc.y * k, enc.y - enc.z * k, enc.z - enc.w * k, enc.w - enc.w * 0.0f};
    if (dir_y < 0.05f) enc = enc * gmax(5.0f, dir_y);
    return enc.x * (1.0f / 1.0f) + enc.y * (1.0f / 255.0f) + enc.z * (1.0f / 65025.0f) + enc.w * (1.0f / 16581375.0f);
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

}  // namespace mt
