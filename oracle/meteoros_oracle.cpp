// TEST INFRASTRUCTURE — the oracle.  Not part of the product.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the checker (or, for bench.py, as the timed CPU
// baseline).  The product path never calls it.
//
// CPU restatement of the reference's compute stage, templated on the scalar
// type: float for FP32 parity with the CUDA kernels, double for the FP64
// oracle of the precision form.  Follows, function by function:
//   src/CloudScapes/shaders/cloudRayMarch.comp   (raymarch, lighting, sky)
//   src/CloudScapes/shaders/reprojection.comp    (10-tap reprojection)
//   src/CloudScapes/shaders/postProcess_TXAA.frag (TXAA resolve)
// Sampler semantics (LINEAR filter, REPEAT for the noise textures,
// CLAMP_TO_BORDER opaque black for frame images, a single mip level) follow
// Texture3D.cpp:92-134, Image.cpp:305-347, Texture2D.cpp:75 and Sky.cpp:47-57.
// The parameters the shader hard-codes come in through mt_params
// (include/meteoros.h); mt_params_reference() reproduces the shader's values.
//
// Build: g++ -O3 -fopenmp -ffp-contract=off -fPIC -shared (see oracle/build.py).
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/meteoros.h"
#include "oracle_math.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------
// Textures.  A texel is read as raw values (0..255 for RGBA8, the stored value
// for float storage); a filtered sample interpolates the raw values with
// exact weights and multiplies by `scale` (1/255 for UNORM8, 1 otherwise).
// Weights follow the Vulkan LINEAR filter: u = s*N - 0.5, i0 = floor(u),
// alpha = u - i0; REPEAT wraps the integer texel coordinate.
// ---------------------------------------------------------------------------
template <class T> struct Tex {
    const uint8_t* u8 = nullptr;
    const float* f32 = nullptr;
    int n = 0;
    T scale = T(1);
    inline V4<T> texel(size_t i) const {
        if (u8) return {T(u8[4 * i]), T(u8[4 * i + 1]), T(u8[4 * i + 2]), T(u8[4 * i + 3])};
        return {T(f32[4 * i]), T(f32[4 * i + 1]), T(f32[4 * i + 2]), T(f32[4 * i + 3])};
    }
};

template <class T> inline T lerp(T p, T q, T t) { return p + t * (q - p); }
template <class T> inline V4<T> lerp4(V4<T> p, V4<T> q, T t) {
    return {lerp(p.x, q.x, t), lerp(p.y, q.y, t), lerp(p.z, q.z, t), lerp(p.w, q.w, t)};
}

template <class T> V4<T> tex3_repeat(const Tex<T>& t, V3<T> s) {
    const int n = t.n;
    const unsigned m = (unsigned)n - 1u;
    const T N = T(n);
    T u = s.x * N - T(0.5), v = s.y * N - T(0.5), w = s.z * N - T(0.5);
    T fu = std::floor(u), fv = std::floor(v), fw = std::floor(w);
    T a = u - fu, b = v - fv, g = w - fw;
    unsigned iu = (unsigned)f2i(fu), iv = (unsigned)f2i(fv), iw = (unsigned)f2i(fw);
    size_t x0 = iu & m, x1 = (iu + 1u) & m, y0 = iv & m, y1 = (iv + 1u) & m, z0 = iw & m, z1 = (iw + 1u) & m;
    const size_t nn = (size_t)n;
    auto at = [&](size_t x, size_t y, size_t z) { return t.texel((z * nn + y) * nn + x); };
    V4<T> c00 = lerp4(at(x0, y0, z0), at(x1, y0, z0), a);
    V4<T> c10 = lerp4(at(x0, y1, z0), at(x1, y1, z0), a);
    V4<T> c01 = lerp4(at(x0, y0, z1), at(x1, y0, z1), a);
    V4<T> c11 = lerp4(at(x0, y1, z1), at(x1, y1, z1), a);
    V4<T> c0 = lerp4(c00, c10, b);
    V4<T> c1 = lerp4(c01, c11, b);
    return lerp4(c0, c1, g) * t.scale;
}

template <class T> V4<T> tex2_repeat(const Tex<T>& t, V2<T> s) {
    const int n = t.n;
    const unsigned m = (unsigned)n - 1u;
    const T N = T(n);
    T u = s.x * N - T(0.5), v = s.y * N - T(0.5);
    T fu = std::floor(u), fv = std::floor(v);
    T a = u - fu, b = v - fv;
    unsigned iu = (unsigned)f2i(fu), iv = (unsigned)f2i(fv);
    size_t x0 = iu & m, x1 = (iu + 1u) & m, y0 = iv & m, y1 = (iv + 1u) & m;
    const size_t nn = (size_t)n;
    auto at = [&](size_t x, size_t y) { return t.texel(y * nn + x); };
    V4<T> c0 = lerp4(at(x0, y0), at(x1, y0), a);
    V4<T> c1 = lerp4(at(x0, y1), at(x1, y1), a);
    return lerp4(c0, c1, b) * t.scale;
}

// Bilinear sample of an RGBA frame image with CLAMP_TO_BORDER, border colour
// VK_BORDER_COLOR_INT_OPAQUE_BLACK = (0,0,0,1) (Texture2D.cpp:75, Image.cpp:324).
template <class T> V4<T> tex2_border(const T* img, int W, int H, V2<T> s) {
    T u = s.x * T(W) - T(0.5), v = s.y * T(H) - T(0.5);
    T fu = std::floor(u), fv = std::floor(v);
    T a = u - fu, b = v - fv;
    int i0 = f2i(fu), j0 = f2i(fv);
    auto at = [&](long long i, long long j) -> V4<T> {
        if (i < 0 || j < 0 || i >= W || j >= H) return {T(0), T(0), T(0), T(1)};
        const T* p = img + 4 * ((size_t)j * (size_t)W + (size_t)i);
        return {p[0], p[1], p[2], p[3]};
    };
    long long i1 = (long long)i0 + 1, j1 = (long long)j0 + 1;
    V4<T> c0 = lerp4(at(i0, j0), at(i1, j0), a);
    V4<T> c1 = lerp4(at(i0, j1), at(i1, j1), a);
    return lerp4(c0, c1, b);
}

// ---------------------------------------------------------------------------
// Per-frame constants
// ---------------------------------------------------------------------------
template <class T> struct Frame {
    Tex<T> base, detail, curl, weather;
    const mt_camera_ubo* cam;
    const mt_camera_ubo* cam_old;
    const mt_time_ubo* tm;
    const mt_params* p;
    T R, Rin, Rout, thickness, inner_alt;
};

template <class T> struct Ray {
    V3<T> origin, direction;
};
template <class T> struct Isect {
    V3<T> normal, point;
    bool valid;
    T t;
};

template <class T> inline V3<T> v3(const float* f) { return {T(f[0]), T(f[1]), T(f[2])}; }

// cloudRayMarch.comp:114-132 / postProcess_TXAA.frag:63-81.  The
// reprojection shader's copy (reprojection.comp:72-90) reads halton 1/2 again
// for index >= 4; `repro_variant` selects that.
template <class T> V2<T> jitter_offset(const mt_time_ubo* tm, int index, int dimx, int dimy, bool repro_variant) {
    V2<T> j{T(0), T(0)};
    index = index / 2;
    if (index < 4) {
        j.x = T(tm->halton_seq1[index]);
        j.y = T(tm->halton_seq2[index]);
    } else {
        index -= 4;
        if (repro_variant) {
            j.x = T(tm->halton_seq1[index]);
            j.y = T(tm->halton_seq2[index]);
        } else {
            j.x = T(tm->halton_seq3[index]);
            j.y = T(tm->halton_seq4[index]);
        }
    }
    return {j.x / T(dimx), j.y / T(dimy)};
}

// cloudRayMarch.comp:194-226 (castRay), reprojection.comp:111-144.
template <class T> Ray<T> cast_ray(V2<T> screen, V3<T> eye, const mt_camera_ubo* cam, const mt_time_ubo* tm,
                                   int pixelID, int dimx, int dimy, bool repro_variant) {
    const float* v = cam->view;
    V3<T> camRight = normalize(V3<T>{T(v[0]), T(v[4]), T(v[8])});
    V3<T> camUp = normalize(V3<T>{T(v[1]), T(v[5]), T(v[9])});
    V3<T> camLook = -normalize(V3<T>{T(v[2]), T(v[6]), T(v[10])});
    V2<T> ndc{screen.x * T(2) - T(1), screen.y * T(2) - T(1)};
    V2<T> jit = jitter_offset<T>(tm, pixelID, dimx, dimy, repro_variant);
    ndc.x = ndc.x + jit.x;
    ndc.y = ndc.y + jit.y;
    V3<T> cam_x = (ndc.x * T(cam->tan_fov_by_2[0])) * camRight;
    V3<T> cam_y = (ndc.y * T(cam->tan_fov_by_2[1])) * camUp;
    V3<T> ref = eye + camLook;
    V3<T> pp = ref + cam_x + cam_y;
    return {eye, normalize(pp - eye)};
}

// cloudRayMarch.comp:229-273.  isect.t = length(p - rO) with rO the
// normalised origin is the reference's own definition and is kept.
template <class T> Isect<T> ray_sphere(V3<T> rO, V3<T> rD, V3<T> c, T radius) {
    Isect<T> is;
    is.valid = false;
    is.point = {T(0), T(0), T(0)};
    is.normal = {T(0), T(1), T(0)};
    is.t = T(0);
    rO = rO - c;
    rO = rO / radius;
    T A = dot(rD, rD);
    T B = T(2) * dot(rD, rO);
    T C = dot(rO, rO) - T(1);
    T disc = B * B - T(4) * A * C;
    if (disc < T(0)) return is;
    T t = (-B - std::sqrt(disc)) / (T(2) * A);
    if (t < T(0)) t = (-B + std::sqrt(disc)) / (T(2) * A);
    if (t >= T(0)) {
        V3<T> pnt = rO + t * rD;
        is.valid = true;
        is.normal = normalize(pnt);
        pnt = pnt * radius;
        pnt = pnt + c;
        is.point = pnt;
        is.t = length(pnt - rO);
    }
    return is;
}

// FP64 shell intersection for the precision form: the same formula evaluated
// in double and rounded back (only used when params->fp64_shells is set).
template <class T> Isect<T> ray_sphere_fp64(V3<T> rO, V3<T> rD, V3<T> c, T radius) {
    Isect<double> d = ray_sphere<double>({double(rO.x), double(rO.y), double(rO.z)},
                                         {double(rD.x), double(rD.y), double(rD.z)},
                                         {double(c.x), double(c.y), double(c.z)}, double(radius));
    Isect<T> r;
    r.valid = d.valid;
    r.point = {T(d.point.x), T(d.point.y), T(d.point.z)};
    r.normal = {T(d.normal.x), T(d.normal.y), T(d.normal.z)};
    r.t = T(d.t);
    return r;
}

// cloudRayMarch.comp:153-169
template <class T> inline T remap(T v, T omin, T omax, T nmin, T nmax) {
    return nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
}
template <class T> inline T remap_clamped(T v, T omin, T omax, T nmin, T nmax) {
    T t = nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
    return gclamp(t, nmin, nmax);
}
template <class T> inline T remap_clamped_ba(T v, T omin, T omax, T nmin, T nmax) {
    v = gclamp(v, omin, omax);
    T t = nmin + (((v - omin) / (omax - omin)) * (nmax - nmin));
    return gclamp(t, nmin, nmax);
}

// cloudRayMarch.comp:171-186
template <class T> T relative_height(const Frame<T>& F, V3<T> point, V3<T> earthCenter, V3<T> startPos, V3<T> rayDir,
                                     V3<T> eye) {
    T lenCam = length(point - eye);
    T lenInner = length(startPos - eye);
    V3<T> p2e = normalize(point - earthCenter);
    T cosTheta = dot(rayDir, p2e);
    T num = std::fabs(cosTheta * (lenCam - lenInner));
    return num / F.thickness;
}

// cloudRayMarch.comp:188-191
template <class T> inline V3<T> relative_position(const Frame<T>& F, V3<T> pos, V3<T> earthCenter) {
    return (pos - V3<T>{earthCenter.x, F.inner_alt, earthCenter.z}) / F.thickness;
}

// cloudRayMarch.comp:475-487 (dead code in the reference; the weather-driven
// presets enable it through params->height_gradient).
template <class T> T height_gradient(T h, T type) {
    h = gclamp(h, T(0), T(1));
    T cumulus = gmax(T(0), remap(h, L(0.01), L(0.3), T(0), T(1)) * remap(h, L(0.6), L(0.95), T(1), T(0)));
    T stratocumulus = gmax(T(0), remap(h, T(0), L(0.25), T(0), T(1)) * remap(h, L(0.3), L(0.65), T(1), T(0)));
    T stratus = gmax(T(0), remap(h, T(0), L(0.1), T(0), T(1)) * remap(h, L(0.2), L(0.3), T(1), T(0)));
    (void)cumulus;  // the reference computes it and never uses it
    T a = gmix(stratus, stratocumulus, gclamp(type * T(2), T(0), T(1)));
    T b = gmix(stratocumulus, stratus, gclamp((type - L(0.5)) * T(2), T(0), T(1)));
    return gmix(a, b, type);
}

// cloudRayMarch.comp:489-497
template <class T> V3<T> skew_with_wind(const Frame<T>& F, V3<T> point, T h) {
    const mt_params* p = F.p;
    point = point + ((h * v3<T>(p->skew_dir)) * T(p->cloud_top_offset)) * L(0.009);
    point = point + (v3<T>(p->wind_dir) * T(p->wind_speed)) * T(F.tm->time[1]);
    return point;
}

// Coverage and cloud type at a sample (weather-driven presets only).
template <class T> struct Weather {
    T coverage_lo;  // remap threshold
    T coverage_mul; // final multiplier
    T type;
};

template <class T> Weather<T> weather_at(const Frame<T>& F, V3<T> pos, V3<T> earthCenter) {
    Weather<T> w;
    const mt_params* p = F.p;
    if (p->coverage_mode == 0) {
        w.coverage_lo = T(p->coverage);
        w.coverage_mul = T(p->coverage);
        w.type = T(0);
        return w;
    }
    T ws = T(p->weather_scale);
    V2<T> uv{(pos.x - earthCenter.x) / ws, (pos.z - earthCenter.z) / ws};
    V4<T> wd = tex2_repeat(F.weather, uv);
    w.coverage_lo = T(1) - wd.x;
    w.coverage_mul = wd.x;
    w.type = wd.z;
    return w;
}

// cloudRayMarch.comp:499-540
template <class T> T sample_low_frequency(const Frame<T>& F, V3<T> point, T relH, const Weather<T>& wt) {
    V4<T> n = tex3_repeat(F.base, point);
    T fbm = (n.y * L(0.625)) + (n.z * L(0.25)) + (n.w * L(0.125));
    fbm = gclamp(fbm, T(0), T(1));
    T baseCloud = remap_clamped(n.x, (fbm - L(0.9)), T(1), T(0), T(1));
    if (F.p->height_gradient) baseCloud = baseCloud * height_gradient(relH, wt.type);
    T cov = wt.coverage_lo;
    T bc = remap_clamped_ba(baseCloud, cov, T(1), T(0), T(1));
    bc = bc * wt.coverage_mul;
    return bc;
}

// cloudRayMarch.comp:542-563, split in two: the texture part (curl offset and
// the detail FBM modifier) depends only on the point and the height, so it is
// shared by the primary erosion and the six cone-light erosions, which the
// reference all evaluate at the primary sample point (:645, :665).
template <class T> T erosion_modifier(const Frame<T>& F, V3<T> point, T h) {
    V4<T> curl = tex2_repeat(F.curl, V2<T>{point.x, point.y});
    point.x = point.x + (curl.x * (T(1) - h)) * L(0.5);
    point.y = point.y + (curl.y * (T(1) - h)) * L(0.5);
    V4<T> hf = tex3_repeat(F.detail, point);
    T hfbm = (hf.x * L(0.625)) + (hf.y * L(0.25)) + (hf.z * L(0.125));
    return gclamp(gmix(hfbm, T(1) - hfbm, gclamp(h * T(2), T(0), T(1))), T(0), T(1));
}
template <class T> inline T erode(T baseCloud, T modifier) {
    return remap(baseCloud, modifier * L(0.005), T(1), T(0), T(1));
}

// cloudRayMarch.comp:295-306
template <class T> T henyey_greenstein(T c, T e) {
    T num = T(1) - e * e;
    T den = std::pow((T(1) + e * e - T(2) * e * c), L(1.5));
    return (num / den) * L(0.07957747154594767);
}
template <class T> T hg_modified(T c, T e, T si, T ss) {
    return gmax(henyey_greenstein(c, e), si * henyey_greenstein(c, L(0.99) - ss));
}

// cloudRayMarch.comp:331-388 (the "THIRD INSTANCE" / "MEDIUM" lines that are live)
template <class T> T light_energy(T h, T dl, T ds, T phase, T cos_angle, T step_size, T brightness) {
    (void)step_size;
    T primary = std::exp(-dl);
    T secondary = std::exp(-dl);
    T att = gmax(remap(cos_angle, L(0.7), T(1), secondary, secondary * L(0.25)), primary);
    T depth = L(0.05) + std::pow(ds, gclamp(remap(h * L(0.125), L(0.3), L(0.85), L(0.5), T(2)), L(0.5), T(2)));
    T vert = std::pow(gclamp(remap(h * L(1.5), L(0.07), L(0.34), L(0.1), T(1)), L(0.1), T(1)), L(0.8));
    T in_scatter = depth * vert;
    return att * primary * in_scatter * phase * brightness;
}

// cloudRayMarch.comp:401-467 (Preetham sky)
template <class T> V3<T> atmosphere_color(const Frame<T>& F, V3<T> dir, V3<T> sunDir, T sunIntensity) {
    const V3<T> skySun = v3<T>(F.p->sky_sun_pos);
    const T PI = L(3.14159265);
    sunDir = normalize(sunDir);
    // calcSunIntensity (:421-425)
    T zenithAngleCos = gclamp(normalize(skySun).y, T(-1), T(1));
    T sunI = L(1000.0) * gmax(T(0), T(1) - std::pow(L(2.718281828459),
                                                    -((L(1.6110731557) - std::acos(zenithAngleCos)) / L(1.5))));
    T sunE = sunIntensity * sunI;
    // calcSkyBetaR (:406-411)
    T sunFade = T(1) - gclamp(T(1) - std::exp(skySun.y / L(450000.0)), T(0), T(1));
    const V3<T> RT{L(5.804542996261093E-6), L(1.3562911419845635E-5), L(3.0265902468824876E-5)};
    V3<T> BetaR = RT * (T(2) - T(1) + sunFade);
    // calcSkyBetaV (:413-419)
    T c = (L(0.2) * L(10.0)) * L(10E-18);
    const V3<T> MIE{L(1.839991851443397), L(2.779802391966052), L(4.079047954386109)};
    V3<T> BetaM = ((L(0.434) * c) * MIE) * L(0.005);

    T zenith = std::acos(gmax(T(0), dir.y));
    T inverse = T(1) / (std::cos(zenith) + L(0.15) * std::pow(L(93.885) - ((zenith * L(180.0)) / PI), L(-1.253)));
    T sR = L(8.4E3) * inverse;
    T sM = L(1.25E3) * inverse;
    V3<T> ex = (-BetaR) * sR + BetaM * sM;
    V3<T> fex{std::exp(ex.x), std::exp(ex.y), std::exp(ex.z)};
    T cosTheta = dot(sunDir, dir);
    T rPhase = L(0.05968310365946075) * (T(1) + (cosTheta * L(0.5) + L(0.5)) * (cosTheta * L(0.5) + L(0.5)));
    V3<T> betaRTheta = BetaR * rPhase;
    T mPhase = henyey_greenstein(cosTheta, L(0.8));
    V3<T> betaMTheta = BetaM * mPhase;
    T yDot = T(1) - sunDir.y;
    yDot = yDot * (yDot * yDot * yDot * yDot);
    V3<T> betas = (betaRTheta + betaMTheta) / (BetaR + BetaM);
    V3<T> a = (sunE * betas) * (V3<T>{T(1), T(1), T(1)} - fex);
    V3<T> Lin{std::pow(a.x, L(1.5)), std::pow(a.y, L(1.5)), std::pow(a.z, L(1.5))};
    V3<T> b = (sunE * betas) * fex;
    V3<T> pb{std::pow(b.x, L(0.5)), std::pow(b.y, L(0.5)), std::pow(b.z, L(0.5))};
    Lin = Lin * vmix(V3<T>{T(1), T(1), T(1)}, pb, gclamp(yDot, T(0), T(1)));
    V3<T> L0 = L(0.1) * fex;
    T sunDisk = gsmoothstep(L(0.999956676946448443553574619906976478926848692873900859324),
                            L(0.999956676946448443553574619906976478926848692873900859324) + L(0.00002), cosTheta);
    L0 = L0 + ((sunE * L(15000.0)) * fex) * sunDisk;
    return (Lin + L0) * L(0.04) + V3<T>{T(0), L(0.0003), L(0.00075)};
}

struct Counters {
    uint64_t primary = 0, light = 0, rays = 0, pixels = 0;
    // Control-flow signature of the last ray marched: an FNV-1a hash over its
    // executed steps of (jitter index | in cloud << 4 | the six light samples'
    // cbl > 0 bits << 5), in step order.  Two marches with equal signatures
    // (and step counts) took the same branches at every threshold.
    uint32_t sig = 2166136261u;
};
inline void sig_step(Counters& c, uint32_t code) { c.sig = (c.sig ^ code) * 16777619u; }

// cloudRayMarch.comp:565-688
template <class T> V3<T> ray_march(const Frame<T>& F, const Ray<T>& ray, V3<T> earthCenter, V3<T> startPos, T start_t,
                                   T end_t, int pixelID, T& accumDensity, Counters& cnt) {
    const mt_params* p = F.p;
    T _dot = dot(ray.direction, V3<T>{T(0), T(1), T(0)});
    const T jitterfactor = L(1.180);
    const T baseDensityFactor = L(0.380);
    T maxSteps;
    if (p->steps_min == p->steps_max)
        maxSteps = T(p->steps_min);
    else
        maxSteps = std::floor(gmix(T(p->steps_min), T(p->steps_max), T(1) - _dot));
    const T thick = end_t - start_t;
    const T stepSize = thick / maxSteps;
    T transmittance = T(1);
    V3<T> returnColor{T(0), T(0), T(0)};

    const V3<T> lightDir = normalize(v3<T>(p->sun_light_pos) - ray.origin);
    const T cos_angle = dot(normalize(ray.direction), lightDir);
    const T HG_light = hg_modified(cos_angle, L(0.6), L(0.7), L(0.1));

    V3<T> maxComp;
    T ax = std::fabs(lightDir.x), ay = std::fabs(lightDir.y), az = std::fabs(lightDir.z);
    if (ax > ay && ax > az)
        maxComp = {ax, T(0), T(0)};
    else if (ay > ax && ay > az)
        maxComp = {T(0), ay, T(0)};
    else
        maxComp = {T(0), T(0), az};
    V3<T> zC = cross(lightDir, maxComp);
    V3<T> xC = cross(zC, lightDir);
    const V3<T> K[6] = {{L(0.1), L(0.25), L(-0.15)}, {L(0.2), L(0.5), L(0.2)},   {L(-0.2), L(0.1), L(-0.1)},
                        {L(-0.05), L(0.75), L(0.05)}, {L(-0.1), T(1), T(0)},     {T(0), T(3), T(0)}};
    V3<T> kernel[6];
    for (int i = 0; i < 6; ++i) kernel[i] = mat3_mul(xC, lightDir, zC, K[i]);

    // Iteration guard (not in the reference): a degenerate interval whose step
    // is below the ulp of t would never advance.  2*steps+8 is never reached
    // by a valid ray (the loop runs steps or steps+1 times).
    const int cap = 2 * f2i(maxSteps) + 8;
    int it = 0;
    cnt.rays++;
    cnt.sig = 2166136261u;
    for (T t = start_t; t < end_t; t += stepSize) {
        if (it++ >= cap) break;
        cnt.primary++;
        int _index = f2i(gmod(T(pixelID + f2i(t)), T(16)));
        uint32_t code = (uint32_t)_index & 15u;
        V2<T> jl = jitter_offset<T>(F.tm, _index, 75, 75, false);
        V3<T> jd = ray.direction + V3<T>{jl.x, (jl.x + jl.y) * jitterfactor, jl.y};
        V3<T> pos = ray.origin + t * jd;
        V3<T> samplePoint = relative_position(F, pos, earthCenter);
        samplePoint = samplePoint / T(p->noise_period);
        T relH = relative_height(F, pos, earthCenter, startPos, ray.direction, ray.origin);
        V3<T> skewed = skew_with_wind(F, samplePoint, relH);
        Weather<T> wt = weather_at(F, pos, earthCenter);
        T baseDensity = sample_low_frequency(F, skewed, relH, wt) * baseDensityFactor;
        if (baseDensity > T(0)) {
            T mod = erosion_modifier(F, skewed, relH);
            T hfd = erode(baseDensity * L(1.4), mod);
            accumDensity = accumDensity + hfd * L(0.5);
            T dl = T(0);
            code |= 16u;
            for (int i = 0; i < 6; ++i) {
                V3<T> lightPos = pos + ((stepSize * kernel[i]) * T(i));
                V3<T> slp = relative_position(F, lightPos, earthCenter);
                cnt.light++;
                T cbl = sample_low_frequency(F, slp, relH, wt);
                if (cbl > T(0)) {
                    dl = dl + erode(L(1.5) * cbl, mod);
                    code |= 32u << i;
                }
            }
            T E = light_energy(relH, dl, baseDensity, HG_light, cos_angle, stepSize, L(5.0));
            transmittance = gmix(transmittance, E, (T(1) - accumDensity));
            returnColor = returnColor + V3<T>{transmittance, transmittance, transmittance};
        }
        sig_step(cnt, code);
        if (accumDensity >= T(p->accum_limit)) {
            accumDensity = T(1);
            break;
        }
    }
    return returnColor;
}

// cloudRayMarch.comp:106-112 and the decode of postProcess_GodRays.frag:36-43:
// the god-ray mask value the consumer reads back, in R32F.
template <class T> T godray_value(T v, T dir_y) {
    V4<T> enc{T(1) * v, L(255.0) * v, L(65025.0) * v, L(16581375.0) * v};
    enc = {gfract(enc.x), gfract(enc.y), gfract(enc.z), gfract(enc.w)};
    const T k = T(1) / L(255.0);
    enc = {enc.x - enc.y * k, enc.y - enc.z * k, enc.z - enc.w * k, enc.w - enc.w * T(0)};
    if (dir_y < L(0.05)) enc = enc * gmax(L(5.0), dir_y);
    V4<T> dec{T(1) / T(1), T(1) / L(255.0), T(1) / L(65025.0), T(1) / L(16581375.0)};
    return enc.x * dec.x + enc.y * dec.y + enc.z * dec.z + enc.w * dec.w;
}

// cloudRayMarch.comp:690-826 for one pixel.  Returns the RGBA colour; *mask
// gets the god-ray value.
template <class T> V4<T> march_pixel(const Frame<T>& F, int px, int py, int W, int H, T* mask, Counters& cnt) {
    const mt_params* p = F.p;
    const int pixelID = F.tm->frame_count_mod16;
    V2<T> uv{T(px) / T(W), T(py) / T(H)};
    uv.y = T(1) - uv.y;
    V3<T> eyePos = T(p->eye_sign) * v3<T>(F.cam->eye);
    Ray<T> ray = cast_ray(uv, eyePos, F.cam, F.tm, pixelID, W, H, false);
    const T sunIntensity = L(0.780);
    V3<T> bg{T(0), T(0), T(0)};
    T _dot = dot(V3<T>{T(0), T(1), T(0)}, ray.direction);
    const T bgMul = gmax(L(0.620), _dot);
    const T fadePoint = L(0.06);
    if (_dot < T(0)) {
        V3<T> cNear = V3<T>{T(0), L(0.16), L(0.51)} * L(0.4);
        V3<T> c2 = V3<T>{T(0), L(0.73), L(0.95)} * L(0.5);
        bg = vmix(cNear, c2, -ray.direction.y * L(5.5));
        *mask = T(0);
        return {bg.x, bg.y, bg.z, T(1)};
    } else if (_dot < fadePoint) {
        bg = atmosphere_color(F, ray.direction, v3<T>(p->sky_sun_pos) - ray.origin, sunIntensity);
        bg = bg * bgMul;
        *mask = T(0);
        return {bg.x, bg.y, bg.z, T(1)};
    }
    bg = atmosphere_color(F, ray.direction, v3<T>(p->sky_sun_pos) - ray.origin, sunIntensity);
    bg = bg * bgMul;
    V3<T> earthCenter = eyePos;
    earthCenter.y = -F.R;
    Isect<T> in, out;
    if (p->fp64_shells) {
        in = ray_sphere_fp64(ray.origin, ray.direction, earthCenter, F.Rin);
        out = ray_sphere_fp64(ray.origin, ray.direction, earthCenter, F.Rout);
    } else {
        in = ray_sphere(ray.origin, ray.direction, earthCenter, F.Rin);
        out = ray_sphere(ray.origin, ray.direction, earthCenter, F.Rout);
    }
    T accum = T(0);
    V3<T> res = ray_march(F, ray, earthCenter, in.point, in.t, out.t, pixelID, accum, cnt);
    T godAccum = accum;
    accum = accum * gsmoothstep(T(0), T(1), gmin(T(1), remap(ray.direction.y, fadePoint, L(0.2), T(0), T(1))));
    V3<T> fc = vmix(bg, res, accum);
    T grey = L(25.0) * gmin(L(0.05), T(1) - godAccum);
    *mask = godray_value(grey, ray.direction.y);
    return {fc.x, fc.y, fc.z, T(1)};
}

// reprojection.comp:193-244 for one pixel.
template <class T> V4<T> reproject_pixel(const Frame<T>& F, int x, int y, int W, int H, const T* prev) {
    const mt_params* p = F.p;
    V2<T> uv{T(x) / T(W), T(y) / T(H)};
    const int pixelID = F.tm->frame_count_mod16;
    V3<T> eyePos = T(p->eye_sign) * v3<T>(F.cam->eye);
    Ray<T> ray = cast_ray(uv, eyePos, F.cam, F.tm, pixelID, W, H, true);
    V3<T> earthCenter = eyePos;
    earthCenter.y = -F.R;
    Isect<T> in = ray_sphere(ray.origin, ray.direction, earthCenter, F.Rin);
    const float* ov = F.cam_old->view;
    V3<T> q = in.point;
    V3<T> od{T(ov[0]) * q.x + T(ov[4]) * q.y + T(ov[8]) * q.z + T(ov[12]) * T(1),
             T(ov[1]) * q.x + T(ov[5]) * q.y + T(ov[9]) * q.z + T(ov[13]) * T(1),
             T(ov[2]) * q.x + T(ov[6]) * q.y + T(ov[10]) * q.z + T(ov[14]) * T(1)};
    od = normalize(od);
    od = od / (-od.z);
    T old_u = (od.x / T(F.cam->tan_fov_by_2[0])) * L(0.5) + L(0.5);
    T old_v = (od.y / T(F.cam->tan_fov_by_2[1])) * L(0.5) + L(0.5);
    V2<T> motion{old_u - uv.x, old_v - uv.y};
    V4<T> blur{T(0), T(0), T(0), T(0)};
    for (int i = 0; i < 10; ++i) {
        T f = T(i) / T(10);
        V2<T> off{motion.x * f, motion.y * f};
        T iu = std::round((old_u - off.x) * T(W));
        T iv = std::round((old_v - off.y) * T(H));
        int ix = f2i(iu), iy = f2i(iv);
        ix = gclamp(ix, 0, W - 1);
        iy = gclamp(iy, 0, H - 1);
        const T* s = prev + 4 * ((size_t)iy * (size_t)W + (size_t)ix);
        blur = blur + V4<T>{s[0], s[1], s[2], s[3]};
    }
    return blur / T(10);
}

// postProcess_TXAA.frag:193-221, 223-269 for one fragment (x, y).
template <class T> V4<T> txaa_pixel(const Frame<T>& F, int x, int y, int W, int H, const T* cur, const T* hist) {
    const mt_params* p = F.p;
    V2<T> in_uv{(T(x) + L(0.5)) / T(W), (T(y) + L(0.5)) / T(H)};
    int ppx = f2i(std::round(T(W) * in_uv.x)), ppy = f2i(std::round(T(H) * in_uv.y));
    ppx = gclamp(ppx, 0, W - 1);
    ppy = gclamp(ppy, 0, H - 1);
    const int pixelID = F.tm->frame_count_mod16;
    V3<T> eyePos = T(p->eye_sign) * v3<T>(F.cam->eye);
    Ray<T> ray = cast_ray(in_uv, eyePos, F.cam, F.tm, pixelID, W, H, false);
    V3<T> earthCenter = eyePos;
    earthCenter.y = -F.R;
    Isect<T> in = ray_sphere(ray.origin, ray.direction, earthCenter, F.Rin);
    const float* ov = F.cam_old->view;
    V3<T> q = in.point;
    V3<T> od{T(ov[0]) * q.x + T(ov[4]) * q.y + T(ov[8]) * q.z + T(ov[12]) * T(1),
             T(ov[1]) * q.x + T(ov[5]) * q.y + T(ov[9]) * q.z + T(ov[13]) * T(1),
             T(ov[2]) * q.x + T(ov[6]) * q.y + T(ov[10]) * q.z + T(ov[14]) * T(1)};
    od = normalize(od);
    od = od / (-od.z);
    T old_u = (od.x / T(F.cam->tan_fov_by_2[0])) * L(0.5) + L(0.5);
    T old_v = (od.y / T(F.cam->tan_fov_by_2[1])) * L(0.5) + L(0.5);

    // imageLoad of an out-of-range coordinate returns zero (robust access).
    auto load = [&](int i, int j) -> V4<T> {
        if (i < 0 || j < 0 || i >= W || j >= H) return {T(0), T(0), T(0), T(0)};
        const T* s = cur + 4 * ((size_t)j * (size_t)W + (size_t)i);
        return {s[0], s[1], s[2], s[3]};
    };
    V4<T> ctl = load(ppx - 1, ppy - 1), ctc = load(ppx, ppy - 1), ctr = load(ppx + 1, ppy - 1);
    V4<T> cml = load(ppx - 1, ppy), cmc = load(ppx, ppy), cmr = load(ppx + 1, ppy);
    V4<T> cbl = load(ppx - 1, ppy + 1), cbc = load(ppx, ppy + 1), cbr = load(ppx + 1, ppy + 1);
    V4<T> cmin = vmin(ctl, vmin(ctc, vmin(ctr, vmin(cml, vmin(cmc, vmin(cmr, vmin(cbl, vmin(cbc, cbr))))))));
    V4<T> cmax = vmax(ctl, vmax(ctc, vmax(ctr, vmax(cml, vmax(cmc, vmax(cmr, vmax(cbl, vmax(cbc, cbr))))))));
    V4<T> cavg = (ctl + ctc + ctr + cml + cmc + cmr + cbl + cbc + cbr) / L(9.0);
    V4<T> cmin5 = vmin(ctc, vmin(cml, vmin(cmc, vmin(cmr, cbc))));
    V4<T> cmax5 = vmax(ctc, vmax(cml, vmax(cmc, vmax(cmr, cbc))));
    V4<T> cavg5 = (ctc + cml + cmc + cmr + cbc) / L(5.0);
    cmin = V4<T>{L(0.5) * (cmin.x + cmin5.x), L(0.5) * (cmin.y + cmin5.y), L(0.5) * (cmin.z + cmin5.z),
                 L(0.5) * (cmin.w + cmin5.w)};
    cmax = V4<T>{L(0.5) * (cmax.x + cmax5.x), L(0.5) * (cmax.y + cmax5.y), L(0.5) * (cmax.z + cmax5.z),
                 L(0.5) * (cmax.w + cmax5.w)};
    cavg = V4<T>{L(0.5) * (cavg.x + cavg5.x), L(0.5) * (cavg.y + cavg5.y), L(0.5) * (cavg.z + cavg5.z),
                 L(0.5) * (cavg.w + cavg5.w)};

    V4<T> currColor = load(ppx, ppy);
    V4<T> prevColor = tex2_border(hist, W, H, V2<T>{old_u, old_v});

    // clip_aabb (:171-191) with p = clamp(cavg, cmin, cmax), q = prevColor
    V4<T> pc = vclamp(cavg, cmin, cmax);
    V3<T> p_clip{L(0.5) * (cmax.x + cmin.x), L(0.5) * (cmax.y + cmin.y), L(0.5) * (cmax.z + cmin.z)};
    const T EPS = L(0.0000000001);
    V3<T> e_clip{L(0.5) * (cmax.x - cmin.x) + EPS, L(0.5) * (cmax.y - cmin.y) + EPS,
                 L(0.5) * (cmax.z - cmin.z) + EPS};
    V4<T> v_clip = prevColor - V4<T>{p_clip.x, p_clip.y, p_clip.z, pc.w};
    V3<T> v_unit{v_clip.x / e_clip.x, v_clip.y / e_clip.y, v_clip.z / e_clip.z};
    V3<T> a_unit{std::fabs(v_unit.x), std::fabs(v_unit.y), std::fabs(v_unit.z)};
    T ma_unit = gmax(a_unit.x, gmax(a_unit.y, a_unit.z));
    if (ma_unit > T(1)) prevColor = V4<T>{p_clip.x, p_clip.y, p_clip.z, pc.w} + v_clip / ma_unit;

    const V3<T> lw{L(0.2125), L(0.7154), L(0.0721)};
    T lum0 = dot(V3<T>{currColor.x, currColor.y, currColor.z}, lw);
    T lum1 = dot(V3<T>{prevColor.x, prevColor.y, prevColor.z}, lw);
    T unbiased_diff = std::fabs(lum0 - lum1) / gmax(lum0, gmax(lum1, L(0.2)));
    T unbiased_weight = T(1) - unbiased_diff;
    T w2 = unbiased_weight * unbiased_weight;
    T k = gmix(T(p->feedback_min), T(p->feedback_max), w2);
    return vmix4(prevColor, currColor, k);
}

template <class T> Tex<T> make_tex(const void* data, int fmt, int n) {
    Tex<T> t;
    t.n = n;
    if (fmt == 0) {
        t.u8 = (const uint8_t*)data;
        t.scale = T(1) / L(255.0);
    } else {
        t.f32 = (const float*)data;
        t.scale = T(1);
    }
    return t;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C ABI (ctypes) — test infrastructure
// ---------------------------------------------------------------------------
extern "C" {

typedef struct orc_volumes {
    const void* base;    // MT_BASE_N^3 RGBA
    const void* detail;  // MT_DETAIL_N^3 RGBA
    const void* curl;    // MT_CURL_N^2 RGBA
    const void* weather; // MT_WEATHER_N^2 RGBA (may be NULL when coverage_mode == 0)
    int32_t fmt;         // 0: uint8 texels, 1: float texel values
    int32_t _pad;
} orc_volumes;

}  // extern "C"

namespace orc {

template <class T> Frame<T> make_frame(const orc_volumes* v, const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                                       const mt_time_ubo* tm, const mt_params* p) {
    Frame<T> F;
    F.base = make_tex<T>(v->base, v->fmt, MT_BASE_N);
    F.detail = make_tex<T>(v->detail, v->fmt, MT_DETAIL_N);
    F.curl = make_tex<T>(v->curl, v->fmt, MT_CURL_N);
    F.weather = make_tex<T>(v->weather ? v->weather : v->curl, v->fmt, v->weather ? MT_WEATHER_N : MT_CURL_N);
    F.cam = cam;
    F.cam_old = cam_old;
    F.tm = tm;
    F.p = p;
    F.R = T(p->earth_radius);
    F.Rin = T(p->shell_inner_radius);
    F.Rout = T(p->shell_outer_radius);
    F.thickness = F.Rout - F.Rin;
    F.inner_alt = F.Rin - F.R;
    return F;
}

// Which pixels the raymarch dispatch writes: Renderer.cpp:713-716 launches
// ceil(floor(W/4)/32) x ceil(floor(H/4)/32) groups of 32x32; each invocation
// marches pixel gid*4 + slot; stores outside the image do nothing.
inline int march_groups(int dim) { return 32 * ((dim / 4 + 31) / 32); }

template <class T> int render(const orc_volumes* v, const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                              const mt_time_ubo* tm, const mt_params* p, const T* prev, T* cur, T* mask, int W,
                              int H, unsigned flags, int nthreads, uint64_t* counters) {
    if (!v || !cam || !cam_old || !tm || !p || !cur || W <= 0 || H <= 0) return 1;
    const bool full = (flags & MT_RENDER_FULL) != 0;
    if (!full && !prev) return 1;
    Frame<T> F = make_frame<T>(v, cam, cam_old, tm, p);
    const int id = tm->frame_count_mod16;
    if (id < 0 || id > 15) return 1;
    const int sx = p->slot_x[id], sy = p->slot_y[id];
    const int gx = march_groups(W), gy = march_groups(H);
    uint64_t c_primary = 0, c_light = 0, c_rays = 0, c_pixels = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : c_primary, c_light, c_rays, c_pixels)
    for (int y = 0; y < H; ++y) {
        Counters cnt;
        for (int x = 0; x < W; ++x) {
            bool marched;
            if (full) {
                marched = true;
            } else {
                int dx = x - sx, dy = y - sy;
                marched = dx >= 0 && dy >= 0 && (dx % 4) == 0 && (dy % 4) == 0 && dx / 4 < gx && dy / 4 < gy;
            }
            T* o = cur + 4 * ((size_t)y * (size_t)W + (size_t)x);
            V4<T> c;
            if (marched) {
                T m;
                c = march_pixel(F, x, y, W, H, &m, cnt);
                if (mask) mask[(size_t)y * (size_t)W + (size_t)x] = m;
            } else {
                c = reproject_pixel(F, x, y, W, H, prev);
            }
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
            o[3] = c.w;
            cnt.pixels++;
        }
        c_primary += cnt.primary;
        c_light += cnt.light;
        c_rays += cnt.rays;
        c_pixels += cnt.pixels;
    }
    if (counters) {
        counters[0] = c_primary;
        counters[1] = c_light;
        counters[2] = c_rays;
        counters[3] = c_pixels;
    }
    return 0;
}

// cloudRayMarch.comp:690-826 for a list of pixels (x, y pairs), each marched
// as in a full-raymarch frame; for error statistics on a sample of a large frame.
// counts (may be NULL): per pixel four uint32, the ray's executed primary
// samples, its in-cloud samples (density > 0, cloudRayMarch.comp:642), its
// control-flow signature (Counters::sig; 0 for a ray that marched no step)
// and 0.
template <class T> int march_pixels(const orc_volumes* v, const mt_camera_ubo* cam, const mt_time_ubo* tm,
                                    const mt_params* p, int W, int H, const int32_t* xy, long long n, T* rgba,
                                    T* mask, uint32_t* counts, int nthreads) {
    if (!v || !cam || !tm || !p || !xy || !rgba || W <= 0 || H <= 0 || n < 0) return 1;
    Frame<T> F = make_frame<T>(v, cam, cam, tm, p);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < n; ++i) {
        Counters cnt;
        T m;
        V4<T> c = march_pixel(F, xy[2 * i], xy[2 * i + 1], W, H, &m, cnt);
        rgba[4 * i] = c.x;
        rgba[4 * i + 1] = c.y;
        rgba[4 * i + 2] = c.z;
        rgba[4 * i + 3] = c.w;
        if (mask) mask[i] = m;
        if (counts) {
            counts[4 * i] = (uint32_t)cnt.primary;
            counts[4 * i + 1] = (uint32_t)(cnt.light / 6);
            counts[4 * i + 2] = cnt.primary ? cnt.sig : 0u;
            counts[4 * i + 3] = 0u;
        }
    }
    return 0;
}

template <class T> int txaa(const mt_camera_ubo* cam, const mt_camera_ubo* cam_old, const mt_time_ubo* tm,
                            const mt_params* p, const T* cur, const T* hist, T* out, int W, int H, int nthreads) {
    if (!cam || !cam_old || !tm || !p || !cur || !hist || !out || W <= 0 || H <= 0) return 1;
    Frame<T> F;
    F.cam = cam;
    F.cam_old = cam_old;
    F.tm = tm;
    F.p = p;
    F.R = T(p->earth_radius);
    F.Rin = T(p->shell_inner_radius);
    F.Rout = T(p->shell_outer_radius);
    F.thickness = F.Rout - F.Rin;
    F.inner_alt = F.Rin - F.R;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            V4<T> c = txaa_pixel(F, x, y, W, H, cur, hist);
            T* o = out + 4 * ((size_t)y * (size_t)W + (size_t)x);
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
            o[3] = c.w;
        }
    return 0;
}

}  // namespace orc

extern "C" {

__attribute__((visibility("default"))) int orc_render_f32(const orc_volumes* v, const mt_camera_ubo* cam,
                                                          const mt_camera_ubo* cam_old, const mt_time_ubo* tm,
                                                          const mt_params* p, const float* prev, float* cur,
                                                          float* mask, int W, int H, unsigned flags, int nthreads,
                                                          uint64_t* counters) {
    return orc::render<float>(v, cam, cam_old, tm, p, prev, cur, mask, W, H, flags, nthreads, counters);
}

__attribute__((visibility("default"))) int orc_render_f64(const orc_volumes* v, const mt_camera_ubo* cam,
                                                          const mt_camera_ubo* cam_old, const mt_time_ubo* tm,
                                                          const mt_params* p, const double* prev, double* cur,
                                                          double* mask, int W, int H, unsigned flags, int nthreads,
                                                          uint64_t* counters) {
    return orc::render<double>(v, cam, cam_old, tm, p, prev, cur, mask, W, H, flags, nthreads, counters);
}

__attribute__((visibility("default"))) int orc_txaa_f32(const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                                                        const mt_time_ubo* tm, const mt_params* p, const float* cur,
                                                        const float* hist, float* out, int W, int H, int nthreads) {
    return orc::txaa<float>(cam, cam_old, tm, p, cur, hist, out, W, H, nthreads);
}

__attribute__((visibility("default"))) int orc_txaa_f64(const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                                                        const mt_time_ubo* tm, const mt_params* p, const double* cur,
                                                        const double* hist, double* out, int W, int H, int nthreads) {
    return orc::txaa<double>(cam, cam_old, tm, p, cur, hist, out, W, H, nthreads);
}

__attribute__((visibility("default"))) int orc_march_pixels_f32(const orc_volumes* v, const mt_camera_ubo* cam,
                                                                const mt_time_ubo* tm, const mt_params* p, int W,
                                                                int H, const int32_t* xy, long long n, float* rgba,
                                                                float* mask, uint32_t* counts, int nthreads) {
    return orc::march_pixels<float>(v, cam, tm, p, W, H, xy, n, rgba, mask, counts, nthreads);
}
__attribute__((visibility("default"))) int orc_march_pixels_f64(const orc_volumes* v, const mt_camera_ubo* cam,
                                                                const mt_time_ubo* tm, const mt_params* p, int W,
                                                                int H, const int32_t* xy, long long n, double* rgba,
                                                                double* mask, uint32_t* counts, int nthreads) {
    return orc::march_pixels<double>(v, cam, tm, p, W, H, xy, n, rgba, mask, counts, nthreads);
}

// Single-function probes for the unit tests (float instantiation).
__attribute__((visibility("default"))) float orc_height_gradient(float h, float type) {
    return orc::height_gradient<float>(h, type);
}
__attribute__((visibility("default"))) float orc_remap(float v, float a, float b, float c, float d) {
    return orc::remap<float>(v, a, b, c, d);
}
__attribute__((visibility("default"))) float orc_remap_clamped(float v, float a, float b, float c, float d) {
    return orc::remap_clamped<float>(v, a, b, c, d);
}
__attribute__((visibility("default"))) float orc_remap_clamped_ba(float v, float a, float b, float c, float d) {
    return orc::remap_clamped_ba<float>(v, a, b, c, d);
}
__attribute__((visibility("default"))) float orc_hg(float c, float e) { return orc::henyey_greenstein<float>(c, e); }
__attribute__((visibility("default"))) float orc_light_energy(float h, float dl, float ds, float phase, float cosA,
                                                              float step, float bright) {
    return orc::light_energy<float>(h, dl, ds, phase, cosA, step, bright);
}
__attribute__((visibility("default"))) float orc_godray_value(float v, float dir_y) {
    return orc::godray_value<float>(v, dir_y);
}
__attribute__((visibility("default"))) int orc_ray_sphere(const float* rO, const float* rD, const float* c,
                                                          float radius, float* point_t) {
    orc::Isect<float> is = orc::ray_sphere<float>({rO[0], rO[1], rO[2]}, {rD[0], rD[1], rD[2]},
                                                  {c[0], c[1], c[2]}, radius);
    point_t[0] = is.point.x;
    point_t[1] = is.point.y;
    point_t[2] = is.point.z;
    point_t[3] = is.t;
    return is.valid ? 1 : 0;
}
__attribute__((visibility("default"))) void orc_tex3(const void* data, int fmt, int n, const float* s, float* out) {
    orc::Tex<float> t = orc::make_tex<float>(data, fmt, n);
    orc::V4<float> r = orc::tex3_repeat(t, orc::V3<float>{s[0], s[1], s[2]});
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

}  // extern "C"
