// TEST INFRASTRUCTURE — the oracle.  Not part of the product.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the checker.
//
// CPU restatement of the two full-screen passes downstream of the compute
// stage, in FP32 with the shaders' operation order (-ffp-contract=off):
//   src/CloudScapes/shaders/postProcess_GodRays.frag:66-149
//   src/CloudScapes/shaders/postProcess_ToneMap.frag:32-84
// Written as the fragment loop the rasteriser runs: one fragment per pixel in
// raster order (rows, then columns) with in_uv at the pixel centre; each
// fragment reads the INPUT image and stores with imageStore at
// pixelPos = clamp(round(dim * in_uv)), so where two fragments store to one
// pixel the later one wins.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/meteoros.h"
#include "oracle_math.hpp"

namespace orp {

using orc::f2i;
using orc::gclamp;
using orc::gmax;
using orc::gmin;

inline float lerp(float p, float q, float t) { return p + t * (q - p); }

struct PixelPos {
    int x, y;
};

// postProcess_GodRays.frag:68-70 / postProcess_ToneMap.frag:70-71
inline void fragment(int x, int y, int W, int H, float& ux, float& uy, PixelPos& pp) {
    ux = ((float)x + 0.5f) / (float)W;
    uy = ((float)y + 0.5f) / (float)H;
    pp.x = std::min(std::max(f2i(std::round((float)W * ux)), 0), W - 1);
    pp.y = std::min(std::max(f2i(std::round((float)H * uy)), 0), H - 1);
}

// texture(godRayCreationDataSampler, uv) of the image whose texels are
// (mask, 0, 0, 0): LINEAR, CLAMP_TO_BORDER opaque black (0, 0, 0, 1)
// (Texture2D.cpp:75, Image.cpp:305-347), then dot(x, bitDec) (:39-43).
float extract(const float* m, int W, int H, float sx, float sy) {
    const float u = sx * (float)W - 0.5f, v = sy * (float)H - 0.5f;
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    const long long i0 = f2i(fu), j0 = f2i(fv);
    float t[2][2][4];
    for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
            const long long i = i0 + di, j = j0 + dj;
            float* o = t[dj][di];
            if (i < 0 || j < 0 || i >= W || j >= H) {
                o[0] = 0.0f, o[1] = 0.0f, o[2] = 0.0f, o[3] = 1.0f;
            } else {
                o[0] = m[(size_t)j * (size_t)W + (size_t)i], o[1] = 0.0f, o[2] = 0.0f, o[3] = 0.0f;
            }
        }
    float x[4];
    for (int c = 0; c < 4; ++c) x[c] = lerp(lerp(t[0][0][c], t[0][1][c], a), lerp(t[1][0][c], t[1][1][c], a), b);
    const float bitDec[4] = {1.0f / 1.0f, 1.0f / 255.0f, 1.0f / 65025.0f, 1.0f / 16581375.0f};
    return x[0] * bitDec[0] + x[1] * bitDec[1] + x[2] * bitDec[2] + x[3] * bitDec[3];
}

bool outside01(float x, float y) { return x < 0.0f || x > 1.0f || y < 0.0f || y > 1.0f; }

void godrays(const mt_camera_ubo* cam, const float* light, const float* mask, const float* in, float* out, int W,
             int H) {
    std::memcpy(out, in, sizeof(float) * 4 * (size_t)W * (size_t)H);
    // :74-87
    const float sx = 0.0f - cam->eye[0], sy = 1.0f - cam->eye[1], sz = 0.0f - cam->eye[2];
    const float sl = std::sqrt(sx * sx + sy * sy + sz * sz);
    const float tsx = sx / sl, tsy = sy / sl, tsz = sz / sl;
    const float fx0 = cam->view[2], fy0 = cam->view[6], fz0 = cam->view[10];
    const float fl = std::sqrt(fx0 * fx0 + fy0 * fy0 + fz0 * fz0);
    const float fx = -(fx0 / fl), fy = -(fy0 / fl), fz = -(fz0 / fl);
    const float blend = tsx * fx + tsy * fy + tsz * fz;
    if (blend < 0.0f) return;  // every fragment returns before its store
    // :90-93, (proj * view) * vec4(0, 1, 0, 1)
    float M[4][4];
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i)
            M[j][i] = cam->proj[0 + i] * cam->view[4 * j + 0] + cam->proj[4 + i] * cam->view[4 * j + 1] +
                      cam->proj[8 + i] * cam->view[4 * j + 2] + cam->proj[12 + i] * cam->view[4 * j + 3];
    const float ndc_x = M[0][0] * 0.0f + M[1][0] * 1.0f + M[2][0] * 0.0f + M[3][0] * 1.0f;
    const float ndc_y = M[0][1] * 0.0f + M[1][1] * 1.0f + M[2][1] * 0.0f + M[3][1] * 1.0f;
    const float ssx = gclamp((ndc_x + 1.0f) / 2.0f, 0.0f, 1.0f), ssy = gclamp((ndc_y + 1.0f) / 2.0f, 0.0f, 1.0f);
    const bool sun_outside = outside01(ssx, ssy);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float ux, uy;
            PixelPos pp;
            fragment(x, y, W, H, ux, uy, pp);
            const float dux = ((ux - ssx) / 100.0f) * 1.0f, duy = ((uy - ssy) / 100.0f) * 1.0f;
            float acc[3] = {0.0f, 0.0f, 0.0f};
            float decay = 1.0f;
            for (int i = 0; i < 100; ++i) {
                float r, g, b, a;
                if (sun_outside && outside01(ux, uy)) {
                    // :110-117: gradient toward the light colour, alpha 1
                    const float t = (ux - ssx) * 0.0f + (uy - ssy) * 1.0f;
                    r = 0.0f * (1.0f - t) + light[0] * t;
                    g = 0.0f * (1.0f - t) + light[1] * t;
                    b = 0.0f * (1.0f - t) + light[2] * t;
                    a = 1.0f;
                } else {
                    r = light[0], g = light[1], b = light[2];
                    a = extract(mask, W, H, ux, uy);
                }
                // godRayLoop (:56-62), WEIGHT_FOR_SAMPLE 0.001, DECAY 1
                const float w = decay * 0.001f;
                acc[0] += (r * a) * w;
                acc[1] += (g * a) * w;
                acc[2] += (b * a) * w;
                decay *= 1.0f;
                ux -= dux;
                uy -= duy;
            }
            if (sun_outside) acc[0] = acc[1] = acc[2] = 0.0f;  // :126
            float* o = out + 4 * ((size_t)pp.y * (size_t)W + (size_t)pp.x);
            const float* s = in + 4 * ((size_t)pp.y * (size_t)W + (size_t)pp.x);
            o[0] = s[0] + (acc[0] * 1.0f) * blend;
            o[1] = s[1] + (acc[1] * 1.0f) * blend;
            o[2] = s[2] + (acc[2] * 1.0f) * blend;
            o[3] = s[3] + 1.0f * blend;
        }
}

// Uncharted2Tonemap (:32-35)
float uncharted2(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}

// WangHashNoise (:52-66)
float wang_hash_noise(uint32_t u, uint32_t v, uint32_t s) {
    uint32_t seed = (u * 1664525u + v) + s;
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return (float)seed * (1.0f / 4294967296.0f);
}

uint32_t f2u(float t) {
    if (!(t > 0.0f)) return 0u;
    if (t >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)t;
}

// out4: float RGBA per pixel (the values the shader stores); pixels no
// fragment stores to are left as the caller filled them.
void tonemap(float time_y, const float* in, float* out4, int W, int H) {
    const float invgamma = 1.0f / 2.2f;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float ux, uy;
            PixelPos pp;
            fragment(x, y, W, H, ux, uy, pp);
            // texture(inputImageSampler, in_uv).rgb, CLAMP_TO_BORDER opaque black
            const float u = ux * (float)W - 0.5f, v = uy * (float)H - 0.5f;
            const float fu = std::floor(u), fv = std::floor(v);
            const float a = u - fu, b = v - fv;
            const long long i0 = f2i(fu), j0 = f2i(fv);
            float c[3];
            for (int ch = 0; ch < 3; ++ch) {
                float t[2][2];
                for (int dj = 0; dj < 2; ++dj)
                    for (int di = 0; di < 2; ++di) {
                        const long long i = i0 + di, j = j0 + dj;
                        t[dj][di] = (i < 0 || j < 0 || i >= W || j >= H)
                                        ? 0.0f
                                        : in[4 * ((size_t)j * (size_t)W + (size_t)i) + ch];
                    }
                c[ch] = lerp(lerp(t[0][0], t[0][1], a), lerp(t[1][0], t[1][1], a), b);
            }
            // tonemap(in_color, 100) (:37-46)
            const float whitemap = 1.0f / uncharted2(100.0f);
            const float noise = wang_hash_noise((uint32_t)pp.x, (uint32_t)pp.y, f2u(time_y)) * 0.01f;
            float* o = out4 + 4 * ((size_t)pp.y * (size_t)W + (size_t)pp.x);
            for (int ch = 0; ch < 3; ++ch) o[ch] = std::pow(uncharted2(2.5f * c[ch]) * whitemap, invgamma) + noise;
            o[3] = 1.0f;
        }
}

// Vulkan float -> UNORM8: clamp to [0, 1], scale by 255, round to nearest even; NaN -> 0.
uint8_t unorm8(float f) {
    const float c = (f > 0.0f) ? (f < 1.0f ? f : 1.0f) : 0.0f;
    return (uint8_t)std::nearbyint(c * 255.0f);
}

}  // namespace orp

extern "C" {

__attribute__((visibility("default"))) int orc_godrays_f32(const mt_camera_ubo* cam, const float* light,
                                                           const float* mask, const float* in, float* out, int W,
                                                           int H) {
    if (!cam || !light || !mask || !in || !out || W < 1 || H < 1) return 1;
    orp::godrays(cam, light, mask, in, out, W, H);
    return 0;
}

// out4 (float RGBA) and/or out8 (RGBA8 words, the UNORM conversion of out4);
// pixels no fragment stores to keep what the caller put there (out8 is
// converted only where a fragment stored).
__attribute__((visibility("default"))) int orc_tonemap_f32(float time_y, const float* in, float* out4,
                                                           uint8_t* out8, int W, int H) {
    if (!in || !out4 || W < 1 || H < 1) return 1;
    const size_t n = (size_t)W * (size_t)H;
    float* tmp = new float[4 * n];
    for (size_t i = 0; i < 4 * n; ++i) tmp[i] = NAN;
    orp::tonemap(time_y, in, tmp, W, H);
    for (size_t i = 0; i < n; ++i) {
        if (std::isnan(tmp[4 * i + 3])) continue;  // alpha is 1 wherever a fragment stored
        for (int c = 0; c < 4; ++c) out4[4 * i + c] = tmp[4 * i + c];
        if (out8)
            for (int c = 0; c < 4; ++c) out8[4 * i + c] = orp::unorm8(tmp[4 * i + c]);
    }
    delete[] tmp;
    return 0;
}

__attribute__((visibility("default"))) float orc_wang_hash_noise(uint32_t u, uint32_t v, uint32_t s) {
    return orp::wang_hash_noise(u, v, s);
}

}  // extern "C"
