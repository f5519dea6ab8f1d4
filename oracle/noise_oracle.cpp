// TEST INFRASTRUCTURE — the oracle.  Not part of the product.
//
// CPU restatement of the seeded noise-volume generator.  The reference has no
// generator (it loads Nubis assets, Sky.cpp:25-58); its one integer hash is
// WangHashNoise (shaders/postProcess_ToneMap.frag:52-66), whose integer core
// `wang()` below restates and which every lattice hash here is built from.
// The algorithms are the published ones: tileable Worley (cellular) noise,
// Perlin's improved gradient noise (Perlin 2002: fade 6t^5-15t^4+10t^3, the
// 12-edge gradient set selected from 4 hash bits) and fBm sums, combined as
// the Nubis cloud textures describe (Schneider, "The real-time volumetric
// cloudscapes of Horizon: Zero Dawn", 2015): R = Perlin-Worley, GBA = Worley
// fBm at rising frequencies.
//
// Every arithmetic step is an IEEE single-precision +, -, *, / or sqrt in a
// fixed order (compiled with -ffp-contract=off), so the CUDA generator can and
// must match it bit for bit.  Layouts follow ImageLoadingUtility.cpp:75-139
// (x fastest, then y, then slice z; RGBA interleaved).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/meteoros.h"

namespace orn {

// Integer core of WangHashNoise (postProcess_ToneMap.frag:55-62).
static inline uint32_t wang(uint32_t u, uint32_t v, uint32_t s) {
    uint32_t seed = (u * 1664525u + v) + s;
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return seed;
}
static inline uint32_t hash3(uint32_t x, uint32_t y, uint32_t z, uint32_t s) { return wang(wang(x, y, s), z, s); }
static inline uint32_t seed32(uint64_t seed) { return (uint32_t)seed ^ (uint32_t)(seed >> 32); }
static inline uint32_t salt(uint32_t s, uint32_t k) { return s + k * 0x9E3779B9u; }

static inline float fmin_(float a, float b) { return b < a ? b : a; }
static inline float fmax_(float a, float b) { return a < b ? b : a; }
static inline float clamp01(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }
static inline float lerp(float a, float b, float t) { return a + t * (b - a); }
static inline float fade(float t) { return ((t * t) * t) * ((t * ((t * 6.0f) - 15.0f)) + 10.0f); }

// Inverted Worley noise, period F cells (F a power of two), p in cell units.
static float worley3(float px, float py, float pz, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
    int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    float rx = px - fx, ry = py - fy, rz = pz - fz;
    float best = 100.0f;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                uint32_t wx = (uint32_t)(cx + dx) & m, wy = (uint32_t)(cy + dy) & m, wz = (uint32_t)(cz + dz) & m;
                uint32_t h = hash3(wx, wy, wz, s);
                float ox = (float)(h & 1023u) * (1.0f / 1024.0f);
                float oy = (float)((h >> 10) & 1023u) * (1.0f / 1024.0f);
                float oz = (float)((h >> 20) & 1023u) * (1.0f / 1024.0f);
                float vx = ((float)dx + ox) - rx;
                float vy = ((float)dy + oy) - ry;
                float vz = ((float)dz + oz) - rz;
                float d2 = vx * vx + vy * vy + vz * vz;
                best = d2 < best ? d2 : best;
            }
    float d = std::sqrt(best);
    return 1.0f - (d < 1.0f ? d : 1.0f);
}

static float worley_fbm3(float x, float y, float z, int F, uint32_t s) {
    float f0 = (float)F, f1 = (float)(2 * F), f2 = (float)(4 * F);
    float w0 = worley3(x * f0, y * f0, z * f0, F, s);
    float w1 = worley3(x * f1, y * f1, z * f1, 2 * F, s + 1u);
    float w2 = worley3(x * f2, y * f2, z * f2, 4 * F, s + 2u);
    return (w0 * 0.625f + w1 * 0.25f) + w2 * 0.125f;
}

static inline float grad3(uint32_t h, float x, float y, float z) {
    h &= 15u;
    float u = h < 8u ? x : y;
    float v = h < 4u ? y : ((h == 12u || h == 14u) ? x : z);
    return ((h & 1u) ? -u : u) + ((h & 2u) ? -v : v);
}

static float perlin3(float px, float py, float pz, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float x = px - fx, y = py - fy, z = pz - fz;
    float u = fade(x), v = fade(y), w = fade(z);
    uint32_t x0 = (uint32_t)ix & m, x1 = (uint32_t)(ix + 1) & m;
    uint32_t y0 = (uint32_t)iy & m, y1 = (uint32_t)(iy + 1) & m;
    uint32_t z0 = (uint32_t)iz & m, z1 = (uint32_t)(iz + 1) & m;
    float g000 = grad3(hash3(x0, y0, z0, s), x, y, z);
    float g100 = grad3(hash3(x1, y0, z0, s), x - 1.0f, y, z);
    float g010 = grad3(hash3(x0, y1, z0, s), x, y - 1.0f, z);
    float g110 = grad3(hash3(x1, y1, z0, s), x - 1.0f, y - 1.0f, z);
    float g001 = grad3(hash3(x0, y0, z1, s), x, y, z - 1.0f);
    float g101 = grad3(hash3(x1, y0, z1, s), x - 1.0f, y, z - 1.0f);
    float g011 = grad3(hash3(x0, y1, z1, s), x, y - 1.0f, z - 1.0f);
    float g111 = grad3(hash3(x1, y1, z1, s), x - 1.0f, y - 1.0f, z - 1.0f);
    float a00 = lerp(g000, g100, u), a10 = lerp(g010, g110, u);
    float a01 = lerp(g001, g101, u), a11 = lerp(g011, g111, u);
    float b0 = lerp(a00, a10, v), b1 = lerp(a01, a11, v);
    return lerp(b0, b1, w);
}

static float perlin_fbm3(float x, float y, float z, int F, int octaves, uint32_t s) {
    float sum = 0.0f, amp = 1.0f, tot = 0.0f;
    int f = F;
    for (int o = 0; o < octaves; ++o) {
        float ff = (float)f;
        sum = sum + amp * perlin3(x * ff, y * ff, z * ff, f, s + (uint32_t)o);
        tot = tot + amp;
        amp = amp * 0.5f;
        f *= 2;
    }
    return sum / tot;
}

static inline float grad2(uint32_t h, float x, float y) {
    switch (h & 7u) {
        case 0: return x + y;
        case 1: return -x + y;
        case 2: return x - y;
        case 3: return -x - y;
        case 4: return x;
        case 5: return -x;
        case 6: return y;
        default: return -y;
    }
}

static float perlin2(float px, float py, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = std::floor(px), fy = std::floor(py);
    int ix = (int)fx, iy = (int)fy;
    float x = px - fx, y = py - fy;
    float u = fade(x), v = fade(y);
    uint32_t x0 = (uint32_t)ix & m, x1 = (uint32_t)(ix + 1) & m;
    uint32_t y0 = (uint32_t)iy & m, y1 = (uint32_t)(iy + 1) & m;
    float g00 = grad2(wang(x0, y0, s), x, y);
    float g10 = grad2(wang(x1, y0, s), x - 1.0f, y);
    float g01 = grad2(wang(x0, y1, s), x, y - 1.0f);
    float g11 = grad2(wang(x1, y1, s), x - 1.0f, y - 1.0f);
    return lerp(lerp(g00, g10, u), lerp(g01, g11, u), v);
}

static float perlin_fbm2(float x, float y, int F, int octaves, uint32_t s) {
    float sum = 0.0f, amp = 1.0f, tot = 0.0f;
    int f = F;
    for (int o = 0; o < octaves; ++o) {
        float ff = (float)f;
        sum = sum + amp * perlin2(x * ff, y * ff, f, s + (uint32_t)o);
        tot = tot + amp;
        amp = amp * 0.5f;
        f *= 2;
    }
    return sum / tot;
}

static inline uint8_t q8(float v) { return (uint8_t)(int)std::floor(clamp01(v) * 255.0f + 0.5f); }

static inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
// IEEE binary32 -> binary16, round to nearest even.
static uint16_t f2h(float f) {
    uint32_t x = fbits(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax < 0x38800000u) {
        float a;
        std::memcpy(&a, &ax, 4);
        return (uint16_t)(sign | (uint32_t)std::nearbyint(a * 16777216.0f));
    }
    return (uint16_t)(sign | ((ax - 0x38000000u + 0xfffu + ((ax >> 13) & 1u)) >> 13));
}
// IEEE binary32 -> bfloat16, round to nearest even (finite inputs).
static uint16_t f2bf(float f) {
    uint32_t x = fbits(f);
    return (uint16_t)((x + 0x7fffu + ((x >> 16) & 1u)) >> 16);
}

struct Out {
    uint8_t* u8;
    uint16_t* h16;
    uint16_t* b16;
    inline void put(size_t texel, float r, float g, float b, float a) const {
        const float v[4] = {clamp01(r), clamp01(g), clamp01(b), clamp01(a)};
        for (int c = 0; c < 4; ++c) {
            if (u8) u8[4 * texel + c] = q8(v[c]);
            if (h16) h16[4 * texel + c] = f2h(v[c]);
            if (b16) b16[4 * texel + c] = f2bf(v[c]);
        }
    }
};

// 128^3: R Perlin-Worley (Perlin fBm 4 octaves at period 4, remapped with the
// Worley fBm of G as its floor), G/B/A Worley fBm at base frequencies 4/8/16.
static void gen_base(uint32_t s, const Out& o) {
    const int N = MT_BASE_N;
    const float inv = 1.0f / (float)N;
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < N; ++z)
        for (int y = 0; y < N; ++y)
            for (int x = 0; x < N; ++x) {
                float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv, pz = ((float)z + 0.5f) * inv;
                float pf = perlin_fbm3(px, py, pz, 4, 4, salt(s, 1));
                float p01 = clamp01(pf * 0.5f + 0.5f);
                float g = worley_fbm3(px, py, pz, 4, salt(s, 2));
                float b = worley_fbm3(px, py, pz, 8, salt(s, 3));
                float a = worley_fbm3(px, py, pz, 16, salt(s, 4));
                float r = (p01 - (g - 1.0f)) / (1.0f - (g - 1.0f));
                o.put(((size_t)z * N + y) * N + x, r, g, b, a);
            }
}

// 32^3: Worley at frequencies 8/16/32 in R/G/B, alpha 1 (unused by the shader).
static void gen_detail(uint32_t s, const Out& o) {
    const int N = MT_DETAIL_N;
    const float inv = 1.0f / (float)N;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < N; ++z)
        for (int y = 0; y < N; ++y)
            for (int x = 0; x < N; ++x) {
                float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv, pz = ((float)z + 0.5f) * inv;
                float r = worley3(px * 8.0f, py * 8.0f, pz * 8.0f, 8, salt(s, 5));
                float g = worley3(px * 16.0f, py * 16.0f, pz * 16.0f, 16, salt(s, 6));
                float b = worley3(px * 32.0f, py * 32.0f, pz * 32.0f, 32, salt(s, 7));
                o.put(((size_t)z * N + y) * N + x, r, g, b, 1.0f);
            }
}

// 128^2 curl of a tileable Perlin fBm potential (central differences one
// texel apart), stored as 0.5 + 0.5 * curl in R/G and |curl| in B.
static void gen_curl(uint32_t s, const Out& o) {
    const int N = MT_CURL_N;
    const float inv = 1.0f / (float)N;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv;
            float dy = perlin_fbm2(px, py + inv, 4, 3, salt(s, 8)) - perlin_fbm2(px, py - inv, 4, 3, salt(s, 8));
            float dx = perlin_fbm2(px + inv, py, 4, 3, salt(s, 8)) - perlin_fbm2(px - inv, py, 4, 3, salt(s, 8));
            float cx = dy * 4.0f;
            float cy = -(dx * 4.0f);
            float mag = std::sqrt(cx * cx + cy * cy);
            o.put((size_t)y * N + x, cx * 0.5f + 0.5f, cy * 0.5f + 0.5f, mag, 1.0f);
        }
}

// 512^2 weather map: R coverage = clamp(fBm6 * 1.2 - 0.2, 0, 1) (fBm mapped to
// [0,1]), G precipitation uniform [0,1), B cloud type in {0, 0.5, 1} per
// 64x64-texel cell, A = 1.
static void gen_weather(uint32_t s, const Out& o) {
    const int N = MT_WEATHER_N;
    const float inv = 1.0f / (float)N;
    const float types[3] = {0.0f, 0.5f, 1.0f};
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv;
            float f = perlin_fbm2(px, py, 4, 6, salt(s, 9)) * 0.5f + 0.5f;
            float cov = clamp01(f * 1.2f - 0.2f);
            float precip = (float)(wang((uint32_t)x, (uint32_t)y, salt(s, 10)) >> 8) * (1.0f / 16777216.0f);
            float type = types[wang((uint32_t)(x >> 6), (uint32_t)(y >> 6), salt(s, 11)) % 3u];
            o.put((size_t)y * N + x, cov, precip, type, 1.0f);
        }
}

}  // namespace orn

extern "C" {

// Any output pointer may be NULL.  *_h16 are IEEE half bits, *_b16 bfloat16 bits.
__attribute__((visibility("default"))) void orc_generate_volumes(uint64_t seed, uint8_t* base, uint8_t* detail,
                                                                uint8_t* curl, uint8_t* weather, uint16_t* base_h16,
                                                                uint16_t* detail_h16, uint16_t* curl_h16,
                                                                uint16_t* weather_h16, uint16_t* base_b16,
                                                                uint16_t* detail_b16, uint16_t* curl_b16,
                                                                uint16_t* weather_b16) {
    const uint32_t s = orn::seed32(seed);
    if (base || base_h16 || base_b16) orn::gen_base(s, {base, base_h16, base_b16});
    if (detail || detail_h16 || detail_b16) orn::gen_detail(s, {detail, detail_h16, detail_b16});
    if (curl || curl_h16 || curl_b16) orn::gen_curl(s, {curl, curl_h16, curl_b16});
    if (weather || weather_h16 || weather_b16) orn::gen_weather(s, {weather, weather_h16, weather_b16});
}

__attribute__((visibility("default"))) uint32_t orc_wang(uint32_t u, uint32_t v, uint32_t s) {
    return orn::wang(u, v, s);
}
__attribute__((visibility("default"))) uint16_t orc_f2h(float f) { return orn::f2h(f); }
__attribute__((visibility("default"))) uint16_t orc_f2bf(float f) { return orn::f2bf(f); }

}  // extern "C"
