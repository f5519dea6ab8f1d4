// Seeded noise-volume generation on the GPU.
//
// The reference loads pre-baked Nubis textures (Sky.cpp:25-58); these kernels
// generate the same four volumes from a seed instead.  Lattice hashing is
// built on the integer core of the reference's WangHashNoise
// (shaders/postProcess_ToneMap.frag:52-66).  Noise families: tileable Worley
// (cellular) noise, Perlin's improved gradient noise (Perlin 2002) and fBm
// sums, arranged as the Nubis cloud textures describe them (R = Perlin-Worley,
// GBA = Worley fBm at rising frequencies).  Every step is an IEEE FP32
// +, -, *, / or sqrt in a fixed order (this file is compiled with
// -fmad=false), so the output is bit-identical to the CPU generator that the
// tests hold it against.
//
// One thread per texel.  Outputs: RGBA8 words plus IEEE half and bfloat16
// copies for the precision form, all in create3DTextureFromMany2DTextures
// layout (x fastest, then y, then slice z).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "mt_kernels.h"

namespace mt {
namespace {

__device__ __forceinline__ uint32_t wang(uint32_t u, uint32_t v, uint32_t s) {
    uint32_t seed = (u * 1664525u + v) + s;
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return seed;
}
__device__ __forceinline__ uint32_t hash3(uint32_t x, uint32_t y, uint32_t z, uint32_t s) {
    return wang(wang(x, y, s), z, s);
}
__device__ __forceinline__ uint32_t salt(uint32_t s, uint32_t k) { return s + k * 0x9E3779B9u; }
__device__ __forceinline__ float clamp01(float x) {
    x = x < 0.0f ? 0.0f : x;
    return 1.0f < x ? 1.0f : x;
}
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }
__device__ __forceinline__ float fade(float t) { return ((t * t) * t) * ((t * ((t * 6.0f) - 15.0f)) + 10.0f); }

// Inverted Worley noise with period F cells; p in cell units.
__device__ float worley3(float px, float py, float pz, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    float rx = px - fx, ry = py - fy, rz = pz - fz;
    float best = 100.0f;
    for (int dz = -1; dz <= 1; ++dz) {
        const uint32_t wz = (uint32_t)(cz + dz) & m;
        for (int dy = -1; dy <= 1; ++dy) {
            const uint32_t wy = (uint32_t)(cy + dy) & m;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const uint32_t wx = (uint32_t)(cx + dx) & m;
                const uint32_t h = hash3(wx, wy, wz, s);
                float ox = (float)(h & 1023u) * (1.0f / 1024.0f);
                float oy = (float)((h >> 10) & 1023u) * (1.0f / 1024.0f);
                float oz = (float)((h >> 20) & 1023u) * (1.0f / 1024.0f);
                float vx = ((float)dx + ox) - rx;
                float vy = ((float)dy + oy) - ry;
                float vz = ((float)dz + oz) - rz;
                float d2 = vx * vx + vy * vy + vz * vz;
                best = d2 < best ? d2 : best;
            }
        }
    }
    float d = sqrtf(best);
    return 1.0f - (d < 1.0f ? d : 1.0f);
}

__device__ float worley_fbm3(float x, float y, float z, int F, uint32_t s) {
    float f0 = (float)F, f1 = (float)(2 * F), f2 = (float)(4 * F);
    float w0 = worley3(x * f0, y * f0, z * f0, F, s);
    float w1 = worley3(x * f1, y * f1, z * f1, 2 * F, s + 1u);
    float w2 = worley3(x * f2, y * f2, z * f2, 4 * F, s + 2u);
    return (w0 * 0.625f + w1 * 0.25f) + w2 * 0.125f;
}

__device__ __forceinline__ float grad3(uint32_t h, float x, float y, float z) {
    h &= 15u;
    float u = h < 8u ? x : y;
    float v = h < 4u ? y : ((h == 12u || h == 14u) ? x : z);
    return ((h & 1u) ? -u : u) + ((h & 2u) ? -v : v);
}

__device__ float perlin3(float px, float py, float pz, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
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
    float a00 = lerpf(g000, g100, u), a10 = lerpf(g010, g110, u);
    float a01 = lerpf(g001, g101, u), a11 = lerpf(g011, g111, u);
    float b0 = lerpf(a00, a10, v), b1 = lerpf(a01, a11, v);
    return lerpf(b0, b1, w);
}

__device__ float perlin_fbm3(float x, float y, float z, int F, int octaves, uint32_t s) {
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

__device__ __forceinline__ float grad2(uint32_t h, float x, float y) {
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

__device__ float perlin2(float px, float py, int F, uint32_t s) {
    const uint32_t m = (uint32_t)F - 1u;
    float fx = floorf(px), fy = floorf(py);
    int ix = (int)fx, iy = (int)fy;
    float x = px - fx, y = py - fy;
    float u = fade(x), v = fade(y);
    uint32_t x0 = (uint32_t)ix & m, x1 = (uint32_t)(ix + 1) & m;
    uint32_t y0 = (uint32_t)iy & m, y1 = (uint32_t)(iy + 1) & m;
    float g00 = grad2(wang(x0, y0, s), x, y);
    float g10 = grad2(wang(x1, y0, s), x - 1.0f, y);
    float g01 = grad2(wang(x0, y1, s), x, y - 1.0f);
    float g11 = grad2(wang(x1, y1, s), x - 1.0f, y - 1.0f);
    return lerpf(lerpf(g00, g10, u), lerpf(g01, g11, u), v);
}

__device__ float perlin_fbm2(float x, float y, int F, int octaves, uint32_t s) {
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

__device__ __forceinline__ uint32_t q8(float v) { return (uint32_t)(int)floorf(clamp01(v) * 255.0f + 0.5f); }

__device__ __forceinline__ void put(const NoiseOut& o, size_t i, float r, float g, float b, float a) {
    r = clamp01(r);
    g = clamp01(g);
    b = clamp01(b);
    a = clamp01(a);
    if (o.u8) o.u8[i] = q8(r) | (q8(g) << 8) | (q8(b) << 16) | (q8(a) << 24);
    if (o.h16) {
        uint32_t lo = (uint32_t)__half_as_ushort(__float2half_rn(r)) |
                      ((uint32_t)__half_as_ushort(__float2half_rn(g)) << 16);
        uint32_t hi = (uint32_t)__half_as_ushort(__float2half_rn(b)) |
                      ((uint32_t)__half_as_ushort(__float2half_rn(a)) << 16);
        o.h16[i] = make_uint2(lo, hi);
    }
    if (o.b16) {
        uint32_t lo = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(r)) |
                      ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(g)) << 16);
        uint32_t hi = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) |
                      ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) << 16);
        o.b16[i] = make_uint2(lo, hi);
    }
}

// 128^3: R Perlin-Worley, G/B/A Worley fBm at base frequencies 4/8/16.
__global__ void __launch_bounds__(128) gen_base_kernel(uint32_t s, NoiseOut o) {
    const int N = MT_BASE_N;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)(N * N * N)) return;
    const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / (N * N));
    const float inv = 1.0f / (float)N;
    float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv, pz = ((float)z + 0.5f) * inv;
    float pf = perlin_fbm3(px, py, pz, 4, 4, salt(s, 1));
    float p01 = clamp01(pf * 0.5f + 0.5f);
    float g = worley_fbm3(px, py, pz, 4, salt(s, 2));
    float b = worley_fbm3(px, py, pz, 8, salt(s, 3));
    float a = worley_fbm3(px, py, pz, 16, salt(s, 4));
    float r = (p01 - (g - 1.0f)) / (1.0f - (g - 1.0f));
    put(o, i, r, g, b, a);
}

// 32^3: Worley at frequencies 8/16/32 in R/G/B.
__global__ void __launch_bounds__(128) gen_detail_kernel(uint32_t s, NoiseOut o) {
    const int N = MT_DETAIL_N;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)(N * N * N)) return;
    const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / (N * N));
    const float inv = 1.0f / (float)N;
    float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv, pz = ((float)z + 0.5f) * inv;
    float r = worley3(px * 8.0f, py * 8.0f, pz * 8.0f, 8, salt(s, 5));
    float g = worley3(px * 16.0f, py * 16.0f, pz * 16.0f, 16, salt(s, 6));
    float b = worley3(px * 32.0f, py * 32.0f, pz * 32.0f, 32, salt(s, 7));
    put(o, i, r, g, b, 1.0f);
}

// 128^2 curl of a tileable Perlin fBm potential (central differences).
__global__ void __launch_bounds__(128) gen_curl_kernel(uint32_t s, NoiseOut o) {
    const int N = MT_CURL_N;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)(N * N)) return;
    const int x = (int)(i % N), y = (int)(i / N);
    const float inv = 1.0f / (float)N;
    float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv;
    const uint32_t sp = salt(s, 8);
    float dy = perlin_fbm2(px, py + inv, 4, 3, sp) - perlin_fbm2(px, py - inv, 4, 3, sp);
    float dx = perlin_fbm2(px + inv, py, 4, 3, sp) - perlin_fbm2(px - inv, py, 4, 3, sp);
    float cx = dy * 4.0f;
    float cy = -(dx * 4.0f);
    float mag = sqrtf(cx * cx + cy * cy);
    put(o, i, cx * 0.5f + 0.5f, cy * 0.5f + 0.5f, mag, 1.0f);
}

// 512^2 weather: R coverage, G precipitation, B cloud type, A = 1.
__global__ void __launch_bounds__(128) gen_weather_kernel(uint32_t s, NoiseOut o) {
    const int N = MT_WEATHER_N;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)(N * N)) return;
    const int x = (int)(i % N), y = (int)(i / N);
    const float inv = 1.0f / (float)N;
    float px = ((float)x + 0.5f) * inv, py = ((float)y + 0.5f) * inv;
    float f = perlin_fbm2(px, py, 4, 6, salt(s, 9)) * 0.5f + 0.5f;
    float cov = clamp01(f * 1.2f - 0.2f);
    float precip = (float)(wang((uint32_t)x, (uint32_t)y, salt(s, 10)) >> 8) * (1.0f / 16777216.0f);
    uint32_t t = wang((uint32_t)(x >> 6), (uint32_t)(y >> 6), salt(s, 11)) % 3u;
    float type = t == 0u ? 0.0f : (t == 1u ? 0.5f : 1.0f);
    put(o, i, cov, precip, type, 1.0f);
}

// RGBA8 UNORM -> half / bfloat16 copies (c / 255, round to nearest even).
__global__ void u8_to_16_kernel(const uint32_t* __restrict__ src, size_t n, uint2* h16, uint2* b16) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t v = src[i];
    NoiseOut o{nullptr, h16, b16};
    put(o, i, (float)(v & 0xffu) / 255.0f, (float)((v >> 8) & 0xffu) / 255.0f, (float)((v >> 16) & 0xffu) / 255.0f,
        (float)(v >> 24) / 255.0f);
}

// Plane-quad layout of an RGBA8 volume (what the plain form's 3D samplers
// read): entry (x, y, z) holds the four texels of plane z a trilinear fetch
// at that cell interpolates, {(x0,y0), (x1,y0), (x0,y1), (x1,y1)} with
// x1 = (x + 1) mod N, y1 likewise (REPEAT), as one 16-byte word: a fetch reads
// two entries, at z0 and z1.
__global__ void quads3_kernel(const uint32_t* __restrict__ vol, int n, uint4* __restrict__ quads) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nn = (size_t)n * n;
    if (i >= nn * n) return;
    const unsigned m = (unsigned)n - 1u;
    const unsigned x = (unsigned)(i % n), y = (unsigned)((i / n) % n), z = (unsigned)(i / nn);
    const unsigned x1 = (x + 1u) & m, y1 = (y + 1u) & m;
    const uint32_t* p = vol + (size_t)z * nn;
    quads[i] = make_uint4(p[y * n + x], p[y * n + x1], p[y1 * n + x], p[y1 * n + x1]);
}

// The same for an RGBA8 image (bilinear cells): {(x0,y0), (x1,y0), (x0,y1), (x1,y1)}.
__global__ void cells2_kernel(const uint32_t* __restrict__ img, int n, uint4* __restrict__ cells) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * n) return;
    const unsigned m = (unsigned)n - 1u;
    const unsigned x = (unsigned)(i % n), y = (unsigned)(i / n);
    const unsigned x1 = (x + 1u) & m, y1 = (y + 1u) & m;
    cells[i] = make_uint4(img[y * n + x], img[y * n + x1], img[y1 * n + x], img[y1 * n + x1]);
}

// Plane-quad layout of a 16-bit volume (what the precision form's 3D samplers
// read): entry (x, y, z) holds the four texels of the z plane a trilinear
// fetch interpolates, as two 16-byte words {(x0,y0), (x1,y0)} and
// {(x0,y1), (x1,y1)}, x1 = (x + 1) mod N (REPEAT): a fetch reads the entries
// at z0 and z1, one 32-byte sector each.
__global__ void quads16_kernel(const uint2* __restrict__ vol, int n, uint4* __restrict__ quads) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nn = (size_t)n * n;
    if (i >= nn * n) return;
    const unsigned m = (unsigned)n - 1u;
    const unsigned x = (unsigned)(i % n), y = (unsigned)((i / n) % n), z = (unsigned)(i / nn);
    const unsigned x1 = (x + 1u) & m, y1 = (y + 1u) & m;
    const uint2* p = vol + (size_t)z * nn;
    const uint2 a = p[y * n + x], b = p[y * n + x1], c = p[y1 * n + x], d = p[y1 * n + x1];
    quads[2 * i] = make_uint4(a.x, a.y, b.x, b.y);
    quads[2 * i + 1] = make_uint4(c.x, c.y, d.x, d.y);
}

}  // namespace

cudaError_t launch_quads16(const uint2* vol, int n, uint4* quads, cudaStream_t s) {
    const size_t texels = (size_t)n * n * n;
    quads16_kernel<<<(unsigned)((texels + 255) / 256), 256, 0, s>>>(vol, n, quads);
    return cudaGetLastError();
}

cudaError_t launch_quads3(const uint32_t* vol, int n, uint4* quads, cudaStream_t s) {
    const size_t texels = (size_t)n * n * n;
    quads3_kernel<<<(unsigned)((texels + 255) / 256), 256, 0, s>>>(vol, n, quads);
    return cudaGetLastError();
}
cudaError_t launch_cells2(const uint32_t* img, int n, uint4* cells, cudaStream_t s) {
    const size_t texels = (size_t)n * n;
    cells2_kernel<<<(unsigned)((texels + 255) / 256), 256, 0, s>>>(img, n, cells);
    return cudaGetLastError();
}

cudaError_t launch_generate_base(uint32_t seed, NoiseOut o, cudaStream_t s) {
    const unsigned n = MT_BASE_N * MT_BASE_N * MT_BASE_N;
    gen_base_kernel<<<(n + 127) / 128, 128, 0, s>>>(seed, o);
    return cudaGetLastError();
}
cudaError_t launch_generate_detail(uint32_t seed, NoiseOut o, cudaStream_t s) {
    const unsigned n = MT_DETAIL_N * MT_DETAIL_N * MT_DETAIL_N;
    gen_detail_kernel<<<(n + 127) / 128, 128, 0, s>>>(seed, o);
    return cudaGetLastError();
}
cudaError_t launch_generate_curl(uint32_t seed, NoiseOut o, cudaStream_t s) {
    const unsigned n = MT_CURL_N * MT_CURL_N;
    gen_curl_kernel<<<(n + 127) / 128, 128, 0, s>>>(seed, o);
    return cudaGetLastError();
}
cudaError_t launch_generate_weather(uint32_t seed, NoiseOut o, cudaStream_t s) {
    const unsigned n = MT_WEATHER_N * MT_WEATHER_N;
    gen_weather_kernel<<<(n + 127) / 128, 128, 0, s>>>(seed, o);
    return cudaGetLastError();
}
cudaError_t launch_u8_to_16(const uint32_t* src, size_t n, uint2* h16, uint2* b16, cudaStream_t s) {
    u8_to_16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, n, h16, b16);
    return cudaGetLastError();
}

}  // namespace mt
