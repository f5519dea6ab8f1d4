// The two downstream full-screen passes that consume the compute stage's
// outputs:
//
//   godrays_kernel  <- shaders/postProcess_GodRays.frag:66-149 (100-sample
//                      radial blur of the god-ray mask, added to the HDR image)
//   tonemap_kernel  <- shaders/postProcess_ToneMap.frag:68-84 (Uncharted-2
//                      filmic curve + WangHash dither)
//
// Both shaders run one fragment per pixel (in_uv at the pixel centre) and
// store with imageStore at pixelPos = clamp(round(dim * in_uv)), which is the
// fragment's own pixel or the next one.  One thread here owns one OUTPUT
// pixel p and finds the fragment whose store lands there: along each axis the
// candidates are fragments p and p - 1, and where both map to p the later one
// in raster order (the larger index) wins.  Each output pixel is written by
// exactly one thread, so the result is defined (in the reference, colliding
// stores race) and out may alias in.
//
// Compiled with -fmad=false and IEEE division: the operation order follows
// the shaders' so the results equal the CPU restatement bit for bit except
// through powf (tone map).
#include <cuda_runtime.h>

#include "mt_kernels.h"
#include "mt_device.cuh"

namespace mt {

namespace {

// pixelPos of the fragment at index f along an axis of size n
// (postProcess_GodRays.frag:69, postProcess_ToneMap.frag:71).
MT_HD float frag_uv(int f, int n) { return ((float)f + 0.5f) / (float)n; }
MT_HD int frag_pixel(int f, int n) { return imin(imax(f2i(roundf((float)n * frag_uv(f, n))), 0), n - 1); }

// The fragment whose store lands on pixel p (the last one in raster order),
// or -1 when none does.
MT_HD int winner_fragment(int p, int n) {
    if (frag_pixel(p, n) == p) return p;
    if (p > 0 && frag_pixel(p - 1, n) == p) return p - 1;
    return -1;
}

// 1 / 16581375 as the shader's bitDec.w (postProcess_GodRays.frag:36-37).
__device__ __forceinline__ float bit_dec_w() { return 1.0f / 16581375.0f; }

// extract32fFromRGBA8f (postProcess_GodRays.frag:39-43) over the R32F mask:
// the texel (m, 0, 0, 0) decodes to m, the opaque-black border (0, 0, 0, 1)
// to bitDec.w.  LINEAR filter with exact FP32 weights, like every sampler
// here: the value channel and the border channel are interpolated x then y,
// then decoded as dot(texel, bitDec) in the shader's order.
MT_HD float mask_decode(const float* __restrict__ m, int W, int H, float sx, float sy) {
    const float u = sx * (float)W - 0.5f, v = sy * (float)H - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int i0 = f2i(fu), j0 = f2i(fv);
    if (i0 >= 0 && j0 >= 0 && i0 < W - 1 && j0 < H - 1) {
        // all four texels inside: the border channel interpolates zeros
        const float* r = m + (size_t)j0 * (size_t)W + (size_t)i0;
        const float x = lerp1(lerp1(__ldg(r), __ldg(r + 1), a), lerp1(__ldg(r + W), __ldg(r + W + 1), a), b);
        const float w = lerp1(lerp1(0.0f, 0.0f, a), lerp1(0.0f, 0.0f, a), b);
        return ((x * 1.0f + 0.0f) + 0.0f) + w * bit_dec_w();
    }
    const long long i1 = (long long)i0 + 1, j1 = (long long)j0 + 1;
    float val[4], brd[4];
    const long long ii[2] = {i0, i1}, jj[2] = {j0, j1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const long long i = ii[k & 1], j = jj[k >> 1];
        const bool out = i < 0 || j < 0 || i >= W || j >= H;
        val[k] = out ? 0.0f : __ldg(m + (size_t)j * (size_t)W + (size_t)i);
        brd[k] = out ? 1.0f : 0.0f;
    }
    const float x = lerp1(lerp1(val[0], val[1], a), lerp1(val[2], val[3], a), b);
    const float w = lerp1(lerp1(brd[0], brd[1], a), lerp1(brd[2], brd[3], a), b);
    // dot(x, bitDec) = x*1 + 0*bitDec.y + 0*bitDec.z + w*bitDec.w, left to right
    return ((x * 1.0f + 0.0f) + 0.0f) + w * bit_dec_w();
}

struct GodrayFrame {
    float blend;   // dot(cam_to_sun, camForward)
    float ssx, ssy;
    bool outside;  // sun outside [0,1]^2 in screen space (never, after the clamp)
};

// The per-frame quantities of postProcess_GodRays.frag:74-93.  Evaluated on
// the device by every thread (a few dozen flops): host compilers may contract
// these into fused multiply-adds.
MT_HD GodrayFrame godray_frame(const mt_camera_ubo& cam) {
    GodrayFrame g;
    const f3 sun{0.0f, 1.0f, 0.0f};
    const f3 cam_to_sun = normalize3(sun - ld3(cam.eye));
    const f3 fwd = -normalize3(f3{cam.view[2], cam.view[6], cam.view[10]});
    g.blend = dot3(cam_to_sun, fwd);
    // camera.proj * camera.view * vec4(sun, 1): the matrix product first,
    // column j = proj * view[j], then that times the vector.
    float M[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            M[j][i] = cam.proj[0 * 4 + i] * cam.view[j * 4 + 0] + cam.proj[1 * 4 + i] * cam.view[j * 4 + 1] +
                      cam.proj[2 * 4 + i] * cam.view[j * 4 + 2] + cam.proj[3 * 4 + i] * cam.view[j * 4 + 3];
    const float nx = M[0][0] * 0.0f + M[1][0] * 1.0f + M[2][0] * 0.0f + M[3][0] * 1.0f;
    const float ny = M[0][1] * 0.0f + M[1][1] * 1.0f + M[2][1] * 0.0f + M[3][1] * 1.0f;
    g.ssx = gclamp((nx + 1.0f) / 2.0f, 0.0f, 1.0f);
    g.ssy = gclamp((ny + 1.0f) / 2.0f, 0.0f, 1.0f);
    g.outside = g.ssx < 0.0f || g.ssx > 1.0f || g.ssy < 0.0f || g.ssy > 1.0f;
    return g;
}

__global__ void __launch_bounds__(256) godrays_kernel(GodrayArgs a) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= a.width || py >= a.height) return;
    const size_t idx = (size_t)py * (size_t)a.width + (size_t)px;
    float4 v = a.in[idx];
    const int fx = winner_fragment(px, a.width), fy = winner_fragment(py, a.height);
    const GodrayFrame g = godray_frame(a.camera);
    if (fx >= 0 && fy >= 0 && !(g.blend < 0.0f)) {
        float ux = frag_uv(fx, a.width), uy = frag_uv(fy, a.height);
        const float dx = ((ux - g.ssx) / 100.0f) * 1.0f, dy = ((uy - g.ssy) / 100.0f) * 1.0f;
        const float w = 1.0f * 0.001f;  // illuminationDecay * WEIGHT_FOR_SAMPLE, DECAY = 1
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
        if (!g.outside) {
#pragma unroll 4
            for (int i = 0; i < 100; ++i) {
                const float s = mask_decode(a.mask, a.width, a.height, ux, uy);
                ax += (a.light[0] * s) * w;
                ay += (a.light[1] * s) * w;
                az += (a.light[2] * s) * w;
                ux -= dx;
                uy -= dy;
            }
        }
        // the out-of-frustum branch discards what it accumulated (:126)
        v.x += (ax * 1.0f) * g.blend;
        v.y += (ay * 1.0f) * g.blend;
        v.z += (az * 1.0f) * g.blend;
        v.w += 1.0f * g.blend;
    }
    a.out[idx] = v;
}

// Uncharted2Tonemap (postProcess_ToneMap.frag:32-35) with A..F = .15 .5 .1 .2 .02 .3
MT_HD float uncharted2(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}

// WangHashNoise (postProcess_ToneMap.frag:52-66)
MT_HD float wang_hash_noise(uint32_t u, uint32_t v, uint32_t s) {
    uint32_t seed = (u * 1664525u + v) + s;
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return __uint2float_rn(seed) * (1.0f / 4294967296.0f);
}

// uint(time.y): truncation; negative and NaN give 0, beyond the range saturates.
MT_HD uint32_t f2u(float t) { return __float2uint_rz(t); }

// tonemap(x, 100) of postProcess_ToneMap.frag:37-46
MT_HD float tonemap1(float x) {
    const float color = uncharted2(2.5f * x);
    const float whitemap = 1.0f / uncharted2(100.0f);
    return powf(color * whitemap, 1.0f / 2.2f);
}

// Vulkan float -> UNORM8: clamp to [0, 1], scale, round to nearest even.
MT_HD uint32_t unorm8(float f) {
    const float c = (f > 0.0f) ? (f < 1.0f ? f : 1.0f) : 0.0f;  // NaN -> 0
    return (uint32_t)__float2uint_rn(c * 255.0f);
}

__global__ void __launch_bounds__(256) tonemap_kernel(TonemapArgs a) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= a.width || py >= a.height) return;
    const int fx = winner_fragment(px, a.width), fy = winner_fragment(py, a.height);
    if (fx < 0 || fy < 0) return;  // no fragment stores here: the pixel keeps its contents
    const f4v c = tex2_border(a.in, a.width, a.height, frag_uv(fx, a.width), frag_uv(fy, a.height));
    const float noise = wang_hash_noise((uint32_t)px, (uint32_t)py, f2u(a.time_y)) * 0.01f;
    const float r = tonemap1(c.x) + noise, g = tonemap1(c.y) + noise, b = tonemap1(c.z) + noise;
    const size_t idx = (size_t)py * (size_t)a.width + (size_t)px;
    if (a.format == MT_LDR_RGBA8) {
        static_cast<uint32_t*>(a.out)[idx] = unorm8(r) | (unorm8(g) << 8) | (unorm8(b) << 16) | (255u << 24);
    } else {
        static_cast<float4*>(a.out)[idx] = make_float4(r, g, b, 1.0f);
    }
}

}  // namespace

cudaError_t launch_godrays(const GodrayArgs& a, cudaStream_t s) {
    const dim3 block(32, 8), grid((a.width + 31) / 32, (a.height + 7) / 8);
    godrays_kernel<<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_tonemap(const TonemapArgs& a, cudaStream_t s) {
    const dim3 block(32, 8), grid((a.width + 31) / 32, (a.height + 7) / 8);
    tonemap_kernel<<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mt
