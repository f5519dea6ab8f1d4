// TEST INFRASTRUCTURE — dispatch driver for the reference's own shader source
// compiled as C++ (see oracle/ref_build.py).  Each shader is included into a
// namespace of the GLSL environment (oracle/glsl_shim.hpp); the functions
// below play the role of the reference's Vulkan dispatches
// (Renderer.cpp:683-716 for the compute shaders, one fragment per pixel for
// the full-screen passes, Renderer.cpp:834-846).
#include <cstdint>
#include <vector>

#include "../include/meteoros.h"
#include "glsl_shim.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace glsl {
namespace sh_march {
thread_local uvec3 gl_GlobalInvocationID;
#include "cloudRayMarch.inc"
}  // namespace sh_march
namespace sh_repro {
thread_local uvec3 gl_GlobalInvocationID;
#include "reprojection.inc"
}  // namespace sh_repro
namespace sh_txaa {
#include "txaa.inc"
}  // namespace sh_txaa
namespace sh_tonemap {
#include "tonemap.inc"
}  // namespace sh_tonemap
namespace sh_godrays {
#include "godrays.inc"
}  // namespace sh_godrays
}  // namespace glsl

namespace {

template <class U> void load_camera(U& dst, const mt_camera_ubo* u) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            dst.view[c][r] = u->view[4 * c + r];
            dst.proj[c][r] = u->proj[4 * c + r];
        }
    dst.eye = glsl::vec4(u->eye[0], u->eye[1], u->eye[2], u->eye[3]);
    dst.tanFovBy2 = glsl::vec2(u->tan_fov_by_2[0], u->tan_fov_by_2[1]);
}

glsl::vec4 v4(const float* f) { return glsl::vec4(f[0], f[1], f[2], f[3]); }

void set_tex(glsl::Texture& t, const void* data, int fmt, int w, int h, int d, glsl::Address mode) {
    t.u8 = fmt == 0 ? (const uint8_t*)data : nullptr;
    t.f32 = fmt == 0 ? nullptr : (const float*)data;
    t.w = w;
    t.h = h;
    t.d = d;
    t.mode = mode;
}

}  // namespace

extern "C" {

// cloudRayMarch.comp dispatch: ceil(floor(W/4)/32) x ceil(floor(H/4)/32)
// groups of 32x32 (Renderer.cpp:713-716).  Writes the marched pixels of
// cur_rgba and godray_rgba (the RGBA value the shader stores) and leaves the
// others untouched.  fmt: 0 uint8 texels, 1 float texel values.
__attribute__((visibility("default"))) int ref_cloud_raymarch(const void* base, const void* detail, const void* curl,
                                                              const void* weather, int fmt, const mt_camera_ubo* cam,
                                                              const mt_time_ubo* tm, float* cur_rgba,
                                                              float* godray_rgba, int width, int height,
                                                              int nthreads) {
    namespace S = glsl::sh_march;
    using glsl::Address;
    S::currentFrameResultImage = glsl::image2D{cur_rgba, cur_rgba, width, height};
    S::previousFrameResultImage = glsl::image2D{nullptr, nullptr, width, height};
    S::godRaysCreationDataImage = glsl::image2D{godray_rgba, godray_rgba, width, height};
    set_tex(S::cloudBaseShapeSampler, base, fmt, MT_BASE_N, MT_BASE_N, MT_BASE_N, Address::Repeat);
    set_tex(S::cloudDetailsHighFreqSampler, detail, fmt, MT_DETAIL_N, MT_DETAIL_N, MT_DETAIL_N, Address::Repeat);
    set_tex(S::curlNoiseSampler, curl, fmt, MT_CURL_N, MT_CURL_N, 1, Address::Repeat);
    set_tex(S::weatherMapSampler, weather ? weather : curl, fmt, weather ? MT_WEATHER_N : MT_CURL_N,
            weather ? MT_WEATHER_N : MT_CURL_N, 1, Address::Repeat);
    load_camera(S::camera, cam);
    S::haltonSeq1 = v4(tm->halton_seq1);
    S::haltonSeq2 = v4(tm->halton_seq2);
    S::haltonSeq3 = v4(tm->halton_seq3);
    S::haltonSeq4 = v4(tm->halton_seq4);
    S::time = glsl::vec2(tm->time[0], tm->time[1]);
    S::frameCountMod16 = tm->frame_count_mod16;
    const long long groups_x = 32LL * ((width / 4 + 31) / 32), groups_y = 32LL * ((height / 4 + 31) / 32);
    const long long total = groups_x * groups_y;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < total; ++i) {
        S::gl_GlobalInvocationID = glsl::uvec3((glsl::uint)(i % groups_x), (glsl::uint)(i / groups_x), 0u);
        S::shader_main();
    }
    return 0;
}

// reprojection.comp dispatch: ceil(W/32) x ceil(H/32) groups of 32x32
// (Renderer.cpp:683-698).  Reads prev_rgba, writes every pixel of cur_rgba.
__attribute__((visibility("default"))) int ref_reprojection(const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                                                            const mt_time_ubo* tm, const float* prev_rgba,
                                                            float* cur_rgba, int width, int height, int nthreads) {
    namespace S = glsl::sh_repro;
    S::currentFrameResultImage = glsl::image2D{nullptr, cur_rgba, width, height};
    S::previousFrameResultImage = glsl::image2D{prev_rgba, nullptr, width, height};
    load_camera(S::camera, cam);
    load_camera(S::cameraOld, cam_old);
    S::haltonSeq1 = v4(tm->halton_seq1);
    S::haltonSeq2 = v4(tm->halton_seq2);
    S::haltonSeq3 = v4(tm->halton_seq3);
    S::haltonSeq4 = v4(tm->halton_seq4);
    S::time = glsl::vec2(tm->time[0], tm->time[1]);
    S::frameCountMod16 = tm->frame_count_mod16;
    const long long gx = 32LL * ((width + 31) / 32), gy = 32LL * ((height + 31) / 32);
    const long long total = gx * gy;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < total; ++i) {
        S::gl_GlobalInvocationID = glsl::uvec3((glsl::uint)(i % gx), (glsl::uint)(i / gx), 0u);
        S::shader_main();
    }
    return 0;
}

// postProcess_TXAA.frag, one fragment per pixel with in_uv at the pixel
// centre.  The shader's neighbourhood reads come from `current`; its
// imageStore goes to a scratch image (the reference reads and writes the same
// image, a race); out_rgba receives outColor.
__attribute__((visibility("default"))) int ref_txaa(const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                                                    const mt_time_ubo* tm, const float* history_rgba,
                                                    const float* current_rgba, float* out_rgba, int width,
                                                    int height, int nthreads) {
    namespace S = glsl::sh_txaa;
    std::vector<float> scratch((size_t)width * (size_t)height * 4);
    set_tex(S::prevFrameImage, history_rgba, 1, width, height, 1, glsl::Address::ClampToBorder);
    S::currentFrameResultImage = glsl::image2D{current_rgba, scratch.data(), width, height};
    load_camera(S::camera, cam);
    load_camera(S::cameraOld, cam_old);
    S::haltonSeq1 = v4(tm->halton_seq1);
    S::haltonSeq2 = v4(tm->halton_seq2);
    S::haltonSeq3 = v4(tm->halton_seq3);
    S::haltonSeq4 = v4(tm->halton_seq4);
    S::time = glsl::vec2(tm->time[0], tm->time[1]);
    S::frameCountMod16 = tm->frame_count_mod16;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            S::in_uv = glsl::vec2(((float)x + 0.5f) / (float)width, ((float)y + 0.5f) / (float)height);
            S::shader_main();
            float* o = out_rgba + 4 * ((size_t)y * (size_t)width + (size_t)x);
            o[0] = S::outColor.x;
            o[1] = S::outColor.y;
            o[2] = S::outColor.z;
            o[3] = S::outColor.w;
        }
    return 0;
}

// postProcess_GodRays.frag, one fragment per pixel in raster order with in_uv
// at the pixel centre.  The mask is the sampler's image as texels
// (mask, 0, 0, 0), which the shader's decode turns back into the mask value;
// imageLoad reads in_rgba, imageStore writes out_rgba (first filled with
// in_rgba), so where two fragments store to one pixel the later one wins.
__attribute__((visibility("default"))) int ref_godrays(const mt_camera_ubo* cam, const float* light_color,
                                                       const float* mask, const float* in_rgba, float* out_rgba,
                                                       int width, int height) {
    namespace S = glsl::sh_godrays;
    const size_t n = (size_t)width * (size_t)height;
    std::vector<float> texels(4 * n, 0.0f);
    for (size_t i = 0; i < n; ++i) texels[4 * i] = mask[i];
    for (size_t i = 0; i < 4 * n; ++i) out_rgba[i] = in_rgba[i];
    set_tex(S::godRayCreationDataSampler, texels.data(), 1, width, height, 1, glsl::Address::ClampToBorder);
    S::currentFrameResultImage = glsl::image2D{in_rgba, out_rgba, width, height};
    load_camera(S::camera, cam);
    S::sunAndSky.lightColor = v4(light_color);
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            S::in_uv = glsl::vec2(((float)x + 0.5f) / (float)width, ((float)y + 0.5f) / (float)height);
            S::shader_main();
        }
    return 0;
}

// postProcess_ToneMap.frag, one fragment per pixel in raster order.  The
// shader's rgba8 image is kept as floats here (the values it stores);
// out_rgba is left as the caller filled it where no fragment stores.
__attribute__((visibility("default"))) int ref_tonemap(const mt_time_ubo* tm, const float* in_rgba, float* out_rgba,
                                                       int width, int height) {
    namespace S = glsl::sh_tonemap;
    set_tex(S::inputImageSampler, in_rgba, 1, width, height, 1, glsl::Address::ClampToBorder);
    S::currentFrameResultImage = glsl::image2D{nullptr, out_rgba, width, height};
    S::haltonSeq1 = v4(tm->halton_seq1);
    S::haltonSeq2 = v4(tm->halton_seq2);
    S::haltonSeq3 = v4(tm->halton_seq3);
    S::haltonSeq4 = v4(tm->halton_seq4);
    S::time = glsl::vec2(tm->time[0], tm->time[1]);
    S::frameCountMod16 = tm->frame_count_mod16;
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            S::in_uv = glsl::vec2(((float)x + 0.5f) / (float)width, ((float)y + 0.5f) / (float)height);
            S::shader_main();
        }
    return 0;
}

// The raymarch shader's helper functions, called one at a time:
// getDensityHeightGradientForPoint (cloudRayMarch.comp:475-487; the shader
// never calls it) and remap / remapClamped / remapClampedBeforeAndAfter
// (:153-169).
__attribute__((visibility("default"))) float ref_height_gradient(float h, float type) {
    return glsl::sh_march::getDensityHeightGradientForPoint(h, type);
}
__attribute__((visibility("default"))) float ref_remap(float v, float a, float b, float c, float d) {
    return glsl::sh_march::remap(v, a, b, c, d);
}
__attribute__((visibility("default"))) float ref_remap_clamped(float v, float a, float b, float c, float d) {
    return glsl::sh_march::remapClamped(v, a, b, c, d);
}
__attribute__((visibility("default"))) float ref_remap_clamped_ba(float v, float a, float b, float c, float d) {
    return glsl::sh_march::remapClampedBeforeAndAfter(v, a, b, c, d);
}

// WangHashNoise of postProcess_ToneMap.frag:52-66, as the shader computes it.
__attribute__((visibility("default"))) float ref_wang_hash_noise(unsigned u, unsigned v, unsigned s) {
    return glsl::sh_tonemap::WangHashNoise(u, v, s);
}

}  // extern "C"
