// Kernel argument blocks and launchers shared by the C ABI (mt_capi.cu) and
// the kernel translation units.  Arguments travel by value as
// __grid_constant__ parameters: the uniform blocks of the reference
// (CameraUBO, TimeUBO) plus mt_params fit easily in the parameter space.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/meteoros.h"

namespace mt {

// The uniform part of the reprojection / TXAA geometry of one frame: the
// camera basis, ray origin and jitter of cast_ray (cloudRayMarch.comp:194-226),
// the shifted origin and constant term of ray_sphere's quadratic (:229-273)
// for the inner shell, the reciprocals of the per-frame denominators (width,
// height, tan(fov/2)) and the previous camera's view matrix.  Computed on the
// host (mt_consts.cpp) with the same IEEE FP32 operations in the same order as
// the per-pixel code it stands for, so every pixel's result is unchanged.
struct ViewConsts {
    float eye[3], right[3], up[3], ref[3], ec[3], ro[3];
    float jx, jy, tanx, tany, C, Rin;
    float r_w[2], r_h[2], r_tanx[2], r_tany[2];  // {b, RN(1/b)}
    float ov[16];
};

void make_view_consts(ViewConsts* v, const mt_params& p, const mt_camera_ubo& cam, const mt_camera_ubo& cam_old,
                      const mt_time_ubo& tm, int W, int H, bool repro);

// A denominator b and its correctly rounded reciprocal y = RN(1/b) (see rdiv).
struct Rcp {
    float b, y;
};

// The per-frame constants of the raymarch (cloudRayMarch.comp:565-688 and the
// helpers it calls), computed on the host (mt_consts.cpp) with the shader's
// IEEE FP32 operations: kept in the kernel's parameter space, they take no
// registers in the march loop.
struct Frame {
    float R, Rin, Rout, thickness, inner_alt;  // earth radius, shell radii, Rout - Rin, Rin - R
    Rcp r_thick, r_period, r_weather;          // thickness, noise_period, weather_scale
    float eye[3];                              // ray origin: eye_sign * camera eye
    float ec[3];                               // earth centre (eye.x, -R, eye.z)
    float wind_t[3];                           // (wind_dir * wind_speed) * time[1]
    float skew[3];                             // skew_dir
    // FP64 shell intersections (precision form), per shell (0 inner, 1 outer):
    // the normalised ray origin (eye - ec) / radius and C = |o|^2 - 1.  Every
    // ray leaves the eye, so both are the same for the whole frame.
    double sh_o[2][3];
    double sh_c[2];
    // The same terms in FP32 for ray_sphere (the plain form)
    float sh32_o[2][3];
    float sh32_c[2];
    // The sun direction normalize(sun - eye) and the six cone-light kernel
    // vectors of cloudRayMarch.comp:598-624, the same for every ray
    float light_dir[3];
    float cone[6][3];
    // atmosphere_color's terms that depend on the sun only (cloudRayMarch.comp:401-467)
    float sky_sun_dir[3];  // normalize(sky_sun_pos - eye)
    float sky_sunE, sky_yDot;
    float sky_betaR[3], sky_betaM[3], sky_betaRM[3];
};

void make_march_frame(Frame* f, const mt_params& p, const mt_camera_ubo& cam, const mt_time_ubo& tm);

struct MarchArgs {
    mt_camera_ubo camera;
    mt_camera_ubo camera_old;
    mt_time_ubo time;
    mt_params params;
    // base (MT_BASE_N^3), detail (MT_DETAIL_N^3), curl (MT_CURL_N^2), weather
    // (MT_WEATHER_N^2, slot params.weather_slot) in params.storage: for RGBA8
    // plane quads of the volumes and bilinear cells of the images (uint4;
    // launch_quads3 / launch_cells2), for the 16-bit storages plane quads of
    // the volumes (2 x uint4; launch_quads16) and four 16-bit values per texel
    // (uint2) of the images
    const void* vol[4];
    const float4* prev;
    float4* cur;
    float* mask;
    unsigned long long* stats;  // 4 counters or NULL
    int32_t width, height;
    int32_t groups_x, groups_y;  // 4x4 blocks covered by the reference's raymarch dispatch
    uint32_t flags;
    int32_t lanes;               // lanes marching one ray together: 1, 4, 8 or 16
    int32_t block;               // march_kernel CTA size: 32, 128 or 256 threads
    // Dispatch order of the ray rows (rows of 4x4 blocks, or of pixels for a
    // full frame): 1 = bottom to top (default), 0 = top to bottom.  Bottom to
    // top runs the rows that do not march (below the fade elevation, 10-50x
    // cheaper) first, which lets the work beside the raymarch start early,
    // then the marching rows from the horizon up.
    int32_t bottom_up;
    const float4* history;       // mt_render_frame only: previous resolved frame
    float4* out;                 // mt_render_frame only: resolved frame
    int32_t fused_resolve;       // mt_render_frame: 1 = reprojection fused with TXAA
    // mt_render / mt_render_frame only (NULL elsewhere): per marched pixel,
    // the ray's executed primary samples, in-cloud samples, control-flow
    // signature and 0 (mt_set_sample_trace)
    uint4* trace;
    ViewConsts vc_repro;         // reprojection geometry (reprojection.comp's jitter)
    ViewConsts vc_txaa;          // TXAA geometry (cloudRayMarch.comp's jitter)
    // The raymarch's per-step jitter (cloudRayMarch.comp:629-633) for each of
    // the 16 values of its index: jx = halton / 1 / 75, jy likewise, and
    // (jx + jy) * 1.18, evaluated on the host in that order (make_march_jitter).
    float jitter[16][3];
    Frame frame;
};

void make_march_jitter(float out[16][3], const mt_time_ubo& tm);

// The k-th of n ray rows in dispatch order.
__host__ __device__ inline int march_row(int k, int n, bool bottom_up) { return bottom_up ? n - 1 - k : k; }

struct TxaaArgs {
    mt_camera_ubo camera;
    mt_camera_ubo camera_old;
    mt_time_ubo time;
    mt_params params;
    const float4* current;
    const float4* history;
    float4* out;
    int32_t width, height;
    ViewConsts vc;
};

// One tile of a batched render: a TW x TH rectangle of one view's ray grid.
struct BatchTile {
    int32_t view;      // index into BatchArgs::views
    int32_t rx0, ry0;  // tile origin in the view's ray grid
    int32_t nrx, nry;  // the view's ray grid: pixels (full) or 4x4 blocks (checkerboard)
};

// A batch of views marched by one persistent launch: every CTA takes tiles
// from `counter` (zeroed before the launch) until all are done.
struct BatchArgs {
    const MarchArgs* views;  // device array, one per view
    const BatchTile* tiles;  // device array, in the order they are handed out
    unsigned* counter;
    unsigned long long* stats;  // or NULL
    int32_t n_tiles;
    int32_t tile_w, tile_h;     // tile shape in rays
};

// Outputs of one generator launch (any pointer may be NULL).
// postProcess_GodRays.frag over an HDR image (mt_godrays)
struct GodrayArgs {
    mt_camera_ubo camera;
    float light[4];  // SunAndSky.lightColor
    const float* mask;
    const float4* in;
    float4* out;  // may equal in
    int32_t width, height;
};

// postProcess_ToneMap.frag (mt_tonemap)
struct TonemapArgs {
    const float4* in;
    void* out;  // uint32 RGBA8 words or float4, by format
    float time_y;
    int32_t format;  // mt_ldr_format
    int32_t width, height;
};

// One TGA file of a volume's slice stack, inside the concatenated upload.
struct TgaSlice {
    long long offset;
    long long size;
};

struct NoiseOut {
    uint32_t* u8;   // RGBA8 words
    uint2* h16;     // 4 x IEEE half per texel
    uint2* b16;     // 4 x bfloat16 per texel
};

// Optional event pairs bracketing each launch (NULL: no timing).
struct LaunchEvents {
    cudaEvent_t reproject[2];
    cudaEvent_t march[2];
    cudaEvent_t resolve[2];
    bool on;
};

// A second stream for the reprojection of a checkerboard frame: it writes the
// pixels the raymarch does not, so the two kernels may run at once (the
// reprojection's blocks fill the SMs the raymarch's uneven rays leave idle).
// fork is recorded on the caller's stream and waited on by aux; join the
// other way.
struct ForkJoin {
    cudaStream_t aux;
    cudaEvent_t fork, join;
};

cudaError_t launch_render(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev, const ForkJoin* fj);
cudaError_t launch_reproject(const MarchArgs& a, cudaStream_t s);
cudaError_t launch_march_u8(const MarchArgs& a, cudaStream_t s, long long rays);
// Persistent batched march: `blocks` CTAs of 128 threads, `lanes` per ray.
cudaError_t launch_batch_u8(const BatchArgs& b, int lanes, int blocks, cudaStream_t s);
cudaError_t launch_batch_f16(const BatchArgs& b, int lanes, int blocks, cudaStream_t s);
cudaError_t launch_batch_bf16(const BatchArgs& b, int lanes, int blocks, cudaStream_t s);
// CTAs of the persistent batched march that fit on the device at once.
int batch_blocks_u8(int device, int lanes);
int batch_blocks_f16(int device, int lanes);
int batch_blocks_bf16(int device, int lanes);
cudaError_t launch_march_f16(const MarchArgs& a, cudaStream_t s, long long rays);
cudaError_t launch_march_bf16(const MarchArgs& a, cudaStream_t s, long long rays);
cudaError_t launch_txaa(const TxaaArgs& a, cudaStream_t s, const cudaEvent_t* ev);
cudaError_t launch_godrays(const GodrayArgs& a, cudaStream_t s);
cudaError_t launch_tga_decode(const unsigned char* blob, const TgaSlice* slices, int n_slices, size_t max_size,
                              uint32_t* vol, int W, int H, cudaStream_t s);
cudaError_t launch_tonemap(const TonemapArgs& a, cudaStream_t s);
// The raymarch, then reprojection fused with TXAA (a.history -> a.out).
cudaError_t launch_frame(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev, const ForkJoin* fj);
cudaError_t launch_selftest_division(const float* a, const float* b, float* out_rdiv, float* out_ieee, int n,
                                     cudaStream_t s);
cudaError_t launch_generate_base(uint32_t seed, NoiseOut o, cudaStream_t s);
cudaError_t launch_generate_detail(uint32_t seed, NoiseOut o, cudaStream_t s);
cudaError_t launch_generate_curl(uint32_t seed, NoiseOut o, cudaStream_t s);
cudaError_t launch_generate_weather(uint32_t seed, NoiseOut o, cudaStream_t s);
cudaError_t launch_u8_to_16(const uint32_t* src, size_t n, uint2* h16, uint2* b16, cudaStream_t s);
// The layouts the plain form's samplers read: plane quads of an RGBA8 volume
// (n^3 x uint4) and bilinear cells of an RGBA8 image (n^2 x uint4).
cudaError_t launch_quads3(const uint32_t* vol, int n, uint4* quads, cudaStream_t s);
cudaError_t launch_cells2(const uint32_t* img, int n, uint4* cells, cudaStream_t s);
// Plane-quad copies of a 16-bit volume (n^3 entries of 2 x uint4), the layout
// the precision form's 3D samplers read.
cudaError_t launch_quads16(const uint2* vol, int n, uint4* quads, cudaStream_t s);

// Number of 4x4 blocks along one axis covered by the reference's raymarch
// dispatch: ceil(floor(dim/4) / 32) groups of 32 (Renderer.cpp:713-716).
inline int march_groups(int dim) { return 32 * ((dim / 4 + 31) / 32); }

}  // namespace mt
