/*
 * meteoros.h — C ABI of the GB300-native Meteoros compute stage.
 *
 * This library replaces the reference renderer's per-frame compute command
 * buffer (Renderer.cpp:653-722): the reprojection dispatch
 * (shaders/reprojection.comp) and the cloud raymarch dispatch
 * (shaders/cloudRayMarch.comp), plus the TXAA resolve
 * (shaders/postProcess_TXAA.frag) and the noise volumes that the reference
 * loads from disk (Sky.cpp:25-58).  All entry points are plain C: pointers,
 * sizes and status codes.  No C++ exception crosses this boundary.
 *
 * Threading: one mt_ctx per host thread.  Calls on one context are ordered on
 * the CUDA stream passed in (NULL = the legacy default stream).  Distinct
 * contexts may be used concurrently from different threads.
 *
 * Image layout: every image is row-major, row 0 first, with no padding.  An
 * RGBA image is width*height*4 floats (RGBA32F); a mask is width*height floats
 * (R32F).  Pixel (x, y) is GLSL imageLoad/imageStore coordinate ivec2(x, y).
 */
#ifndef METEOROS_H
#define METEOROS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MT_API __attribute__((visibility("default")))
#else
#define MT_API
#endif

#define MT_ABI_VERSION 1

/* Noise volume sizes.  Fixed by the reference's asset set:
 * Sky.cpp:31 (128^3 RGBA8 base shape), Sky.cpp:40 (32^3 RGBA8 detail),
 * Sky.cpp:47 (128^2 RGBA8 curl), Sky.cpp:54 (512^2 RGBA8 weather map). */
#define MT_BASE_N 128
#define MT_DETAIL_N 32
#define MT_CURL_N 128
#define MT_WEATHER_N 512
#define MT_MAX_WEATHER_SLOTS 256
#define MT_MAX_DIM 16384

/* Status codes.  The reference throws std::runtime_error on a VkResult other
 * than VK_SUCCESS (Renderer.cpp:139-141, 430-432); here each call returns one
 * of these, and mt_last_error() gives the message. */
typedef enum mt_status {
    MT_OK = 0,
    MT_ERR_INVALID_ARG = 1,  /* null pointer, bad size, bad slot, bad flags */
    MT_ERR_NO_VOLUMES = 2,   /* render before any volume upload/generation */
    MT_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    MT_ERR_OUT_OF_MEMORY = 4,
    MT_ERR_UNSUPPORTED = 5,  /* e.g. no sm_103a device */
    MT_ERR_BUDGET = 6,       /* serving: request does not fit the HBM budget */
    MT_ERR_TIMEOUT = 7       /* a bounded wait gave up */
} mt_status;

/* CameraUBO: camera.h:12-18 and cloudRayMarch.comp:15-21 (std140, 152 bytes,
 * padded here to 160).  Matrices are column-major: view[c*4 + r] is GLSL
 * view[c][r], as glm stores them. */
typedef struct mt_camera_ubo {
    float view[16];
    float proj[16];
    float eye[4];
    float tan_fov_by_2[2]; /* .x = aspect * tan(fovy/2), .y = tan(fovy/2) */
    float _pad[2];
} mt_camera_ubo;

/* TimeUBO: Scene.h:12-21 and cloudRayMarch.comp:23-31 (std140, 80 bytes). */
typedef struct mt_time_ubo {
    float halton_seq1[4];
    float halton_seq2[4];
    float halton_seq3[4];
    float halton_seq4[4];
    float time[2]; /* .x = delta time, .y = total time (seconds) */
    int32_t frame_count_mod16;
    int32_t _pad;
} mt_time_ubo;

/* Storage precision of the noise volumes read by the raymarch. */
typedef enum mt_storage {
    MT_STORAGE_U8 = 0,   /* RGBA8 UNORM, as the reference's textures */
    MT_STORAGE_F16 = 1,  /* precision form: IEEE half volumes, half2 density math */
    MT_STORAGE_BF16 = 2  /* precision form: bfloat16 volumes, half2 density math */
} mt_storage;

/* Render flags. */
#define MT_RENDER_CHECKERBOARD 0u /* 1 pixel per 4x4 block marched, the rest reprojected (the reference) */
#define MT_RENDER_FULL 1u         /* every pixel marched, no reprojection (config 0) */
#define MT_RENDER_COUNT 2u        /* accumulate executed-sample counters (mt_get_stats) */

/* Parameters the reference compiles in as #defines and literals.
 * mt_params_reference() fills the reference's values; mt_params_config()
 * fills the physically parameterised values of the benchmark configurations.
 * Both run the same kernels. */
typedef struct mt_params {
    /* Atmosphere shells: cloudRayMarch.comp:75-78 */
    float earth_radius;        /* EARTH_RADIUS */
    float shell_inner_radius;  /* ATMOSPHERE_RADIUS_INNER (from the Earth's centre) */
    float shell_outer_radius;  /* ATMOSPHERE_RADIUS_OUTER */
    float noise_period;        /* samplePoint /= 8.0 (cloudRayMarch.comp:635) */
    /* Primary march: cloudRayMarch.comp:572, 680-684 */
    int32_t steps_min;         /* floor(mix(steps_min, steps_max, 1 - dir.y)); equal = fixed */
    int32_t steps_max;
    float accum_limit;         /* stop once accumulated density >= accum_limit (1.0 in the reference) */
    /* Coverage / weather map: cloudRayMarch.comp:515-537 */
    int32_t coverage_mode;     /* 0: constant `coverage`; 1: weather map R with threshold 1 - R */
    float coverage;            /* cloud_coverage = 0.6 */
    int32_t height_gradient;   /* 1: multiply by getDensityHeightGradientForPoint(h, weather B) */
    float weather_scale;       /* weather uv = (pos - earthCentre).xz / weather_scale */
    int32_t weather_slot;      /* which uploaded/generated weather map to read */
    /* Wind: cloudRayMarch.comp:88-91, 489-497 */
    float wind_dir[3];         /* WIND_DIRECTION + vec3(0, 0.1, 0) */
    float wind_speed;          /* CLOUD_SPEED (noise units per second) */
    float skew_dir[3];         /* WIND_DIRECTION for the top skew */
    float cloud_top_offset;    /* CLOUD_TOP_OFFSET (times 0.009) */
    /* Sun: cloudRayMarch.comp:93-99 */
    float sun_light_pos[3];    /* SUN_LOCATION: lights the clouds */
    float sky_sun_pos[3];      /* BACKGROUND_SKY_SUN_LOCATION: Preetham sky */
    float eye_sign;            /* ray origin = eye_sign * camera.eye (-1 in the reference, :707) */
    /* TXAA feedback: postProcess_TXAA.frag:52-53 */
    float feedback_min;
    float feedback_max;
    /* Checkerboard slot order: cloudRayMarch.comp:695-701 (slot i -> (i/4, i%4)) */
    int32_t slot_x[16];
    int32_t slot_y[16];
    /* Precision form */
    int32_t storage;           /* mt_storage */
    int32_t fp64_shells;       /* 1: shell intersection in FP64 (precision form) */
    int32_t _reserved[7];
} mt_params;

/* Counters of the last render call made with MT_RENDER_COUNT. */
typedef struct mt_stats {
    uint64_t primary_samples; /* executed iterations of cloudRayMarch.comp:627-686 */
    uint64_t light_samples;   /* executed cone-light base-shape fetches (:654-668) */
    uint64_t marched_rays;    /* rays that reached the march loop */
    uint64_t pixels;          /* pixels written (marched + reprojected + horizon) */
} mt_stats;

/* Device durations of the most recent launches made while timing was on
 * (mt_set_timing).  A kernel that did not run since timing was switched on
 * reads 0. */
typedef struct mt_kernel_times {
    float reproject_ms; /* the reprojection (mt_render_frame: with the TXAA history taps, one kernel) */
    float march_ms;     /* the raymarch */
    float txaa_ms;      /* mt_txaa */
    float resolve_ms;   /* mt_render_frame's TXAA resolve (fused_resolve: reprojection fused with TXAA) */
} mt_kernel_times;

/* Launch-shape choices of the kernels.  Results do not depend on them (the
 * tests hold every choice to the same output); only speed does. */
typedef struct mt_tuning {
    int32_t march_lanes;  /* lanes that march one ray together: 1, 4, 8 or 16; 0 = chosen from the ray count */
    int32_t fused_resolve; /* mt_render_frame: 0 = the raymarch, the TXAA history taps and the
                            * reprojection in one kernel beside it, then the TXAA resolve (default);
                            * 1 = the raymarch, then the reprojection fused with the TXAA resolve */
    int32_t batch_tile_w;  /* mt_render_batch: tile of rays a CTA takes at a time (default 16 x 8) */
    int32_t batch_tile_h;
    int32_t batch_lanes;   /* mt_render_batch: lanes per ray, 1, 4, 8 or 16 (default 1) */
    int32_t batch_direct;  /* mt_render_batch: 0 = one CUDA graph per batch (default); 1 = the same
                            * copies and launches issued directly on the stream (no capture
                            * cost per batch: the serving loop's small batches) */
    int32_t reproject_serial; /* mt_render / mt_render_frame, checkerboard: 0 = the reprojection
                               * runs on a second stream beside the raymarch (default; the call
                               * still completes in `stream` order); 1 = before it on `stream` */
    int32_t march_block;   /* mt_render: raymarch CTA size, 32, 128 or 256 threads; 0 = default (256) */
    int32_t march_order;   /* mt_render: 0 = ray rows dispatched bottom to top (default: the rows
                            * below the horizon, which do not march, first, then the marching rows
                            * from the horizon up); 1 = top to bottom */
    int32_t batch_order;   /* mt_render_batch: the order each view's tile rows are handed out in,
                            * 0 = bottom to top (default), 1 = top to bottom */
    int32_t _reserved[2];
} mt_tuning;

/* One view of a batched render (config 3). */
typedef struct mt_view {
    mt_camera_ubo camera;
    mt_camera_ubo camera_old;
    mt_time_ubo time;
    mt_params params;
    const float* prev_rgba;  /* device, may be NULL with MT_RENDER_FULL */
    float* cur_rgba;         /* device */
    float* godray_mask;      /* device, may be NULL */
    int32_t width;
    int32_t height;
    uint32_t flags;
    int32_t _pad;
} mt_view;

typedef struct mt_ctx mt_ctx;

/* ---- library / context -------------------------------------------------- */

MT_API int mt_abi_version(void);

/* Replaces VulkanInstance/VulkanDevice creation (main.cpp:135-156) for the
 * compute path: binds CUDA device `device` and checks it is sm_103. */
MT_API mt_status mt_create(mt_ctx** out, int device);
MT_API void mt_destroy(mt_ctx* ctx);
/* Message of the last failed call on ctx (or of the last failed mt_create when
 * ctx is NULL).  Never NULL. */
MT_API const char* mt_last_error(const mt_ctx* ctx);

/* ---- parameters and uniform producers (host only, no GPU work) ---------- */

MT_API void mt_params_reference(mt_params* out);
MT_API void mt_params_config(mt_params* out);
/* Scene::InitializeTime (Scene.cpp:86-119): Halton base 3, i = 1..16;
 * frame count 0; time zero. */
MT_API void mt_time_init(mt_time_ubo* out);
/* Scene::UpdateTime (Scene.cpp:65-85): time.x = dt, time.y += dt,
 * frameCount = (frameCount + 1) % 16. */
MT_API void mt_time_advance(mt_time_ubo* t, float dt);
/* Camera::UpdateBuffer (camera.cpp:31-42): view = lookAt(eye, ref, up),
 * proj = perspective with proj[1][1] negated, eye, tan(fovy/2). */
MT_API void mt_camera_look_at(mt_camera_ubo* out, const float eye[3], const float ref[3],
                              float fovy_deg, float aspect, float near_clip, float far_clip);
/* Scene::HaltonSequenceAt (Scene.cpp:125-138). */
MT_API float mt_halton(int index, int base);

/* ---- noise volumes (Sky::CreateCloudResources, Sky.cpp:25-58) ----------- */

/* Upload RGBA8 volumes from host memory, in create3DTextureFromMany2DTextures
 * layout (ImageLoadingUtility.cpp:75-139: x fastest, then y, then slice z).
 * Any pointer may be NULL to keep the current volume.  `weather` goes to slot 0. */
MT_API mt_status mt_upload_volumes(mt_ctx* ctx, const uint8_t* base_rgba8, const uint8_t* detail_rgba8,
                                   const uint8_t* curl_rgba8, const uint8_t* weather_rgba8);
MT_API mt_status mt_upload_weather(mt_ctx* ctx, int slot, const uint8_t* weather_rgba8);

/* A noise volume from its stack of TGA slices, decoded on the device, in place
 * of Sky::CreateCloudResources' stb_image loads (Sky.cpp:25-45,
 * ImageLoadingUtility.cpp:75-139).  files[z] / sizes[z]: the bytes of slice z
 * (the reference's "<name>(z+1).tga"), in host memory; MT_BASE_N slices of
 * MT_BASE_N^2 for MT_VOLUME_BASE, MT_DETAIL_N of MT_DETAIL_N^2 for
 * MT_VOLUME_DETAIL.  Decoded as the reference's loader does: image types 2
 * (raw) and 10 (run-length) with colour-map type 0, 24 or 32 bits per pixel
 * (24-bit pixels get alpha 255), rows flipped to top-first unless the origin
 * is top-left, bytes past the end of a file read as 0.  Other files are
 * rejected with MT_ERR_INVALID_ARG, as is a slice above
 * MT_TGA_MAX_SLICE_BYTES.  Returns when the volume (and its FP16/BF16
 * copies) is ready. */
#define MT_VOLUME_BASE 0
#define MT_VOLUME_DETAIL 1
#define MT_TGA_MAX_SLICE_BYTES 200000
MT_API mt_status mt_decode_tga_volume(mt_ctx* ctx, int volume, const uint8_t* const* files, const size_t* sizes,
                                      int n_slices, void* stream);
/* Generate the four noise volumes on the GPU from `seed` (no reference
 * counterpart: the reference loads pre-baked assets).  Writes RGBA8 and the
 * FP16/BF16 precision-form copies.  Weather goes to slot 0. */
MT_API mt_status mt_generate_volumes(mt_ctx* ctx, uint64_t seed, void* stream);
MT_API mt_status mt_generate_weather(mt_ctx* ctx, int slot, uint64_t seed, void* stream);
/* Copy volumes back to host memory (any pointer may be NULL). */
MT_API mt_status mt_download_volumes(mt_ctx* ctx, uint8_t* base_rgba8, uint8_t* detail_rgba8,
                                     uint8_t* curl_rgba8, uint8_t* weather_rgba8, int weather_slot);
/* Copy the half-precision copies back (raw IEEE half or bfloat16 bits). */
MT_API mt_status mt_download_volumes_16(mt_ctx* ctx, int storage, uint16_t* base_rgba, uint16_t* detail_rgba,
                                        uint16_t* curl_rgba, uint16_t* weather_rgba, int weather_slot);

/* ---- the compute stage -------------------------------------------------- */

/* One compute command buffer of the reference (Renderer.cpp:653-722): with
 * MT_RENDER_CHECKERBOARD, every pixel of cur_rgba is the 10-tap reprojection of
 * prev_rgba (reprojection.comp:193-244) except the one pixel per 4x4 block
 * selected by time->frame_count_mod16, which is raymarched
 * (cloudRayMarch.comp:690-826).  With MT_RENDER_FULL every pixel is marched
 * and prev_rgba is not read.  godray_mask (may be NULL) receives, for each
 * marched pixel only, the scalar the god-ray pass decodes
 * (postProcess_GodRays.frag:39-43); other mask pixels keep their contents, as
 * the reference's god-ray image does.  Device pointers; stream-ordered. */
MT_API mt_status mt_render(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                           const mt_time_ubo* time, const mt_params* params, const float* prev_rgba,
                           float* cur_rgba, float* godray_mask, int width, int height, uint32_t flags,
                           void* stream);

/* One whole frame: the reprojection and raymarch of mt_render and the TXAA
 * resolve of mt_txaa (with mt_tuning.fused_resolve, the raymarch then the
 * reprojection fused with TXAA in a second launch).  cur_rgba receives the
 * raw frame (what the next frame reprojects from, as with mt_render), out_rgba
 * the resolved frame (the next frame's TXAA history).  Results equal
 * mt_render followed by mt_txaa(current = cur_rgba, history_rgba, out_rgba).
 * With MT_RENDER_FULL every pixel is marched and prev_rgba is not read. */
MT_API mt_status mt_render_frame(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                                 const mt_time_ubo* time, const mt_params* params, const float* prev_rgba,
                                 float* cur_rgba, const float* history_rgba, float* out_rgba,
                                 float* godray_mask, int width, int height, uint32_t flags, void* stream);

/* TXAA resolve (postProcess_TXAA.frag:223-269) of `current` against
 * `history` (the previous resolved frame), written to `out` (distinct from
 * both).  Device pointers; stream-ordered. */
MT_API mt_status mt_txaa(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                         const mt_time_ubo* time, const mt_params* params, const float* current_rgba,
                         const float* history_rgba, float* out_rgba, int width, int height, void* stream);

/* Many views, uneven sizes, one persistent launch (config 3).  `views` is a
 * host array; its image pointers are device pointers.  All views share one
 * storage.  Checkerboard views are reprojected first, then one persistent
 * raymarch launch takes tiles of every view from a work counter; the whole
 * batch is a CUDA graph launched on `stream`.  Results equal mt_render per view.
 * Two batches may be in flight at once (on two streams they overlap on the
 * device); a third waits for the first.  The views' images of batches in
 * flight together must not overlap. */
MT_API mt_status mt_render_batch(mt_ctx* ctx, const mt_view* views, int n_views, void* stream);

/* Diagnostic, no counterpart in the reference: while `counts` is not NULL,
 * every mt_render / mt_render_frame of this context writes, for each marched
 * pixel (x, y), four uint32 at counts[4 * (y * width + x)]: the ray's executed
 * primary samples, its in-cloud samples (density > 0,
 * cloudRayMarch.comp:642), its control-flow signature and 0.  The signature
 * is an FNV-1a hash (offset 2166136261, prime 16777619) over the executed
 * steps, in order, of (jitter index | in cloud << 4 | light sample i's
 * cbl > 0 << (5 + i)); 0 for a ray that marched no step.  `counts` is a
 * 16-byte-aligned device buffer of width x height x 4 uint32 the caller owns,
 * for the size of the frames rendered.  It records each ray's control flow,
 * e.g. to tell pixels whose march took the same branches as an oracle's from
 * pixels where a threshold flipped.  NULL turns it off.  Traced renders use
 * 1 or 4 lanes per ray and 256-thread CTAs; batched renders never write it. */
MT_API mt_status mt_set_sample_trace(mt_ctx* ctx, void* counts);

/* Times mt_render_batch on these views over the tile shapes {8x8, 16x8,
 * 16x16, 32x8} and the step schedule -- the lanes that march one ray (1, 4
 * or 8: a ray's primary steps evaluated one at a time, or 4 / 8 at once with
 * the in-order scan) and the order the tile rows are handed out (bottom to
 * top or top to bottom) -- keeps the fastest in the context's tuning
 * (batch_tile_w/h, batch_lanes, batch_order) and returns it.  Each point is
 * timed twice and its faster run kept; the views are rendered 49 times. */
MT_API mt_status mt_autotune_batch(mt_ctx* ctx, const mt_view* views, int n_views, void* stream,
                                   mt_tuning* best);

/* mt_render_batch without any device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory on the render
 * path: cudaMalloc and cudaFree synchronise the device and stall every other
 * stream of a frame loop, and a host that has handed its HBM budget to its
 * own pool has none left to give.  The view table, tile list and work
 * counter live in one fixed device array of the library (about 0.76 MB):
 * at most MT_NOALLOC_MAX_VIEWS views and MT_NOALLOC_MAX_TILES tiles of the
 * context's batch tile shape; a batch beyond either limit is rejected with
 * MT_ERR_INVALID_ARG before anything is launched.  Nothing is staged in
 * host memory and the call never waits for the device: the view tables reach
 * the array as the parameters of small store kernels launched on `stream`,
 * the tile list is generated there by another kernel, then the reprojections
 * and the persistent raymarch follow on the same stream.  Results equal
 * mt_render_batch.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  Every call on a device shares the one array and
 * leaves its tables there (the next call rewrites them and zeroes the work
 * counter): calls on one stream are ordered, but calls whose work may overlap
 * on the device (two streams not ordered by events) race on the array. */
#define MT_NOALLOC_MAX_VIEWS 64
#define MT_NOALLOC_MAX_TILES 32768
MT_API mt_status mt_render_batch_noalloc(mt_ctx* ctx, const mt_view* views, int n_views, void* stream);

/* ---- Downstream passes (the consumers of the compute stage's outputs) ----
 * Both are full-screen fragment passes in the reference: one fragment per
 * pixel with in_uv at the pixel centre, storing with imageStore at
 * pixelPos = clamp(round(dim * in_uv)), which is the fragment's own pixel or
 * the next one (round half away from zero).  Where two fragments store to
 * one pixel the later fragment in raster order wins; pixels no fragment
 * stores to keep their input value (mt_godrays) or their previous contents
 * (mt_tonemap's output).  Device pointers, stream-ordered. */

/* postProcess_GodRays.frag:66-149: 100-sample screen-space radial blur of the
 * god-ray mask toward the static sun at (0, 1, 0), added to the HDR image.
 * `mask` is the R32F mask the raymarch writes (the decoded value the shader's
 * extract32fFromRGBA8f reads; LINEAR filtering with exact FP32 weights,
 * border = the decode of opaque black).  `light_color` is SunAndSky.lightColor
 * (Sky.cpp:71: 1, 1, 0.57, 1).  out_rgba may equal in_rgba.  The pass is
 * disabled in the reference's command buffer (Renderer.cpp:826-832). */
MT_API mt_status mt_godrays(mt_ctx* ctx, const mt_camera_ubo* camera, const float light_color[4],
                            const float* mask, const float* in_rgba, float* out_rgba, int width, int height,
                            void* stream);

/* postProcess_ToneMap.frag:68-84: Uncharted-2 filmic curve (exposure 2.5,
 * white point 100, gamma 1/2.2) of the LINEAR-filtered HDR image
 * (clamp-to-border opaque black) plus WangHash dither * 0.01 seeded with
 * uint(time.y).  out_format MT_LDR_RGBA8: 4 bytes per pixel, UNORM
 * (clamp to [0, 1], x255, round to nearest even, NaN -> 0; the shader's
 * `rgba8` image); MT_LDR_RGBA32F: the float values the shader stores. */
typedef enum mt_ldr_format { MT_LDR_RGBA8 = 0, MT_LDR_RGBA32F = 1 } mt_ldr_format;
MT_API mt_status mt_tonemap(mt_ctx* ctx, const mt_time_ubo* time, const float* in_rgba, void* out, int width,
                            int height, int out_format, void* stream);

/* Counters accumulated by render calls made with MT_RENDER_COUNT since the
 * last reset.  Synchronises the stream. */
MT_API mt_status mt_get_stats(mt_ctx* ctx, mt_stats* out, int reset, void* stream);

/* Launch-shape tuning (no counterpart in the reference, whose workgroup is a
 * fixed 32x32, cloudRayMarch.comp:4-5). */
MT_API mt_status mt_set_tuning(mt_ctx* ctx, const mt_tuning* tuning);
MT_API mt_status mt_get_tuning(mt_ctx* ctx, mt_tuning* tuning);

/* Numerical self-test of the kernels' division by a reused denominator:
 * out_rdiv[i] is that routine's a[i] / b[i], out_ieee[i] the device's IEEE
 * division.  The two must agree bit for bit.  Device pointers. */
MT_API mt_status mt_selftest_division(mt_ctx* ctx, const float* a, const float* b, float* out_rdiv,
                                      float* out_ieee, int n, void* stream);

/* Per-kernel CUDA-event timing (no counterpart in the reference, which only
 * reports frame rates read off externally, README.md:266-294).  While on,
 * each kernel launch is bracketed by events on its stream. */
MT_API mt_status mt_set_timing(mt_ctx* ctx, int enabled);
/* Synchronises on the recorded events and returns their durations. */
MT_API mt_status mt_get_kernel_times(mt_ctx* ctx, mt_kernel_times* out);

/* ---- Serving (config 4): continuous batching of per-session frames ----
 * No counterpart in the reference, whose one window renders one view per
 * frame (main.cpp:172-194).  A server owns a worker thread that batches
 * requests over the context's shared volumes; the context must not be used
 * by anything else while the server exists.  A session keeps its two raw
 * frames (the reprojection ping-pong, Renderer.cpp:131-136), its god-ray
 * mask and its previous camera resident in HBM; sessions are admitted while
 * width * height * 36 bytes each fit hbm_budget_bytes (after waiting up to
 * admission_wait_ms for sessions to close; else MT_ERR_BUDGET).
 * Each request is one frame of one session: the first marches every pixel,
 * later ones march one pixel per 4x4 block and reproject the previous frame.
 * A batch takes every queued request whose session has no frame in flight
 * (up to max_batch, in arrival order) into one mt_render_batch; with
 * streams = 2 a batch formed while another runs overlaps it on the device.
 * Results equal the same requests rendered one at a time. */
typedef struct mt_server mt_server;

typedef struct mt_server_config {
    uint64_t hbm_budget_bytes;  /* admission limit for session state */
    int32_t max_batch;          /* requests per batch, >= 1 */
    int32_t streams;            /* batches in flight at once: 1 or 2 */
    int32_t batch_lanes;        /* 0 = keep the context's tuning, else 1, 4, 8 or 16 */
    int32_t per_request;        /* 1 = no batching: one mt_render per request (the plain
                                   per-request launch the batched loop is compared with) */
    int32_t use_graph;          /* 1 = each batch as a CUDA graph; 0 = direct launches (lower
                                   host cost per batch) */
    int32_t admission_wait_ms;  /* mt_server_open_session waits up to this long for closing
                                   sessions to free budget before MT_ERR_BUDGET (0 = no wait) */
} mt_server_config;

typedef struct mt_request_info {
    uint64_t id;
    int64_t session;
    double submit_s, start_s, done_s;  /* mt_server_clock() at submit, batch launch, completion */
    int32_t batch_size;                /* requests in the batch that ran it */
    int32_t status;                    /* mt_status of the request */
} mt_request_info;

/* Seconds on the monotonic clock the request times use. */
MT_API double mt_server_clock(void);
MT_API mt_status mt_server_create(mt_ctx* ctx, const mt_server_config* cfg, mt_server** out);
/* Waits (at most 30 s) for the batches in flight, then frees every session. */
MT_API void mt_server_destroy(mt_server* srv);
MT_API const char* mt_server_last_error(const mt_server* srv);
MT_API mt_status mt_server_open_session(mt_server* srv, int width, int height, const mt_params* params,
                                        int64_t* session);
/* Waits (at most 30 s, else MT_ERR_TIMEOUT) for the session's frame in flight. */
MT_API mt_status mt_server_close_session(mt_server* srv, int64_t session);
/* Queues one frame of `session`; the camera of the session's previous frame
 * is its camera_old.  Host structures, copied before the call returns. */
MT_API mt_status mt_server_submit(mt_server* srv, int64_t session, const mt_camera_ubo* camera,
                                  const mt_time_ubo* time, uint64_t* request);
/* Waits at most timeout_ms for the request (MT_ERR_TIMEOUT, request kept),
 * fills `info` and forgets the request; returns the request's status. */
MT_API mt_status mt_server_wait(mt_server* srv, uint64_t request, int timeout_ms, mt_request_info* info);
/* Copies the session's last frame (RGBA32F) and mask (R32F) to host memory
 * (either may be NULL); waits (at most 30 s) for its frame in flight. */
MT_API mt_status mt_server_read_frame(mt_server* srv, int64_t session, float* host_rgba, float* host_mask);
MT_API mt_status mt_server_memory(mt_server* srv, uint64_t* used_bytes, uint64_t* budget_bytes);

#ifdef __cplusplus
}
#endif

#endif /* METEOROS_H */
