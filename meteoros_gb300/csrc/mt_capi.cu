// The C ABI of include/meteoros.h: context, volume ownership, argument
// checking and kernel dispatch.
//
// Replaces, on the compute path:
//   Renderer::RecordComputeCommandBuffer / Frame  (Renderer.cpp:653-722, 122-141)
//   Sky::CreateCloudResources                    (Sky.cpp:25-58)
//   the descriptor sets binding images, samplers and uniform blocks
//                                                (Renderer.cpp:914-1086)
// Errors: every entry point returns an mt_status and records a message that
// mt_last_error() returns; no exception crosses the boundary.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mt_kernels.h"

struct mt_ctx {
    int device = 0;
    std::string err;
    uint32_t* base = nullptr;
    uint32_t* detail = nullptr;
    uint32_t* curl = nullptr;
    uint2* base16[2] = {nullptr, nullptr};    // [0] IEEE half, [1] bfloat16
    uint2* detail16[2] = {nullptr, nullptr};
    uint2* curl16[2] = {nullptr, nullptr};
    std::vector<uint32_t*> weather;           // MT_MAX_WEATHER_SLOTS entries, allocated on demand
    std::vector<uint2*> weather16[2];
    // plane-quad / bilinear-cell copies of the RGBA8 volumes (the plain form's samplers read these)
    uint4* base_c = nullptr;                  // MT_BASE_N^3 plane quads
    uint4* detail_c = nullptr;                // MT_DETAIL_N^3 plane quads
    uint4* curl_c = nullptr;                  // MT_CURL_N^2 cells
    std::vector<uint4*> weather_c;            // MT_WEATHER_N^2 cells per slot
    // plane-quad copies of the 16-bit volumes (the precision form's 3D samplers read these)
    uint4* base16q[2] = {nullptr, nullptr};   // MT_BASE_N^3 x 2
    uint4* detail16q[2] = {nullptr, nullptr}; // MT_DETAIL_N^3 x 2
    bool have_base = false, have_detail = false, have_curl = false;
    unsigned long long* stats = nullptr;      // 4 counters
    bool timing = false;
    cudaEvent_t ev[8] = {};                   // reproject, march, txaa, resolve (start, end)
    bool ran[4] = {false, false, false, false};
    int march_lanes = 0;                      // step-parallel lanes per ray (mt_set_tuning); 0 = auto
    int march_block = 256;                    // march_kernel CTA size (mt_set_tuning)
    int march_order = 0;                      // ray rows: 0 bottom to top, 1 top to bottom
    int batch_order = 0;                      // mt_render_batch tile rows: 0 bottom to top, 1 top to bottom
    int fused_resolve = 0;                    // mt_render_frame: reprojection fused with TXAA
    // mt_render_batch
    int batch_tile_w = 16, batch_tile_h = 8, batch_lanes = 1;
    int batch_direct = 0;                     // 1: no graph, copies and launches issued on the stream
    // Two slots used in turn, so two batches may run at once on two streams.
    mt::MarchArgs* d_views[2] = {nullptr, nullptr};  // device view tables
    mt::BatchTile* d_tiles[2] = {nullptr, nullptr};  // device tile lists
    unsigned* d_counter[2] = {nullptr, nullptr};     // work counters
    mt::MarchArgs* h_views[2] = {nullptr, nullptr};  // pinned staging, two slots used in turn
    mt::BatchTile* h_tiles[2] = {nullptr, nullptr};
    cudaEvent_t slot_done[2] = {nullptr, nullptr};   // the batch that last used the slot has finished
    bool slot_pending[2] = {false, false};
    int slot = 0;
    size_t cap_views = 0, cap_tiles = 0;
    cudaStream_t cap_stream = nullptr;        // private stream the batch graphs are captured on
    cudaGraphExec_t batch_exec[2] = {nullptr, nullptr};
    // mt_render / mt_render_frame: the reprojection runs beside the raymarch
    // on this stream (fork/join events); overlap = 0 keeps one stream
    cudaStream_t aux = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    int overlap = 1;
    uint4* trace = nullptr;                   // mt_set_sample_trace
};

namespace {

thread_local std::string g_create_error;

constexpr size_t kBaseTexels = (size_t)MT_BASE_N * MT_BASE_N * MT_BASE_N;
constexpr size_t kDetailTexels = (size_t)MT_DETAIL_N * MT_DETAIL_N * MT_DETAIL_N;
constexpr size_t kCurlTexels = (size_t)MT_CURL_N * MT_CURL_N;
constexpr size_t kWeatherTexels = (size_t)MT_WEATHER_N * MT_WEATHER_N;

mt_status fail(mt_ctx* ctx, mt_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->err = buf;
    else
        g_create_error = buf;
    return st;
}

#define MT_CUDA(ctx, call)                                                                                 \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? MT_ERR_OUT_OF_MEMORY : MT_ERR_CUDA,       \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                                   \
    } while (0)

template <class T> mt_status alloc(mt_ctx* ctx, T** p, size_t count) {
    if (*p) return MT_OK;
    MT_CUDA(ctx, cudaMalloc((void**)p, count * sizeof(T)));
    return MT_OK;
}

mt_status bind_device(mt_ctx* ctx) {
    MT_CUDA(ctx, cudaSetDevice(ctx->device));
    return MT_OK;
}

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

mt_status check_params(mt_ctx* ctx, const mt_params* p, const mt_time_ubo* t) {
    if (!p || !t) return fail(ctx, MT_ERR_INVALID_ARG, "params and time must not be NULL");
    if (t->frame_count_mod16 < 0 || t->frame_count_mod16 > 15)
        return fail(ctx, MT_ERR_INVALID_ARG, "time.frame_count_mod16 = %d is outside 0..15", t->frame_count_mod16);
    if (!(p->earth_radius > 0.0f) || !(p->shell_inner_radius > p->earth_radius) ||
        !(p->shell_outer_radius > p->shell_inner_radius))
        return fail(ctx, MT_ERR_INVALID_ARG, "shell radii must satisfy 0 < earth < inner < outer");
    if (!(p->noise_period > 0.0f)) return fail(ctx, MT_ERR_INVALID_ARG, "noise_period must be > 0");
    if (p->steps_min < 1 || p->steps_max < 1 || p->steps_min > 4096 || p->steps_max > 4096)
        return fail(ctx, MT_ERR_INVALID_ARG, "steps_min/steps_max must be in 1..4096");
    if (p->coverage_mode != 0 && p->coverage_mode != 1)
        return fail(ctx, MT_ERR_INVALID_ARG, "coverage_mode must be 0 or 1");
    if (p->coverage_mode == 1 && !(p->weather_scale > 0.0f))
        return fail(ctx, MT_ERR_INVALID_ARG, "weather_scale must be > 0");
    if (p->weather_slot < 0 || p->weather_slot >= MT_MAX_WEATHER_SLOTS)
        return fail(ctx, MT_ERR_INVALID_ARG, "weather_slot %d is outside 0..%d", p->weather_slot,
                    MT_MAX_WEATHER_SLOTS - 1);
    for (int i = 0; i < 16; ++i)
        if (p->slot_x[i] < 0 || p->slot_x[i] > 3 || p->slot_y[i] < 0 || p->slot_y[i] > 3)
            return fail(ctx, MT_ERR_INVALID_ARG, "checkerboard slot %d is outside the 4x4 block", i);
    if (p->storage != MT_STORAGE_U8 && p->storage != MT_STORAGE_F16 && p->storage != MT_STORAGE_BF16)
        return fail(ctx, MT_ERR_INVALID_ARG, "unknown storage %d", p->storage);
    return MT_OK;
}

mt_status check_image(mt_ctx* ctx, int w, int h) {
    if (w < 1 || h < 1 || w > MT_MAX_DIM || h > MT_MAX_DIM)
        return fail(ctx, MT_ERR_INVALID_ARG, "image size %dx%d is outside 1..%d", w, h, MT_MAX_DIM);
    return MT_OK;
}

mt_status ensure_weather(mt_ctx* ctx, int slot) {
    if (ctx->weather[slot]) return MT_OK;
    mt_status st = alloc(ctx, &ctx->weather[slot], kWeatherTexels);
    if (st != MT_OK) return st;
    st = alloc(ctx, &ctx->weather16[0][slot], kWeatherTexels);
    if (st != MT_OK) return st;
    st = alloc(ctx, &ctx->weather_c[slot], kWeatherTexels);
    if (st != MT_OK) return st;
    return alloc(ctx, &ctx->weather16[1][slot], kWeatherTexels);
}

// The plane-quad copies of a volume's two 16-bit versions, after they change.
cudaError_t refresh_quads(mt_ctx* ctx, int volume, cudaStream_t s) {
    const bool base = volume == MT_VOLUME_BASE;
    for (int k = 0; k < 2; ++k) {
        const cudaError_t e = mt::launch_quads16(base ? ctx->base16[k] : ctx->detail16[k],
                                                 base ? MT_BASE_N : MT_DETAIL_N,
                                                 base ? ctx->base16q[k] : ctx->detail16q[k], s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

mt_status ensure_volumes(mt_ctx* ctx) {
    mt_status st;
    if ((st = alloc(ctx, &ctx->base, kBaseTexels)) != MT_OK) return st;
    if ((st = alloc(ctx, &ctx->detail, kDetailTexels)) != MT_OK) return st;
    if ((st = alloc(ctx, &ctx->curl, kCurlTexels)) != MT_OK) return st;
    if ((st = alloc(ctx, &ctx->base_c, kBaseTexels)) != MT_OK) return st;
    if ((st = alloc(ctx, &ctx->detail_c, kDetailTexels)) != MT_OK) return st;
    if ((st = alloc(ctx, &ctx->curl_c, kCurlTexels)) != MT_OK) return st;
    for (int k = 0; k < 2; ++k) {
        if ((st = alloc(ctx, &ctx->base16[k], kBaseTexels)) != MT_OK) return st;
        if ((st = alloc(ctx, &ctx->detail16[k], kDetailTexels)) != MT_OK) return st;
        if ((st = alloc(ctx, &ctx->curl16[k], kCurlTexels)) != MT_OK) return st;
        if ((st = alloc(ctx, &ctx->base16q[k], 2 * kBaseTexels)) != MT_OK) return st;
        if ((st = alloc(ctx, &ctx->detail16q[k], 2 * kDetailTexels)) != MT_OK) return st;
    }
    return MT_OK;
}

uint32_t seed32(uint64_t s) { return (uint32_t)s ^ (uint32_t)(s >> 32); }

mt_status build_march_args(mt_ctx* ctx, const mt_camera_ubo* cam, const mt_camera_ubo* cam_old,
                           const mt_time_ubo* tm, const mt_params* p, const float* prev, float* cur, float* mask,
                           int w, int h, uint32_t flags, mt::MarchArgs* a) {
    if (!cam || !cam_old) return fail(ctx, MT_ERR_INVALID_ARG, "camera and camera_old must not be NULL");
    mt_status st;
    if ((st = check_params(ctx, p, tm)) != MT_OK) return st;
    if ((st = check_image(ctx, w, h)) != MT_OK) return st;
    if (flags & ~(MT_RENDER_FULL | MT_RENDER_COUNT)) return fail(ctx, MT_ERR_INVALID_ARG, "unknown flags 0x%x", flags);
    if (!cur) return fail(ctx, MT_ERR_INVALID_ARG, "cur_rgba must not be NULL");
    if (!aligned(cur, 16) || (prev && !aligned(prev, 16)) || (mask && !aligned(mask, 4)))
        return fail(ctx, MT_ERR_INVALID_ARG, "images must be 16-byte aligned (mask 4-byte)");
    const bool full = (flags & MT_RENDER_FULL) != 0;
    if (!full && !prev) return fail(ctx, MT_ERR_INVALID_ARG, "prev_rgba is required without MT_RENDER_FULL");
    if (!full && prev == cur) return fail(ctx, MT_ERR_INVALID_ARG, "prev_rgba and cur_rgba must be distinct images");
    if (!ctx->have_base || !ctx->have_detail || !ctx->have_curl)
        return fail(ctx, MT_ERR_NO_VOLUMES, "noise volumes have not been uploaded or generated");
    if (p->coverage_mode == 1 && !ctx->weather[p->weather_slot])
        return fail(ctx, MT_ERR_NO_VOLUMES, "weather slot %d holds no weather map", p->weather_slot);
    std::memset(a, 0, sizeof(*a));
    a->camera = *cam;
    a->camera_old = *cam_old;
    a->time = *tm;
    a->params = *p;
    const int k = p->storage == MT_STORAGE_BF16 ? 1 : 0;
    const uint4* weather8 = (p->coverage_mode == 1) ? ctx->weather_c[p->weather_slot] : ctx->curl_c;
    const uint2* weather16 = (p->coverage_mode == 1) ? ctx->weather16[k][p->weather_slot] : ctx->curl16[k];
    if (p->storage == MT_STORAGE_U8) {
        a->vol[0] = ctx->base_c;
        a->vol[1] = ctx->detail_c;
        a->vol[2] = ctx->curl_c;
        a->vol[3] = weather8;  // never read when coverage_mode == 0
    } else {
        a->vol[0] = ctx->base16q[k];
        a->vol[1] = ctx->detail16q[k];
        a->vol[2] = ctx->curl16[k];
        a->vol[3] = weather16;
    }
    a->prev = (const float4*)prev;
    a->cur = (float4*)cur;
    a->mask = mask;
    a->stats = (flags & MT_RENDER_COUNT) ? ctx->stats : nullptr;
    a->width = w;
    a->height = h;
    a->groups_x = mt::march_groups(w);
    a->groups_y = mt::march_groups(h);
    a->flags = flags;
    a->block = ctx->march_block;
    mt::make_view_consts(&a->vc_repro, *p, *cam, *cam_old, *tm, w, h, true);
    mt::make_view_consts(&a->vc_txaa, *p, *cam, *cam_old, *tm, w, h, false);
    mt::make_march_jitter(a->jitter, *tm);
    mt::make_march_frame(&a->frame, *p, *cam, *tm);
    a->bottom_up = ctx->march_order == 0 ? 1 : 0;
    a->lanes = ctx->march_lanes;
    if (a->lanes == 0) {
        // Auto: enough rays fill the GPU one lane per ray; fewer rays (a
        // checkerboard frame marches 1/16 of the pixels) get 4 lanes each.
        const long long rays = full ? (long long)w * h : (long long)a->groups_x * a->groups_y;
        a->lanes = rays >= 262144 ? 1 : 4;
    }
    return MT_OK;
}

}  // namespace

namespace mt {
int ctx_device(const mt_ctx* ctx) { return ctx->device; }
}  // namespace mt

extern "C" {

MT_API mt_status mt_create(mt_ctx** out, int device) {
    if (!out) return fail(nullptr, MT_ERR_INVALID_ARG, "out must not be NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, MT_ERR_UNSUPPORTED, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(nullptr, MT_ERR_INVALID_ARG, "device %d of %d", device, n);
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return fail(nullptr, MT_ERR_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    if (prop.major != 10 || prop.minor != 3)
        return fail(nullptr, MT_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a", device,
                    prop.major, prop.minor);
    mt_ctx* ctx = new (std::nothrow) mt_ctx();
    if (!ctx) return fail(nullptr, MT_ERR_OUT_OF_MEMORY, "host allocation failed");
    ctx->device = device;
    ctx->weather.assign(MT_MAX_WEATHER_SLOTS, nullptr);
    ctx->weather_c.assign(MT_MAX_WEATHER_SLOTS, nullptr);
    ctx->weather16[0].assign(MT_MAX_WEATHER_SLOTS, nullptr);
    ctx->weather16[1].assign(MT_MAX_WEATHER_SLOTS, nullptr);
    if (bind_device(ctx) != MT_OK || alloc(ctx, &ctx->stats, 4) != MT_OK ||
        cudaMemset(ctx->stats, 0, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) != cudaSuccess) {
        g_create_error = ctx->err.empty() ? "context set-up failed" : ctx->err;
        mt_destroy(ctx);
        return MT_ERR_CUDA;
    }
    *out = ctx;
    return MT_OK;
}

MT_API void mt_destroy(mt_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaFree(ctx->base);
    cudaFree(ctx->detail);
    cudaFree(ctx->curl);
    cudaFree(ctx->base_c);
    cudaFree(ctx->detail_c);
    cudaFree(ctx->curl_c);
    for (uint4* w : ctx->weather_c) cudaFree(w);
    for (int k = 0; k < 2; ++k) {
        cudaFree(ctx->base16[k]);
        cudaFree(ctx->base16q[k]);
        cudaFree(ctx->detail16q[k]);
        cudaFree(ctx->detail16[k]);
        cudaFree(ctx->curl16[k]);
        for (uint2* w : ctx->weather16[k]) cudaFree(w);
    }
    for (uint32_t* w : ctx->weather) cudaFree(w);
    cudaFree(ctx->stats);
    for (cudaEvent_t e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
        if (ctx->slot_pending[k]) cudaEventSynchronize(ctx->slot_done[k]);
        cudaFree(ctx->d_views[k]);
        cudaFree(ctx->d_tiles[k]);
        cudaFree(ctx->d_counter[k]);
        cudaFreeHost(ctx->h_views[k]);
        cudaFreeHost(ctx->h_tiles[k]);
        if (ctx->slot_done[k]) cudaEventDestroy(ctx->slot_done[k]);
        if (ctx->batch_exec[k]) cudaGraphExecDestroy(ctx->batch_exec[k]);
    }
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    delete ctx;
}

MT_API const char* mt_last_error(const mt_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

MT_API mt_status mt_upload_volumes(mt_ctx* ctx, const uint8_t* base, const uint8_t* detail, const uint8_t* curl,
                                   const uint8_t* weather) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if ((st = ensure_volumes(ctx)) != MT_OK) return st;
    if (base) {
        MT_CUDA(ctx, cudaMemcpy(ctx->base, base, kBaseTexels * 4, cudaMemcpyHostToDevice));
        MT_CUDA(ctx, mt::launch_u8_to_16(ctx->base, kBaseTexels, ctx->base16[0], ctx->base16[1], 0));
        MT_CUDA(ctx, mt::launch_quads3(ctx->base, MT_BASE_N, ctx->base_c, 0));
        MT_CUDA(ctx, refresh_quads(ctx, MT_VOLUME_BASE, 0));
        ctx->have_base = true;
    }
    if (detail) {
        MT_CUDA(ctx, cudaMemcpy(ctx->detail, detail, kDetailTexels * 4, cudaMemcpyHostToDevice));
        MT_CUDA(ctx, mt::launch_u8_to_16(ctx->detail, kDetailTexels, ctx->detail16[0], ctx->detail16[1], 0));
        MT_CUDA(ctx, mt::launch_quads3(ctx->detail, MT_DETAIL_N, ctx->detail_c, 0));
        MT_CUDA(ctx, refresh_quads(ctx, MT_VOLUME_DETAIL, 0));
        ctx->have_detail = true;
    }
    if (curl) {
        MT_CUDA(ctx, cudaMemcpy(ctx->curl, curl, kCurlTexels * 4, cudaMemcpyHostToDevice));
        MT_CUDA(ctx, mt::launch_u8_to_16(ctx->curl, kCurlTexels, ctx->curl16[0], ctx->curl16[1], 0));
        MT_CUDA(ctx, mt::launch_cells2(ctx->curl, MT_CURL_N, ctx->curl_c, 0));
        ctx->have_curl = true;
    }
    if (weather) {
        if ((st = mt_upload_weather(ctx, 0, weather)) != MT_OK) return st;
    }
    MT_CUDA(ctx, cudaDeviceSynchronize());
    return MT_OK;
}

MT_API mt_status mt_decode_tga_volume(mt_ctx* ctx, int volume, const uint8_t* const* files, const size_t* sizes,
                                      int n_slices, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (volume != MT_VOLUME_BASE && volume != MT_VOLUME_DETAIL)
        return fail(ctx, MT_ERR_INVALID_ARG, "volume must be MT_VOLUME_BASE or MT_VOLUME_DETAIL");
    const int n = volume == MT_VOLUME_BASE ? MT_BASE_N : MT_DETAIL_N;
    if (n_slices != n) return fail(ctx, MT_ERR_INVALID_ARG, "%d slices given, the volume has %d", n_slices, n);
    if (!files || !sizes) return fail(ctx, MT_ERR_INVALID_ARG, "files and sizes must not be NULL");
    std::vector<mt::TgaSlice> table((size_t)n);
    size_t total = 0, max_size = 0;
    for (int z = 0; z < n; ++z) {
        const uint8_t* f = files[z];
        const size_t sz = sizes[z];
        if (!f || sz < 18) return fail(ctx, MT_ERR_INVALID_ARG, "slice %d: not a TGA file (%zu bytes)", z, sz);
        if (sz > MT_TGA_MAX_SLICE_BYTES)
            return fail(ctx, MT_ERR_INVALID_ARG, "slice %d: %zu bytes, above the %d-byte limit", z, sz,
                        MT_TGA_MAX_SLICE_BYTES);
        const int type = f[2], bpp = f[16], w = f[12] | (f[13] << 8), h = f[14] | (f[15] << 8);
        if (f[1] != 0 || (type != 2 && type != 10) || (bpp != 24 && bpp != 32))
            return fail(ctx, MT_ERR_INVALID_ARG,
                        "slice %d: unsupported TGA (colour-map type %d, image type %d, %d bits per pixel)", z, f[1],
                        type, bpp);
        if (w != n || h != n)
            return fail(ctx, MT_ERR_INVALID_ARG, "slice %d is %dx%d, the volume's slices are %dx%d", z, w, h, n, n);
        table[(size_t)z] = mt::TgaSlice{(long long)total, (long long)sz};
        total += sz;
        max_size = std::max(max_size, sz);
    }
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if ((st = ensure_volumes(ctx)) != MT_OK) return st;
    std::vector<uint8_t> blob(total);
    for (int z = 0; z < n; ++z) std::memcpy(blob.data() + table[(size_t)z].offset, files[z], sizes[z]);
    unsigned char* d_blob = nullptr;
    mt::TgaSlice* d_table = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* vol = volume == MT_VOLUME_BASE ? ctx->base : ctx->detail;
    cudaError_t e = cudaMalloc((void**)&d_blob, total);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_table, table.size() * sizeof(mt::TgaSlice));
    if (e == cudaSuccess) e = cudaMemcpy(d_blob, blob.data(), total, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_table, table.data(), table.size() * sizeof(mt::TgaSlice), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = mt::launch_tga_decode(d_blob, d_table, n, max_size, vol, n, n, s);
    const size_t texels = (size_t)n * n * n;
    if (e == cudaSuccess)
        e = mt::launch_u8_to_16(vol, texels, volume == MT_VOLUME_BASE ? ctx->base16[0] : ctx->detail16[0],
                                volume == MT_VOLUME_BASE ? ctx->base16[1] : ctx->detail16[1], s);
    if (e == cudaSuccess) e = mt::launch_quads3(vol, n, volume == MT_VOLUME_BASE ? ctx->base_c : ctx->detail_c, s);
    if (e == cudaSuccess) e = refresh_quads(ctx, volume, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_blob);
    cudaFree(d_table);
    if (e != cudaSuccess)
        return fail(ctx, e == cudaErrorMemoryAllocation ? MT_ERR_OUT_OF_MEMORY : MT_ERR_CUDA, "TGA decode: %s",
                    cudaGetErrorString(e));
    if (volume == MT_VOLUME_BASE)
        ctx->have_base = true;
    else
        ctx->have_detail = true;
    return MT_OK;
}

MT_API mt_status mt_upload_weather(mt_ctx* ctx, int slot, const uint8_t* weather) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!weather) return fail(ctx, MT_ERR_INVALID_ARG, "weather must not be NULL");
    if (slot < 0 || slot >= MT_MAX_WEATHER_SLOTS) return fail(ctx, MT_ERR_INVALID_ARG, "weather slot %d", slot);
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if ((st = ensure_weather(ctx, slot)) != MT_OK) return st;
    MT_CUDA(ctx, cudaMemcpy(ctx->weather[slot], weather, kWeatherTexels * 4, cudaMemcpyHostToDevice));
    MT_CUDA(ctx, mt::launch_u8_to_16(ctx->weather[slot], kWeatherTexels, ctx->weather16[0][slot],
                                     ctx->weather16[1][slot], 0));
    MT_CUDA(ctx, mt::launch_cells2(ctx->weather[slot], MT_WEATHER_N, ctx->weather_c[slot], 0));
    MT_CUDA(ctx, cudaDeviceSynchronize());
    return MT_OK;
}

MT_API mt_status mt_generate_volumes(mt_ctx* ctx, uint64_t seed, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if ((st = ensure_volumes(ctx)) != MT_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t s32 = seed32(seed);
    MT_CUDA(ctx, mt::launch_generate_base(s32, mt::NoiseOut{ctx->base, ctx->base16[0], ctx->base16[1]}, s));
    MT_CUDA(ctx, mt::launch_generate_detail(s32, mt::NoiseOut{ctx->detail, ctx->detail16[0], ctx->detail16[1]}, s));
    MT_CUDA(ctx, mt::launch_generate_curl(s32, mt::NoiseOut{ctx->curl, ctx->curl16[0], ctx->curl16[1]}, s));
    MT_CUDA(ctx, mt::launch_quads3(ctx->base, MT_BASE_N, ctx->base_c, s));
    MT_CUDA(ctx, mt::launch_quads3(ctx->detail, MT_DETAIL_N, ctx->detail_c, s));
    MT_CUDA(ctx, mt::launch_cells2(ctx->curl, MT_CURL_N, ctx->curl_c, s));
    MT_CUDA(ctx, refresh_quads(ctx, MT_VOLUME_BASE, s));
    MT_CUDA(ctx, refresh_quads(ctx, MT_VOLUME_DETAIL, s));
    ctx->have_base = ctx->have_detail = ctx->have_curl = true;
    return mt_generate_weather(ctx, 0, seed, stream);
}

MT_API mt_status mt_generate_weather(mt_ctx* ctx, int slot, uint64_t seed, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (slot < 0 || slot >= MT_MAX_WEATHER_SLOTS) return fail(ctx, MT_ERR_INVALID_ARG, "weather slot %d", slot);
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if ((st = ensure_weather(ctx, slot)) != MT_OK) return st;
    MT_CUDA(ctx, mt::launch_generate_weather(
                     seed32(seed), mt::NoiseOut{ctx->weather[slot], ctx->weather16[0][slot], ctx->weather16[1][slot]},
                     (cudaStream_t)stream));
    MT_CUDA(ctx, mt::launch_cells2(ctx->weather[slot], MT_WEATHER_N, ctx->weather_c[slot], (cudaStream_t)stream));
    return MT_OK;
}

MT_API mt_status mt_download_volumes(mt_ctx* ctx, uint8_t* base, uint8_t* detail, uint8_t* curl, uint8_t* weather,
                                     int weather_slot) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    MT_CUDA(ctx, cudaDeviceSynchronize());
    if ((base || detail || curl) && !(ctx->have_base && ctx->have_detail && ctx->have_curl))
        return fail(ctx, MT_ERR_NO_VOLUMES, "no volumes to download");
    if (base) MT_CUDA(ctx, cudaMemcpy(base, ctx->base, kBaseTexels * 4, cudaMemcpyDeviceToHost));
    if (detail) MT_CUDA(ctx, cudaMemcpy(detail, ctx->detail, kDetailTexels * 4, cudaMemcpyDeviceToHost));
    if (curl) MT_CUDA(ctx, cudaMemcpy(curl, ctx->curl, kCurlTexels * 4, cudaMemcpyDeviceToHost));
    if (weather) {
        if (weather_slot < 0 || weather_slot >= MT_MAX_WEATHER_SLOTS || !ctx->weather[weather_slot])
            return fail(ctx, MT_ERR_NO_VOLUMES, "weather slot %d holds no weather map", weather_slot);
        MT_CUDA(ctx, cudaMemcpy(weather, ctx->weather[weather_slot], kWeatherTexels * 4, cudaMemcpyDeviceToHost));
    }
    return MT_OK;
}

MT_API mt_status mt_download_volumes_16(mt_ctx* ctx, int storage, uint16_t* base, uint16_t* detail, uint16_t* curl,
                                        uint16_t* weather, int weather_slot) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (storage != MT_STORAGE_F16 && storage != MT_STORAGE_BF16)
        return fail(ctx, MT_ERR_INVALID_ARG, "storage must be MT_STORAGE_F16 or MT_STORAGE_BF16");
    const int k = storage == MT_STORAGE_F16 ? 0 : 1;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    MT_CUDA(ctx, cudaDeviceSynchronize());
    if ((base || detail || curl) && !(ctx->have_base && ctx->have_detail && ctx->have_curl))
        return fail(ctx, MT_ERR_NO_VOLUMES, "no volumes to download");
    if (base) MT_CUDA(ctx, cudaMemcpy(base, ctx->base16[k], kBaseTexels * 8, cudaMemcpyDeviceToHost));
    if (detail) MT_CUDA(ctx, cudaMemcpy(detail, ctx->detail16[k], kDetailTexels * 8, cudaMemcpyDeviceToHost));
    if (curl) MT_CUDA(ctx, cudaMemcpy(curl, ctx->curl16[k], kCurlTexels * 8, cudaMemcpyDeviceToHost));
    if (weather) {
        if (weather_slot < 0 || weather_slot >= MT_MAX_WEATHER_SLOTS || !ctx->weather[weather_slot])
            return fail(ctx, MT_ERR_NO_VOLUMES, "weather slot %d holds no weather map", weather_slot);
        MT_CUDA(ctx, cudaMemcpy(weather, ctx->weather16[k][weather_slot], kWeatherTexels * 8, cudaMemcpyDeviceToHost));
    }
    return MT_OK;
}

MT_API mt_status mt_set_sample_trace(mt_ctx* ctx, void* counts) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (counts && !aligned(counts, 16)) return fail(ctx, MT_ERR_INVALID_ARG, "counts must be 16-byte aligned");
    ctx->trace = static_cast<uint4*>(counts);
    return MT_OK;
}

MT_API mt_status mt_render(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                           const mt_time_ubo* time, const mt_params* params, const float* prev_rgba, float* cur_rgba,
                           float* godray_mask, int width, int height, uint32_t flags, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt::MarchArgs a;
    mt_status st = build_march_args(ctx, camera, camera_old, time, params, prev_rgba, cur_rgba, godray_mask, width,
                                    height, flags, &a);
    if (st != MT_OK) return st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    a.trace = ctx->trace;
    mt::LaunchEvents ev{{ctx->ev[0], ctx->ev[1]}, {ctx->ev[2], ctx->ev[3]}, {ctx->ev[6], ctx->ev[7]}, ctx->timing};
    const mt::ForkJoin fj{ctx->aux, ctx->fork_ev, ctx->join_ev};
    MT_CUDA(ctx, mt::launch_render(a, (cudaStream_t)stream, &ev, ctx->overlap ? &fj : nullptr));
    if (ctx->timing) {
        ctx->ran[0] = !(flags & MT_RENDER_FULL) || ctx->ran[0];
        ctx->ran[1] = true;
    }
    return MT_OK;
}

MT_API mt_status mt_render_frame(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                                 const mt_time_ubo* time, const mt_params* params, const float* prev_rgba,
                                 float* cur_rgba, const float* history_rgba, float* out_rgba, float* godray_mask,
                                 int width, int height, uint32_t flags, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt::MarchArgs a;
    mt_status st = build_march_args(ctx, camera, camera_old, time, params, prev_rgba, cur_rgba, godray_mask, width,
                                    height, flags, &a);
    if (st != MT_OK) return st;
    if (!history_rgba || !out_rgba) return fail(ctx, MT_ERR_INVALID_ARG, "history and out must not be NULL");
    a.trace = ctx->trace;
    if (!aligned(history_rgba, 16) || !aligned(out_rgba, 16))
        return fail(ctx, MT_ERR_INVALID_ARG, "images must be 16-byte aligned");
    if (out_rgba == cur_rgba || out_rgba == history_rgba || out_rgba == prev_rgba)
        return fail(ctx, MT_ERR_INVALID_ARG, "out_rgba must differ from cur, prev and history");
    if (history_rgba == cur_rgba)
        return fail(ctx, MT_ERR_INVALID_ARG, "history_rgba must differ from cur_rgba");
    a.history = (const float4*)history_rgba;
    a.out = (float4*)out_rgba;
    a.fused_resolve = ctx->fused_resolve;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    mt::LaunchEvents ev{{ctx->ev[0], ctx->ev[1]}, {ctx->ev[2], ctx->ev[3]}, {ctx->ev[6], ctx->ev[7]}, ctx->timing};
    const mt::ForkJoin fj{ctx->aux, ctx->fork_ev, ctx->join_ev};
    MT_CUDA(ctx, mt::launch_frame(a, (cudaStream_t)stream, &ev, ctx->overlap ? &fj : nullptr));
    if (ctx->timing) {
        ctx->ran[0] = ctx->ran[0] || (!(flags & MT_RENDER_FULL) && !ctx->fused_resolve);
        ctx->ran[1] = true;
        ctx->ran[3] = true;
    }
    return MT_OK;
}

MT_API mt_status mt_txaa(mt_ctx* ctx, const mt_camera_ubo* camera, const mt_camera_ubo* camera_old,
                         const mt_time_ubo* time, const mt_params* params, const float* current_rgba,
                         const float* history_rgba, float* out_rgba, int width, int height, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!camera || !camera_old) return fail(ctx, MT_ERR_INVALID_ARG, "camera and camera_old must not be NULL");
    mt_status st;
    if ((st = check_params(ctx, params, time)) != MT_OK) return st;
    if ((st = check_image(ctx, width, height)) != MT_OK) return st;
    if (!current_rgba || !history_rgba || !out_rgba)
        return fail(ctx, MT_ERR_INVALID_ARG, "current, history and out must not be NULL");
    if (!aligned(current_rgba, 16) || !aligned(history_rgba, 16) || !aligned(out_rgba, 16))
        return fail(ctx, MT_ERR_INVALID_ARG, "images must be 16-byte aligned");
    if (out_rgba == current_rgba || out_rgba == history_rgba)
        return fail(ctx, MT_ERR_INVALID_ARG, "out_rgba must differ from current_rgba and history_rgba");
    if ((st = bind_device(ctx)) != MT_OK) return st;
    mt::TxaaArgs a;
    std::memset(&a, 0, sizeof(a));
    a.camera = *camera;
    a.camera_old = *camera_old;
    a.time = *time;
    a.params = *params;
    a.current = (const float4*)current_rgba;
    a.history = (const float4*)history_rgba;
    a.out = (float4*)out_rgba;
    a.width = width;
    a.height = height;
    mt::make_view_consts(&a.vc, *params, *camera, *camera_old, *time, width, height, false);
    MT_CUDA(ctx, mt::launch_txaa(a, (cudaStream_t)stream, ctx->timing ? &ctx->ev[4] : nullptr));
    if (ctx->timing) ctx->ran[2] = true;
    return MT_OK;
}

MT_API mt_status mt_godrays(mt_ctx* ctx, const mt_camera_ubo* camera, const float light_color[4], const float* mask,
                            const float* in_rgba, float* out_rgba, int width, int height, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!camera || !light_color) return fail(ctx, MT_ERR_INVALID_ARG, "camera and light_color must not be NULL");
    mt_status st;
    if ((st = check_image(ctx, width, height)) != MT_OK) return st;
    if (!mask || !in_rgba || !out_rgba) return fail(ctx, MT_ERR_INVALID_ARG, "mask, in and out must not be NULL");
    if (!aligned(in_rgba, 16) || !aligned(out_rgba, 16) || !aligned(mask, 4))
        return fail(ctx, MT_ERR_INVALID_ARG, "images must be 16-byte aligned (mask 4-byte)");
    if ((st = bind_device(ctx)) != MT_OK) return st;
    mt::GodrayArgs a;
    std::memset(&a, 0, sizeof(a));
    a.camera = *camera;
    for (int i = 0; i < 4; ++i) a.light[i] = light_color[i];
    a.mask = mask;
    a.in = (const float4*)in_rgba;
    a.out = (float4*)out_rgba;
    a.width = width;
    a.height = height;
    MT_CUDA(ctx, mt::launch_godrays(a, (cudaStream_t)stream));
    return MT_OK;
}

MT_API mt_status mt_tonemap(mt_ctx* ctx, const mt_time_ubo* time, const float* in_rgba, void* out, int width,
                            int height, int out_format, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!time) return fail(ctx, MT_ERR_INVALID_ARG, "time must not be NULL");
    mt_status st;
    if ((st = check_image(ctx, width, height)) != MT_OK) return st;
    if (out_format != MT_LDR_RGBA8 && out_format != MT_LDR_RGBA32F)
        return fail(ctx, MT_ERR_INVALID_ARG, "out_format must be MT_LDR_RGBA8 or MT_LDR_RGBA32F");
    if (!in_rgba || !out) return fail(ctx, MT_ERR_INVALID_ARG, "in and out must not be NULL");
    if (!aligned(in_rgba, 16) || !aligned(out, out_format == MT_LDR_RGBA8 ? 4 : 16))
        return fail(ctx, MT_ERR_INVALID_ARG, "in must be 16-byte aligned, out 4 (RGBA8) or 16 (RGBA32F)");
    if ((const void*)in_rgba == out) return fail(ctx, MT_ERR_INVALID_ARG, "out must differ from in");
    if ((st = bind_device(ctx)) != MT_OK) return st;
    mt::TonemapArgs a;
    std::memset(&a, 0, sizeof(a));
    a.in = (const float4*)in_rgba;
    a.out = out;
    a.time_y = time->time[1];
    a.format = out_format;
    a.width = width;
    a.height = height;
    MT_CUDA(ctx, mt::launch_tonemap(a, (cudaStream_t)stream));
    return MT_OK;
}

namespace {

mt_status ensure_batch_buffers(mt_ctx* ctx, size_t n_views, size_t n_tiles) {
    if (!ctx->cap_stream) {
        MT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            MT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->slot_done[k], cudaEventDisableTiming));
            MT_CUDA(ctx, cudaMalloc((void**)&ctx->d_counter[k], sizeof(unsigned)));
        }
    }
    if (n_views > ctx->cap_views || n_tiles > ctx->cap_tiles) {
        // Nothing in flight may still read the old buffers.
        for (int k = 0; k < 2; ++k)
            if (ctx->slot_pending[k]) MT_CUDA(ctx, cudaEventSynchronize(ctx->slot_done[k]));
    }
    if (n_views > ctx->cap_views) {
        const size_t cap = std::max<size_t>(n_views, 64);
        for (int k = 0; k < 2; ++k) {
            cudaFree(ctx->d_views[k]);
            cudaFreeHost(ctx->h_views[k]);
            ctx->d_views[k] = nullptr;
            ctx->h_views[k] = nullptr;
        }
        ctx->cap_views = 0;
        for (int k = 0; k < 2; ++k) {
            MT_CUDA(ctx, cudaMalloc((void**)&ctx->d_views[k], cap * sizeof(mt::MarchArgs)));
            MT_CUDA(ctx, cudaHostAlloc((void**)&ctx->h_views[k], cap * sizeof(mt::MarchArgs), cudaHostAllocDefault));
        }
        ctx->cap_views = cap;
    }
    if (n_tiles > ctx->cap_tiles) {
        const size_t cap = std::max<size_t>(n_tiles, 4096);
        for (int k = 0; k < 2; ++k) {
            cudaFree(ctx->d_tiles[k]);
            cudaFreeHost(ctx->h_tiles[k]);
            ctx->d_tiles[k] = nullptr;
            ctx->h_tiles[k] = nullptr;
        }
        ctx->cap_tiles = 0;
        for (int k = 0; k < 2; ++k) {
            MT_CUDA(ctx, cudaMalloc((void**)&ctx->d_tiles[k], cap * sizeof(mt::BatchTile)));
            MT_CUDA(ctx, cudaHostAlloc((void**)&ctx->h_tiles[k], cap * sizeof(mt::BatchTile), cudaHostAllocDefault));
        }
        ctx->cap_tiles = cap;
    }
    return MT_OK;
}

// The ray grid of a view: pixels (full) or the 4x4 blocks whose slot pixel
// lies in the image and in the reference's dispatch (checkerboard).
void ray_grid(const mt::MarchArgs& a, int* nrx, int* nry) {
    if (a.flags & MT_RENDER_FULL) {
        *nrx = a.width;
        *nry = a.height;
        return;
    }
    const int id = a.time.frame_count_mod16;
    const int sx = a.params.slot_x[id], sy = a.params.slot_y[id];
    *nrx = a.width > sx ? std::min(a.groups_x, (a.width - sx + 3) / 4) : 0;
    *nry = a.height > sy ? std::min(a.groups_y, (a.height - sy + 3) / 4) : 0;
}

}  // namespace

MT_API mt_status mt_render_batch(mt_ctx* ctx, const mt_view* views, int n_views, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (n_views < 0 || (n_views > 0 && !views)) return fail(ctx, MT_ERR_INVALID_ARG, "bad view list");
    if (n_views == 0) return MT_OK;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    std::vector<mt::MarchArgs> args((size_t)n_views);
    bool count = false;
    for (int i = 0; i < n_views; ++i) {
        const mt_view& v = views[i];
        st = build_march_args(ctx, &v.camera, &v.camera_old, &v.time, &v.params, v.prev_rgba, v.cur_rgba,
                              v.godray_mask, v.width, v.height, v.flags, &args[(size_t)i]);
        if (st != MT_OK) {
            std::string m = ctx->err;
            return fail(ctx, st, "view %d: %s", i, m.c_str());
        }
        if (v.params.storage != views[0].params.storage)
            return fail(ctx, MT_ERR_INVALID_ARG, "view %d: all views of a batch must share one storage", i);
        count = count || (v.flags & MT_RENDER_COUNT);
        args[(size_t)i].bottom_up = ctx->batch_order == 0 ? 1 : 0;  // the order tile rows are handed out
    }
    // Tiles, most expensive views first (rays x steps), so the persistent
    // launch does not end on one large view.
    const int tw = ctx->batch_tile_w, th = ctx->batch_tile_h;
    std::vector<int> order((size_t)n_views);
    for (int i = 0; i < n_views; ++i) order[(size_t)i] = i;
    auto cost = [&](int i) {
        int nx, ny;
        ray_grid(args[(size_t)i], &nx, &ny);
        return (double)nx * ny * std::max(args[(size_t)i].params.steps_min, args[(size_t)i].params.steps_max);
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    std::vector<mt::BatchTile> tiles;
    for (int i : order) {
        int nx, ny;
        ray_grid(args[(size_t)i], &nx, &ny);
        // tile rows in the view's ray-row order (march_row)
        const int nty = (ny + th - 1) / th;
        for (int k = 0; k < nty; ++k) {
            const int y = mt::march_row(k, nty, args[(size_t)i].bottom_up != 0) * th;
            for (int x = 0; x < nx; x += tw) tiles.push_back(mt::BatchTile{i, x, y, nx, ny});
        }
    }
    if ((st = ensure_batch_buffers(ctx, (size_t)n_views, tiles.size())) != MT_OK) return st;
    // Slot: the batch that used it last (two calls ago) must have finished
    // before its staging is overwritten (host) and its tables reused (device).
    const int k = ctx->slot;
    ctx->slot ^= 1;
    if (ctx->slot_pending[k]) MT_CUDA(ctx, cudaEventSynchronize(ctx->slot_done[k]));
    mt::MarchArgs* h_views = ctx->h_views[k];
    mt::BatchTile* h_tiles = ctx->h_tiles[k];
    std::memcpy(h_views, args.data(), args.size() * sizeof(mt::MarchArgs));
    if (!tiles.empty()) std::memcpy(h_tiles, tiles.data(), tiles.size() * sizeof(mt::BatchTile));

    mt::BatchArgs b;
    b.views = ctx->d_views[k];
    b.tiles = ctx->d_tiles[k];
    b.counter = ctx->d_counter[k];
    b.stats = count ? ctx->stats : nullptr;
    b.n_tiles = (int32_t)tiles.size();
    b.tile_w = tw;
    b.tile_h = th;
    const int storage = views[0].params.storage;
    const int lanes = ctx->batch_lanes;
    int blocks = storage == MT_STORAGE_F16    ? mt::batch_blocks_f16(ctx->device, lanes)
                 : storage == MT_STORAGE_BF16 ? mt::batch_blocks_bf16(ctx->device, lanes)
                                              : mt::batch_blocks_u8(ctx->device, lanes);

    if (ctx->batch_direct) {
        // The same work as the graph below, issued on the caller's stream.
        cudaStream_t s = (cudaStream_t)stream;
        if (ctx->slot_pending[k]) MT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->slot_done[k], 0));
        MT_CUDA(ctx, cudaMemcpyAsync(ctx->d_views[k], h_views, args.size() * sizeof(mt::MarchArgs),
                                     cudaMemcpyHostToDevice, s));
        if (!tiles.empty())
            MT_CUDA(ctx, cudaMemcpyAsync(ctx->d_tiles[k], h_tiles, tiles.size() * sizeof(mt::BatchTile),
                                         cudaMemcpyHostToDevice, s));
        MT_CUDA(ctx, cudaMemsetAsync(ctx->d_counter[k], 0, sizeof(unsigned), s));
        for (int i = 0; i < n_views; ++i)
            if (!(args[(size_t)i].flags & MT_RENDER_FULL)) MT_CUDA(ctx, mt::launch_reproject(args[(size_t)i], s));
        if (!tiles.empty())
            MT_CUDA(ctx, storage == MT_STORAGE_F16    ? mt::launch_batch_f16(b, lanes, blocks, s)
                         : storage == MT_STORAGE_BF16 ? mt::launch_batch_bf16(b, lanes, blocks, s)
                                                      : mt::launch_batch_u8(b, lanes, blocks, s));
        MT_CUDA(ctx, cudaEventRecord(ctx->slot_done[k], s));
        ctx->slot_pending[k] = true;
        return MT_OK;
    }

    cudaGraph_t graph = nullptr;
    cudaStream_t cs = ctx->cap_stream;
    MT_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemcpyAsync(ctx->d_views[k], h_views, args.size() * sizeof(mt::MarchArgs),
                                    cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && !tiles.empty())
        e = cudaMemcpyAsync(ctx->d_tiles[k], h_tiles, tiles.size() * sizeof(mt::BatchTile), cudaMemcpyHostToDevice,
                            cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_counter[k], 0, sizeof(unsigned), cs);
    for (int i = 0; e == cudaSuccess && i < n_views; ++i)
        if (!(args[(size_t)i].flags & MT_RENDER_FULL)) e = mt::launch_reproject(args[(size_t)i], cs);
    if (e == cudaSuccess && !tiles.empty()) {
        e = storage == MT_STORAGE_F16    ? mt::launch_batch_f16(b, lanes, blocks, cs)
            : storage == MT_STORAGE_BF16 ? mt::launch_batch_bf16(b, lanes, blocks, cs)
                                         : mt::launch_batch_u8(b, lanes, blocks, cs);
    }
    cudaError_t e_end = cudaStreamEndCapture(cs, &graph);
    if (e != cudaSuccess || e_end != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(ctx, MT_ERR_CUDA, "batch graph capture failed: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e_end));
    }
    bool updated = false;
    cudaGraphExec_t& exec = ctx->batch_exec[k];
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess;
        if (!updated) {
            cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    if (!updated) {
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            return fail(ctx, MT_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
        }
    }
    cudaGraphDestroy(graph);
    // The slot's previous batch must be done with its device tables,
    // whatever stream it ran on; batches in the other slot may overlap.
    if (ctx->slot_pending[k]) MT_CUDA(ctx, cudaStreamWaitEvent((cudaStream_t)stream, ctx->slot_done[k], 0));
    MT_CUDA(ctx, cudaGraphLaunch(exec, (cudaStream_t)stream));
    MT_CUDA(ctx, cudaEventRecord(ctx->slot_done[k], (cudaStream_t)stream));
    ctx->slot_pending[k] = true;
    return MT_OK;
}

MT_API mt_status mt_autotune_batch(mt_ctx* ctx, const mt_view* views, int n_views, void* stream, mt_tuning* best) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!best) return fail(ctx, MT_ERR_INVALID_ARG, "best must not be NULL");
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    const int shapes[4][2] = {{8, 8}, {16, 8}, {16, 16}, {32, 8}};
    const int lane_choices[3] = {1, 4, 8};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaError_t e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e != cudaSuccess) {
        if (t0) cudaEventDestroy(t0);
        return fail(ctx, MT_ERR_CUDA, "CUDA error %s (%s) creating the autotuner's events", cudaGetErrorName(e),
                    cudaGetErrorString(e));
    }
    float best_ms = -1.0f;
    int bw = ctx->batch_tile_w, bh = ctx->batch_tile_h, bl = ctx->batch_lanes, bo = ctx->batch_order;
    st = mt_render_batch(ctx, views, n_views, stream);  // warm-up
    for (int oi = 0; st == MT_OK && oi < 2; ++oi)
        for (int li = 0; st == MT_OK && li < 3; ++li)
            for (int si = 0; st == MT_OK && si < 4; ++si) {
                ctx->batch_tile_w = shapes[si][0];
                ctx->batch_tile_h = shapes[si][1];
                ctx->batch_lanes = lane_choices[li];
                ctx->batch_order = oi;
                float ms = -1.0f;
                for (int rep = 0; st == MT_OK && rep < 2; ++rep) {  // the faster of two runs
                    cudaEventRecord(t0, (cudaStream_t)stream);
                    st = mt_render_batch(ctx, views, n_views, stream);
                    cudaEventRecord(t1, (cudaStream_t)stream);
                    if (st != MT_OK) break;
                    float m = 0.0f;
                    e = cudaEventSynchronize(t1);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&m, t0, t1);
                    if (e != cudaSuccess) {
                        st = fail(ctx, MT_ERR_CUDA, "CUDA error %s (%s) timing a tuning candidate", cudaGetErrorName(e),
                                  cudaGetErrorString(e));
                        break;
                    }
                    if (ms < 0.0f || m < ms) ms = m;
                }
                if (st == MT_OK && (best_ms < 0.0f || ms < best_ms)) {
                    best_ms = ms;
                    bw = shapes[si][0];
                    bh = shapes[si][1];
                    bl = lane_choices[li];
                    bo = oi;
                }
            }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    ctx->batch_tile_w = bw;
    ctx->batch_tile_h = bh;
    ctx->batch_lanes = bl;
    ctx->batch_order = bo;
    if (st != MT_OK) return st;
    return mt_get_tuning(ctx, best);
}

MT_API mt_status mt_get_stats(mt_ctx* ctx, mt_stats* out, int reset, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, MT_ERR_INVALID_ARG, "out must not be NULL");
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    MT_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    unsigned long long h[4];
    MT_CUDA(ctx, cudaMemcpy(h, ctx->stats, sizeof(h), cudaMemcpyDeviceToHost));
    out->primary_samples = h[0];
    out->light_samples = h[1];
    out->marched_rays = h[2];
    out->pixels = h[3];
    if (reset) MT_CUDA(ctx, cudaMemset(ctx->stats, 0, sizeof(h)));
    return MT_OK;
}

MT_API mt_status mt_set_tuning(mt_ctx* ctx, const mt_tuning* t) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!t) return fail(ctx, MT_ERR_INVALID_ARG, "tuning must not be NULL");
    if (t->march_lanes != 0 && t->march_lanes != 1 && t->march_lanes != 4 && t->march_lanes != 8 &&
        t->march_lanes != 16)
        return fail(ctx, MT_ERR_INVALID_ARG, "march_lanes must be 0 (auto), 1, 4, 8 or 16 (got %d)",
                    t->march_lanes);
    if (t->fused_resolve != 0 && t->fused_resolve != 1)
        return fail(ctx, MT_ERR_INVALID_ARG, "fused_resolve must be 0 or 1");
    if (t->batch_tile_w < 1 || t->batch_tile_h < 1 || t->batch_tile_w * t->batch_tile_h > 4096)
        return fail(ctx, MT_ERR_INVALID_ARG, "batch tile must be 1..4096 rays");
    if (t->batch_lanes != 1 && t->batch_lanes != 4 && t->batch_lanes != 8 && t->batch_lanes != 16)
        return fail(ctx, MT_ERR_INVALID_ARG, "batch_lanes must be 1, 4, 8 or 16");
    if (t->batch_direct != 0 && t->batch_direct != 1) return fail(ctx, MT_ERR_INVALID_ARG, "batch_direct must be 0 or 1");
    if (t->reproject_serial != 0 && t->reproject_serial != 1)
        return fail(ctx, MT_ERR_INVALID_ARG, "reproject_serial must be 0 or 1");
    if (t->march_block != 0 && t->march_block != 32 && t->march_block != 128 && t->march_block != 256)
        return fail(ctx, MT_ERR_INVALID_ARG, "march_block must be 0 (default 256), 32, 128 or 256");
    if (t->march_order != 0 && t->march_order != 1) return fail(ctx, MT_ERR_INVALID_ARG, "march_order must be 0 or 1");
    if (t->batch_order != 0 && t->batch_order != 1) return fail(ctx, MT_ERR_INVALID_ARG, "batch_order must be 0 or 1");
    ctx->march_lanes = t->march_lanes;
    ctx->fused_resolve = t->fused_resolve;
    ctx->batch_tile_w = t->batch_tile_w;
    ctx->batch_tile_h = t->batch_tile_h;
    ctx->batch_lanes = t->batch_lanes;
    ctx->batch_direct = t->batch_direct;
    ctx->overlap = t->reproject_serial ? 0 : 1;
    ctx->march_block = t->march_block == 0 ? 256 : t->march_block;
    ctx->march_order = t->march_order;
    ctx->batch_order = t->batch_order;
    return MT_OK;
}

MT_API mt_status mt_get_tuning(mt_ctx* ctx, mt_tuning* t) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!t) return fail(ctx, MT_ERR_INVALID_ARG, "tuning must not be NULL");
    std::memset(t, 0, sizeof(*t));
    t->march_lanes = ctx->march_lanes;
    t->fused_resolve = ctx->fused_resolve;
    t->batch_tile_w = ctx->batch_tile_w;
    t->batch_tile_h = ctx->batch_tile_h;
    t->batch_lanes = ctx->batch_lanes;
    t->batch_direct = ctx->batch_direct;
    t->reproject_serial = ctx->overlap ? 0 : 1;
    t->march_block = ctx->march_block;
    t->march_order = ctx->march_order;
    t->batch_order = ctx->batch_order;
    return MT_OK;
}

MT_API mt_status mt_selftest_division(mt_ctx* ctx, const float* a, const float* b, float* out_rdiv, float* out_ieee,
                                      int n, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (n < 0 || (n > 0 && (!a || !b || !out_rdiv || !out_ieee)))
        return fail(ctx, MT_ERR_INVALID_ARG, "bad self-test buffers");
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    MT_CUDA(ctx, mt::launch_selftest_division(a, b, out_rdiv, out_ieee, n, (cudaStream_t)stream));
    return MT_OK;
}

MT_API mt_status mt_set_timing(mt_ctx* ctx, int enabled) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    if (enabled && !ctx->ev[0])
        for (cudaEvent_t& e : ctx->ev) MT_CUDA(ctx, cudaEventCreate(&e));
    ctx->timing = enabled != 0;
    ctx->ran[0] = ctx->ran[1] = ctx->ran[2] = ctx->ran[3] = false;
    return MT_OK;
}

MT_API mt_status mt_get_kernel_times(mt_ctx* ctx, mt_kernel_times* out) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, MT_ERR_INVALID_ARG, "out must not be NULL");
    std::memset(out, 0, sizeof(*out));
    if (!ctx->ev[0]) return MT_OK;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    float* dst[4] = {&out->reproject_ms, &out->march_ms, &out->txaa_ms, &out->resolve_ms};
    for (int k = 0; k < 4; ++k) {
        if (!ctx->ran[k]) continue;
        MT_CUDA(ctx, cudaEventSynchronize(ctx->ev[2 * k + 1]));
        MT_CUDA(ctx, cudaEventElapsedTime(dst[k], ctx->ev[2 * k], ctx->ev[2 * k + 1]));
    }
    return MT_OK;
}

}  // extern "C"

// ---- mt_render_batch_noalloc -------------------------------------------
// The batched raymarch with its view table, tile list and work counter in one
// fixed device array of this library instead of buffers the context
// allocates.  Layout (bytes): [0, 256) work counter; [256, 256 + views)
// MT_NOALLOC_MAX_VIEWS view tables; then MT_NOALLOC_MAX_TILES tiles.
//
// Nothing is staged in host memory: the view tables travel to the device as
// the parameters of small store kernels (kNoallocStoreViews views a launch;
// the launch copies its parameters, so nothing on the host is read after the
// call returns), and the tile list is generated on the device from a small
// per-view description, in the order mt_render_batch builds it on the host.
// The call never waits for the device.
namespace {

constexpr size_t kNoallocViewsOff = 256;
constexpr size_t kNoallocViewsBytes =
    ((MT_NOALLOC_MAX_VIEWS * sizeof(mt::MarchArgs) + 255) / 256) * 256;
constexpr size_t kNoallocTilesOff = kNoallocViewsOff + kNoallocViewsBytes;
constexpr size_t kNoallocBytes = kNoallocTilesOff + MT_NOALLOC_MAX_TILES * sizeof(mt::BatchTile);
constexpr int kNoallocMaxDevices = 64;
static_assert(alignof(mt::MarchArgs) <= 256 && alignof(mt::BatchTile) <= 256, "scratch layout");
static_assert(sizeof(mt::MarchArgs) % 4 == 0, "view tables are stored as 32-bit words");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Views per store launch: 16 view tables (~26 KB) stay inside the 32 KB of
// kernel parameter space.
constexpr int kNoallocStoreViews = 16;
constexpr int kViewWords = (int)(sizeof(mt::MarchArgs) / 4);

struct NoallocStore {
    uint32_t words[kNoallocStoreViews * kViewWords];  // the view tables, as words
    int32_t first_view, n_views;
};
static_assert(sizeof(NoallocStore) <= 32000, "kernel parameter space");

// Copies n_views view tables into the array at view first_view, one CTA a
// view (a warp's parameter-space reads at 32 different words are served one
// word at a time, so the copies are spread over SMs); the launch holding
// view 0 also zeroes the work counter.
__global__ void noalloc_store_kernel(const __grid_constant__ NoallocStore p, unsigned char* scratch) {
    const int v = blockIdx.x;
    if (v >= p.n_views) return;
    uint32_t* dst = reinterpret_cast<uint32_t*>(scratch + kNoallocViewsOff) + (size_t)(p.first_view + v) * kViewWords;
    const uint32_t* src = p.words + (size_t)v * kViewWords;
    for (int i = threadIdx.x; i < kViewWords; i += blockDim.x) dst[i] = src[i];
    if (p.first_view == 0 && v == 0 && threadIdx.x == 0) *reinterpret_cast<unsigned*>(scratch) = 0u;
}

// The tile list's description: views in hand-out order with their ray grids
// and the running tile count before each.
struct NoallocTileSpec {
    int32_t n_views, n_tiles, tile_w, tile_h;
    int32_t view[MT_NOALLOC_MAX_VIEWS];
    int32_t nx[MT_NOALLOC_MAX_VIEWS], ny[MT_NOALLOC_MAX_VIEWS];
    int32_t bottom_up[MT_NOALLOC_MAX_VIEWS];
    int32_t first[MT_NOALLOC_MAX_VIEWS + 1];
};

// Tile t of the list: the ordered view o with first[o] <= t < first[o + 1],
// then its tile rows in march_row order, tw-wide tiles left to right in each
// (the host loop of mt_render_batch, unrolled by index).
__global__ void noalloc_tiles_kernel(const __grid_constant__ NoallocTileSpec p, unsigned char* scratch) {
    mt::BatchTile* tiles = reinterpret_cast<mt::BatchTile*>(scratch + kNoallocTilesOff);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < p.n_tiles; t += gridDim.x * blockDim.x) {
        int lo = 0, hi = p.n_views - 1;  // last o with first[o] <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (p.first[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const int o = lo, nx = p.nx[o], ny = p.ny[o];
        const int ntx = (nx + p.tile_w - 1) / p.tile_w, nty = (ny + p.tile_h - 1) / p.tile_h;
        const int local = t - p.first[o];
        const int k = local / ntx, xi = local - k * ntx;
        tiles[t] = mt::BatchTile{p.view[o], xi * p.tile_w, mt::march_row(k, nty, p.bottom_up[o] != 0) * p.tile_h,
                                 nx, ny};
    }
}

// Address of the array on each device, looked up (cudaGetSymbolAddress, with
// the device current) on the first call made on that device.
std::mutex g_noalloc_lookup_mu;
unsigned char* g_noalloc_dev[kNoallocMaxDevices] = {};

mt_status noalloc_scratch(mt_ctx* ctx, unsigned char** out) {
    if (ctx->device < 0 || ctx->device >= kNoallocMaxDevices)
        return fail(ctx, MT_ERR_UNSUPPORTED, "device %d is beyond the %d devices of the fixed scratch table",
                    ctx->device, kNoallocMaxDevices);
    std::lock_guard<std::mutex> lk(g_noalloc_lookup_mu);
    if (!g_noalloc_dev[ctx->device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(ctx, MT_ERR_CUDA, "cudaGetSymbolAddress of the batch scratch: %s", cudaGetErrorString(e));
        g_noalloc_dev[ctx->device] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_dev[ctx->device];
    return MT_OK;
}

}  // namespace

extern "C" {

MT_API mt_status mt_render_batch_noalloc(mt_ctx* ctx, const mt_view* views, int n_views, void* stream) {
    if (!ctx) return MT_ERR_INVALID_ARG;
    if (n_views < 0 || (n_views > 0 && !views)) return fail(ctx, MT_ERR_INVALID_ARG, "bad view list");
    if (n_views > MT_NOALLOC_MAX_VIEWS)
        return fail(ctx, MT_ERR_INVALID_ARG, "%d views exceed the fixed table of %d views", n_views,
                    MT_NOALLOC_MAX_VIEWS);
    if (n_views == 0) return MT_OK;
    mt_status st;
    if ((st = bind_device(ctx)) != MT_OK) return st;
    unsigned char* dev = nullptr;
    if ((st = noalloc_scratch(ctx, &dev)) != MT_OK) return st;
    // Pass 1: validate every view and describe its ray grid, before anything
    // is launched (a rejected batch leaves the array as it was).
    NoallocTileSpec spec;
    std::memset(&spec, 0, sizeof(spec));
    mt::MarchArgs a;
    double cost[MT_NOALLOC_MAX_VIEWS];
    int nx[MT_NOALLOC_MAX_VIEWS], ny[MT_NOALLOC_MAX_VIEWS], bu[MT_NOALLOC_MAX_VIEWS], order[MT_NOALLOC_MAX_VIEWS];
    bool count = false;
    for (int i = 0; i < n_views; ++i) {
        const mt_view& v = views[i];
        st = build_march_args(ctx, &v.camera, &v.camera_old, &v.time, &v.params, v.prev_rgba, v.cur_rgba,
                              v.godray_mask, v.width, v.height, v.flags, &a);
        if (st != MT_OK) {
            const std::string m = ctx->err;
            return fail(ctx, st, "view %d: %s", i, m.c_str());
        }
        if (v.params.storage != views[0].params.storage)
            return fail(ctx, MT_ERR_INVALID_ARG, "view %d: all views of a batch must share one storage", i);
        count = count || (v.flags & MT_RENDER_COUNT);
        ray_grid(a, &nx[i], &ny[i]);
        bu[i] = ctx->batch_order == 0 ? 1 : 0;  // the order tile rows are handed out
        // most expensive views first, stable (mt_render_batch's order)
        cost[i] = (double)nx[i] * ny[i] * std::max(a.params.steps_min, a.params.steps_max);
        int j = i;
        while (j > 0 && cost[order[j - 1]] < cost[i]) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = i;
    }
    const int tw = ctx->batch_tile_w, th = ctx->batch_tile_h;
    long long n_tiles = 0;
    for (int o = 0; o < n_views; ++o) {
        const int i = order[o];
        spec.view[o] = i;
        spec.nx[o] = nx[i];
        spec.ny[o] = ny[i];
        spec.bottom_up[o] = bu[i];
        spec.first[o] = (int32_t)std::min<long long>(n_tiles, MT_NOALLOC_MAX_TILES + 1);
        n_tiles += (long long)((nx[i] + tw - 1) / tw) * ((ny[i] + th - 1) / th);
    }
    if (n_tiles > MT_NOALLOC_MAX_TILES)
        return fail(ctx, MT_ERR_INVALID_ARG,
                    "the batch needs %lld tiles of %dx%d rays; the fixed tile list holds %d", n_tiles, tw, th,
                    MT_NOALLOC_MAX_TILES);
    spec.first[n_views] = (int32_t)n_tiles;
    spec.n_views = n_views;
    spec.n_tiles = (int32_t)n_tiles;
    spec.tile_w = tw;
    spec.tile_h = th;
    // Pass 2: the view tables, kNoallocStoreViews views per store launch
    // (the first launch also zeroes the work counter), then the tile list.
    cudaStream_t s = (cudaStream_t)stream;
    NoallocStore store;
    for (int v0 = 0; v0 < n_views; v0 += kNoallocStoreViews) {
        store.first_view = v0;
        store.n_views = std::min(kNoallocStoreViews, n_views - v0);
        for (int k = 0; k < store.n_views; ++k) {
            const mt_view& v = views[v0 + k];
            build_march_args(ctx, &v.camera, &v.camera_old, &v.time, &v.params, v.prev_rgba, v.cur_rgba,
                             v.godray_mask, v.width, v.height, v.flags, &a);  // validated above
            std::memcpy(store.words + (size_t)k * kViewWords, &a, sizeof(a));
            // the view's reprojection reads nothing of the array: launched as its table is built
            if (!(a.flags & MT_RENDER_FULL)) MT_CUDA(ctx, mt::launch_reproject(a, s));
        }
        noalloc_store_kernel<<<store.n_views, 256, 0, s>>>(store, dev);
        MT_CUDA(ctx, cudaGetLastError());
    }
    if (n_tiles == 0) return MT_OK;
    {
        const int blocks = (int)std::min<long long>((n_tiles + 255) / 256, 128);
        noalloc_tiles_kernel<<<blocks, 256, 0, s>>>(spec, dev);
        MT_CUDA(ctx, cudaGetLastError());
    }
    mt::BatchArgs b;
    b.views = reinterpret_cast<const mt::MarchArgs*>(dev + kNoallocViewsOff);
    b.tiles = reinterpret_cast<const mt::BatchTile*>(dev + kNoallocTilesOff);
    b.counter = reinterpret_cast<unsigned*>(dev);
    b.stats = count ? ctx->stats : nullptr;
    b.n_tiles = (int32_t)n_tiles;
    b.tile_w = tw;
    b.tile_h = th;
    const int storage = views[0].params.storage;
    const int lanes = ctx->batch_lanes;
    const int blocks = storage == MT_STORAGE_F16    ? mt::batch_blocks_f16(ctx->device, lanes)
                       : storage == MT_STORAGE_BF16 ? mt::batch_blocks_bf16(ctx->device, lanes)
                                                    : mt::batch_blocks_u8(ctx->device, lanes);
    MT_CUDA(ctx, storage == MT_STORAGE_F16    ? mt::launch_batch_f16(b, lanes, blocks, s)
                 : storage == MT_STORAGE_BF16 ? mt::launch_batch_bf16(b, lanes, blocks, s)
                                              : mt::launch_batch_u8(b, lanes, blocks, s));
    return MT_OK;
}

}  // extern "C"
