// Reprojection and TXAA kernels of the compute stage, and the launchers of
// every render kernel (the raymarch itself lives in mt_march.cuh).
//
//   march_kernel        <- shaders/cloudRayMarch.comp:690-826 (one thread per
//                          marched pixel)
//   reproject_kernel    <- shaders/reprojection.comp:193-244 (one thread per
//                          pixel not marched this frame)
//   txaa_kernel         <- shaders/postProcess_TXAA.frag:223-269 (one thread
//                          per pixel)
//
// The reference runs reprojection over every pixel and then the raymarch over
// one pixel per 4x4 block with no barrier between the two dispatches
// (Renderer.cpp:688-716); the marched pixel is meant to win.  Here the two
// kernels write disjoint pixel sets, so the outcome is defined and the two
// launches can overlap.
//
// Compiled with -fmad=false: see mt_device.cuh.  The divisions are inlined
// (MT_DIV_INLINE): these kernels are small enough for the instruction cache.
#define MT_DIV_INLINE 1
#include <cuda_runtime.h>

#include "mt_shared.cuh"

namespace mt {

// Pixels the checkerboard raymarch writes this frame (cloudRayMarch.comp:695-701
// under the dispatch of Renderer.cpp:713-716).
MT_HD bool is_marched(const MarchArgs& a, int x, int y) {
    const int id = a.time.frame_count_mod16;
    const int dx = x - a.params.slot_x[id], dy = y - a.params.slot_y[id];
    return dx >= 0 && dy >= 0 && (dx & 3) == 0 && (dy & 3) == 0 && (dx >> 2) < a.groups_x && (dy >> 2) < a.groups_y;
}

// The previous camera's uv of the inner-shell hit of the ray through screen
// point (sx, sy) (reprojection.comp:205-222, postProcess_TXAA.frag:230-247):
// cast_ray (cloudRayMarch.comp:194-226) and ray_sphere (:229-273) with the
// uniform parts taken from `v`.
MT_HD Rcp rcp_of(const float r[2]) { return Rcp{r[0], r[1]}; }

MT_HD void old_uv(const ViewConsts& v, float sx, float sy, float& old_u, float& old_v) {
    const f3 rD = cast_ray(v, ld3(v.eye), sx, sy).direction;
    const f3 ro = ld3(v.ro);
    f3 q{0.0f, 0.0f, 0.0f};
    const float A = dot3(rD, rD);
    const float B = 2.0f * dot3(rD, ro);
    const float disc = B * B - 4.0f * A * v.C;
    if (!(disc < 0.0f)) {
        // the first root's sign is its numerator's (2A > 0): one division
        const float sq = sqrtf(disc), n1 = -B - sq;
        const float t = (n1 < 0.0f ? -B + sq : n1) / (2.0f * A);
        if (t >= 0.0f) {
            f3 pnt = ro + t * rD;
            pnt = pnt * v.Rin;
            q = pnt + ld3(v.ec);
        }
    }
    const float* ov = v.ov;
    f3 od{ov[0] * q.x + ov[4] * q.y + ov[8] * q.z + ov[12] * 1.0f, ov[1] * q.x + ov[5] * q.y + ov[9] * q.z + ov[13] * 1.0f,
          ov[2] * q.x + ov[6] * q.y + ov[10] * q.z + ov[14] * 1.0f};
    od = normalize3_r(od);
    od = rdiv3(od, make_rcp(-od.z));
    old_u = rdiv(od.x, rcp_of(v.r_tanx)) * 0.5f + 0.5f;
    old_v = rdiv(od.y, rcp_of(v.r_tany)) * 0.5f + 0.5f;
}

// reprojection.comp:193-244 for pixel (x, y).
MT_HD f4v reproject_pixel(const MarchArgs& a, const ViewConsts& v, int x, int y) {
    const int W = a.width, H = a.height;
    const float ux = rdiv((float)x, rcp_of(v.r_w)), uy = rdiv((float)y, rcp_of(v.r_h));
    float old_u, old_v;
    old_uv(v, ux, uy, old_u, old_v);
    const float mx = old_u - ux, my = old_v - uy;
    // (old - m * f) * (W, H) for u and v as one packed pair; the blur sum in pairs
    const float2 o2 = make_float2(old_u, old_v), m2 = make_float2(mx, my), wh = make_float2((float)W, (float)H);
    f4p blur{make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const float f = (float)i / 10.0f;
        const float2 q = mul2(sub2(o2, mul2(m2, splat2(f))), wh);
        const int ix = imin(imax(f2i(roundf(q.x)), 0), W - 1);
        const int iy = imin(imax(f2i(roundf(q.y)), 0), H - 1);
        const float4 s = __ldg(a.prev + (size_t)iy * (size_t)W + (size_t)ix);
        blur = add4p(blur, f4p{make_float2(s.x, s.y), make_float2(s.z, s.w)});
    }
    return unpack4(rdiv4p(blur, MT_RCP(0.0f, 10.0f)));
}

// The centre pixel of fragment (x, y)'s neighbourhood: pixelPos of
// postProcess_TXAA.frag:227 with in_uv at the fragment centre.
MT_HD void txaa_centre(const ViewConsts& v, int x, int y, int W, int H, float& iux, float& iuy, int& ppx, int& ppy) {
    iux = rdiv((float)x + 0.5f, rcp_of(v.r_w));
    iuy = rdiv((float)y + 0.5f, rcp_of(v.r_h));
    ppx = imin(imax(f2i(roundf((float)W * iux)), 0), W - 1);
    ppy = imin(imax(f2i(roundf((float)H * iuy)), 0), H - 1);
}

// A value the TXAA fast path accepts: non-negative and not NaN (+0 up to +inf).
MT_HD bool txaa_plain(float4 c) {
    const unsigned lim = 0x7f800000u;
    return (__float_as_uint(c.x) <= lim) & (__float_as_uint(c.y) <= lim) & (__float_as_uint(c.z) <= lim) &
           (__float_as_uint(c.w) <= lim);
}
MT_HD f4v fmin4(f4v a, f4v b) { return f4v{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w)}; }
MT_HD f4v fmax4(f4v a, f4v b) { return f4v{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w)}; }

// postProcess_TXAA.frag:223-269 for fragment (x, y); `load(i, j)` reads the
// current frame (0 outside the image, as imageLoad does).  PLAIN: every value
// `load` can return is non-negative and not NaN (txaa_plain).  Then the
// neighbourhood minimum and maximum are the same value whatever the order of
// comparison (equal non-negative floats have equal bits), so min/max
// instructions over shared partial results replace the shader's nested
// compare-selects, bit for bit.
template <bool PLAIN, class Load>
MT_HD f4v txaa_resolve(const mt_params& p, const ViewConsts& v, f4v prev, int x, int y, int W, int H, Load load) {
    float iux, iuy;
    int ppx, ppy;
    txaa_centre(v, x, y, W, H, iux, iuy, ppx, ppy);
    f4v ctl = load(ppx - 1, ppy - 1), ctc = load(ppx, ppy - 1), ctr = load(ppx + 1, ppy - 1);
    f4v cml = load(ppx - 1, ppy), cmc = load(ppx, ppy), cmr = load(ppx + 1, ppy);
    f4v cbl = load(ppx - 1, ppy + 1), cbc = load(ppx, ppy + 1), cbr = load(ppx + 1, ppy + 1);
    f4v cmin, cmax, cmin5, cmax5;
    if (PLAIN) {
        cmin5 = fmin4(fmin4(fmin4(ctc, cml), fmin4(cmc, cmr)), cbc);
        cmax5 = fmax4(fmax4(fmax4(ctc, cml), fmax4(cmc, cmr)), cbc);
        cmin = fmin4(cmin5, fmin4(fmin4(ctl, ctr), fmin4(cbl, cbr)));
        cmax = fmax4(cmax5, fmax4(fmax4(ctl, ctr), fmax4(cbl, cbr)));
    } else {
        cmin = min4(ctl, min4(ctc, min4(ctr, min4(cml, min4(cmc, min4(cmr, min4(cbl, min4(cbc, cbr))))))));
        cmax = max4(ctl, max4(ctc, max4(ctr, max4(cml, max4(cmc, max4(cmr, max4(cbl, max4(cbc, cbr))))))));
        cmin5 = min4(ctc, min4(cml, min4(cmc, min4(cmr, cbc))));
        cmax5 = max4(ctc, max4(cml, max4(cmc, max4(cmr, cbc))));
    }
    // sums left to right as the shader adds them, channels in packed pairs
    const f4p pctc = pack4(ctc), pcml = pack4(cml), pcmc = pack4(cmc), pcmr = pack4(cmr), pcbc = pack4(cbc);
    const f4p s9 = add4p(add4p(add4p(add4p(add4p(add4p(add4p(add4p(pack4(ctl), pctc), pack4(ctr)), pcml), pcmc), pcmr),
                                     pack4(cbl)), pcbc), pack4(cbr));
    const f4p s5 = add4p(add4p(add4p(add4p(pctc, pcml), pcmc), pcmr), pcbc);
    const Rcp r9 = MT_RCP(0.0f, 9.0f), r5 = MT_RCP(0.0f, 5.0f);
    const f4p cavg9 = rdiv4p(s9, r9), cavg5 = rdiv4p(s5, r5);
    // 0.5 * (a + b) per channel
    cmin = unpack4(mul4p(add4p(pack4(cmin), pack4(cmin5)), 0.5f));
    cmax = unpack4(mul4p(add4p(pack4(cmax), pack4(cmax5)), 0.5f));
    const f4v cavg = unpack4(mul4p(add4p(cavg9, cavg5), 0.5f));
    f4v curr = cmc;
    // clip_aabb (:171-191)
    f4v pc = min4(max4(cavg, cmin), cmax);
    f3 p_clip{0.5f * (cmax.x + cmin.x), 0.5f * (cmax.y + cmin.y), 0.5f * (cmax.z + cmin.z)};
    const float EPS = 0.0000000001f;
    f3 e_clip{0.5f * (cmax.x - cmin.x) + EPS, 0.5f * (cmax.y - cmin.y) + EPS, 0.5f * (cmax.z - cmin.z) + EPS};
    f4v v_clip = prev - f4v{p_clip.x, p_clip.y, p_clip.z, pc.w};
    float vux = fabsf(v_clip.x / e_clip.x), vuy = fabsf(v_clip.y / e_clip.y), vuz = fabsf(v_clip.z / e_clip.z);
    float ma = gmax(vux, gmax(vuy, vuz));
    if (ma > 1.0f) {
        const Rcp rm = make_rcp(ma);
        prev = f4v{p_clip.x, p_clip.y, p_clip.z, pc.w} +
               f4v{rdiv(v_clip.x, rm), rdiv(v_clip.y, rm), rdiv(v_clip.z, rm), rdiv(v_clip.w, rm)};
    }
    const f3 lw{0.2125f, 0.7154f, 0.0721f};
    float lum0 = dot3(f3{curr.x, curr.y, curr.z}, lw);
    float lum1 = dot3(f3{prev.x, prev.y, prev.z}, lw);
    float ud = fabsf(lum0 - lum1) / gmax(lum0, gmax(lum1, 0.2f));
    float uw = 1.0f - ud;
    float k = gmix(p.feedback_min, p.feedback_max, uw * uw);
    // mix(prev, curr, k) = prev * (1 - k) + curr * k per channel
    return unpack4(add4p(mul4p(pack4(prev), 1.0f - k), mul4p(pack4(curr), k)));
}

// The history tap of fragment (x, y): the previous resolved frame sampled at
// the previous camera's uv (postProcess_TXAA.frag:230-249).  It depends on the
// uniforms and the history only, not on the current frame.
MT_HD f4v txaa_history(const ViewConsts& v, const float4* __restrict__ history, int x, int y, int W, int H) {
    float iux, iuy;
    int ppx, ppy;
    txaa_centre(v, x, y, W, H, iux, iuy, ppx, ppy);
    float old_u, old_v;
    old_uv(v, iux, iuy, old_u, old_v);
    return tex2_border(history, W, H, old_u, old_v);
}

template <bool PLAIN, class Load>
MT_HD f4v txaa_pixel(const mt_params& p, const ViewConsts& v, const float4* __restrict__ history, int x, int y, int W,
                     int H, Load load) {
    return txaa_resolve<PLAIN>(p, v, txaa_history(v, history, x, y, W, H), x, y, W, H, load);
}

// reprojection.comp:193-244 for every pixel the march does not write.
// 2D grid of 32x8-pixel CTAs (no index division; neighbouring taps share L1).
__global__ void __launch_bounds__(256) reproject_kernel(const __grid_constant__ MarchArgs a) {
    const int W = a.width, H = a.height;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const bool active = x < W && y < H && !is_marched(a, x, y);
    if (active) {
        const f4v b = reproject_pixel(a, a.vc_repro, x, y);
        a.cur[(size_t)y * (size_t)W + (size_t)x] = make_float4(b.x, b.y, b.z, b.w);
    }
    if (a.stats) {
        Counts none{0u, 0u, 0u};
        flush_counts(a.stats, none, active ? 1u : 0u);
    }
}

// postProcess_TXAA.frag:223-269 per output pixel (fragment).  A CTA stages
// the current frame over its pixels plus the halo the neighbourhoods reach
// (the centre is the fragment's pixel or the next one: one column/row before,
// two after) in shared memory, zero outside the image as imageLoad returns;
// the nine taps per pixel then read shared memory.
constexpr int kTxaaTW = 32, kTxaaTH = 8;

// The two per-pixel passes of a frame that do not depend on its raymarch, in
// one kernel run beside it: every pixel's TXAA history tap, into `out`
// (which the resolve then reads back and overwrites, pixel by pixel), and
// the reprojection of every pixel the raymarch does not write, into `cur`.
// One launch instead of two, and each thread has two independent chains.
__global__ void __launch_bounds__(kTxaaTW * kTxaaTH) history_reproject_kernel(const __grid_constant__ MarchArgs a,
                                                                              const __grid_constant__ TxaaArgs t) {
    const int W = a.width, H = a.height;
    const int x = blockIdx.x * kTxaaTW + threadIdx.x, y = blockIdx.y * kTxaaTH + threadIdx.y;
    const bool inside = x < W && y < H;
    const bool reproject = inside && !is_marched(a, x, y);
    if (inside) {
        const size_t o = (size_t)y * (size_t)W + (size_t)x;
        const f4v h = txaa_history(t.vc, t.history, x, y, W, H);
        if (reproject) {
            const f4v b = reproject_pixel(a, a.vc_repro, x, y);
            a.cur[o] = make_float4(b.x, b.y, b.z, b.w);
        }
        t.out[o] = make_float4(h.x, h.y, h.z, h.w);
    }
    if (a.stats) {
        Counts none{0u, 0u, 0u};
        flush_counts(a.stats, none, reproject ? 1u : 0u);
    }
}

// The resolve: a 32x8 CTA owns a 32x32 tile, each thread four pixels 8 rows
// apart (the halo and the barrier are shared by four times the pixels).
// HISTORY_IN_OUT: the history taps were stored in `out` by history_reproject_kernel.
constexpr int kTxaaRows = 4;
template <bool HISTORY_IN_OUT>
__global__ void __launch_bounds__(kTxaaTW * kTxaaTH, 4) txaa_kernel(const __grid_constant__ TxaaArgs a) {
    constexpr int TH = kTxaaTH * kTxaaRows, SW = kTxaaTW + 3, SH = TH + 3;
    __shared__ float4 tile[SH][SW];
    const int W = a.width, H = a.height;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int x0 = blockIdx.x * kTxaaTW - 1, y0 = blockIdx.y * TH - 1;
    const int x = blockIdx.x * kTxaaTW + threadIdx.x;
    const int ya = blockIdx.y * TH + threadIdx.y;
    bool plain = true;
    // every load of the tile in flight before the first shared-memory store
    constexpr int NT = kTxaaTW * kTxaaTH, NL = (SW * SH + NT - 1) / NT;
    float4 c[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) {
        const int i = tid + k * NT;
        const int gx = x0 + i % SW, gy = y0 + i / SW;
        c[k] = (i < SW * SH && gx >= 0 && gy >= 0 && gx < W && gy < H)
                   ? __ldg(a.current + (size_t)gy * (size_t)W + (size_t)gx)
                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
#pragma unroll
    for (int k = 0; k < NL; ++k) {
        const int i = tid + k * NT;
        if (i < SW * SH) {
            plain = plain & txaa_plain(c[k]);
            tile[i / SW][i % SW] = c[k];
        }
    }
    // the whole tile non-negative and NaN-free: the block takes the min/max path
    plain = __syncthreads_and(plain) != 0;
    auto load = [&](int i, int j) -> f4v {
        const float4 s = tile[j - y0][i - x0];
        return f4v{s.x, s.y, s.z, s.w};
    };
#pragma unroll 1
    for (int r = 0; r < kTxaaRows; ++r) {
        const int y = ya + r * kTxaaTH;
        if (!(x < W && y < H)) continue;
        const size_t o = (size_t)y * (size_t)W + (size_t)x;
        f4v prev;
        if (HISTORY_IN_OUT) {
            const float4 h = a.out[o];
            prev = f4v{h.x, h.y, h.z, h.w};
        } else {
            prev = txaa_history(a.vc, a.history, x, y, W, H);
        }
        const f4v res = plain ? txaa_resolve<true>(a.params, a.vc, prev, x, y, W, H, load)
                              : txaa_resolve<false>(a.params, a.vc, prev, x, y, W, H, load);
        a.out[o] = make_float4(res.x, res.y, res.z, res.w);
    }
}

// Reprojection fused with the TXAA resolve, after the raymarch of the frame.
// A block owns a TW x TH tile of output pixels.  It first builds the current
// frame over the tile plus the halo its TXAA neighbourhoods reach (one pixel
// left/up, two right/down: the neighbourhood centre is the fragment's pixel or
// the next one): marched pixels come from the march's output, the others are
// reprojected here.  It stores the reprojected pixels it owns (the raw frame
// the next frame reprojects from), then resolves every owned pixel's TXAA
// from shared memory.  Values equal those of reproject_kernel + txaa_kernel.
template <int TW, int TH>
__global__ void __launch_bounds__(TW * TH) resolve_kernel(const __grid_constant__ MarchArgs a) {
    constexpr int SW = TW + 3, SH = TH + 3;
    __shared__ float4 tile[SH][SW];
    const int W = a.width, H = a.height;
    const int x0 = blockIdx.x * TW - 1, y0 = blockIdx.y * TH - 1;
    const bool full = (a.flags & MT_RENDER_FULL) != 0;
    unsigned reprojected = 0;
    bool plain = true;
    for (int i = threadIdx.x; i < SW * SH; i += TW * TH) {
        const int sx = i % SW, sy = i / SW;
        const int x = x0 + sx, y = y0 + sy;
        f4v v{0.0f, 0.0f, 0.0f, 0.0f};
        if (x >= 0 && y >= 0 && x < W && y < H) {
            const size_t o = (size_t)y * (size_t)W + (size_t)x;
            if (full || is_marched(a, x, y)) {
                const float4 c = a.cur[o];
                v = f4v{c.x, c.y, c.z, c.w};
            } else {
                v = reproject_pixel(a, a.vc_repro, x, y);
                const bool owned = sx >= 1 && sy >= 1 && sx <= TW && sy <= TH;
                if (owned) {
                    a.cur[o] = make_float4(v.x, v.y, v.z, v.w);
                    ++reprojected;
                }
            }
        }
        const float4 c = make_float4(v.x, v.y, v.z, v.w);
        plain = plain & txaa_plain(c);
        tile[sy][sx] = c;
    }
    plain = __syncthreads_and(plain) != 0;
    const int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
    const int x = x0 + 1 + tx, y = y0 + 1 + ty;
    if (x < W && y < H) {
        auto load = [&](int i, int j) -> f4v {
            if (i < 0 || j < 0 || i >= W || j >= H) return f4v{0.0f, 0.0f, 0.0f, 0.0f};
            const float4 s = tile[j - y0][i - x0];
            return f4v{s.x, s.y, s.z, s.w};
        };
        const f4v r = plain ? txaa_pixel<true>(a.params, a.vc_txaa, a.history, x, y, W, H, load)
                            : txaa_pixel<false>(a.params, a.vc_txaa, a.history, x, y, W, H, load);
        a.out[(size_t)y * (size_t)W + (size_t)x] = make_float4(r.x, r.y, r.z, r.w);
    }
    if (a.stats) {
        Counts none{0u, 0u, 0u};
        flush_counts(a.stats, none, reprojected);
    }
}

// rdiv(a, 1/b) against the device's IEEE division, element by element.
__global__ void selftest_division_kernel(const float* __restrict__ a, const float* __restrict__ b, float* out_rdiv,
                                         float* out_ieee, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out_rdiv[i] = rdiv(a[i], make_rcp(b[i]));
    out_ieee[i] = a[i] / b[i];
}

}  // namespace mt

// ---------------------------------------------------------------------------
// Launchers (called from the C ABI in mt_capi.cu)
// ---------------------------------------------------------------------------
namespace mt {

static cudaError_t launch_march(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev) {
    const bool timed = ev && ev->on;
    const long long m = (a.flags & MT_RENDER_FULL) ? (long long)a.width * a.height
                                                   : (long long)a.groups_x * a.groups_y;
    // Images narrower or shorter than 4 pixels give the reference an empty
    // raymarch dispatch (Renderer.cpp:713-716): nothing is marched.
    if (timed) cudaEventRecord(ev->march[0], s);
    cudaError_t e = cudaSuccess;
    if (m > 0) {
        switch (a.params.storage) {
            case MT_STORAGE_F16: e = launch_march_f16(a, s, m); break;
            case MT_STORAGE_BF16: e = launch_march_bf16(a, s, m); break;
            default: e = launch_march_u8(a, s, m); break;
        }
    }
    if (timed) cudaEventRecord(ev->march[1], s);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_reproject(const MarchArgs& a, cudaStream_t s) {
    const dim3 block(32, 8), grid((unsigned)((a.width + 31) / 32), (unsigned)((a.height + 7) / 8));
    reproject_kernel<<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_render(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev, const ForkJoin* fj) {
    const bool timed = ev && ev->on;
    if (a.flags & MT_RENDER_FULL) return launch_march(a, s, ev);
    if (!fj) {
        if (timed) cudaEventRecord(ev->reproject[0], s);
        cudaError_t e = launch_reproject(a, s);
        if (timed) cudaEventRecord(ev->reproject[1], s);
        if (e != cudaSuccess) return e;
        return launch_march(a, s, ev);
    }
    // raymarch on s, reprojection beside it on aux (launched second, so the
    // raymarch's blocks are dispatched first and the reprojection fills in)
    cudaError_t e = cudaEventRecord(fj->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(fj->aux, fj->fork, 0);
    if (e != cudaSuccess) return e;
    e = launch_march(a, s, ev);
    if (e != cudaSuccess) return e;
    if (timed) cudaEventRecord(ev->reproject[0], fj->aux);
    e = launch_reproject(a, fj->aux);
    if (timed) cudaEventRecord(ev->reproject[1], fj->aux);
    if (e == cudaSuccess) e = cudaEventRecord(fj->join, fj->aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, fj->join, 0);
    return e;
}

constexpr int kResolveTW = 32, kResolveTH = 8;

cudaError_t launch_frame(const MarchArgs& a, cudaStream_t s, const LaunchEvents* ev, const ForkJoin* fj) {
    const bool timed = ev && ev->on;
    if (!a.fused_resolve) {
        TxaaArgs t;
        t.camera = a.camera;
        t.camera_old = a.camera_old;
        t.time = a.time;
        t.params = a.params;
        t.current = a.cur;
        t.history = a.history;
        t.out = a.out;
        t.width = a.width;
        t.height = a.height;
        t.vc = a.vc_txaa;
        if (!fj || (a.flags & MT_RENDER_FULL)) {
            // reprojection, raymarch, TXAA on one stream
            cudaError_t e = launch_render(a, s, ev, fj);
            if (e != cudaSuccess) return e;
            return launch_txaa(t, s, timed ? ev->resolve : nullptr);
        }
        // the raymarch on s, launched first so that its CTAs take the SMs
        // first; then on aux the TXAA history taps (they need only the
        // previous resolved frame) and the reprojection in one kernel, which
        // fills the raymarch's last waves; then the TXAA resolve on s
        const dim3 block(kTxaaTW, kTxaaTH),
            grid((unsigned)((a.width + kTxaaTW - 1) / kTxaaTW), (unsigned)((a.height + kTxaaTH - 1) / kTxaaTH));
        cudaError_t e = cudaEventRecord(fj->fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(fj->aux, fj->fork, 0);
        if (e == cudaSuccess) e = launch_march(a, s, ev);
        if (e != cudaSuccess) return e;
        if (timed) cudaEventRecord(ev->reproject[0], fj->aux);
        history_reproject_kernel<<<grid, block, 0, fj->aux>>>(a, t);
        e = cudaGetLastError();
        if (timed) cudaEventRecord(ev->reproject[1], fj->aux);
        if (e == cudaSuccess) e = cudaEventRecord(fj->join, fj->aux);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, fj->join, 0);
        if (e != cudaSuccess) return e;
        if (timed) cudaEventRecord(ev->resolve[0], s);
        const dim3 grid_r(grid.x, (unsigned)((a.height + kTxaaTH * kTxaaRows - 1) / (kTxaaTH * kTxaaRows)));
        txaa_kernel<true><<<grid_r, block, 0, s>>>(t);
        if (timed) cudaEventRecord(ev->resolve[1], s);
        return cudaGetLastError();
    }
    cudaError_t e = launch_march(a, s, ev);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((a.width + kResolveTW - 1) / kResolveTW), (unsigned)((a.height + kResolveTH - 1) / kResolveTH));
    if (timed) cudaEventRecord(ev->resolve[0], s);
    resolve_kernel<kResolveTW, kResolveTH><<<grid, kResolveTW * kResolveTH, 0, s>>>(a);
    if (timed) cudaEventRecord(ev->resolve[1], s);
    return cudaGetLastError();
}

cudaError_t launch_selftest_division(const float* a, const float* b, float* out_rdiv, float* out_ieee, int n,
                                     cudaStream_t s) {
    if (n > 0) selftest_division_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, b, out_rdiv, out_ieee, n);
    return cudaGetLastError();
}

cudaError_t launch_txaa(const TxaaArgs& a, cudaStream_t s, const cudaEvent_t* ev) {
    if (ev) cudaEventRecord(ev[0], s);
    const dim3 block(kTxaaTW, kTxaaTH), grid((unsigned)((a.width + kTxaaTW - 1) / kTxaaTW),
                                             (unsigned)((a.height + kTxaaTH * kTxaaRows - 1) / (kTxaaTH * kTxaaRows)));
    txaa_kernel<false><<<grid, block, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    return cudaGetLastError();
}

}  // namespace mt
