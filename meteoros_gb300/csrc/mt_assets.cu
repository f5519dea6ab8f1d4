// Noise-volume assets: a 3D volume from its stack of TGA slices, decoded on the
// device.  The reference loads slice z from the file "<name>(z+1).tga" with
// stb_image (forced to 4 components) and copies it to depth z of an RGBA8
// volume (ImageLoadingUtility.cpp:75-139); its assets are run-length encoded
// 32-bit TGAs (image type 10) with the bottom-left origin.
//
// TGA decoding, as the reference's decoder does it:
//   * header: id length (byte 0), colour-map type (1, must be 0), image type
//     (2: raw, 10: run-length), width (12-13), height (14-15), bits per pixel
//     (16: 24 or 32), descriptor (17: bit 5 set = top-left origin); the pixel
//     data follow the image id;
//   * run-length packets: a count byte c (1 + (c & 127) pixels), a run of one
//     pixel value when c & 128, else that many literal pixels; packets run on
//     across scanlines; bytes past the end of the file read as 0;
//   * pixels are B, G, R[, A]; 24-bit pixels get A = 255; rows are flipped to
//     top-first unless the origin is top-left.
//
// One CTA per slice: the file is staged in shared memory, one thread walks the
// packet headers (a serial dependency chain, cheap from shared memory) in
// chunks, and the CTA expands each chunk's packets in parallel.
#include <cuda_runtime.h>

#include "mt_kernels.h"

namespace mt {

namespace {

constexpr int kChunk = 1024;  // packets per walk/expand round

__device__ __forceinline__ unsigned sbyte(const unsigned char* sm, long long size, long long p) {
    return (p >= 0 && p < size) ? (unsigned)sm[p] : 0u;
}

__device__ __forceinline__ uint32_t rgba_word(const unsigned char* sm, long long size, long long p, int bytes_pp) {
    const unsigned b = sbyte(sm, size, p), g = sbyte(sm, size, p + 1), r = sbyte(sm, size, p + 2);
    const unsigned a = bytes_pp == 4 ? sbyte(sm, size, p + 3) : 255u;
    return r | (g << 8) | (b << 16) | (a << 24);
}

__global__ void __launch_bounds__(256) tga_decode_kernel(const unsigned char* __restrict__ blob,
                                                         const TgaSlice* __restrict__ slices, uint32_t* vol, int W,
                                                         int H) {
    extern __shared__ unsigned char sm[];
    __shared__ int p_first[kChunk], p_pos[kChunk], p_cnt[kChunk];
    __shared__ int s_n, s_pos, s_pix;
    const TgaSlice sl = slices[blockIdx.x];
    const long long size = sl.size;
    for (long long i = threadIdx.x; i < size; i += blockDim.x) sm[i] = blob[sl.offset + i];
    __syncthreads();
    const int bpp = (int)sbyte(sm, size, 16) / 8;
    // colour-map type 0 (checked on the host): the pixels follow the image id
    const long long data = 18 + (long long)sbyte(sm, size, 0);
    const bool rle = sbyte(sm, size, 2) == 10;
    const bool flip = !(sbyte(sm, size, 17) & 32u);
    const int N = W * H;
    uint32_t* out = vol + (size_t)blockIdx.x * (size_t)N;
    auto store = [&](int i, uint32_t v) {
        const int x = i % W, y = i / W;
        out[(size_t)(flip ? H - 1 - y : y) * (size_t)W + (size_t)x] = v;
    };
    if (!rle) {
        for (int i = threadIdx.x; i < N; i += blockDim.x) store(i, rgba_word(sm, size, data + (long long)i * bpp, bpp));
        return;
    }
    if (threadIdx.x == 0) {
        s_pos = (int)data;
        s_pix = 0;
    }
    __syncthreads();
    // every round covers at least one pixel, so at most N rounds
    for (int round = 0; round <= N; ++round) {
        const int pix_now = s_pix;
        __syncthreads();  // every thread has read s_pix before thread 0 moves it
        if (pix_now >= N) break;
        if (threadIdx.x == 0) {
            int pos = s_pos, pix = s_pix, n = 0;
            while (n < kChunk && pix < N) {
                const unsigned c = sbyte(sm, size, pos);
                const int count = 1 + (int)(c & 127u);
                p_first[n] = pix;
                p_pos[n] = pos + 1;
                p_cnt[n] = (c & 128u) ? -count : count;  // negative: a run of one value
                pos += 1 + ((c & 128u) ? bpp : count * bpp);
                pix += count;
                ++n;
            }
            s_n = n;
            s_pos = pos;
            s_pix = pix;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < s_n; k += blockDim.x) {
            const int first = p_first[k], c = p_cnt[k], pos = p_pos[k];
            const int count = c < 0 ? -c : c;
            const int end = first + count < N ? first + count : N;
            if (c < 0) {
                const uint32_t v = rgba_word(sm, size, pos, bpp);
                for (int i = first; i < end; ++i) store(i, v);
            } else {
                for (int i = first; i < end; ++i) store(i, rgba_word(sm, size, pos + (long long)(i - first) * bpp, bpp));
            }
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_tga_decode(const unsigned char* blob, const TgaSlice* slices, int n_slices, size_t max_size,
                              uint32_t* vol, int W, int H, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(tga_decode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_size);
    if (e != cudaSuccess) return e;
    tga_decode_kernel<<<n_slices, 256, max_size, s>>>(blob, slices, vol, W, H);
    return cudaGetLastError();
}

}  // namespace mt
