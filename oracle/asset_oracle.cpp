// TEST INFRASTRUCTURE — the oracle.  Not part of the product: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
// only as the checker.
//
// CPU restatement of the TGA decoding the reference's asset loader performs
// (ImageLoadingUtility.cpp:75-139 loads every slice with stb_image v2.16,
// external/stb_image.h:5416-5610, forced to 4 components), for the files the
// product accepts: image types 2 (raw) and 10 (run-length), colour-map type
// 0, 24 or 32 bits per pixel.  Pixels are decoded one at a time as a stream
// (run-length packets run on across scanlines; a byte past the end of the file
// reads as 0), then the rows are flipped unless the origin is top-left, then
// B and R are swapped and 24-bit pixels get alpha 255.
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Reader {
    const uint8_t* p;
    size_t n, pos;
    unsigned get() { return pos < n ? p[pos++] : (pos++, 0u); }
};

}  // namespace

extern "C" {

// out: width*height*4 bytes (RGBA, top row first).  Returns 0, or 1 for a
// file outside the accepted subset (out untouched).
__attribute__((visibility("default"))) int orc_decode_tga(const uint8_t* file, size_t size, int* width, int* height,
                                                          uint8_t* out) {
    if (!file || size < 18) return 1;
    const int idlen = file[0], cmtype = file[1], type = file[2], bpp = file[16], desc = file[17];
    const int w = file[12] | (file[13] << 8), h = file[14] | (file[15] << 8);
    if (cmtype != 0 || (type != 2 && type != 10) || (bpp != 24 && bpp != 32) || w < 1 || h < 1) return 1;
    if (width) *width = w;
    if (height) *height = h;
    if (!out) return 0;
    const int comp = bpp / 8;
    const bool rle = type == 10;
    const bool top_left = (desc >> 5) & 1;
    Reader r{file, size, (size_t)18 + (size_t)idlen};
    std::vector<uint8_t> px((size_t)w * h * comp);
    uint8_t raw[4] = {0, 0, 0, 0};
    int run_left = 0;
    bool repeating = false;
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        bool read = true;
        if (rle) {
            if (run_left == 0) {
                const unsigned c = r.get();
                run_left = 1 + (int)(c & 127u);
                repeating = (c >> 7) != 0;
            } else if (repeating) {
                read = false;
            }
        }
        if (read)
            for (int j = 0; j < comp; ++j) raw[j] = (uint8_t)r.get();
        std::memcpy(&px[i * comp], raw, (size_t)comp);
        --run_left;
    }
    for (int y = 0; y < h; ++y) {
        const int src_row = top_left ? y : h - 1 - y;
        for (int x = 0; x < w; ++x) {
            const uint8_t* s = &px[((size_t)src_row * w + x) * comp];
            uint8_t* o = out + ((size_t)y * w + x) * 4;
            o[0] = s[2];
            o[1] = s[1];
            o[2] = s[0];
            o[3] = comp == 4 ? s[3] : 255;
        }
    }
    return 0;
}

}  // extern "C"
