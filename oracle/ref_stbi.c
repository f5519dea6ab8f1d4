/* TEST INFRASTRUCTURE — the reference's own image loader, stb_image v2.16 as
 * vendored in the reference (external/stb_image.h), compiled from where it
 * lies by oracle/ref_build.py into oracle/_ref/.  Used only to pin the TGA
 * restatement (oracle/asset_oracle.cpp) and to make golden hashes of the
 * reference's shipped noise volumes. */
#define STB_IMAGE_IMPLEMENTATION
#define STBI_NO_STDIO
#include <string.h>

#include "stb_image.h"

/* Decodes an image file held in memory to RGBA8 (4 components, as
 * ImageLoadingUtility.cpp:88 asks).  Returns 0 and fills out (cap bytes) on
 * success, 1 when stb_image rejects the file, 2 when out is too small. */
__attribute__((visibility("default"))) int ref_stbi_load_rgba(const unsigned char* buf, int len, int* w, int* h,
                                                               unsigned char* out, long long cap) {
    int comp = 0;
    unsigned char* px = stbi_load_from_memory(buf, len, w, h, &comp, 4);
    if (!px) return 1;
    long long need = (long long)(*w) * (long long)(*h) * 4;
    if (!out || need > cap) {
        stbi_image_free(px);
        return 2;
    }
    memcpy(out, px, (size_t)need);
    stbi_image_free(px);
    return 0;
}
