// image_io.cpp — headless image files in place of the sample apps' output
// (SDK/optixMotionBlur/optixMotionBlur.cpp:795-840: the film, its
// "-density" image and, after ConvertToBytes, the 8-bit image, written by
// sutil::saveImage).  The reference writes floating-point images as OpenEXR
// through a third-party library; here they are Portable Float Maps (PFM: a
// text header "PF", width height, -1.0 for little-endian, then RGB float32
// rows from the bottom up), which every HDR tool reads and numpy parses in a
// few lines.  8-bit images are binary PPM (P6, RGB rows from the top), as
// sutil writes a .ppm.  The alpha channel of the float4/uchar4 pixels is
// dropped, as both formats hold RGB.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "mdas.h"

namespace {

// float bits in little-endian byte order, whatever the host's
void put_le(unsigned char* dst, float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    dst[0] = (unsigned char)(u & 0xffu);
    dst[1] = (unsigned char)((u >> 8) & 0xffu);
    dst[2] = (unsigned char)((u >> 16) & 0xffu);
    dst[3] = (unsigned char)((u >> 24) & 0xffu);
}

}  // namespace

extern "C" int mdas_save_image(const char* path, const void* pixels, int width, int height, int format) {
    if (!path || !pixels || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    if (format != MDAS_IMAGE_FLOAT4 && format != MDAS_IMAGE_UCHAR4) return MDAS_ERR_INVALID;
    FILE* f = fopen(path, "wb");
    if (!f) return MDAS_ERR_INVALID;
    bool ok = true;
    const size_t W = (size_t)width, H = (size_t)height;
    if (format == MDAS_IMAGE_FLOAT4) {
        ok = fprintf(f, "PF\n%d %d\n-1.0\n", width, height) > 0;
        const float* px = static_cast<const float*>(pixels);
        std::vector<unsigned char> row(12 * W);
        for (size_t y = 0; y < H && ok; ++y) {
            const float* src = px + 4 * W * (H - 1 - y);  // PFM rows run bottom to top
            for (size_t x = 0; x < W; ++x)
                for (int c = 0; c < 3; ++c) put_le(&row[12 * x + 4 * c], src[4 * x + c]);
            ok = fwrite(row.data(), 1, row.size(), f) == row.size();
        }
    } else {
        ok = fprintf(f, "P6\n%d %d\n255\n", width, height) > 0;
        const unsigned char* px = static_cast<const unsigned char*>(pixels);
        std::vector<unsigned char> row(3 * W);
        for (size_t y = 0; y < H && ok; ++y) {
            const unsigned char* src = px + 4 * W * y;
            for (size_t x = 0; x < W; ++x)
                for (int c = 0; c < 3; ++c) row[3 * x + c] = src[4 * x + c];
            ok = fwrite(row.data(), 1, row.size(), f) == row.size();
        }
    }
    if (fclose(f) != 0) ok = false;
    return ok ? MDAS_OK : MDAS_ERR_INVALID;
}
