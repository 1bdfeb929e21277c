// ingest.cu -- host-side helpers of the scene loader (no device code).
//
// vct_png_unfilter reverses the per-scanline filters of a PNG image after the
// zlib stream has been inflated (PNG specification, ISO/IEC 15948:2004,
// section 9: filter types 0 None, 1 Sub, 2 Up, 3 Average, 4 Paeth, each row
// prefixed by its filter byte, byte arithmetic modulo 256, bpp = bytes per
// complete pixel rounded up to 1).  The glTF loader uses it to decode the
// PNG images a scene references (GLTFLoader::loadScene gets them decoded
// from tinygltf, VFS/Util/GLTFLoader.cpp:118-123).
#include <stdint.h>
#include <stdlib.h>

#include "common.cuh"

namespace {

inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

}  // namespace

extern "C" int vct_png_unfilter(const uint8_t* filtered_host, int64_t row_bytes, int64_t rows, int32_t bpp,
                                uint8_t* out_host) {
    VCT_CHECK_ARG(filtered_host && out_host, "vct_png_unfilter: null argument");
    VCT_CHECK_ARG(row_bytes > 0 && rows > 0 && bpp >= 1 && bpp <= 8, "vct_png_unfilter: bad image geometry");
    for (int64_t y = 0; y < rows; ++y) {
        const uint8_t* f = filtered_host + y * (row_bytes + 1);
        const uint8_t type = f[0];
        ++f;
        uint8_t* r = out_host + y * row_bytes;
        const uint8_t* up = y > 0 ? r - row_bytes : nullptr;
        switch (type) {
            case 0:
                for (int64_t i = 0; i < row_bytes; ++i) r[i] = f[i];
                break;
            case 1:
                for (int64_t i = 0; i < row_bytes; ++i) r[i] = (uint8_t)(f[i] + (i >= bpp ? r[i - bpp] : 0));
                break;
            case 2:
                for (int64_t i = 0; i < row_bytes; ++i) r[i] = (uint8_t)(f[i] + (up ? up[i] : 0));
                break;
            case 3:
                for (int64_t i = 0; i < row_bytes; ++i) {
                    const int a = i >= bpp ? r[i - bpp] : 0, b = up ? up[i] : 0;
                    r[i] = (uint8_t)(f[i] + ((a + b) >> 1));
                }
                break;
            case 4:
                for (int64_t i = 0; i < row_bytes; ++i) {
                    const int a = i >= bpp ? r[i - bpp] : 0, b = up ? up[i] : 0;
                    const int c = (up && i >= bpp) ? up[i - bpp] : 0;
                    r[i] = (uint8_t)(f[i] + paeth(a, b, c));
                }
                break;
            default:
                return vct::fail(VCT_E_BAD_ARG, "vct_png_unfilter: unknown filter type");
        }
    }
    return VCT_OK;
}
