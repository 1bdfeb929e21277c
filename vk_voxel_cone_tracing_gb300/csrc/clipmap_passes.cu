// clipmap_passes.cu -- CUDA kernels for the clipmap maintenance passes:
// region clear, copy-alpha, anisotropic 2x2x2 downsample, border wrap.
//
// All four are HBM-streaming integer/unorm8 work.  This translation unit is
// compiled with -fmad=false and the float math is written with explicit
// round-to-nearest intrinsics, so every RGBA8 result is bit-identical to the
// FP32 evaluation of the reference's GLSL expressions in their written order.
#include "common.cuh"

namespace vct {

// ------------------------------------------------------------------ clear
// clipmapCleaning.comp:17-31.  One thread per (x, y, z) of the region; the
// 6 face copies are 6 strided stores.
__global__ void k_clear_region(uint32_t* __restrict__ atlas, AtlasDims A, int3 rmin, uint3 ext, int level,
                               int faces) {
    const int64_t n = (int64_t)ext.x * ext.y * ext.z;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int gx = (int)(t % ext.x);
        int64_t r = t / ext.x;
        int gy = (int)(r % ext.y);
        int gz = (int)(r / ext.y);
        int px = (gx + rmin.x) % A.R + 1;
        int py = (gy + rmin.y) % A.R + 1 + level * A.rb;
        int pz = (gz + rmin.z) % A.R + 1;
        for (int f = 0; f < faces; ++f) atlas[A.index(px + A.rb * f, py, pz)] = 0u;
    }
}

// ------------------------------------------------------------- copy alpha
// copyAlphaImage.comp:16-30: dst.a = src.a over the R^3 interior, all faces.
// Thread per texel of one face row (x fastest) -> coalesced 4-byte RMW.
// blockIdx.y = face; R is a power of two, so the (x, y, z) split is shifts.
__global__ void k_copy_alpha(uint32_t* __restrict__ dst, const uint32_t* __restrict__ src, AtlasDims A, int level,
                             int lg) {
    const int f = blockIdx.y;
    const uint32_t n = 1u << (3 * lg), m = (1u << lg) - 1u;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int x = (int)(t & m), y = (int)((t >> lg) & m), z = (int)(t >> (2 * lg));
        const int64_t i = A.index(x + 1 + A.rb * f, y + 1 + level * A.rb, z + 1);
        dst[i] = (dst[i] & 0x00ffffffu) | (__ldg(src + i) & 0xff000000u);
    }
}

// ---------------------------------------------------------------- border
// borderWrapping.comp:14-37: invocations over ((R+2)>>3)*8 per axis; the
// ones with a zero coordinate copy the toroidal neighbour into the border
// for every clip level and face.
__global__ void k_wrap_border(uint32_t* __restrict__ atlas, AtlasDims A, int rwb, int faces, int regions, int n) {
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int x = (int)(t % n);
        int64_t r = t / n;
        int y = (int)(r % n);
        int z = (int)(r / n);
        if (x >= rwb || y >= rwb || z >= rwb) continue;
        if (x < A.R + 1 && y < A.R + 1 && z < A.R + 1 && x > 0 && y > 0 && z > 0) continue;
        const int m = A.R - 1;
        int rx = ((x + A.R - 1) & m) + 1, ry = ((y + A.R - 1) & m) + 1, rz = ((z + A.R - 1) & m) + 1;
        int wy = y;
        for (int i = 0; i < regions; ++i) {
            for (int j = 0; j < faces; ++j) atlas[A.index(x + rwb * j, wy, z)] = atlas[A.index(rx + rwb * j, ry, rz)];
            ry += rwb;
            wy += rwb;
        }
    }
}

// ------------------------------------------------------------- downsample
// opacityDownSample.comp / radianceDownSample.comp.  Thread per output voxel
// of level l (an (R/2)^3 grid, x fastest); per face it gathers the 2x2x2
// block of level l-1, composites front-to-back along the face's direction,
// blends with the level's own texel in the outer band and stores.
__device__ __forceinline__ int ds_wrap(int p, int R) { return (p + R * (abs(p / R) + 1)) & (R - 1); }

__constant__ int c_pairs[6][4][2] = {
    {{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{1, 0}, {3, 2}, {5, 4}, {7, 6}}, {{0, 2}, {1, 3}, {4, 6}, {5, 7}},
    {{2, 0}, {3, 1}, {6, 4}, {7, 5}}, {{0, 4}, {1, 5}, {2, 6}, {3, 7}}, {{4, 0}, {5, 1}, {6, 2}, {7, 3}}};

template <int MODE>
__global__ void k_downsample(uint32_t* __restrict__ atlas, AtlasDims A, int3 pmin, int level, int band, int lgh) {
    const int half = A.R >> 1;
    const uint32_t n = 1u << (3 * lgh), m = (1u << lgh) - 1u;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int gx = (int)(t & m);
        const int gy = (int)((t >> lgh) & m);
        const int gz = (int)(t >> (2 * lgh));
        const int cur[3] = {(pmin.x >> 1) + gx, (pmin.y >> 1) + gy, (pmin.z >> 1) + gz};
        const int pm[3] = {pmin.x, pmin.y, pmin.z};
        int wpos[3], ps[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            wpos[a] = ds_wrap(cur[a], A.R) + 1;
            ps[a] = ds_wrap(cur[a] << 1, A.R) + 1;
        }
        wpos[1] += A.rb * level;
        ps[1] += A.rb * (level - 1);

        // lerpFactor (opacityDownSample.comp:55-64).
        float dist[3];
        bool any_ge = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float center = __fadd_rn((float)(pm[a] >> 1), (float)(half >> 1));
            dist[a] = __fsub_rn(fabsf(__fsub_rn(__fadd_rn((float)cur[a], 0.5f), center)), 0.5f);
            any_ge |= dist[a] >= (float)((half >> 1) - band);
        }
        float lerp = 0.0f;
        const float inv = 1.0f / __fadd_rn((float)band, 1.0f);
        if (any_ge) {
            lerp = __fadd_rn(__fsub_rn(fmaxf(dist[0], fmaxf(dist[1], dist[2])), (float)((half >> 1) - band)), 1.0f);
            lerp = __fmul_rn(lerp, inv);
        }

        for (int f = 0; f < 6; ++f) {
            uint32_t raw[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                raw[i] = atlas[A.index(ps[0] + (i & 1) + A.rb * f, ps[1] + ((i >> 1) & 1), ps[2] + ((i >> 2) & 1))];
            const int64_t wi = A.index(wpos[0] + A.rb * f, wpos[1], wpos[2]);
            const uint32_t own_raw = atlas[wi];
            if (MODE == 0) {
                float s = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float a0 = unorm8_load(raw[c_pairs[f][k][0]], 3);
                    const float a1 = unorm8_load(raw[c_pairs[f][k][1]], 3);
                    const float tt = __fmul_rn(__fsub_rn(1.0f, a0), a1);
                    s = (k == 0) ? __fadd_rn(a0, tt) : __fadd_rn(__fadd_rn(s, a0), tt);
                }
                const float res = __fmul_rn(s, 0.25f);
                const float own_r = unorm8_load(own_raw, 0);
                const float a = mix_rn(res, own_r, lerp);
                const uint32_t q = unorm8_store(a);
                atlas[wi] = (own_raw & 0x00ff00ffu) | (q << 8) | (q << 24);
            } else {
                float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t r0 = raw[c_pairs[f][k][0]], r1 = raw[c_pairs[f][k][1]];
                    const float tt = __fsub_rn(1.0f, unorm8_load(r0, 3));
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float a0 = unorm8_load(r0, c);
                        const float b = __fmul_rn(tt, unorm8_load(r1, c));
                        s[c] = (k == 0) ? __fadd_rn(a0, b) : __fadd_rn(__fadd_rn(s[c], a0), b);
                    }
                }
                uint32_t out = 0;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float res = __fmul_rn(s[c], 0.25f);
                    out |= unorm8_store(mix_rn(res, unorm8_load(own_raw, c), lerp)) << (8 * c);
                }
                atlas[wi] = out;
            }
        }
    }
}

static int grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g > 152 * 64) g = 152 * 64;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace vct

using namespace vct;

extern "C" int vct_clear_region(uint32_t* atlas, const vct_image_cleaning_desc* d, void* stream) {
    VCT_CHECK_ARG(atlas && d, "vct_clear_region: null argument");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "vct_clear_region: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 0 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "vct_clear_region: clip level out of range");
    VCT_CHECK_ARG(d->face_count <= VCT_FACE_COUNT, "vct_clear_region: face count > 6");
    for (int a = 0; a < 3; ++a) {
        VCT_CHECK_ARG(d->region_min_corner[a] >= 0, "vct_clear_region: region min corner must be non-negative (wrap it first)");
        VCT_CHECK_ARG(d->clip_max_extent[a] <= (uint32_t)d->clipmap_resolution, "vct_clear_region: extent > resolution");
    }
    AtlasDims A(d->clipmap_resolution);
    const int64_t n = (int64_t)d->clip_max_extent[0] * d->clip_max_extent[1] * d->clip_max_extent[2];
    if (n == 0 || d->face_count == 0) return VCT_OK;
    k_clear_region<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        atlas, A, make_int3(d->region_min_corner[0], d->region_min_corner[1], d->region_min_corner[2]),
        make_uint3(d->clip_max_extent[0], d->clip_max_extent[1], d->clip_max_extent[2]), d->clip_level,
        (int)d->face_count);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_copy_alpha(uint32_t* dst, const uint32_t* src, const vct_copy_alpha_desc* d, void* stream) {
    VCT_CHECK_ARG(dst && src && d, "vct_copy_alpha: null argument");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "vct_copy_alpha: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 0 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "vct_copy_alpha: clip level out of range");
    VCT_CHECK_ARG(d->face_count >= 0 && d->face_count <= VCT_FACE_COUNT, "vct_copy_alpha: face count out of range");
    VCT_CHECK_ARG(dst != src, "vct_copy_alpha: source and destination atlases must differ");
    AtlasDims A(d->clipmap_resolution);
    if (d->face_count == 0) return VCT_OK;
    const int lg = 31 - __builtin_clz((unsigned)A.R);
    const int64_t n = (int64_t)A.R * A.R * A.R;
    dim3 grid((unsigned)grid_for(n, 256), (unsigned)d->face_count);
    k_copy_alpha<<<grid, 256, 0, as_stream(stream)>>>(dst, src, A, d->clip_level, lg);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_wrap_border(uint32_t* atlas, const vct_border_wrapping_desc* d, void* stream) {
    VCT_CHECK_ARG(atlas && d, "vct_wrap_border: null argument");
    VCT_CHECK_ARG(valid_resolution((int)d->clipmap_resolution), "vct_wrap_border: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_border_width == VCT_VOXEL_BORDER, "vct_wrap_border: border width must be 2 (one texel per side)");
    VCT_CHECK_ARG(d->face_count <= VCT_FACE_COUNT && d->clip_region_count <= VCT_CLIP_LEVEL_COUNT,
                  "vct_wrap_border: face/region count out of range");
    AtlasDims A((int)d->clipmap_resolution);
    const int n = ((A.R + 2) >> 3) * 8;
    const int64_t total = (int64_t)n * n * n;
    k_wrap_border<<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(atlas, A, A.R + (int)d->clip_border_width,
                                                                       (int)d->face_count, (int)d->clip_region_count, n);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_downsample(uint32_t* atlas, const vct_downsample_desc* d, int32_t mode, void* stream) {
    VCT_CHECK_ARG(atlas && d, "vct_downsample: null argument");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "vct_downsample: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 1 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "vct_downsample: clip level must be 1..5");
    VCT_CHECK_ARG(mode == VCT_DOWNSAMPLE_OPACITY || mode == VCT_DOWNSAMPLE_RADIANCE, "vct_downsample: bad mode");
    VCT_CHECK_ARG(d->downsample_region_size >= 0 && d->downsample_region_size <= 4096,
                  "vct_downsample: downsample band out of range");
    AtlasDims A(d->clipmap_resolution);
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    int3 pm = make_int3(d->prev_region_min_corner[0], d->prev_region_min_corner[1], d->prev_region_min_corner[2]);
    const int lgh = 31 - __builtin_clz((unsigned)half);
    if (mode == VCT_DOWNSAMPLE_OPACITY)
        k_downsample<0><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(atlas, A, pm, d->clip_level, d->downsample_region_size, lgh);
    else
        k_downsample<1><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(atlas, A, pm, d->clip_level, d->downsample_region_size, lgh);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_downsample_all(uint32_t* atlas, const vct_clipmap_region regions[6], int32_t R, int32_t mode,
                                  void* stream) {
    VCT_CHECK_ARG(regions, "vct_downsample_all: null regions");
    for (int l = 1; l < VCT_CLIP_LEVEL_COUNT; ++l) {
        vct_downsample_desc d;
        for (int a = 0; a < 3; ++a) d.prev_region_min_corner[a] = regions[l - 1].min_corner[a];
        d.clip_level = l;
        d.clipmap_resolution = R;
        d.downsample_region_size = VCT_DOWNSAMPLE_REGION_SIZE;
        int rc = vct_downsample(atlas, &d, mode, stream);
        if (rc != VCT_OK) return rc;
    }
    return VCT_OK;
}
