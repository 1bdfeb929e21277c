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
    // extents <= R <= 1024 and corners in [0, 2^30]: 32-bit arithmetic; R is
    // a power of two, so the (non-negative) % R is a mask
    const uint32_t n = ext.x * ext.y * ext.z, m = (uint32_t)A.R - 1u;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t gx = t % ext.x, r = t / ext.x;
        const uint32_t gy = r % ext.y, gz = r / ext.y;
        const int px = (int)((gx + (uint32_t)rmin.x) & m) + 1;
        const int py = (int)((gy + (uint32_t)rmin.y) & m) + 1 + level * A.rb;
        const int pz = (int)((gz + (uint32_t)rmin.z) & m) + 1;
        for (int f = 0; f < faces; ++f) atlas[A.index(px + A.rb * f, py, pz)] = 0u;
    }
}

// ------------------------------------------------------------- copy alpha
// copyAlphaImage.comp:16-30: dst.a = src.a over the R^3 interior, all faces.
// Thread per texel position (cube_texel order: coalesced 4-byte RMW), all
// faces; R is a power of two, so the (x, y, z) split is shifts.
// `mirror` (0 = none): a texture array's surface that receives the same texels.
// `touched` (may be null): texels whose bit is clear read as zero rgb.
// (Both words are loaded unconditionally and selected, so the loads of a
// thread's texels stay independent and in flight together.)
__device__ __forceinline__ uint32_t rgb_of(const uint32_t* __restrict__ atlas, const uint32_t* __restrict__ touched,
                                           int64_t i) {
    const uint32_t r = atlas[i];
    const uint32_t w = touched ? __ldg(touched + (i >> 5)) : 0xffffffffu;
    return ((w >> (i & 31)) & 1u) ? (r & 0x00ffffffu) : 0u;
}

// Texel order of the passes that also store into a texture: a warp takes 16
// x-neighbours of two neighbouring rows, so each 32-byte sector of the
// array's block-linear layout (16 B of two neighbouring rows) is written
// whole by one warp.  (On the 8-byte FP16 conversion, row-by-row warps cost
// a DRAM read-modify-write per sector; with these 4-byte texels the frame
// time is the same either way.)  t -> (x, y, z) of a 2^lg cube, a bijection.
__device__ __forceinline__ void cube_texel(uint32_t t, int lg, int& x, int& y, int& z) {
    const uint32_t m = (1u << lg) - 1u;
    if (lg >= 4) {
        x = (int)((t & 15u) | (((t >> 5) & (m >> 4)) << 4));
        y = (int)(((t >> 4) & 1u) | (((t >> (lg + 1)) & (m >> 1)) << 1));
    } else {
        x = (int)(t & m);
        y = (int)((t >> lg) & m);
    }
    z = (int)(t >> (2 * lg));
}

// The alpha byte of opacity texel i in the alpha position of an RGBA8 word:
// the reference's RGBA8 opacity atlas (OT = uint32_t) or the one-byte-per-
// texel form (OT = uint8_t, the same texel order), which holds the alpha only.
__device__ __forceinline__ uint32_t opa_alpha(const uint32_t* __restrict__ opa, int64_t i) {
    return __ldg(opa + i) & 0xff000000u;
}
__device__ __forceinline__ uint32_t opa_alpha(const uint8_t* __restrict__ opa, int64_t i) {
    return (uint32_t)__ldg(opa + i) << 24;
}

template <class OT>
__global__ void k_copy_alpha(uint32_t* __restrict__ dst, const OT* __restrict__ src, AtlasDims A, int level,
                             int lg, int faces, cudaSurfaceObject_t mirror, const uint32_t* __restrict__ touched) {
    const uint32_t n = 1u << (3 * lg);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int x, y, z;
        cube_texel(t, lg, x, y, z);
        x += 1;
        y += 1 + level * A.rb;
        z += 1;
        const int64_t i0 = A.index(x, y, z);
        // every face's texel loaded before the first store: six loads in flight per thread
        uint32_t v[6];
#pragma unroll
        for (int f = 0; f < 6; ++f)
            if (f < faces) v[f] = rgb_of(dst, touched, i0 + A.rb * f) | opa_alpha(src, i0 + A.rb * f);
#pragma unroll
        for (int f = 0; f < 6; ++f)
            if (f < faces) {
                dst[i0 + A.rb * f] = v[f];
                if (mirror) surf3Dwrite(v[f], mirror, (x + A.rb * f) * 4, y, z);
            }
    }
}

// The same pass four texels at a time: each thread takes an aligned group of
// four texels of a row (rows are 16-byte aligned: W = 6 (R + 2) is a multiple
// of four), with 16-byte loads and stores and one 16-byte surface store; the
// group's texels outside the faces' interiors (the border columns, which no
// pass writes in the radiance atlas) are stored back unchanged.  A warp covers
// 512 contiguous bytes of a row.
__device__ __forceinline__ uint4 opa_alpha4(const uint32_t* __restrict__ opa, int64_t i) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(opa + i));
    return make_uint4(v.x & 0xff000000u, v.y & 0xff000000u, v.z & 0xff000000u, v.w & 0xff000000u);
}
__device__ __forceinline__ uint4 opa_alpha4(const uint8_t* __restrict__ opa, int64_t i) {
    const uint32_t b = __ldg(reinterpret_cast<const uint32_t*>(opa + i));
    return make_uint4(b << 24, (b << 16) & 0xff000000u, (b << 8) & 0xff000000u, b & 0xff000000u);
}

template <class OT>
__global__ void k_copy_alpha4(uint32_t* __restrict__ dst, const OT* __restrict__ src, AtlasDims A, int level,
                              int faces, cudaSurfaceObject_t mirror, const uint32_t* __restrict__ touched) {
    const int lane = threadIdx.x & 31;
    const uint32_t groups = (uint32_t)(A.rb * faces + 3) >> 2;  // x groups of a row
    const uint32_t g32 = (groups + 31u) & ~31u;                  // a row's groups padded to whole warps
    const uint32_t R = (uint32_t)A.R;
    const uint32_t n = g32 * R * R;  // R <= 1024: < 2^31
    // warp-uniform trip count: a warp's 32 groups lie in one row
    for (uint32_t t0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; t0 < n; t0 += gridDim.x * blockDim.x) {
        const uint32_t t = t0 + (uint32_t)lane;
        const uint32_t gx = t % g32, r = t / g32;
        const int y = (int)(r & (R - 1u)) + 1 + level * A.rb, z = (int)(r / R) + 1;
        const int x0 = (int)gx * 4;
        const bool valid = gx < groups;
        const int64_t i = A.index(x0, y, z);
        uint32_t v[4] = {0u, 0u, 0u, 0u};
        if (valid) {
            const uint4 d = *reinterpret_cast<const uint4*>(dst + i);
            const uint4 a = opa_alpha4(src, i);
            const uint32_t w = touched ? __ldg(touched + (i >> 5)) : 0xffffffffu;
            v[0] = d.x, v[1] = d.y, v[2] = d.z, v[3] = d.w;
            const uint32_t av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int x = x0 + k, xf = x % A.rb;
                if (x < A.rb * faces && xf >= 1 && xf <= A.R)
                    v[k] = (((w >> ((i + k) & 31)) & 1u) ? (v[k] & 0x00ffffffu) : 0u) | av[k];
            }
            *reinterpret_cast<uint4*>(dst + i) = make_uint4(v[0], v[1], v[2], v[3]);
        }
        if (mirror) {
            // the texture's texel stores coalesced: in round k lane L stores texel 32 k + L of the warp's 128,
            // which lane 8 k + L / 4 holds as its element L % 4
            const int xw = (int)(gx - (uint32_t)lane) * 4;  // the warp's first texel
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int o = 8 * k + (lane >> 2), e = lane & 3;
                const uint32_t c0 = __shfl_sync(0xffffffffu, v[0], o), c1 = __shfl_sync(0xffffffffu, v[1], o);
                const uint32_t c2 = __shfl_sync(0xffffffffu, v[2], o), c3 = __shfl_sync(0xffffffffu, v[3], o);
                const uint32_t c = e == 0 ? c0 : (e == 1 ? c1 : (e == 2 ? c2 : c3));
                const int x = xw + 32 * k + lane;
                if (t0 < n && (uint32_t)x < groups * 4u) surf3Dwrite(c, mirror, x * 4, y, z);
            }
        }
    }
}

// ---------------------------------------------------------------- border
// borderWrapping.comp:14-37: the dispatch covers ((R+2)>>3)*8 = R
// invocations per axis (R a power of two >= 8), and an invocation whose
// position has a zero coordinate copies its toroidal interior neighbour into
// that border texel, for every clip level and face; the R+1 side is never
// reached.  One thread per (level, face, position of [0,R)^3 with a zero
// coordinate): the z = 0 plane, then the y = 0 rows, then the x = 0 column,
// x fastest where it varies.  Sources are interior texels, never written here.
template <class T>
__global__ void k_wrap_border(T* __restrict__ atlas, AtlasDims A, int faces, int regions) {
    // R <= 1024: (3R^2 - 3R + 1) * 36 < 2^27
    const uint32_t R = (uint32_t)A.R, lg = 31u - __clz(A.R);
    const uint32_t zf = R * R, yr = R * (R - 1u), shell = zf + yr + (R - 1u) * (R - 1u);
    const uint32_t total = shell * (uint32_t)faces * (uint32_t)regions;
    const int m = A.R - 1, W = A.R + 2;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        uint32_t s = t % shell;
        const uint32_t fl = t / shell;
        const int j = (int)(fl % (uint32_t)faces), i = (int)(fl / (uint32_t)faces);
        int x, y, z;
        if (s < zf) {
            z = 0;
            x = (int)(s & (R - 1u));
            y = (int)(s >> lg);
        } else if ((s -= zf) < yr) {
            y = 0;
            x = (int)(s & (R - 1u));
            z = 1 + (int)(s >> lg);
        } else {
            s -= yr;
            x = 0;
            y = 1 + (int)(s % (R - 1u));
            z = 1 + (int)(s / (R - 1u));
        }
        const int rx = ((x + A.R - 1) & m) + 1, ry = ((y + A.R - 1) & m) + 1, rz = ((z + A.R - 1) & m) + 1;
        atlas[A.index(x + W * j, y + W * i, z)] = atlas[A.index(rx + W * j, ry + W * i, rz)];
    }
}

// ------------------------------------------------------------- downsample
// opacityDownSample.comp / radianceDownSample.comp.  Thread per output voxel
// of level l (an (R/2)^3 grid, x fastest); per face it gathers the 2x2x2
// block of level l-1, composites front-to-back along the face's direction,
// blends with the level's own texel in the outer band and stores.
__device__ __forceinline__ int ds_wrap(int p, int R) { return (p + R * (abs(p / R) + 1)) & (R - 1); }

}  // namespace vct
#include "mip_pairs.cuh"
namespace vct {

// `prev` is `atlas` again, read only at level l - 1 (which this pass does not
// write): as a second restrict pointer its loads are free to run ahead of the
// stores of level l, so all six faces' 2x2x2 blocks are loaded before the
// first store (one memory round trip per output voxel instead of six).
template <int MODE>
__global__ void k_downsample(uint32_t* __restrict__ atlas, const uint32_t* __restrict__ prev, AtlasDims A, int3 pmin,
                             int level, int band, int lgh) {
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

        uint32_t raw6[6][8], own6[6];
        const int64_t c0 = A.index(ps[0], ps[1], ps[2]), w0 = A.index(wpos[0], wpos[1], wpos[2]);
        const int64_t dy = A.W, dz = (int64_t)A.W * A.H;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                raw6[f][i] = __ldg(prev + c0 + A.rb * f + (i & 1) + ((i >> 1) & 1) * dy + ((i >> 2) & 1) * dz);
            own6[f] = atlas[w0 + A.rb * f];
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const uint32_t* raw = raw6[f];
            const int64_t wi = w0 + A.rb * f;
            const uint32_t own_raw = own6[f];
            if (MODE == 0) {
                float s = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float a0 = unorm8_load(raw[ds_pair(f, k, 0)], 3);
                    const float a1 = unorm8_load(raw[ds_pair(f, k, 1)], 3);
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
                    const uint32_t r0 = raw[ds_pair(f, k, 0)], r1 = raw[ds_pair(f, k, 1)];
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

// opacityDownSample.comp on the one-byte opacity form.  The RGBA8 pass reads
// the children's alpha and the target's red byte (the level's own voxelised
// value), and writes the result into green and alpha, keeping red.  Within a
// full revoxelisation a target's red byte is read only by this pass, before
// the store, and every other reader of the opacity atlas (the next level's
// pass, the border wrap, copy-alpha) reads alpha; outside the target block
// red == alpha (the voxeliser writes all four bytes).  So one byte per texel
// -- the voxelised value until this pass stores the alpha over it -- gives
// every reader the byte it reads from the RGBA8 atlas.  (The toroidal update
// re-reads red of texels voxelised in earlier frames, so it keeps RGBA8.)
__global__ void k_downsample_r8(uint8_t* __restrict__ atlas, const uint8_t* __restrict__ prev, AtlasDims A, int3 pmin,
                                int level, int band, int lgh) {
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
        uint32_t raw6[6][8], own6[6];
        const int64_t c0 = A.index(ps[0], ps[1], ps[2]), w0 = A.index(wpos[0], wpos[1], wpos[2]);
        const int64_t dy = A.W, dz = (int64_t)A.W * A.H;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                raw6[f][i] = (uint32_t)__ldg(prev + c0 + A.rb * f + (i & 1) + ((i >> 1) & 1) * dy + ((i >> 2) & 1) * dz)
                             << 24;
            own6[f] = atlas[w0 + A.rb * f];
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const uint32_t* raw = raw6[f];
            const int64_t wi = w0 + A.rb * f;
            float s = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float a0 = unorm8_load(raw[ds_pair(f, k, 0)], 3);
                const float a1 = unorm8_load(raw[ds_pair(f, k, 1)], 3);
                const float tt = __fmul_rn(__fsub_rn(1.0f, a0), a1);
                s = (k == 0) ? __fadd_rn(a0, tt) : __fadd_rn(__fadd_rn(s, a0), tt);
            }
            const float res = __fmul_rn(s, 0.25f);
            const float own_r = unorm8_load(own6[f], 0);
            atlas[wi] = (uint8_t)unorm8_store(mix_rn(res, own_r, lerp));
        }
    }
}

// copyAlphaImage.comp then radianceDownSample.comp for one level l >= 1 in
// one launch, same result as the two passes in sequence.  Two grid-stride
// loops: (a) copy-alpha of the level's R^3 interior texels outside the
// downsample's target block (the (R/2)^3 block from the previous region's
// corner / 2 on, toroidally), in cube_texel order; (b) the target block in a
// compact index space (x fastest): each target takes its copy-alpha value
// as the blend's own texel and blends the 2x2x2 composite of level l - 1
// with it as k_downsample<1> does -- every lane of a loop does the same kind
// of work (one loop over the mixed texels was 3 % slower per frame at
// R = 256).  The target block depends only on level l - 1, which earlier
// launches finished.  All six faces per thread.
// Faces whose 2x2x2 blocks of level l - 1 a target loads together, ahead of
// their stores (through `prev`, the radiance atlas again as a read-only
// restrict pointer: level l - 1 is not written by this pass).
constexpr int kAlphaDsFacesPerRound = 2;

template <class OT>
__global__ void __launch_bounds__(128, 8) k_alpha_downsample(uint32_t* __restrict__ rad,
                                                                    const uint32_t* __restrict__ prev,
                                                                    const OT* __restrict__ opa, AtlasDims A,
                                                                    int3 pmin, int level, int band, int lg,
                                                                    cudaSurfaceObject_t mirror,
                                                                    const uint32_t* __restrict__ touched) {
    const int half = A.R >> 1;
    const int pm[3] = {pmin.x, pmin.y, pmin.z};
    const uint32_t stride = gridDim.x * blockDim.x;
    // (a) copy-alpha outside the target block
    const uint32_t n = 1u << (3 * lg);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        int w[3];
        cube_texel(t, lg, w[0], w[1], w[2]);
        bool target = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) target = target && ((w[a] - (pm[a] >> 1)) & (A.R - 1)) < half;
        if (target) continue;
        const int64_t w0 = A.index(w[0] + 1, w[1] + 1 + A.rb * level, w[2] + 1);
        uint32_t own6[6];
#pragma unroll
        for (int f = 0; f < 6; ++f)
            own6[f] = rgb_of(rad, touched, w0 + A.rb * f) | opa_alpha(opa, w0 + A.rb * f);
        const int my = w[1] + 1 + A.rb * level, mz = w[2] + 1;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            rad[w0 + A.rb * f] = own6[f];
            if (mirror) surf3Dwrite(own6[f], mirror, (w[0] + 1 + A.rb * f) * 4, my, mz);
        }
    }
    // (b) the target block: copy-alpha value, then the 2x2x2 composite of level l - 1
    const int lgh = lg - 1;
    const uint32_t nh = 1u << (3 * lgh), mh = (1u << lgh) - 1u;
    const float inv = 1.0f / __fadd_rn((float)band, 1.0f);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nh; t += stride) {
        const int g[3] = {(int)(t & mh), (int)((t >> lgh) & mh), (int)(t >> (2 * lgh))};
        int cur[3], wpos[3], ps[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            cur[a] = (pm[a] >> 1) + g[a];
            wpos[a] = ds_wrap(cur[a], A.R) + 1;
            ps[a] = ds_wrap(cur[a] << 1, A.R) + 1;
        }
        wpos[1] += A.rb * level;
        ps[1] += A.rb * (level - 1);
        float dist[3];
        bool any_ge = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float center = __fadd_rn((float)(pm[a] >> 1), (float)(half >> 1));
            dist[a] = __fsub_rn(fabsf(__fsub_rn(__fadd_rn((float)cur[a], 0.5f), center)), 0.5f);
            any_ge |= dist[a] >= (float)((half >> 1) - band);
        }
        float lerp = 0.0f;
        if (any_ge) {
            lerp = __fadd_rn(__fsub_rn(fmaxf(dist[0], fmaxf(dist[1], dist[2])), (float)((half >> 1) - band)), 1.0f);
            lerp = __fmul_rn(lerp, inv);
        }
        const int64_t w0 = A.index(wpos[0], wpos[1], wpos[2]);
        uint32_t own6[6];
#pragma unroll
        for (int f = 0; f < 6; ++f)
            own6[f] = rgb_of(rad, touched, w0 + A.rb * f) | opa_alpha(opa, w0 + A.rb * f);
        const int64_t c0 = A.index(ps[0], ps[1], ps[2]);
        const int64_t dy = A.W, dz = (int64_t)A.W * A.H;
#pragma unroll
        for (int f0 = 0; f0 < 6; f0 += kAlphaDsFacesPerRound) {
          uint32_t rawr[kAlphaDsFacesPerRound][8];
#pragma unroll
          for (int h = 0; h < kAlphaDsFacesPerRound; ++h)
#pragma unroll
            for (int i = 0; i < 8; ++i)
                rawr[h][i] = __ldg(prev + c0 + A.rb * (f0 + h) + (i & 1) + ((i >> 1) & 1) * dy + ((i >> 2) & 1) * dz);
#pragma unroll
          for (int h = 0; h < kAlphaDsFacesPerRound; ++h) {
            const int f = f0 + h;
            const uint32_t* raw = rawr[h];
            float sc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t r0 = raw[ds_pair(f, k, 0)], r1 = raw[ds_pair(f, k, 1)];
                const float tt = __fsub_rn(1.0f, unorm8_load(r0, 3));
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float a0 = unorm8_load(r0, c);
                    const float b = __fmul_rn(tt, unorm8_load(r1, c));
                    sc[c] = (k == 0) ? __fadd_rn(a0, b) : __fadd_rn(__fadd_rn(sc[c], a0), b);
                }
            }
            uint32_t out = 0;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float res = __fmul_rn(sc[c], 0.25f);
                out |= unorm8_store(mix_rn(res, unorm8_load(own6[f], c), lerp)) << (8 * c);
            }
            rad[w0 + A.rb * f] = out;
            if (mirror) surf3Dwrite(out, mirror, (wpos[0] + A.rb * f) * 4, wpos[1], wpos[2]);
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
        VCT_CHECK_ARG(d->region_min_corner[a] >= 0 && d->region_min_corner[a] <= (1 << 30),
                      "vct_clear_region: region min corner must be in [0, 2^30] (wrap it first)");
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

namespace vct {

int copy_alpha_pass(uint32_t* dst, const void* src, const vct_copy_alpha_desc* d, cudaSurfaceObject_t mirror,
                    const uint32_t* touched, cudaStream_t st, bool src_r8) {
    VCT_CHECK_ARG(dst && src && d, "vct_copy_alpha: null argument");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "vct_copy_alpha: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 0 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "vct_copy_alpha: clip level out of range");
    VCT_CHECK_ARG(d->face_count >= 0 && d->face_count <= VCT_FACE_COUNT, "vct_copy_alpha: face count out of range");
    VCT_CHECK_ARG(dst != src, "vct_copy_alpha: source and destination atlases must differ");
    AtlasDims A(d->clipmap_resolution);
    if (d->face_count == 0) return VCT_OK;
    const int lg = 31 - __builtin_clz((unsigned)A.R);
    const int64_t n = (int64_t)A.R * A.R * A.R;
    const int grid = grid_for(n, 256);
    const bool aligned = (((uintptr_t)dst | (uintptr_t)src) & 15) == 0;  // 16-byte row groups (R8: 4 bytes)
    if (aligned) {
        const int64_t n4 = (int64_t)((((A.rb * d->face_count + 3) >> 2) + 31) & ~31) * A.R * A.R;
        const int grid4 = grid_for(n4, 256);
        if (src_r8)
            k_copy_alpha4<<<grid4, 256, 0, st>>>(dst, static_cast<const uint8_t*>(src), A, d->clip_level,
                                                 d->face_count, mirror, touched);
        else
            k_copy_alpha4<<<grid4, 256, 0, st>>>(dst, static_cast<const uint32_t*>(src), A, d->clip_level,
                                                 d->face_count, mirror, touched);
    } else if (src_r8)
        k_copy_alpha<<<grid, 256, 0, st>>>(dst, static_cast<const uint8_t*>(src), A, d->clip_level, lg, d->face_count,
                                           mirror, touched);
    else
        k_copy_alpha<<<grid, 256, 0, st>>>(dst, static_cast<const uint32_t*>(src), A, d->clip_level, lg, d->face_count,
                                           mirror, touched);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

int copy_alpha_downsample_pass(uint32_t* radiance, const void* opacity, const vct_downsample_desc* d,
                               cudaSurfaceObject_t mirror, const uint32_t* touched, cudaStream_t st, bool opa_r8) {
    VCT_CHECK_ARG(radiance && opacity && d, "vct_copy_alpha_downsample: null argument");
    VCT_CHECK_ARG((const void*)radiance != opacity, "vct_copy_alpha_downsample: radiance and opacity atlases must differ");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution),
                  "vct_copy_alpha_downsample: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 1 && d->clip_level < VCT_CLIP_LEVEL_COUNT,
                  "vct_copy_alpha_downsample: clip level must be 1..5");
    VCT_CHECK_ARG(d->downsample_region_size >= 0 && d->downsample_region_size <= 4096,
                  "vct_copy_alpha_downsample: downsample band out of range");
    AtlasDims A(d->clipmap_resolution);
    const int64_t n = (int64_t)A.R * A.R * A.R;
    int3 pm = make_int3(d->prev_region_min_corner[0], d->prev_region_min_corner[1], d->prev_region_min_corner[2]);
    const int lg = 31 - __builtin_clz((unsigned)A.R);
    const int grid = grid_for(n, 128);
    const int band = d->downsample_region_size, l = d->clip_level;
    if (opa_r8)
        k_alpha_downsample<<<grid, 128, 0, st>>>(radiance, radiance, static_cast<const uint8_t*>(opacity), A, pm, l,
                                                 band, lg, mirror, touched);
    else
        k_alpha_downsample<<<grid, 128, 0, st>>>(radiance, radiance, static_cast<const uint32_t*>(opacity), A, pm, l,
                                                 band, lg, mirror, touched);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

// The one-byte opacity form's mips 1..5 and border wrap (VoxelizationPass's
// end-of-pass dispatches on that form).
int opacity_r8_mips(uint8_t* atlas, const vct_clipmap_region regions[6], int R, cudaStream_t st) {
    AtlasDims A(R);
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    const int lgh = 31 - __builtin_clz((unsigned)half);
    for (int l = 1; l < VCT_CLIP_LEVEL_COUNT; ++l) {
        const int3 pm = make_int3(regions[l - 1].min_corner[0], regions[l - 1].min_corner[1], regions[l - 1].min_corner[2]);
        k_downsample_r8<<<grid_for(n, 128), 128, 0, st>>>(atlas, atlas, A, pm, l, VCT_DOWNSAMPLE_REGION_SIZE, lgh);
        VCT_LAUNCH_CHECK();
    }
    return VCT_OK;
}

int wrap_border_r8(uint8_t* atlas, int R, cudaStream_t st) {
    AtlasDims A(R);
    const int64_t shell = 3 * (int64_t)A.R * A.R - 3 * (int64_t)A.R + 1;
    const int64_t total = shell * VCT_FACE_COUNT * VCT_CLIP_LEVEL_COUNT;
    k_wrap_border<<<grid_for(total, 256), 256, 0, st>>>(atlas, A, VCT_FACE_COUNT, VCT_CLIP_LEVEL_COUNT);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

// The mirror texture must be an RGBA8 texture of the same resolution.
static int mirror_surface(vct_texture_s* t, int R, const char* who, cudaSurfaceObject_t* out) {
    *out = 0;
    if (!t) return VCT_OK;
    if (texture_format(t) != VCT_TEX_RGBA8 || texture_resolution(t) != R)
        return fail(VCT_E_BAD_ARG, who);
    *out = texture_surface(t);
    return VCT_OK;
}

}  // namespace vct

extern "C" int vct_copy_alpha(uint32_t* dst, const uint32_t* src, const vct_copy_alpha_desc* d, void* stream) {
    return copy_alpha_pass(dst, src, d, 0, nullptr, as_stream(stream), false);
}

extern "C" int vct_copy_alpha_downsample(uint32_t* radiance, const uint32_t* opacity, const vct_downsample_desc* d,
                                         vct_texture_s* mirror, void* stream) {
    VCT_CHECK_ARG(d, "vct_copy_alpha_downsample: null argument");
    cudaSurfaceObject_t surf = 0;
    int rc = mirror_surface(mirror, d->clipmap_resolution,
                            "vct_copy_alpha_downsample: the mirror must be an RGBA8 texture of the same resolution", &surf);
    if (rc != VCT_OK) return rc;
    return copy_alpha_downsample_pass(radiance, opacity, d, surf, nullptr, as_stream(stream), false);
}

extern "C" int vct_wrap_border(uint32_t* atlas, const vct_border_wrapping_desc* d, void* stream) {
    VCT_CHECK_ARG(atlas && d, "vct_wrap_border: null argument");
    VCT_CHECK_ARG(valid_resolution((int)d->clipmap_resolution), "vct_wrap_border: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_border_width == VCT_VOXEL_BORDER, "vct_wrap_border: border width must be 2 (one texel per side)");
    VCT_CHECK_ARG(d->face_count <= VCT_FACE_COUNT && d->clip_region_count <= VCT_CLIP_LEVEL_COUNT,
                  "vct_wrap_border: face/region count out of range");
    AtlasDims A((int)d->clipmap_resolution);
    if (d->face_count == 0 || d->clip_region_count == 0) return VCT_OK;
    const int64_t shell = 3 * (int64_t)A.R * A.R - 3 * (int64_t)A.R + 1;  // ((R+2)>>3)*8 == R here
    const int64_t total = shell * d->face_count * d->clip_region_count;
    k_wrap_border<<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(atlas, A, (int)d->face_count,
                                                                       (int)d->clip_region_count);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

// ----------------------------------------------- differentiable (float) mips
// The same level downsample on float RGBA texels (no 8-bit store), and its
// adjoint.  One output voxel g of level l per thread: its write position,
// the corner of its 2x2x2 child block in level l-1 and the band's lerp
// factor, as k_downsample computes them.
struct DsSite {
    int wpos[3], ps[3];
    float lerp;
};

__device__ __forceinline__ DsSite ds_site(const AtlasDims& A, int3 pmin, int level, int band, int lgh, uint32_t t) {
    const int half = A.R >> 1;
    const uint32_t m = (1u << lgh) - 1u;
    const int g[3] = {(int)(t & m), (int)((t >> lgh) & m), (int)(t >> (2 * lgh))};
    const int pm[3] = {pmin.x, pmin.y, pmin.z};
    DsSite s;
    float dist[3];
    bool any_ge = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int cur = (pm[a] >> 1) + g[a];
        s.wpos[a] = ds_wrap(cur, A.R) + 1;
        s.ps[a] = ds_wrap(cur << 1, A.R) + 1;
        const float center = __fadd_rn((float)(pm[a] >> 1), (float)(half >> 1));
        dist[a] = __fsub_rn(fabsf(__fsub_rn(__fadd_rn((float)cur, 0.5f), center)), 0.5f);
        any_ge |= dist[a] >= (float)((half >> 1) - band);
    }
    s.wpos[1] += A.rb * level;
    s.ps[1] += A.rb * (level - 1);
    s.lerp = 0.0f;
    if (any_ge) {
        const float inv = 1.0f / __fadd_rn((float)band, 1.0f);
        s.lerp = __fmul_rn(__fadd_rn(__fsub_rn(fmaxf(dist[0], fmaxf(dist[1], dist[2])), (float)((half >> 1) - band)), 1.0f), inv);
    }
    return s;
}

__device__ __forceinline__ int64_t ds_child(const AtlasDims& A, const DsSite& s, int f, int i) {
    return A.index(s.ps[0] + (i & 1) + A.rb * f, s.ps[1] + ((i >> 1) & 1), s.ps[2] + ((i >> 2) & 1));
}

template <int MODE>
__global__ void k_downsample_f32(float4* __restrict__ atlas, AtlasDims A, int3 pmin, int level, int band, int lgh) {
    const uint32_t n = 1u << (3 * lgh);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const DsSite st = ds_site(A, pmin, level, band, lgh, t);
        #pragma unroll
        for (int f = 0; f < 6; ++f) {
            float4 v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = atlas[ds_child(A, st, f, i)];
            const int64_t wi = A.index(st.wpos[0] + A.rb * f, st.wpos[1], st.wpos[2]);
            const float4 own = atlas[wi];
            if (MODE == 0) {
                float s = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float a0 = v[ds_pair(f, k, 0)].w, a1 = v[ds_pair(f, k, 1)].w;
                    const float tt = __fmul_rn(__fsub_rn(1.0f, a0), a1);
                    s = (k == 0) ? __fadd_rn(a0, tt) : __fadd_rn(__fadd_rn(s, a0), tt);
                }
                const float a = mix_rn(__fmul_rn(s, 0.25f), own.x, st.lerp);
                atlas[wi] = make_float4(own.x, a, own.z, a);
            } else {
                float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float4 a0 = v[ds_pair(f, k, 0)], a1 = v[ds_pair(f, k, 1)];
                    const float tt = __fsub_rn(1.0f, a0.w);
                    const float av[4] = {a0.x, a0.y, a0.z, a0.w}, bv[4] = {a1.x, a1.y, a1.z, a1.w};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float b = __fmul_rn(tt, bv[c]);
                        s[c] = (k == 0) ? __fadd_rn(av[c], b) : __fadd_rn(__fadd_rn(s[c], av[c]), b);
                    }
                }
                atlas[wi] = make_float4(mix_rn(__fmul_rn(s[0], 0.25f), own.x, st.lerp),
                                        mix_rn(__fmul_rn(s[1], 0.25f), own.y, st.lerp),
                                        mix_rn(__fmul_rn(s[2], 0.25f), own.z, st.lerp),
                                        mix_rn(__fmul_rn(s[3], 0.25f), own.w, st.lerp));
            }
        }
    }
}

// The adjoint of k_downsample_f32 for one level: G holds dL/d(atlas after
// the pass) and leaves with dL/d(atlas before it).  A written texel's
// gradient becomes its share through the blend (lerp; opacity: only x and
// the blended alpha's lerp share, y and w are overwritten); its child block
// gains the composite's shares: d/d a0 = 1 per channel and -sum_c g_c a1_c
// on a0's alpha, d/d a1 = (1 - a0.w) (opacity: 1 - a1 and 1 - a0 on the
// alphas).  Each (voxel, face) owns its written texel and its child block,
// so no two threads touch the same gradient.  `atlas` holds the forward's
// final values (a level's children are final before the level is mipped).
template <int MODE>
__global__ void k_downsample_backward(const float4* __restrict__ atlas, float4* __restrict__ G, AtlasDims A, int3 pmin,
                                      int level, int band, int lgh) {
    const uint32_t n = 1u << (3 * lgh);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const DsSite st = ds_site(A, pmin, level, band, lgh, t);
        #pragma unroll
        for (int f = 0; f < 6; ++f) {
            float4 v[8], gc[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                v[i] = atlas[ds_child(A, st, f, i)];
                gc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            const int64_t wi = A.index(st.wpos[0] + A.rb * f, st.wpos[1], st.wpos[2]);
            const float4 go = G[wi];
            if (MODE == 0) {
                const float ga = go.y + go.w;
                G[wi] = make_float4(go.x + ga * st.lerp, 0.0f, go.z, 0.0f);
                const float gs = ga * (1.0f - st.lerp) * 0.25f;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i0 = ds_pair(f, k, 0), i1 = ds_pair(f, k, 1);
                    gc[i0].w += gs * (1.0f - v[i1].w);
                    gc[i1].w += gs * (1.0f - v[i0].w);
                }
            } else {
                G[wi] = make_float4(go.x * st.lerp, go.y * st.lerp, go.z * st.lerp, go.w * st.lerp);
                const float w = (1.0f - st.lerp) * 0.25f;
                const float4 gs = make_float4(go.x * w, go.y * w, go.z * w, go.w * w);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i0 = ds_pair(f, k, 0), i1 = ds_pair(f, k, 1);
                    const float tt = 1.0f - v[i0].w;
                    gc[i0].x += gs.x;
                    gc[i0].y += gs.y;
                    gc[i0].z += gs.z;
                    gc[i0].w += gs.w - (gs.x * v[i1].x + gs.y * v[i1].y + gs.z * v[i1].z + gs.w * v[i1].w);
                    gc[i1].x += gs.x * tt;
                    gc[i1].y += gs.y * tt;
                    gc[i1].z += gs.z * tt;
                    gc[i1].w += gs.w * tt;
                }
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int64_t ci = ds_child(A, st, f, i);
                float4 g = G[ci];
                G[ci] = make_float4(g.x + gc[i].x, g.y + gc[i].y, g.z + gc[i].z, g.w + gc[i].w);
            }
        }
    }
}

static int check_ds_desc(const vct_downsample_desc* d, int32_t mode, const char* who) {
    VCT_CHECK_ARG(d, who);
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "downsample: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(d->clip_level >= 1 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "downsample: clip level must be 1..5");
    VCT_CHECK_ARG(mode == VCT_DOWNSAMPLE_OPACITY || mode == VCT_DOWNSAMPLE_RADIANCE, "downsample: bad mode");
    VCT_CHECK_ARG(d->downsample_region_size >= 0 && d->downsample_region_size <= 4096, "downsample: band out of range");
    return VCT_OK;
}

extern "C" int vct_downsample_f32(float* atlas4, const vct_downsample_desc* d, int32_t mode, void* stream) {
    VCT_CHECK_ARG(atlas4 && ((uintptr_t)atlas4 & 15) == 0, "vct_downsample_f32: null or unaligned atlas");
    int rc = check_ds_desc(d, mode, "vct_downsample_f32: null desc");
    if (rc != VCT_OK) return rc;
    AtlasDims A(d->clipmap_resolution);
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    const int3 pm = make_int3(d->prev_region_min_corner[0], d->prev_region_min_corner[1], d->prev_region_min_corner[2]);
    const int lgh = 31 - __builtin_clz((unsigned)half);
    float4* a = reinterpret_cast<float4*>(atlas4);
    if (mode == VCT_DOWNSAMPLE_OPACITY)
        k_downsample_f32<0><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(a, A, pm, d->clip_level, d->downsample_region_size, lgh);
    else
        k_downsample_f32<1><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(a, A, pm, d->clip_level, d->downsample_region_size, lgh);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_downsample_backward(const float* atlas4, float* grad4, const vct_downsample_desc* d, int32_t mode,
                                       void* stream) {
    VCT_CHECK_ARG(atlas4 && grad4 && (((uintptr_t)atlas4 | (uintptr_t)grad4) & 15) == 0 && atlas4 != grad4,
                  "vct_downsample_backward: null, unaligned or aliased atlases");
    int rc = check_ds_desc(d, mode, "vct_downsample_backward: null desc");
    if (rc != VCT_OK) return rc;
    AtlasDims A(d->clipmap_resolution);
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    const int3 pm = make_int3(d->prev_region_min_corner[0], d->prev_region_min_corner[1], d->prev_region_min_corner[2]);
    const int lgh = 31 - __builtin_clz((unsigned)half);
    const float4* a = reinterpret_cast<const float4*>(atlas4);
    float4* g = reinterpret_cast<float4*>(grad4);
    if (mode == VCT_DOWNSAMPLE_OPACITY)
        k_downsample_backward<0><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(a, g, A, pm, d->clip_level, d->downsample_region_size, lgh);
    else
        k_downsample_backward<1><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(a, g, A, pm, d->clip_level, d->downsample_region_size, lgh);
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
        k_downsample<0><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(atlas, atlas, A, pm, d->clip_level,
                                                                         d->downsample_region_size, lgh);
    else
        k_downsample<1><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(atlas, atlas, A, pm, d->clip_level,
                                                                         d->downsample_region_size, lgh);
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
