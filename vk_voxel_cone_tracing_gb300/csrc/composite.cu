// composite.cu -- the passes after the cone trace: SpecularFilterPass
// (VFS/RenderPass/SpecularFilterPass.cpp, specularFilter.frag, filter.glsl,
// tonemapping.glsl) and FinalPass's copy into the B8G8R8A8_SRGB swapchain
// image (VFS/RenderPass/FinalPass.cpp, finalPass.frag, VFS/SwapChain.cpp:400-412),
// over headless RGBA32F device images (row-major, width x height float4).
//
// Sampling.  The filter samples the trace's RGBA32F contribution images with
// a LINEAR, CLAMP_TO_EDGE sampler at texCoord = pixel centre (a full-screen
// strip).  Pinned here as:
//   * a tap at a whole-texel offset (the centre, the bilateral's 15 x 15
//     window) reads that texel, the coordinate clamped to the image;
//   * the "Gaussian" blur's taps lie within blurSize = 0.01 texel of the
//     centre (radius = blurSize / textureSize in uv), so each bilinear tap
//     touches only the 3 x 3 neighbourhood and the whole blur is one fixed
//     3 x 3 stencil: the sum over the 32 directions x 8 rings of the taps'
//     exact bilinear weights plus the centre tap, divided by 8 * 32 - 15 = 241
//     (the shader's normaliser; with 257 taps the blur brightens by 257 / 241,
//     a quirk kept as is).  The stencil is accumulated in double on the host
//     (directions d from the shader's FP32 loop, cos / sin in double) and
//     rounded to FP32 once;
//   * the bilateral filter's weights follow normpdf3 / KERNEL in FP32 up to a
//     few ulp: the range term is one ex2 per tap and the constant factors
//     are folded into a 15 x 15 table.
// Everything else is FP32 without contraction (this unit is built with
// -fmad=false) in the shader's evaluation order.
#include <math.h>

#include "common.cuh"

namespace vct {
namespace {

constexpr int kBX = 32, kBY = 8, kHalo = 7;

struct FilterParams {
    float gamma, exposure;
    int tonemap, method;
    float stencil[9];        // Gaussian: [(dy + 1) * 3 + (dx + 1)], divided by 241
    float bilateral_exp2;    // -0.5 / sigma^2 * log2(e)
    float bw[225];           // bilateral weights without the range term, [i][j] = [x offset + 7][y offset + 7]
};

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// tonemapping.glsl Uncharted2Tonemap for one channel.
__device__ inline float uncharted2(float c) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F)) - E / F;
}

// tonemap(): Uncharted2 of colour * exposure, white-scaled by 1 / U2(11.2),
// then pow(., 1 / gamma); alpha passes through.
__device__ inline float4 tonemap(float4 c, float gamma, float exposure) {
    const float white = 1.0f / uncharted2(11.2f);
    const float e = 1.0f / gamma;
    return make_float4(powf(uncharted2(c.x * exposure) * white, e), powf(uncharted2(c.y * exposure) * white, e),
                       powf(uncharted2(c.z * exposure) * white, e), c.w);
}

__device__ inline float4 finish(float4 diffuse, float3 spec, const FilterParams& P) {
    float4 c = make_float4(diffuse.x + spec.x, diffuse.y + spec.y, diffuse.z + spec.z, diffuse.w);
    return P.tonemap == 1 ? tonemap(c, P.gamma, P.exposure) : c;
}

// Gaussian path: the 3 x 3 stencil at every pixel (its taps hit L1).
__global__ void __launch_bounds__(256) k_composite_gaussian(const float4* __restrict__ diffuse,
                                                            const float4* __restrict__ specular, int W, int H,
                                                            const FilterParams P, float4* __restrict__ out) {
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    if (x >= W || y >= H) return;
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int yy = min(max(y + r - 1, 0), H - 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int xx = min(max(x + c - 1, 0), W - 1);
            const float4 t = specular[(int64_t)yy * W + xx];
            const float w = P.stencil[r * 3 + c];
            acc = make_float3(acc.x + w * t.x, acc.y + w * t.y, acc.z + w * t.z);
        }
    }
    const int64_t i = (int64_t)y * W + x;
    out[i] = finish(diffuse[i], acc, P);
}

// Bilateral path (filter.glsl bilateralFilter): a 15 x 15 window staged in
// shared memory per 32 x 8 block.
__global__ void __launch_bounds__(256) k_composite_bilateral(const float4* __restrict__ diffuse,
                                                             const float4* __restrict__ specular, int W, int H,
                                                             const FilterParams P, float4* __restrict__ out) {
    constexpr int TW = kBX + 2 * kHalo, TH = kBY + 2 * kHalo;
    __shared__ float3 tile[TH][TW];
    const int x0 = blockIdx.x * kBX, y0 = blockIdx.y * kBY;
    for (int k = threadIdx.y * kBX + threadIdx.x; k < TW * TH; k += kBX * kBY) {
        const int ty = k / TW, tx = k - ty * TW;
        const int gx = min(max(x0 + tx - kHalo, 0), W - 1), gy = min(max(y0 + ty - kHalo, 0), H - 1);
        const float4 v = specular[(int64_t)gy * W + gx];
        tile[ty][tx] = make_float3(v.x, v.y, v.z);
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= W || y >= H) return;
    const float3 cc = tile[threadIdx.y + kHalo][threadIdx.x + kHalo];
    // factor = normpdf3(s - c, 10) * bZ * KERNEL[7+j] * KERNEL[7+i] as exp2(dd * c_e) * c_w[i][j]:
    // the constant part of normpdf3 times bZ times the two KERNEL entries is folded into c_w
    // (host-computed in the shader's order), the exp becomes one ex2 of dd * (-0.5 / sigma^2) * log2(e).
    // Within a few ulp of the shader's factor; the sums use fused multiply-adds.
    float Z = 0.0f;
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    const float ce = P.bilateral_exp2;
#pragma unroll 1
    for (int i = 0; i < 2 * kHalo + 1; ++i) {
#pragma unroll
        for (int j = 0; j < 2 * kHalo + 1; ++j) {
            const float3 s = tile[threadIdx.y + j][threadIdx.x + i];
            const float vx = s.x - cc.x, vy = s.y - cc.y, vz = s.z - cc.z;
            const float dd = __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, __fmul_rn(vx, vx)));
            const float f = __fmul_rn(ex2_approx(__fmul_rn(dd, ce)), P.bw[i * (2 * kHalo + 1) + j]);
            Z = __fadd_rn(Z, f);
            acc = make_float3(__fmaf_rn(f, s.x, acc.x), __fmaf_rn(f, s.y, acc.y), __fmaf_rn(f, s.z, acc.z));
        }
    }
    const int64_t idx = (int64_t)y * W + x;
    out[idx] = finish(diffuse[idx], make_float3(acc.x / Z, acc.y / Z, acc.z / Z), P);
}

// FinalPass into B8G8R8A8_SRGB: clamp to [0, 1], the sRGB transfer function
// on rgb (IEC 61966-2-1: 12.92 c below 0.0031308, else 1.055 c^(1/2.4) -
// 0.055), the pinned UNORM8 store; bytes B, G, R, A.
__device__ inline float srgb_encode(float c) {
    c = fminf(fmaxf(c, 0.0f), 1.0f);
    return c <= 0.0031308f ? c * 12.92f : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}

__global__ void __launch_bounds__(256) k_present_srgb8(const float4* __restrict__ rgba, int64_t n,
                                                       uint32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 c = rgba[i];
        out[i] = unorm8_store(srgb_encode(c.z)) | (unorm8_store(srgb_encode(c.y)) << 8) |
                 (unorm8_store(srgb_encode(c.x)) << 16) | (unorm8_store(c.w) << 24);
    }
}

// The Gaussian blur's 3 x 3 stencil (see the file comment).
void gaussian_stencil(float out[9]) {
    const float blur_size = 0.01f;
    const float two_pi = 6.28318530718f, directions = 32.0f, quality = 8.0f;
    double S[3][3] = {{0.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 0.0}};  // the centre tap
    for (float d = 0.0f; d < two_pi; d += two_pi / directions) {
        const double cd = cos((double)d), sd = sin((double)d);
        for (float i = 1.0f / quality; i <= 1.0f; i += 1.0f / quality) {
            const double ox = cd * (double)blur_size * (double)i, oy = sd * (double)blur_size * (double)i;
            const double bx = floor(ox), by = floor(oy);
            const double fx = ox - bx, fy = oy - by;
            const int cx = (int)bx + 1, cy = (int)by + 1;  // stencil cell of the lower texel (0 or 1)
            S[cy][cx] += (1.0 - fx) * (1.0 - fy);
            S[cy][cx + 1] += fx * (1.0 - fy);
            S[cy + 1][cx] += (1.0 - fx) * fy;
            S[cy + 1][cx + 1] += fx * fy;
        }
    }
    const double norm = (double)(quality * directions - 15.0f);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r * 3 + c] = (float)(S[r][c] / norm);
}

// normpdf's constant factor times bZ times KERNEL[7+j] * KERNEL[7+i], in the shader's order
// (filter.glsl KERNEL[15] = normpdf(x, 10) at x = -7..7, as the shader lists it).
void bilateral_weights(float w[225]) {
    static const float K[15] = {0.031225216f, 0.033322271f, 0.035206333f, 0.036826804f, 0.038138565f,
                                0.039104044f, 0.039695028f, 0.039894000f, 0.039695028f, 0.039104044f,
                                0.038138565f, 0.036826804f, 0.035206333f, 0.033322271f, 0.031225216f};
    const float sigma = 10.0f;
    const float bz = 1.0f / (0.39894f * 1.0f / sigma);  // 1 / normpdf(0, sigma)
    for (int i = 0; i < 15; ++i)
        for (int j = 0; j < 15; ++j) w[i * 15 + j] = 0.39894f / sigma * bz * K[j] * K[i];
}

int grid1(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

}  // namespace
}  // namespace vct

using namespace vct;

extern "C" int vct_specular_filter_stencil(float out_host[9]) {
    VCT_CHECK_ARG(out_host, "vct_specular_filter_stencil: null output");
    gaussian_stencil(out_host);
    return VCT_OK;
}

extern "C" int vct_specular_filter(const vct_specular_filter_desc* desc, const float* diffuse_rgba,
                                   const float* specular_rgba, int32_t width, int32_t height, float* out_rgba,
                                   void* stream) {
    vct::NvtxRange nvtx_range("vct_specular_filter");
    VCT_CHECK_ARG(desc && diffuse_rgba && specular_rgba && out_rgba, "vct_specular_filter: null argument");
    VCT_CHECK_ARG(width > 0 && height > 0 && width <= 32768 && height <= 32768, "vct_specular_filter: bad image size");
    VCT_CHECK_ARG(out_rgba != specular_rgba, "vct_specular_filter: the output must not alias the specular image");
    VCT_CHECK_ARG((((uintptr_t)diffuse_rgba | (uintptr_t)specular_rgba | (uintptr_t)out_rgba) & 15) == 0,
                  "vct_specular_filter: images must be 16-byte aligned");
    FilterParams P;
    P.gamma = desc->tonemap_gamma;
    P.exposure = desc->tonemap_exposure;
    P.tonemap = desc->tonemap_enable;
    P.method = desc->filter_method;
    gaussian_stencil(P.stencil);
    P.bilateral_exp2 = (float)(-0.5 / 100.0 * 1.4426950408889634);
    bilateral_weights(P.bw);
    const dim3 block(kBX, kBY), grid((width + kBX - 1) / kBX, (height + kBY - 1) / kBY);
    cudaStream_t st = as_stream(stream);
    const float4* d = reinterpret_cast<const float4*>(diffuse_rgba);
    const float4* s = reinterpret_cast<const float4*>(specular_rgba);
    float4* o = reinterpret_cast<float4*>(out_rgba);
    if (P.method == VCT_FILTER_GAUSSIAN) k_composite_gaussian<<<grid, block, 0, st>>>(d, s, width, height, P, o);
    else k_composite_bilateral<<<grid, block, 0, st>>>(d, s, width, height, P, o);  // 0 and any other value
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_present_srgb8(const float* rgba, int32_t width, int32_t height, uint32_t* out_bgra8, void* stream) {
    VCT_CHECK_ARG(rgba && out_bgra8, "vct_present_srgb8: null argument");
    VCT_CHECK_ARG(width > 0 && height > 0, "vct_present_srgb8: bad image size");
    VCT_CHECK_ARG(((uintptr_t)rgba & 15) == 0, "vct_present_srgb8: the image must be 16-byte aligned");
    const int64_t n = (int64_t)width * height;
    k_present_srgb8<<<grid1(n), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float4*>(rgba), n, out_bgra8);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}
