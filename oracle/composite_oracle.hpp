// composite_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the passes after the cone trace:
//   * SpecularFilterPass (VFS/RenderPass/SpecularFilterPass.cpp:72-86) with
//     specularFilter.frag:26-56, filter.glsl (gaussianBlur :9-23,
//     bilateralFilter :40-60) and tonemapping.glsl (Uncharted2Tonemap :11-22,
//     tonemap :24-29), sampled through a LINEAR / CLAMP_TO_EDGE sampler at
//     pixel centres.  Pinned sampling: whole-texel taps read the clamped
//     texel; the Gaussian blur's sub-texel taps are evaluated as exact
//     bilinear weights, accumulated over all 257 taps in double into a 3 x 3
//     stencil divided by the shader's 241 and rounded to FP32 once;
//   * FinalPass into B8G8R8A8_SRGB (VFS/SwapChain.cpp:400-412): clamp, sRGB
//     transfer function, UNORM8 store with round half up.
// FP32 without contraction otherwise; exp / pow are the host libm's.
#pragma once

#include <cmath>
#include <cstdint>

namespace vcto {

struct FilterDesc {  // SpecularFilterPass push constants
    float gamma, exposure;
    int32_t tonemap, method;
};

// Exact bilinear weights of every tap of gaussianBlur(tex, uv, 0.01) on the
// 3 x 3 texel neighbourhood, divided by 8 * 32 - 15.
inline void gaussian_stencil(float w[9]) {
    double acc[9] = {0, 0, 0, 0, 1.0, 0, 0, 0, 0};  // the centre tap
    const float dpi = 6.28318530718f;
    const float blur = 0.01f;
    for (float d = 0.0f; d < dpi; d += dpi / 32.0f) {  // the shader's FP32 loop
        const double c = std::cos((double)d), s = std::sin((double)d);
        for (float i = 0.125f; i <= 1.0f; i += 0.125f) {
            const double px = c * (double)blur * (double)i, py = s * (double)blur * (double)i;
            const int x0 = (int)std::floor(px), y0 = (int)std::floor(py);  // -1 or 0
            const double ax = px - x0, ay = py - y0;
            const int col = x0 + 1, row = y0 + 1;
            acc[row * 3 + col] += (1.0 - ax) * (1.0 - ay);
            acc[row * 3 + col + 1] += ax * (1.0 - ay);
            acc[(row + 1) * 3 + col] += (1.0 - ax) * ay;
            acc[(row + 1) * 3 + col + 1] += ax * ay;
        }
    }
    for (int k = 0; k < 9; ++k) w[k] = (float)(acc[k] / 241.0);
}

inline float u2_tonemap(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    const float num = x * (A * x + C * B) + D * E;
    const float den = x * (A * x + B) + D * F;
    return num / den - E / F;
}

// specularFilter.frag over whole images (RGBA32F, row-major).
inline void specular_filter(const FilterDesc& fd, const float* diffuse, const float* specular, int W, int H,
                            float* out) {
    auto texel = [&](int x, int y) {
        x = x < 0 ? 0 : (x >= W ? W - 1 : x);
        y = y < 0 ? 0 : (y >= H ? H - 1 : y);
        return specular + 4 * ((int64_t)y * W + x);
    };
    float stencil[9];
    gaussian_stencil(stencil);
    static const float K[15] = {0.031225216f, 0.033322271f, 0.035206333f, 0.036826804f, 0.038138565f,
                                0.039104044f, 0.039695028f, 0.039894000f, 0.039695028f, 0.039104044f,
                                0.038138565f, 0.036826804f, 0.035206333f, 0.033322271f, 0.031225216f};
    const float sigma = 10.0f;
    const float bz = 1.0f / (0.39894f * std::exp(-0.5f * 0.0f * 0.0f / (sigma * sigma)) / sigma);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float sp[3] = {0.0f, 0.0f, 0.0f};
            if (fd.method == 1) {
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) {
                        const float* t = texel(x + c - 1, y + r - 1);
                        for (int k = 0; k < 3; ++k) sp[k] = sp[k] + stencil[r * 3 + c] * t[k];
                    }
            } else {
                const float* ctr = texel(x, y);
                float Z = 0.0f;
                for (int i = -7; i <= 7; ++i)
                    for (int j = -7; j <= 7; ++j) {
                        const float* t = texel(x + i, y + j);
                        const float v0 = t[0] - ctr[0], v1 = t[1] - ctr[1], v2 = t[2] - ctr[2];
                        const float dot = (v0 * v0 + v1 * v1) + v2 * v2;
                        const float g = 0.39894f * std::exp(-0.5f * dot / (sigma * sigma)) / sigma;
                        const float f = g * bz * K[7 + j] * K[7 + i];
                        Z = Z + f;
                        for (int k = 0; k < 3; ++k) sp[k] = sp[k] + f * t[k];
                    }
                for (int k = 0; k < 3; ++k) sp[k] = sp[k] / Z;
            }
            const float* d = diffuse + 4 * ((int64_t)y * W + x);
            float* o = out + 4 * ((int64_t)y * W + x);
            for (int k = 0; k < 3; ++k) o[k] = d[k] + sp[k];
            o[3] = d[3];
            if (fd.tonemap == 1) {
                const float white = 1.0f / u2_tonemap(11.2f);
                for (int k = 0; k < 3; ++k) o[k] = std::pow(u2_tonemap(o[k] * fd.exposure) * white, 1.0f / fd.gamma);
            }
        }
}

inline float srgb_oetf(float c) {
    c = std::fmin(std::fmax(c, 0.0f), 1.0f);
    if (c <= 0.0031308f) return c * 12.92f;
    return 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f;
}

inline uint32_t unorm8_round_half_up(float x) {
    const float c = std::fmin(std::fmax(x, 0.0f), 1.0f);
    return (uint32_t)std::floor(c * 255.0f + 0.5f);
}

inline void present_srgb8(const float* rgba, int64_t n, uint32_t* out) {
    for (int64_t i = 0; i < n; ++i) {
        const float* p = rgba + 4 * i;
        out[i] = unorm8_round_half_up(srgb_oetf(p[2])) | (unorm8_round_half_up(srgb_oetf(p[1])) << 8) |
                 (unorm8_round_half_up(srgb_oetf(p[0])) << 16) | (unorm8_round_half_up(p[3]) << 24);
    }
}

}  // namespace vcto
