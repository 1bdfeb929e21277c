// trace_common.cuh -- device-side pieces of voxelConeTracing.frag shared by
// the cone-tracing kernels: cone tables, calcMinLevel, the PBR direct term,
// the shadow "PCF" and the per-sample epilogue (rendering-mode switch).
#pragma once

#include "common.cuh"

namespace vct {

// voxelConeTracing.frag:78-135.
__constant__ float c_dirs16[16][3] = {
    {0.57735f, 0.57735f, 0.57735f},       {0.57735f, -0.57735f, -0.57735f},     {-0.57735f, 0.57735f, -0.57735f},
    {-0.57735f, -0.57735f, 0.57735f},     {-0.903007f, -0.182696f, -0.388844f}, {-0.903007f, 0.182696f, 0.388844f},
    {0.903007f, -0.182696f, 0.388844f},   {0.903007f, 0.182696f, -0.388844f},   {-0.388844f, -0.903007f, -0.182696f},
    {0.388844f, -0.903007f, 0.182696f},   {0.388844f, 0.903007f, -0.182696f},   {-0.388844f, 0.903007f, 0.182696f},
    {-0.182696f, -0.388844f, -0.903007f}, {0.182696f, 0.388844f, -0.903007f},   {-0.182696f, 0.388844f, 0.903007f},
    {0.182696f, -0.388844f, 0.903007f}};
__constant__ float c_dirs32[32][3] = {
    {0.898904f, 0.435512f, 0.0479745f},   {0.898904f, -0.435512f, -0.0479745f}, {0.898904f, 0.0479745f, -0.435512f},
    {0.898904f, -0.0479745f, 0.435512f},  {-0.898904f, 0.435512f, -0.0479745f}, {-0.898904f, -0.435512f, 0.0479745f},
    {-0.898904f, 0.0479745f, 0.435512f},  {-0.898904f, -0.0479745f, -0.435512f}, {0.0479745f, 0.898904f, 0.435512f},
    {-0.0479745f, 0.898904f, -0.435512f}, {-0.435512f, 0.898904f, 0.0479745f},  {0.435512f, 0.898904f, -0.0479745f},
    {-0.0479745f, -0.898904f, 0.435512f}, {0.0479745f, -0.898904f, -0.435512f}, {0.435512f, -0.898904f, 0.0479745f},
    {-0.435512f, -0.898904f, -0.0479745f}, {0.435512f, 0.0479745f, 0.898904f},  {-0.435512f, -0.0479745f, 0.898904f},
    {0.0479745f, -0.435512f, 0.898904f},  {-0.0479745f, 0.435512f, 0.898904f},  {0.435512f, -0.0479745f, -0.898904f},
    {-0.435512f, 0.0479745f, -0.898904f}, {0.0479745f, 0.435512f, -0.898904f},  {-0.0479745f, -0.435512f, -0.898904f},
    {0.57735f, 0.57735f, 0.57735f},       {0.57735f, 0.57735f, -0.57735f},      {0.57735f, -0.57735f, 0.57735f},
    {0.57735f, -0.57735f, -0.57735f},     {-0.57735f, 0.57735f, 0.57735f},      {-0.57735f, 0.57735f, -0.57735f},
    {-0.57735f, -0.57735f, 0.57735f},     {-0.57735f, -0.57735f, -0.57735f}};

constexpr float kAperture16 = 0.872665f;
constexpr float kAperture32 = 0.628319f;
constexpr float kMinTraceStepFactor = 0.2f;
constexpr float kMaxTraceDistance = 30.0f;
constexpr float kMinSpecularAperture = 0.05f;
constexpr int kClipLevels = 6;
constexpr int kFaces = 6;

// Trace parameters as the kernels consume them (the 52-byte push constants
// plus the camera eye and the lighting inputs of the direct term).
struct TraceParams {
    vct_cone_tracing_desc d;
    float eye[3];
    vct_directional_light_desc light;
    vct_directional_light_shadow_desc shadow_desc;
    const float* shadow;  // may be null: visibility 1
    int shadow_w, shadow_h;
    float diffuse_aperture;  // the diffuse cones' aperture: the shader's constant unless an option sets it
};

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 normalize3(float3 a) {
    float inv = 1.0f / sqrtf(dot3(a, a));
    return a * inv;
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }

// calcMinLevel (voxelConeTracing.frag:394-414).
__device__ __forceinline__ float calc_min_level(const vct_cone_tracing_desc& d, float3 wp) {
    float3 c = f3(d.volume_center[0], d.volume_center[1], d.volume_center[2]);
    float dist = sqrtf(dot3(c - wp, c - wp));
    float min_radius = d.voxel_size * d.volume_dimension * 0.5f;
    float min_level = fmaxf(log2f(dist / min_radius), 0.0f);
    float radius = min_radius * exp2f(ceilf(min_level));
    float f = dist / radius;
    const float ts = 0.5f;
    float cc = 1.0f / (1.0f - ts);
    if (f > ts) return ceilf(min_level) + (f - ts) * cc;
    return ceilf(min_level);
}

// One bilinear CLAMP_TO_BORDER(0) tap of the D32 shadow map.
__device__ __forceinline__ float shadow_tap(const float* __restrict__ depth, int W, int H, float s, float t) {
    float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    int i0 = (int)fu, j0 = (int)fv;
    auto at = [&](int i, int j) -> float {
        if (i < 0 || j < 0 || i >= W || j >= H) return 0.0f;
        return __ldg(depth + (int64_t)j * W + i);
    };
    float t00 = at(i0, j0), t10 = at(i0 + 1, j0), t01 = at(i0, j0 + 1), t11 = at(i0 + 1, j0 + 1);
    float r0 = t00 + (t10 - t00) * a;
    float r1 = t01 + (t11 - t01) * a;
    return r0 + (r1 - r0) * b;
}

// calcVisibility + calcShadowCoefficientPCF16 (shadow.glsl:8-36).
__device__ __forceinline__ float calc_visibility(const TraceParams& p, float3 wp) {
    if (!p.shadow) return 1.0f;
    const float* V = p.shadow_desc.view;
    const float* P = p.shadow_desc.proj;
    float lx = V[0] * wp.x + V[4] * wp.y + V[8] * wp.z + V[12] * 1.0f;
    float ly = V[1] * wp.x + V[5] * wp.y + V[9] * wp.z + V[13] * 1.0f;
    float px = P[0] * lx + P[4] * ly + P[8] * 0.0f + P[12] * 1.0f;
    float py = P[1] * lx + P[5] * ly + P[9] * 0.0f + P[13] * 1.0f;
    float sx = px * 0.5f + 0.5f, sy = py * 0.5f + 0.5f;
    float scx = 1.0f / (float)p.shadow_w, scy = 1.0f / (float)p.shadow_h;
    float sum = 0.0f;
    for (int yi = 0; yi < 4; ++yi)
        for (int xi = 0; xi < 4; ++xi) {
            float ox = -1.5f + (float)xi, oy = -1.5f + (float)yi;
            sum += shadow_tap(p.shadow, p.shadow_w, p.shadow_h, sx + ox * scx * 1.0f, sy + oy * scy * 1.0f);
        }
    return sum * 0.0625f;
}

// microfacetBRDF (brdf.glsl:28-78) for the PBRInfo of voxelConeTracing.frag:225-252.
__device__ __forceinline__ float3 microfacet_brdf(float NdotL, float NdotV, float NdotH, float VdotH, float3 r0,
                                                  float3 r90, float alpha_r, float3 dcol) {
    const float kPi = 3.141592f;
    float fres = powf(clampf(1.0f - VdotH, 0.0f, 1.0f), 5.0f);
    float F[3] = {r0.x + (r90.x - r0.x) * fres, r0.y + (r90.y - r0.y) * fres, r0.z + (r90.z - r0.z) * fres};
    float r = alpha_r;
    float attL = 2.0f * NdotL / (NdotL + sqrtf(r * r + (1.0f - r * r) * (NdotL * NdotL)));
    float attV = 2.0f * NdotV / (NdotV + sqrtf(r * r + (1.0f - r * r) * (NdotV * NdotV)));
    float G = attL * attV;
    float rsq = alpha_r * alpha_r;
    float f = (NdotH * rsq - NdotH) * NdotH + 1.0f;
    float D = rsq / (kPi * f * f);
    float diff[3] = {dcol.x / kPi, dcol.y / kPi, dcol.z / kPi};
    float out[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float dc = (1.0f - F[i]) * diff[i];
        float sc = F[i] * G * D / (4.0f * NdotL * NdotV);
        out[i] = NdotL * 1.0f * (dc + sc);
    }
    return f3(out[0], out[1], out[2]);
}

// Decoded G-buffer texel set of one sample.
struct GSample {
    float3 wp, normal, view, diffuse_color, specular_color, emission;
    float roughness, metallic, depth;
};

__device__ __forceinline__ GSample load_sample(const vct_surface_sample* __restrict__ s, const float eye[3]) {
    const float4* p = reinterpret_cast<const float4*>(s);
    float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4);
    GSample g;
    g.wp = f3(a.x, a.y, a.z);
    g.depth = a.w;
    g.view = normalize3(f3(eye[0], eye[1], eye[2]) - g.wp);
    g.normal = normalize3(f3(b.x * 2.0f - 1.0f, b.y * 2.0f - 1.0f, b.z * 2.0f - 1.0f));
    g.diffuse_color = f3(c.x, c.y, c.z);
    g.roughness = c.w;
    g.specular_color = f3(d.x, d.y, d.z);
    g.metallic = d.w;
    g.emission = f3(e.x, e.y, e.z);
    return g;
}

__device__ __forceinline__ bool has_specular_cone(const GSample& g) {
    return (g.specular_color.x > 1e-6f || g.specular_color.y > 1e-6f || g.specular_color.z > 1e-6f) &&
           g.metallic > 1e-6f;
}

__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - n * (2.0f * dot3(n, i)); }

// The direct term of main() (voxelConeTracing.frag:218-253).
__device__ __forceinline__ float3 direct_term(const TraceParams& p, const GSample& g) {
    bool has_emission = g.emission.x > 0.0f || g.emission.y > 0.0f || g.emission.z > 0.0f;
    if (has_emission) return g.emission;
    float alpha_r = g.roughness * g.roughness;
    float reflectance = fmaxf(fmaxf(g.specular_color.x, g.specular_color.y), g.specular_color.z);
    float r90v = clampf(reflectance * 50.0f, 0.0f, 1.0f);
    float3 l = normalize3(f3(-p.light.direction[0], -p.light.direction[1], -p.light.direction[2]));
    float3 h = normalize3(l + g.view);
    float NdotL = clampf(dot3(g.normal, l), 0.001f, 1.0f);
    float NdotV = clampf(fabsf(dot3(g.normal, g.view)), 0.001f, 1.0f);
    float NdotH = clampf(dot3(g.normal, h), 0.0f, 1.0f);
    float VdotH = clampf(dot3(g.view, h), 0.0f, 1.0f);
    float vis = calc_visibility(p, g.wp);
    float3 b = microfacet_brdf(NdotL, NdotV, NdotH, VdotH, g.specular_color, f3(r90v, r90v, r90v), alpha_r,
                               g.diffuse_color);
    return b * vis;
}

// The rendering-mode switch at the end of main() (voxelConeTracing.frag:255-293).
// `indirect` is the normalised, AO-scaled, albedo-scaled diffuse sum.
__device__ __forceinline__ void write_outputs(const TraceParams& p, const GSample& g, float min_level, float4 indirect,
                                              float3 ispec, float3 direct, float* __restrict__ dout,
                                              float* __restrict__ sout) {
    float4 D = make_float4(0.f, 0.f, 0.f, 1.f), S = make_float4(0.f, 0.f, 0.f, 1.f);
    switch (p.d.rendering_mode) {
        case 0: D = make_float4(g.diffuse_color.x, g.diffuse_color.y, g.diffuse_color.z, 1.f); break;
        case 1: D = make_float4(g.specular_color.x, g.specular_color.y, g.specular_color.z, 1.f); break;
        case 2:
            D = make_float4(g.normal.x * 0.5f + 0.5f, g.normal.y * 0.5f + 0.5f, g.normal.z * 0.5f + 0.5f, 1.f);
            break;
        case 3: {
            const float colors[7][4] = {{1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {1, 1, 0, 1},
                                        {0, 1, 1, 1}, {1, 0, 1, 1}, {1, 1, 1, 1}};
            int lo = min(max((int)floorf(min_level), 0), 5);
            float f = fractf(min_level);
            float v[4];
            for (int c = 0; c < 4; ++c) v[c] = (colors[lo][c] * (1.0f - f) + colors[lo + 1][c] * f) * 0.5f;
            D = make_float4(v[0], v[1], v[2], v[3]);
            break;
        }
        case 4:
            direct = direct * indirect.w;
            D = make_float4(direct.x, direct.y, direct.z, 1.f);
            break;
        case 5:
            direct = direct * indirect.w;
            D.x = D.x + direct.x + indirect.x;
            D.y = D.y + direct.y + indirect.y;
            D.z = D.z + direct.z + indirect.z;
            break;
        case 6:
            S.x += ispec.x;
            S.y += ispec.y;
            S.z += ispec.z;
            break;
        case 7: D = make_float4(indirect.w, indirect.w, indirect.w, 1.f); break;
        default:
            direct = direct * indirect.w;
            D.x = D.x + direct.x + indirect.x;
            D.y = D.y + direct.y + indirect.y;
            D.z = D.z + direct.z + indirect.z;
            S.x += ispec.x;
            S.y += ispec.y;
            S.z += ispec.z;
            break;
    }
    reinterpret_cast<float4*>(dout)[0] = D;
    reinterpret_cast<float4*>(sout)[0] = S;
}

// A coherent processing order of G-buffer samples: radix-sorted by normal
// class (6 bits, octahedral 8 x 8) and then by the Morton code of the
// position on a grid of two level-0 voxels per cell around the volume centre
// (10 bits per axis, 64-bit keys).  Per-sample results do not depend on the processing
// order, so the per-thread kernels walk this permutation: a warp's lanes skip
// the same diffuse cones and their texel fetches (and the adjoint's gradient
// atomics) land on neighbouring cache lines.  Allocates its buffers
// stream-ordered: `*block` is freed with cudaFreeAsync after the last kernel
// that reads `*order`.  For n >= 2^31 it returns VCT_OK with *order = nullptr
// (identity order).
struct SampleOrder {
    uint32_t* order = nullptr;
    void* block = nullptr;
};
int sample_coherent_order(const vct_surface_sample* samples, int64_t n, const vct_cone_tracing_desc& d,
                        SampleOrder* out, cudaStream_t st);

}  // namespace vct
