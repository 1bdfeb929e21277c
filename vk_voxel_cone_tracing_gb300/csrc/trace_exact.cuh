// trace_exact.cuh -- the FP32 cone march of voxelConeTracing.frag over a
// linear atlas in the reference's layout, generic in the atlas's texel type:
// ExactAtlas (RGBA8, the drop-in) and F4Atlas (float RGBA, the
// differentiable form).  Software trilinear filter with FP32 weights and
// REPEAT addressing; the units that include it build with -fmad=false, so
// every form runs the same arithmetic in the same order.
#pragma once

#include "trace_common.cuh"

namespace vct {

struct ExactAtlas {
    const uint32_t* __restrict__ p;
    AtlasDims A;
    __device__ __forceinline__ float4 fetch(int x, int y, int z) const { return unpack_rgba8(__ldg(p + A.index(x, y, z))); }
};

// The RGBA8 atlas's texels read through a radiance texture holding the same
// texels (point filter at texel centres, unnormalised coordinates): one
// texture instruction returns the four channels decoded to float by the
// texture unit, in place of the 64-bit address arithmetic, the 4-byte load
// and the four-channel decode.  The unit's unorm8 conversion gives c/255
// correctly rounded, the float unorm8_decode computes (the tests compare whole
// traces through both reads bit for bit), so the trace's arithmetic, in its
// order, is unchanged.
struct TexelAtlas {
    cudaTextureObject_t t;
    AtlasDims A;
    __device__ __forceinline__ float4 fetch(int x, int y, int z) const {
        return tex3D<float4>(t, (float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f);
    }
};

// Float RGBA texels (16 B each), the layout of the FP16 form widened to FP32.
struct F4Atlas {
    const float4* __restrict__ p;
    AtlasDims A;
    __device__ __forceinline__ float4 fetch(int x, int y, int z) const { return __ldg(p + A.index(x, y, z)); }
};

__device__ __forceinline__ int wrap_rep(int i, int n) {
    int m = i % n;
    return m < 0 ? m + n : m;
}

// REPEAT of a texel index that a sampler coordinate in [0, 1) produces
// (i in [-1, n]): one compare and select on that range; the general
// modulo for anything else, so no index leaves [0, n).
__device__ __forceinline__ int wrap_tap(int i, int n) {
    const int m = i < 0 ? i + n : (i >= n ? i - n : i);
    return (unsigned)m < (unsigned)n ? m : wrap_rep(i, n);
}

__device__ __forceinline__ float4 lerp4(float4 p, float4 q, float t) {
    return make_float4(p.x + (q.x - p.x) * t, p.y + (q.y - p.y) * t, p.z + (q.z - p.z) * t, p.w + (q.w - p.w) * t);
}

// Linear-filtered sampler3D fetch (Vulkan linear filter, REPEAT, one mip).
template <class Atlas>
__device__ __forceinline__ float4 texture3d(const Atlas& T, float ux, float uy, float uz) {
    const AtlasDims& A = T.A;
    float u = ux * (float)A.W - 0.5f, v = uy * (float)A.H - 0.5f, w = uz * (float)A.D - 0.5f;
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    float a = u - fu, b = v - fv, c = w - fw;
    int i0 = wrap_tap((int)fu, A.W), i1 = wrap_tap((int)fu + 1, A.W);
    int j0 = wrap_tap((int)fv, A.H), j1 = wrap_tap((int)fv + 1, A.H);
    int k0 = wrap_tap((int)fw, A.D), k1 = wrap_tap((int)fw + 1, A.D);
    float4 x00 = lerp4(T.fetch(i0, j0, k0), T.fetch(i1, j0, k0), a);
    float4 x10 = lerp4(T.fetch(i0, j1, k0), T.fetch(i1, j1, k0), a);
    float4 x01 = lerp4(T.fetch(i0, j0, k1), T.fetch(i1, j0, k1), a);
    float4 x11 = lerp4(T.fetch(i0, j1, k1), T.fetch(i1, j1, k1), a);
    return lerp4(lerp4(x00, x10, b), lerp4(x01, x11, b), c);
}

// sampleClipmap (voxelConeTracing.frag:313-327).
template <class Atlas>
__device__ __forceinline__ float4 sample_clipmap(const Atlas& T, const vct_cone_tracing_desc& d, float3 p,
                                                 int level, float3 fo, float3 wt) {
    float vs = d.voxel_size * exp2f((float)level);
    float extent = vs * d.volume_dimension;
    float dim = d.volume_dimension;
    float sx = (fractf(p.x / extent) * dim + 1.0f) / (dim + 2.0f);
    float sy = (fractf(p.y / extent) * dim + 1.0f) / (dim + 2.0f);
    float sz = (fractf(p.z / extent) * dim + 1.0f) / (dim + 2.0f);
    sy = sy + (float)level;
    sy = sy / (float)kClipLevels;
    sx = sx / (float)kFaces;
    float4 a = texture3d(T, sx + fo.x, sy, sz);
    float4 b = texture3d(T, sx + fo.y, sy, sz);
    float4 c = texture3d(T, sx + fo.z, sy, sz);
    return make_float4(a.x * wt.x + b.x * wt.y + c.x * wt.z, a.y * wt.x + b.y * wt.y + c.y * wt.z,
                       a.z * wt.x + b.z * wt.y + c.z * wt.z, a.w * wt.x + b.w * wt.y + c.w * wt.z);
}

// traceCone (voxelConeTracing.frag:341-392).
template <class Atlas>
__device__ float4 trace_cone(const Atlas& T, const vct_cone_tracing_desc& d, float3 start, float3 dir,
                             float aperture, float max_dist, float start_level, float step_factor,
                             unsigned long long& steps) {
    float4 result = make_float4(0.f, 0.f, 0.f, 0.f);
    const float uvs = d.voxel_size;
    const float cone_coef = 2.0f * tanf(aperture * 0.5f);
    float cur_level = start_level;
    float vs = uvs * exp2f(cur_level);
    start = start + dir * (vs * d.trace_start_offset * 0.5f);
    float step = 0.0f;
    float diameter = fmaxf(step * cone_coef, uvs);
    float occlusion = 0.0f;
    const float3 fo = f3(dir.x > 0.0f ? 0.0f : 1.0f / 6.0f, dir.y > 0.0f ? 2.0f / 6.0f : 3.0f / 6.0f,
                         dir.z > 0.0f ? 4.0f / 6.0f : 5.0f / 6.0f);
    const float3 wt = f3(dir.x * dir.x, dir.y * dir.y, dir.z * dir.z);
    float seg = vs;
    const float min_radius = uvs * d.volume_dimension * 0.5f;
    const float3 center = f3(d.volume_center[0], d.volume_center[1], d.volume_center[2]);
    while (step < max_dist && occlusion < 1.0f) {
        ++steps;
        float3 pos = start + dir * step;
        float dist = sqrtf(dot3(center - pos, center - pos));
        float min_level = ceilf(log2f(dist / min_radius));
        cur_level = log2f(diameter / uvs);
        cur_level = fminf(fmaxf(fmaxf(start_level, cur_level), min_level), (float)(kClipLevels - 1));
        int lower = (int)floorf(cur_level), upper = (int)ceilf(cur_level);
        float4 lo = sample_clipmap(T, d, pos, lower, fo, wt);
        // an integral level mixes lo with itself at fr = 0: lo * 1 + hi * 0 == lo exactly
        float4 hi = upper != lower ? sample_clipmap(T, d, pos, upper, fo, wt) : lo;
        float fr = fractf(cur_level);
        float4 s = make_float4(lo.x * (1.0f - fr) + hi.x * fr, lo.y * (1.0f - fr) + hi.y * fr,
                               lo.z * (1.0f - fr) + hi.z * fr, lo.w * (1.0f - fr) + hi.w * fr);
        vs = uvs * exp2f(cur_level);
        float correction = seg / vs;
        float rx = s.x * correction, ry = s.y * correction, rz = s.z * correction;
        // a filtered alpha rounded above 1 (the face weights sum to 1 + ulp) would make the base of pow
        // negative, which GLSL leaves undefined (NaN, then clamped to a transparent 0 on hardware); the
        // base is taken as 0 there: the sample is opaque
        float opacity = clampf(1.0f - powf(fmaxf(1.0f - s.w, 0.0f), correction), 0.0f, 1.0f);
        float k = clampf(1.0f - result.w, 0.0f, 1.0f);
        result = make_float4(result.x + k * rx, result.y + k * ry, result.z + k * rz, result.w + k * opacity);
        occlusion = occlusion + (1.0f - occlusion) * opacity / (1.0f + (step + vs) * d.occlusion_decay);
        float prev = step;
        step = step + fmaxf(diameter, uvs) * step_factor;
        seg = step - prev;
        diameter = step * cone_coef;
    }
    return make_float4(result.x, result.y, result.z, 1.0f - occlusion);
}

// The visiting plan of the exact forms and their adjoint: the samples in the
// coherent order (normal class, then Morton) and the specular samples listed
// grouped by aperture (log-spaced buckets of max(roughness, 0.05)), each group
// in the coherent order, with their count (device).  A cone's step count is
// about proportional to 1 / aperture, so the 32 cones of a warp taken from
// one group march nearly the same number of steps.  Stream-ordered scratch:
// release it with exact_plan_free after the last kernel that reads it.
struct ExactPlan {
    const uint32_t* order;
    uint32_t* spec_list;
    unsigned int* spec_count;
    void* block;
    void* order_block;
};
int exact_plan(const vct_surface_sample* samples, int64_t n, const vct_cone_tracing_desc& d, ExactPlan* plan,
               cudaStream_t st);
void exact_plan_free(ExactPlan* plan, cudaStream_t st);

// ---------------------------------------------------------------------------
// traceCone split into its volume-independent geometry, its step schedule
// and one step, for the adjoint's recomputation of a march.

// The cone as trace_cone sets it up (start already offset by half a step).
struct ConeGeo {
    float3 start, dir, fo, wt, center;
    float uvs, coef, start_level, step_factor, min_radius;
};

__device__ __forceinline__ ConeGeo make_cone(const vct_cone_tracing_desc& d, float3 start, float3 dir, float aperture,
                                             float start_level, float step_factor) {
    ConeGeo K;
    K.uvs = d.voxel_size;
    K.coef = 2.0f * tanf(aperture * 0.5f);
    const float vs = K.uvs * exp2f(start_level);
    K.start = start + dir * (vs * d.trace_start_offset * 0.5f);
    K.dir = dir;
    K.fo = f3(dir.x > 0.0f ? 0.0f : 1.0f / 6.0f, dir.y > 0.0f ? 2.0f / 6.0f : 3.0f / 6.0f,
              dir.z > 0.0f ? 4.0f / 6.0f : 5.0f / 6.0f);
    K.wt = f3(dir.x * dir.x, dir.y * dir.y, dir.z * dir.z);
    K.center = f3(d.volume_center[0], d.volume_center[1], d.volume_center[2]);
    K.min_radius = K.uvs * d.volume_dimension * 0.5f;
    K.start_level = start_level;
    K.step_factor = step_factor;
    return K;
}

// The loop's schedule at one step: distance, segment length, diameter.
struct Sched {
    float step, seg, diameter;
};

__device__ __forceinline__ Sched first_sched(const ConeGeo& K) {
    return Sched{0.0f, K.uvs * exp2f(K.start_level), fmaxf(0.0f * K.coef, K.uvs)};
}

// step += max(diameter, uvs) * stepFactor (the loop's expressions and order).
__device__ __forceinline__ void sched_advance(Sched& s, const ConeGeo& K) {
    const float prev = s.step;
    s.step = s.step + fmaxf(s.diameter, K.uvs) * K.step_factor;
    s.seg = s.step - prev;
    s.diameter = s.step * K.coef;
}

// Everything one step computes: its tap geometry (position, the two levels
// and the mix fraction), the filtered sample, the opacity correction, the raw
// and clamped opacity and the occlusion divisor.
struct StepDetail {
    float3 pos;
    int lower, upper;
    float fr, correction, op_raw, op, q;
    float4 smp;
};

template <class Atlas>
__device__ __forceinline__ StepDetail exact_step_detail(const Atlas& T, const vct_cone_tracing_desc& d,
                                                        const ConeGeo& K, const Sched& s) {
    StepDetail e;
    e.pos = K.start + K.dir * s.step;
    const float dist = sqrtf(dot3(K.center - e.pos, K.center - e.pos));
    const float min_level = ceilf(log2f(dist / K.min_radius));
    float cur_level = log2f(s.diameter / K.uvs);
    cur_level = fminf(fmaxf(fmaxf(K.start_level, cur_level), min_level), (float)(kClipLevels - 1));
    e.lower = (int)floorf(cur_level);
    e.upper = (int)ceilf(cur_level);
    const float4 lo = sample_clipmap(T, d, e.pos, e.lower, K.fo, K.wt);
    const float4 hi = e.upper != e.lower ? sample_clipmap(T, d, e.pos, e.upper, K.fo, K.wt) : lo;
    e.fr = fractf(cur_level);
    const float fr = e.fr;
    e.smp = make_float4(lo.x * (1.0f - fr) + hi.x * fr, lo.y * (1.0f - fr) + hi.y * fr,
                        lo.z * (1.0f - fr) + hi.z * fr, lo.w * (1.0f - fr) + hi.w * fr);
    const float vs = K.uvs * exp2f(cur_level);
    e.correction = s.seg / vs;
    e.op_raw = 1.0f - powf(fmaxf(1.0f - e.smp.w, 0.0f), e.correction);  // base >= 0 as in trace_cone
    e.op = clampf(e.op_raw, 0.0f, 1.0f);
    e.q = 1.0f + (s.step + vs) * d.occlusion_decay;
    return e;
}

}  // namespace vct
