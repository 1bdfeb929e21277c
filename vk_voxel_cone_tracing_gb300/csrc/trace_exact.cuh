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
    int i0 = wrap_rep((int)fu, A.W), i1 = wrap_rep((int)fu + 1, A.W);
    int j0 = wrap_rep((int)fv, A.H), j1 = wrap_rep((int)fv + 1, A.H);
    int k0 = wrap_rep((int)fw, A.D), k1 = wrap_rep((int)fw + 1, A.D);
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
        float opacity = clampf(1.0f - powf(1.0f - s.w, correction), 0.0f, 1.0f);
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

// ---------------------------------------------------------------------------
// traceCone split into its volume-independent geometry, its step schedule
// and one step, for kernels that march a cone's steps on several lanes.

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

// One step of the loop at schedule s: the filtered sample scaled by the
// opacity correction (rgb), the corrected opacity and the occlusion divisor
// q = 1 + (step + vs) * decay.
struct ExactStep {
    float r, g, b, op, q;
};

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
    e.op_raw = 1.0f - powf(1.0f - e.smp.w, e.correction);
    e.op = clampf(e.op_raw, 0.0f, 1.0f);
    e.q = 1.0f + (s.step + vs) * d.occlusion_decay;
    return e;
}

template <class Atlas>
__device__ __forceinline__ ExactStep exact_step(const Atlas& T, const vct_cone_tracing_desc& d, const ConeGeo& K,
                                                const Sched& s) {
    const StepDetail e = exact_step_detail(T, d, K, s);
    return ExactStep{e.smp.x * e.correction, e.smp.y * e.correction, e.smp.z * e.correction, e.op, e.q};
}

// A run of steps composited front to back: rgb and alpha by the "over"
// operator, t = the product of (1 - op / q) (1 - occlusion).
struct Composite {
    float r, g, b, a, t;
};

__device__ __forceinline__ Composite over(const Composite& p, const Composite& q) {
    const float k = clampf(1.0f - p.a, 0.0f, 1.0f);
    return Composite{p.r + k * q.r, p.g + k * q.g, p.b + k * q.b, p.a + k * q.a, p.t * q.t};
}

__device__ __forceinline__ Composite as_composite(const ExactStep& e) {
    return Composite{e.r, e.g, e.b, e.op, 1.0f - e.op / e.q};
}

__device__ __forceinline__ Composite shfl_composite(const Composite& c, int src) {
    return Composite{__shfl_sync(0xffffffffu, c.r, src), __shfl_sync(0xffffffffu, c.g, src),
                     __shfl_sync(0xffffffffu, c.b, src), __shfl_sync(0xffffffffu, c.a, src),
                     __shfl_sync(0xffffffffu, c.t, src)};
}

// Consecutive steps of one cone per lane in the warp-cooperative march.
constexpr int kExactStepsPerLane = 2;

// traceCone marched by a whole warp, 64 steps per round: lane j takes steps
// 2j, 2j + 1 of the round.  The schedule is a serial FP32 recurrence, so each
// lane advances it from the round's first step to its own (the positions are
// the loop's, bit for bit); the composite is the associative "over" operator
// and 1 - occlusion a product, so a warp scan composes the lanes.  The first
// lane whose composite reaches occlusion 1 marches its steps again with the
// loop's own update from the state before them and stops where the loop
// does.  Returns (rgb, 1 - occlusion) to every lane.
template <class Atlas>
__device__ float4 trace_cone_warp_exact(const Atlas& T, const vct_cone_tracing_desc& d, const ConeGeo& K,
                                        float max_dist, unsigned long long& steps) {
    constexpr int S = kExactStepsPerLane;
    const int lane = threadIdx.x & 31;
    const Composite id{0.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    Composite carried = id;
    Sched round0 = first_sched(K);
    unsigned long long it = 0;
    for (;;) {
        Sched s = round0;
        for (int k = 0; k < S * lane; ++k) sched_advance(s, K);
        const Sched mine = s;
        Composite x = id;
        int nvalid = 0;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            if (s.step < max_dist) {
                x = over(x, as_composite(exact_step(T, d, K, s)));
                ++nvalid;
            }
            sched_advance(s, K);
        }
        // inclusive scan of the lanes' composites
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const Composite p = shfl_composite(x, (lane - o) & 31);
            if (lane >= o) x = over(p, x);
        }
        const Composite after = over(carried, x);
        const unsigned tmask = __ballot_sync(0xffffffffu, nvalid > 0 && (1.0f - after.t) >= 1.0f);
        if (tmask) {  // occlusion reaches 1 within lane L's steps: the loop stops after that step
            const int L = __ffs(tmask) - 1;
            const Composite prior = shfl_composite(x, (lane - 1) & 31);
            Composite y = carried;
            int done = 0;
            if (lane == L) {
                const Composite before = lane == 0 ? carried : over(carried, prior);
                float4 result = make_float4(before.r, before.g, before.b, before.a);
                float occ = 1.0f - before.t;
                Sched q = mine;
                for (int k = 0; k < S && q.step < max_dist && occ < 1.0f; ++k) {
                    const ExactStep e = exact_step(T, d, K, q);
                    const float kk = clampf(1.0f - result.w, 0.0f, 1.0f);
                    result = make_float4(result.x + kk * e.r, result.y + kk * e.g, result.z + kk * e.b,
                                         result.w + kk * e.op);
                    occ = occ + (1.0f - occ) * e.op / e.q;
                    ++done;
                    sched_advance(q, K);
                }
                y = Composite{result.x, result.y, result.z, result.w, 1.0f - occ};
            }
            carried = shfl_composite(y, L);
            it += (unsigned long long)(S * L + __shfl_sync(0xffffffffu, done, L));
            break;
        }
        carried = shfl_composite(after, 31);
        int nv = nvalid;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nv += __shfl_xor_sync(0xffffffffu, nv, o);
        it += (unsigned long long)nv;
        if (nv < 32 * S) break;  // maxDistance reached within the round
        round0 = Sched{__shfl_sync(0xffffffffu, s.step, 31), __shfl_sync(0xffffffffu, s.seg, 31),
                       __shfl_sync(0xffffffffu, s.diameter, 31)};
    }
    if (lane == 0) steps += it;
    const float occlusion = 1.0f - carried.t;
    return make_float4(carried.r, carried.g, carried.b, 1.0f - occlusion);
}

}  // namespace vct
