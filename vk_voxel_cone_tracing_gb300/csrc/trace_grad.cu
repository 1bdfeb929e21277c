// trace_grad.cu -- the adjoint of the FP32 cone trace over a float atlas
// (vct_cone_trace_f32): given dL/d(diffuse out) and dL/d(specular out) per
// sample, accumulate dL/d(texel) into a float RGBA atlas of the same layout.
//
// The march's step schedule, levels, tap positions, opacity corrections and
// occlusion divisors depend on geometry only; the number of steps depends on
// the volume through the occlusion stop and is held fixed (the derivative of
// a piecewise-smooth function away from its switches).  The clamps of the
// opacity and of 1 - alpha pass the derivative of their argument when it lies
// in [0, 1], bounds included: from an empty texel (alpha 0) the opacity's
// right derivative reaches it, which is the one inverse fitting needs.
//
// With T_i = prod_{m<i} (1 - op_m) (the weight clamp(1 - alpha) of step i),
// U_i = prod_{m<i} (1 - op_m / q_m) (1 - occlusion before step i),
// q_i = 1 + (t_i + vs_i) decay and c_i the opacity correction, the cone
// returns C = sum_i T_i c_i s_i.rgb and O = 1 - U_n, so for L = gC . C + gO O
//     dL/d(s_i.rgb) = gC T_i c_i
//     dL/d(op_i)    = -T_i R_i + gO U_i V_i / q_i,
//     R_i = sum_{j>i} prod_{i<m<j} (1 - op_m) c_j gC . s_j.rgb,
//     V_i = prod_{j>i} (1 - op_j / q_j),
//     dL/d(s_i.a)   = dL/d(op_i) c_i (1 - s_i.a)^(c_i - 1).
// g(s_i) is split over the two levels (1 - fr, fr), the three faces (the
// direction weights) and the eight texels of each trilinear tap (the products
// of the lerp fractions) and added to the gradient atlas with float4 atomics.
// Same FP32 expressions as the forward kernels (this unit is built with
// -fmad=false like them), so the recomputed steps are the forward's.
//
// Each cone is walked by one lane, the warp's lanes in lock step: one march
// forward keeps each of the first 128 steps' record (the state before the
// step, its sample, opacity terms, position and levels) in device scratch,
// and a checkpoint of the march state every 32 steps after those; the walk
// backward with the recurrences above in sequential form reads the records,
// and recomputes a later segment from its checkpoint.  Diffuse cones all share one step schedule; specular
// cones are taken from the exact forward's aperture-grouped list, so a
// warp's cones also march nearly the same number of steps.
#include <algorithm>

#include "trace_exact.cuh"

namespace vct {

int fill_trace_params(TraceParams& P, const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                      const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow);

namespace {

constexpr int kSegSteps = 32;
constexpr int kMaxSegments = 256;  // 8192 steps per cone: the specular cone at R = 1024 takes ~7.1k

// A cone's first kStoredSteps steps keep what the reverse walk reads in a
// record block of the lane's warp (device scratch, one block per warp of the
// grid, fields outermost and lanes innermost: a warp's store or load of a
// field is one 128-byte line), so those segments are walked backward without
// a second march; later segments are recomputed from checkpoints.
constexpr int kStoredSteps = 128;
static_assert(kStoredSteps % kSegSteps == 0, "stored steps are whole segments");
enum RecField { kRecAlpha, kRecOcc, kRecCorr, kRecQ, kRecOp, kRecSlope, kRecR, kRecG, kRecB, kRecStep, kRecFr,
                kRecLevels, kRecFields };
constexpr size_t kRecWarpFloats = (size_t)kRecFields * kStoredSteps * 32;
__device__ __forceinline__ void rec_put(float* p, float v) { *p = v; }
__device__ __forceinline__ float rec_get(const float* p) { return *p; }

// Diffuse cones per warp group: 0 deals them cone-major (each cone slot over
// all samples of the coherent order in turn); T > 0 deals all slots of T
// consecutive samples before the next T.
constexpr int kDiffuseTile = 1024;

struct MarchState {
    float step, seg, diameter, alpha, occ;
};

__device__ __forceinline__ void add4(float4* p, float4 v) {
    if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) atomicAdd(p, v);
}

// Adjoint of texture3d: the eight texels' shares of g.
__device__ __forceinline__ void texture3d_grad(float4* __restrict__ G, const AtlasDims& A, float ux, float uy, float uz,
                                               float4 g) {
    float u = ux * (float)A.W - 0.5f, v = uy * (float)A.H - 0.5f, w = uz * (float)A.D - 0.5f;
    float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    float a = u - fu, b = v - fv, c = w - fw;
    int i0 = wrap_tap((int)fu, A.W), i1 = wrap_tap((int)fu + 1, A.W);
    int j0 = wrap_tap((int)fv, A.H), j1 = wrap_tap((int)fv + 1, A.H);
    int k0 = wrap_tap((int)fw, A.D), k1 = wrap_tap((int)fw + 1, A.D);
    const float wi[2] = {1.0f - a, a}, wj[2] = {1.0f - b, b}, wk[2] = {1.0f - c, c};
    const int ii[2] = {i0, i1}, jj[2] = {j0, j1}, kk[2] = {k0, k1};
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const float wt = wi[x] * wj[y] * wk[z];
                add4(G + A.index(ii[x], jj[y], kk[z]), make_float4(g.x * wt, g.y * wt, g.z * wt, g.w * wt));
            }
}

// Adjoint of sample_clipmap: the three face taps' shares (one copy of the
// tap code, looped: the kernel is instruction-fetch bound when it is inlined
// six times per step).
__device__ __forceinline__ void sample_clipmap_grad(float4* __restrict__ G, const AtlasDims& A,
                                                    const vct_cone_tracing_desc& d, float3 p, int level, float3 fo,
                                                    float3 wt, float4 g) {
    float vs = d.voxel_size * exp2f((float)level);
    float extent = vs * d.volume_dimension;
    float dim = d.volume_dimension;
    float sx = (fractf(p.x / extent) * dim + 1.0f) / (dim + 2.0f);
    float sy = (fractf(p.y / extent) * dim + 1.0f) / (dim + 2.0f);
    float sz = (fractf(p.z / extent) * dim + 1.0f) / (dim + 2.0f);
    sy = sy + (float)level;
    sy = sy / (float)kClipLevels;
    sx = sx / (float)kFaces;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        const float off = f == 0 ? fo.x : (f == 1 ? fo.y : fo.z);
        const float w = f == 0 ? wt.x : (f == 1 ? wt.y : wt.z);
        texture3d_grad(G, A, sx + off, sy, sz, make_float4(g.x * w, g.y * w, g.z * w, g.w * w));
    }
}

// g(s) of one step spread over its levels, faces and texels.
__device__ __forceinline__ void scatter_step(float4* __restrict__ G, const AtlasDims& A, const vct_cone_tracing_desc& d,
                                             const ConeGeo& K, float3 pos, int lower, int upper, float fr, float4 gs) {
    // s = lo (1 - fr) + hi fr: the lower level's share, then the upper's (zero when fr = 0)
#pragma unroll 1
    for (int lv = 0; lv < 2; ++lv) {
        const float f = lv ? fr : 1.0f - fr;
        if (f == 0.0f) continue;
        sample_clipmap_grad(G, A, d, pos, lv ? upper : lower, K.fo, K.wt,
                            make_float4(gs.x * f, gs.y * f, gs.z * f, gs.w * f));
    }
}

// d(op)/d(s.a) for op = clamp(1 - (1 - s.a)^c, 0, 1), the bounds inside.
__device__ __forceinline__ float opacity_slope(const StepDetail& e) {
    const float base = 1.0f - e.smp.w;
    return (e.op_raw >= 0.0f && e.op_raw <= 1.0f && base > 0.0f) ? e.correction * powf(base, e.correction - 1.0f)
                                                                   : 0.0f;
}

// One step of trace_cone (same expressions) at march state m: advances m
// (alpha, occlusion, schedule) and returns the step.
__device__ __forceinline__ StepDetail march_step(const F4Atlas& T, const vct_cone_tracing_desc& d, const ConeGeo& K,
                                                 MarchState& m) {
    const Sched s{m.step, m.seg, m.diameter};
    const StepDetail e = exact_step_detail(T, d, K, s);
    const float k = clampf(1.0f - m.alpha, 0.0f, 1.0f);
    m.alpha = m.alpha + k * e.op;
    m.occ = m.occ + (1.0f - m.occ) * e.op / e.q;
    Sched n = s;
    sched_advance(n, K);
    m.step = n.step;
    m.seg = n.seg;
    m.diameter = n.diameter;
    return e;
}

// The adjoint of one cone per lane: gC (rgb) and gO (d/d occlusion)
// at the end of the march.  The warp's lanes run in lock step: every loop
// runs to the warp's longest march and a lane sits out the steps its cone
// does not have (or all of them when `active` is false).  The reverse walk
// reads no texels: a stored step's record, or the recompute of a later
// segment, kept in local arrays.
// `rec`: the warp's record block (kRecWarpFloats floats), written and read
// by each lane for its own cone only.
__device__ void cone_backward_lane(const F4Atlas& T, float4* __restrict__ G, const vct_cone_tracing_desc& d,
                                   const ConeGeo& K, float3 gC, float gO, bool active, float max_dist,
                                   float* rec, int* __restrict__ err) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    MarchState ckpt[kMaxSegments];
    const Sched s0 = first_sched(K);
    MarchState m{s0.step, s0.seg, s0.diameter, 0.0f, 0.0f};
    int n = 0;
    bool running = active && m.step < max_dist && m.occ < 1.0f;
    for (int j = 0; __any_sync(kFull, running); ++j) {
        if ((j % kSegSteps) == 0 && j / kSegSteps >= kMaxSegments) {  // j is warp-uniform
            if (running) atomicOr(err, 1);
            return;
        }
        if (running) {
            if ((j % kSegSteps) == 0 && j >= kStoredSteps) ckpt[j / kSegSteps] = m;
            const float alpha0 = m.alpha, occ0 = m.occ, step0 = m.step;
            const StepDetail e = march_step(T, d, K, m);
            if (j < kStoredSteps) {
                float* r = rec + (size_t)j * 32 + lane;
                constexpr size_t F = (size_t)kStoredSteps * 32;  // one field's floats
                rec_put(r + kRecAlpha * F, alpha0);
                rec_put(r + kRecOcc * F, occ0);
                rec_put(r + kRecCorr * F, e.correction);
                rec_put(r + kRecQ * F, e.q);
                rec_put(r + kRecOp * F, e.op);
                rec_put(r + kRecSlope * F, opacity_slope(e));
                rec_put(r + kRecR * F, e.smp.x);
                rec_put(r + kRecG * F, e.smp.y);
                rec_put(r + kRecB * F, e.smp.z);
                rec_put(r + kRecStep * F, step0);
                rec_put(r + kRecFr * F, e.fr);
                rec_put(r + kRecLevels * F, __int_as_float((e.lower & 0xffff) | (e.upper << 16)));
            }
            ++n;
            running = m.step < max_dist && m.occ < 1.0f;
        }
    }
    const int nmax = __reduce_max_sync(kFull, n);
    float gA = 0.0f;
    MarchState seg[kSegSteps];
    StepDetail seg_step[kSegSteps];
    for (int sidx = (nmax - 1) / kSegSteps; nmax > 0 && sidx >= 0; --sidx) {
        const int first = sidx * kSegSteps, last = min(nmax, first + kSegSteps);
        const int mine = min(n, first + kSegSteps);  // this lane's steps of the segment: first .. mine - 1
        if (first < kStoredSteps) {  // warp-uniform: the segment's steps are in the record block
            for (int i = last - 1; i >= first; --i) {
                if (i >= mine) continue;
                const float* rr = rec + (size_t)i * 32 + lane;
                constexpr size_t F = (size_t)kStoredSteps * 32;
                const float alpha = rec_get(rr + kRecAlpha * F), occ = rec_get(rr + kRecOcc * F);
                const float c = rec_get(rr + kRecCorr * F), q = rec_get(rr + kRecQ * F), op = rec_get(rr + kRecOp * F);
                const float slope = rec_get(rr + kRecSlope * F);
                const float sr = rec_get(rr + kRecR * F), sg = rec_get(rr + kRecG * F), sb = rec_get(rr + kRecB * F);
                const float step = rec_get(rr + kRecStep * F), fr = rec_get(rr + kRecFr * F);
                const int lv = __float_as_int(rec_get(rr + kRecLevels * F));
                const float k_raw = 1.0f - alpha;
                const float k = clampf(k_raw, 0.0f, 1.0f);
                float4 gs;
                gs.x = gC.x * k * c;
                gs.y = gC.y * k * c;
                gs.z = gC.z * k * c;
                const float gop = gA * k + gO * (1.0f - occ) / q;
                gs.w = gop * slope;
                if (k_raw >= 0.0f && k_raw <= 1.0f) gA = gA - ((gC.x * sr + gC.y * sg + gC.z * sb) * c + gA * op);
                gO = gO * (1.0f - op / q);
                const float3 pos = K.start + K.dir * step;  // exact_step_detail's expression
                scatter_step(G, T.A, d, K, pos, (int)(short)(lv & 0xffff), lv >> 16, fr, gs);
            }
            continue;
        }
        MarchState r;
        if (first < n) r = ckpt[sidx];
        for (int i = first; i < last; ++i) {
            if (i < mine) {
                seg[i - first] = r;
                seg_step[i - first] = march_step(T, d, K, r);
            }
        }
        for (int i = last - 1; i >= first; --i) {
            if (i >= mine) continue;
            const MarchState& mi = seg[i - first];
            const StepDetail& e = seg_step[i - first];
            const float c = e.correction;
            const float k_raw = 1.0f - mi.alpha;
            const float k = clampf(k_raw, 0.0f, 1.0f);
            float4 gs;
            gs.x = gC.x * k * c;
            gs.y = gC.y * k * c;
            gs.z = gC.z * k * c;
            const float gop = gA * k + gO * (1.0f - mi.occ) / e.q;
            gs.w = gop * opacity_slope(e);
            if (k_raw >= 0.0f && k_raw <= 1.0f)
                gA = gA - ((gC.x * e.smp.x + gC.y * e.smp.y + gC.z * e.smp.z) * c + gA * e.op);
            gO = gO * (1.0f - e.op / e.q);
            scatter_step(G, T.A, d, K, e.pos, e.lower, e.upper, e.fr, gs);
        }
    }
}

// dL/d(indirect) -> the diffuse cones' gC and gO; false when the mode does
// not read the volume through the diffuse cones.
__device__ __forceinline__ bool diffuse_seeds(const TraceParams& P, const GSample& g, float4 GD, float cos_t, int nc,
                                              float3& gC, float& gO) {
    const vct_cone_tracing_desc& d = P.d;
    const uint32_t mode = d.rendering_mode;
    // D.rgb = direct * ind.w + ind.rgb (modes 5 and the default), direct * ind.w (4), ind.w (7)
    float3 g_ind = f3(0.f, 0.f, 0.f);
    float g_ao = 0.0f;
    const bool rgb_mode = mode == 5 || mode >= 8;
    if (rgb_mode) g_ind = f3(GD.x, GD.y, GD.z);
    if (rgb_mode || mode == 4) {
        const float3 direct = direct_term(P, g);
        g_ao = GD.x * direct.x + GD.y * direct.y + GD.z * direct.z;
    } else if (mode == 7) {
        g_ao = GD.x + GD.y + GD.z;
    }
    const float w = cos_t / (float)nc;
    gC = f3(g_ind.x * w * (g.diffuse_color.x * d.indirect_diffuse_intensity),
            g_ind.y * w * (g.diffuse_color.y * d.indirect_diffuse_intensity),
            g_ind.z * w * (g.diffuse_color.z * d.indirect_diffuse_intensity));
    gO = -(g_ao * w * d.ambient_occlusion_factor);  // the cone returns 1 - occlusion
    return !(gC.x == 0.0f && gC.y == 0.0f && gC.z == 0.0f && gO == 0.0f);
}

__global__ void __launch_bounds__(128) k_cone_backward_diffuse(TraceParams P, F4Atlas T,
                                                               const vct_surface_sample* __restrict__ samples,
                                                               int64_t n, const uint32_t* __restrict__ order,
                                                               const float4* __restrict__ gd, float4* __restrict__ G,
                                                               float* rec_all, int* __restrict__ err) {
    const vct_cone_tracing_desc& d = P.d;
    float* rec = rec_all + (size_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRecWarpFloats;
    const bool c32 = d.enable_32_cones != 0;
    const int nc = c32 ? 32 : 16;
    const int lane = threadIdx.x & 31;
    const int64_t total = n * nc;
    // warp-uniform trip count: a warp's lanes enter cone_backward_lane together
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; t0 < total;
         t0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = t0 + lane;
        bool active = t < total;
        // a warp's lanes march the same cone of consecutive samples in the coherent order (the same direction
        // from neighbouring points: the lanes stay in step and share texels), all cones of kDiffuseTile samples
        // before the next kDiffuseTile (the resident warps' gradient scatter then stays near one patch)
        int slot = 0;
        int64_t u = 0;
        if (active && kDiffuseTile > 0) {
            const int64_t per = (int64_t)kDiffuseTile * nc, tile = t / per, base = tile * kDiffuseTile;
            const int64_t len = min((int64_t)kDiffuseTile, n - base), r = t - tile * per;
            slot = (int)(r / len);
            u = base + (r - (int64_t)slot * len);
        } else if (active) {
            slot = (int)(t / n);
            u = t - (int64_t)slot * n;
        }
        const int64_t i = order ? (int64_t)__ldg(order + u) : u;
        const GSample g = load_sample(samples + i, P.eye);
        active = active && g.depth != 1.0f;
        const float min_level = calc_min_level(d, g.wp);
        const float vs = d.voxel_size * exp2f(min_level);
        const float3 start = g.wp + g.normal * (vs * d.trace_start_offset);
        const float3 dir = c32 ? f3(c_dirs32[slot][0], c_dirs32[slot][1], c_dirs32[slot][2])
                               : f3(c_dirs16[slot][0], c_dirs16[slot][1], c_dirs16[slot][2]);
        const float cos_t = dot3(g.normal, dir);
        active = active && cos_t >= 0.0f;
        float3 gC = f3(0.f, 0.f, 0.f);
        float gO = 0.0f;
        active = active && diffuse_seeds(P, g, gd[i], cos_t, nc, gC, gO);
        const ConeGeo K = make_cone(d, start, dir, P.diffuse_aperture, min_level,
                                    fmaxf(kMinTraceStepFactor, d.min_trace_step_factor));
        cone_backward_lane(T, G, d, K, gC, gO, active, kMaxTraceDistance, rec, err);
    }
}

// One lane per specular cone of the aperture-grouped list (a warp's cones
// share their step schedule, so the lock-step walk keeps its lanes busy).
__global__ void __launch_bounds__(128) k_cone_backward_specular(
    TraceParams P, F4Atlas T, const vct_surface_sample* __restrict__ samples, const uint32_t* __restrict__ list,
    const unsigned int* __restrict__ spec_count, const float4* __restrict__ gsp, float4* __restrict__ G,
    float* rec_all, int* __restrict__ err) {
    const vct_cone_tracing_desc& d = P.d;
    float* rec = rec_all + (size_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRecWarpFloats;
    if (!(d.rendering_mode == 6 || d.rendering_mode >= 8)) return;
    const int lane = threadIdx.x & 31;
    const int64_t m = *spec_count;
    // warp-uniform trip count: a warp's lanes enter cone_backward_lane together
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; t0 < m;
         t0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = t0 + lane;
        bool active = t < m;
        const uint32_t i = __ldg(list + (active ? t : t0));
        const GSample g = load_sample(samples + i, P.eye);
        const float4 GS = gsp[i];
        const float isi = d.indirect_specular_intensity;
        const float3 gC = f3(GS.x * g.specular_color.x * isi, GS.y * g.specular_color.y * isi,
                             GS.z * g.specular_color.z * isi);
        active = active && !(gC.x == 0.0f && gC.y == 0.0f && gC.z == 0.0f);
        const float min_level = calc_min_level(d, g.wp);
        const float vs = d.voxel_size * exp2f(min_level);
        const float3 start = g.wp + g.normal * (vs * d.trace_start_offset);
        const float3 sdir = reflect3(f3(-g.view.x, -g.view.y, -g.view.z), g.normal);
        const ConeGeo K = make_cone(d, start, sdir, fmaxf(g.roughness, kMinSpecularAperture), min_level, d.voxel_size);
        cone_backward_lane(T, G, d, K, gC, 0.0f, active, kMaxTraceDistance, rec, err);
    }
}

}  // namespace
}  // namespace vct

using namespace vct;

extern "C" int vct_cone_trace_backward(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                       const float* atlas4, int32_t R, const vct_shadow_map* shadow,
                                       const vct_directional_light_desc* light,
                                       const vct_directional_light_shadow_desc* light_shadow,
                                       const vct_surface_sample* samples, int64_t n, const float* grad_diffuse,
                                       const float* grad_specular, float* grad_atlas4, void* stream) {
    vct::NvtxRange nvtx_range("vct_cone_trace_backward");
    VCT_CHECK_ARG(atlas4 && grad_atlas4 && valid_resolution(R), "vct_cone_trace_backward: bad atlas / resolution");
    VCT_CHECK_ARG((((uintptr_t)atlas4 | (uintptr_t)grad_atlas4) & 15) == 0,
                  "vct_cone_trace_backward: atlases must be 16-byte aligned");
    VCT_CHECK_ARG(n >= 0, "vct_cone_trace_backward: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && grad_diffuse && grad_specular, "vct_cone_trace_backward: null sample or gradient buffer");
    VCT_CHECK_ARG((((uintptr_t)samples | (uintptr_t)grad_diffuse | (uintptr_t)grad_specular) & 15) == 0,
                  "vct_cone_trace_backward: sample / gradient buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    cudaStream_t st = as_stream(stream);
    const int nc = desc->enable_32_cones ? 32 : 16;
    // grids of resident blocks (grid-stride loops): the record scratch holds one block per warp of the grid
    int dev = 0, sms = 0, occ_d = 0, occ_s = 0;
    VCT_CUDA_TRY(cudaGetDevice(&dev));
    VCT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    VCT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_d, k_cone_backward_diffuse, 128, 0));
    VCT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_cone_backward_specular, 128, 0));
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n * nc + 127) / 128, (int64_t)sms * std::max(occ_d, 1)));
    const int64_t lblocks = std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, (int64_t)sms * std::max(occ_s, 1)));
    const size_t rec_bytes = (size_t)std::max(blocks, lblocks) * (128 / 32) * kRecWarpFloats * sizeof(float);
    int* err = nullptr;
    VCT_CUDA_TRY(cudaMallocAsync(&err, sizeof(int), st));
    VCT_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    float* rec = nullptr;
    if (cudaMallocAsync(&rec, rec_bytes, st) != cudaSuccess) {
        cudaFreeAsync(err, st);
        return fail(VCT_E_CUDA, "vct_cone_trace_backward: record scratch allocation failed");
    }
    F4Atlas T{reinterpret_cast<const float4*>(atlas4), AtlasDims(R)};
    ExactPlan plan;
    rc = exact_plan(samples, n, P.d, &plan, st);
    if (rc != VCT_OK) {
        cudaFreeAsync(rec, st);
        cudaFreeAsync(err, st);
        return rc;
    }
    float4* G = reinterpret_cast<float4*>(grad_atlas4);
    k_cone_backward_diffuse<<<(int)blocks, 128, 0, st>>>(P, T, samples, n, plan.order,
                                                          reinterpret_cast<const float4*>(grad_diffuse), G, rec, err);
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) {
        k_cone_backward_specular<<<(int)lblocks, 128, 0, st>>>(P, T, samples, plan.spec_list, plan.spec_count,
                                                               reinterpret_cast<const float4*>(grad_specular), G, rec,
                                                               err);
        le = cudaGetLastError();
    }
    int h_err = 0;
    cudaError_t ce = cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t se = cudaStreamSynchronize(st);
    cudaFreeAsync(rec, st);
    cudaFreeAsync(err, st);
    exact_plan_free(&plan, st);
    if (le != cudaSuccess) return cuda_fail(le, "vct_cone_trace_backward kernels");
    if (ce != cudaSuccess) return cuda_fail(ce, "vct_cone_trace_backward readback");
    if (se != cudaSuccess) return cuda_fail(se, "vct_cone_trace_backward");
    if (h_err) return fail(VCT_E_OVERFLOW, "vct_cone_trace_backward: a cone marched more than 8192 steps");
    return VCT_OK;
}

// ------------------------------------------------------ inverse fitting ops
namespace vct {
namespace {

constexpr int kSqErrBlocks = 152 * 4;
constexpr int kSqErrThreads = 256;

// Squared error and its gradient; one double partial sum per block, each
// thread summing its grid-stride elements in index order, the block in a
// fixed tree order: the result does not depend on scheduling.
__global__ void __launch_bounds__(kSqErrThreads) k_sq_error(const float4* __restrict__ out,
                                                            const float4* __restrict__ target, int64_t n, float scale,
                                                            float4* __restrict__ grad, double* __restrict__ partial) {
    __shared__ double red[kSqErrThreads / 32];
    const float two_scale = 2.0f * scale;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 o = out[i], t = target[i];
        const float dx = o.x - t.x, dy = o.y - t.y, dz = o.z - t.z, dw = o.w - t.w;
        if (grad) grad[i] = make_float4(two_scale * dx, two_scale * dy, two_scale * dz, two_scale * dw);
        acc += ((double)dx * dx + (double)dy * dy) + ((double)dz * dz + (double)dw * dw);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kSqErrThreads / 32; ++w) s += red[w];
        partial[blockIdx.x] = s;
    }
}

__global__ void k_sq_error_fold(const double* __restrict__ partial, int blocks, double scale,
                                double* __restrict__ loss) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < blocks; ++b) s += partial[b];
        *loss = s * scale;
    }
}

struct AdamArgs {
    float lr, b1, omb1, b2, omb2, eps, c1, c2;
    float lo[4], hi[4];
    int zero_grad;
};

// One rounding per operation (the file is compiled without contraction), so
// a float32 host restatement in the same order reproduces every bit.
__device__ __forceinline__ float adam1(float& p, float g, float& m, float& v, const AdamArgs& a, int c) {
    m = a.b1 * m + a.omb1 * g;
    v = a.b2 * v + (a.omb2 * g) * g;
    const float mh = m * a.c1, vh = v * a.c2;
    const float upd = (a.lr * mh) / (__fsqrt_rn(vh) + a.eps);
    p = fminf(fmaxf(p - upd, a.lo[c]), a.hi[c]);
    return p;
}

__global__ void __launch_bounds__(256) k_adam(float4* __restrict__ p, float4* __restrict__ g, float4* __restrict__ m,
                                              float4* __restrict__ v, int64_t n4, const AdamArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
        float4 P = p[i], G = g[i], M = m[i], V = v[i];
        adam1(P.x, G.x, M.x, V.x, a, 0);
        adam1(P.y, G.y, M.y, V.y, a, 1);
        adam1(P.z, G.z, M.z, V.z, a, 2);
        adam1(P.w, G.w, M.w, V.w, a, 3);
        p[i] = P;
        m[i] = M;
        v[i] = V;
        if (a.zero_grad) g[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

}  // namespace
}  // namespace vct

extern "C" int vct_sq_error(const float* out4, const float* target4, int64_t n, float scale, float* grad4,
                            double* loss, void* stream) {
    vct::NvtxRange nvtx_range("vct_sq_error");
    VCT_CHECK_ARG(n >= 0 && loss, "vct_sq_error: bad size or null loss");
    VCT_CHECK_ARG(n == 0 || (out4 && target4), "vct_sq_error: null output / target");
    VCT_CHECK_ARG((((uintptr_t)out4 | (uintptr_t)target4 | (uintptr_t)grad4) & 15) == 0,
                  "vct_sq_error: buffers must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    double* partial = nullptr;
    VCT_CUDA_TRY(cudaMallocAsync(&partial, sizeof(double) * kSqErrBlocks, st));
    int64_t blocks = (n + kSqErrThreads - 1) / kSqErrThreads;
    blocks = blocks < 1 ? 1 : (blocks > kSqErrBlocks ? kSqErrBlocks : blocks);
    k_sq_error<<<(int)blocks, kSqErrThreads, 0, st>>>(reinterpret_cast<const float4*>(out4),
                                                      reinterpret_cast<const float4*>(target4), n, scale,
                                                      reinterpret_cast<float4*>(grad4), partial);
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) {
        k_sq_error_fold<<<1, 32, 0, st>>>(partial, (int)blocks, (double)scale, loss);
        le = cudaGetLastError();
    }
    cudaFreeAsync(partial, st);
    if (le != cudaSuccess) return cuda_fail(le, "k_sq_error");
    return VCT_OK;
}

extern "C" int vct_adam_step(float* param, float* grad, float* m, float* v, int64_t n, const vct_adam_desc* desc,
                             void* stream) {
    vct::NvtxRange nvtx_range("vct_adam_step");
    VCT_CHECK_ARG(desc && n >= 0 && (n & 3) == 0, "vct_adam_step: null descriptor or n not a multiple of 4");
    VCT_CHECK_ARG(desc->step >= 1, "vct_adam_step: step counts from 1");
    VCT_CHECK_ARG(desc->beta1 >= 0.0f && desc->beta1 < 1.0f && desc->beta2 >= 0.0f && desc->beta2 < 1.0f &&
                      desc->eps > 0.0f,
                  "vct_adam_step: betas must lie in [0, 1) and eps be positive");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(param && grad && m && v, "vct_adam_step: null buffer");
    VCT_CHECK_ARG((((uintptr_t)param | (uintptr_t)grad | (uintptr_t)m | (uintptr_t)v) & 15) == 0,
                  "vct_adam_step: buffers must be 16-byte aligned");
    AdamArgs a;
    a.lr = desc->lr;
    a.b1 = desc->beta1;
    a.omb1 = 1.0f - desc->beta1;
    a.b2 = desc->beta2;
    a.omb2 = 1.0f - desc->beta2;
    a.eps = desc->eps;
    a.c1 = (float)(1.0 / (1.0 - pow((double)desc->beta1, (double)desc->step)));
    a.c2 = (float)(1.0 / (1.0 - pow((double)desc->beta2, (double)desc->step)));
    for (int c = 0; c < 3; ++c) {
        a.lo[c] = desc->rgb_lo;
        a.hi[c] = desc->rgb_hi;
    }
    a.lo[3] = desc->alpha_lo;
    a.hi[3] = desc->alpha_hi;
    a.zero_grad = desc->zero_grad;
    cudaStream_t st = as_stream(stream);
    const int64_t n4 = n / 4;
    int64_t blocks = (n4 + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_adam<<<(int)blocks, 256, 0, st>>>(reinterpret_cast<float4*>(param), reinterpret_cast<float4*>(grad),
                                        reinterpret_cast<float4*>(m), reinterpret_cast<float4*>(v), n4, a);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}
