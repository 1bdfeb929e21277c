// trace_fast.cu -- the GB300 form of voxelConeTracing.frag.
//
// Same pass contract and arithmetic as the exact tracer, reorganised for the
// hardware:
//   1. samples are visited in Morton order of their position (a 30-bit key,
//      radix-sorted), so neighbouring lanes march through the same texels and
//      the taps hit L1/TEX and L2 instead of HBM;
//   2. diffuse cones are compacted per warp: the (sample, cone) pairs with
//      cos >= 0 of 32 samples are dealt to the 32 lanes in rounds, so no lane
//      idles on a back-facing cone; every sample's cone results are summed by
//      its owner lane in cone order (the shader's order);
//   3. specular cones (57..780 marching steps, depending on the aperture) run
//      in their own kernel, one cone per warp with consecutive steps on
//      consecutive lanes (the steps of one cone are a fraction of a voxel
//      apart, so the 32 lanes share texels) and warp scans for the composite;
//   4. the clipmap is sampled through a 3D texture object (hardware trilinear
//      filter, WRAP addressing = the reference's REPEAT sampler), RGBA8 or
//      RGBA16F storage, FP32 compositing.
// Scratch memory (sort keys, orders, cub temporary storage) is provided by
// the caller; vct_cone_trace_fast_scratch_bytes() gives its size.
#include <cstring>
#include <mutex>
#include <vector>

#include <cub/cub.cuh>

#include "trace_deal.cuh"

struct vct_texture_s;

namespace vct {

cudaTextureObject_t texture_object(const vct_texture_s* t);
int texture_resolution(const vct_texture_s* t);
int texture_format(const vct_texture_s* t);
int fill_trace_params(TraceParams& P, const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                      const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow);
int apply_trace_options(TraceParams& P, const vct_trace_options* o);

struct FastConsts {
    float uvs, inv_uvs, min_radius, inv_min_radius, inv_min_radius2, decay, start_off;
    float coef_diffuse, sf_diffuse, aperture_diffuse;
    float cx, cy, cz;
    float inv_ext[kClipLevels];
    float ax, bx, ay, az, bz;
    float by[kClipLevels];
    int ncones;
    int need_diffuse, need_specular;
};

struct FastArgs {
    TraceParams P;
    FastConsts C;
    cudaTextureObject_t tex;
    const vct_surface_sample* __restrict__ samples;
    int64_t n;
    float* __restrict__ dout;
    float* __restrict__ sout;
    unsigned long long* steps;
};

// 2^x by the hardware approximation (PTX ex2.approx: about 2 ulp, flushes
// subnormal results): the per-step level size and opacity correction of the
// texture form, whose error bar (8-bit texture filter weights) dominates.
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float4 fma4(float4 a, float s, float4 b) {
    return make_float4(fmaf(a.x, s, b.x), fmaf(a.y, s, b.y), fmaf(a.z, s, b.z), fmaf(a.w, s, b.w));
}

// sampleClipmap at integer level l: three face taps along the cone's signs.
__device__ __forceinline__ float4 sample_level(cudaTextureObject_t tex, const FastConsts& C, float3 p, int l, float fox,
                                               float foy, float foz, float3 wt) {
    const float ie = C.inv_ext[l];
    float fx = p.x * ie, fy = p.y * ie, fz = p.z * ie;
    fx -= floorf(fx);
    fy -= floorf(fy);
    fz -= floorf(fz);
    const float sx = fmaf(fx, C.ax, C.bx), sy = fmaf(fy, C.ay, C.by[l]), sz = fmaf(fz, C.az, C.bz);
    float4 a = tex3D<float4>(tex, sx + fox, sy, sz);
    float4 b = tex3D<float4>(tex, sx + foy, sy, sz);
    float4 c = tex3D<float4>(tex, sx + foz, sy, sz);
    float4 r = make_float4(a.x * wt.x, a.y * wt.x, a.z * wt.x, a.w * wt.x);
    r = fma4(b, wt.y, r);
    return fma4(c, wt.z, r);
}

// traceCone (voxelConeTracing.frag:341-392); the upper-level fetch is skipped
// when curLevel is integral (mix(x, x, 0) == x).
__device__ __forceinline__ float4 trace_cone_fast(cudaTextureObject_t tex, const FastConsts& C, float3 start, float3 dir,
                                                  float coef, float start_level, float step_factor,
                                                  unsigned long long& steps) {
    float4 result = make_float4(0.f, 0.f, 0.f, 0.f);
    const float uvs = C.uvs;
    float vs = uvs * exp2f(start_level);
    const float off = vs * C.start_off * 0.5f;
    start = f3(fmaf(dir.x, off, start.x), fmaf(dir.y, off, start.y), fmaf(dir.z, off, start.z));
    float step = 0.0f, diameter = uvs, occlusion = 0.0f, seg = vs;
    const float fox = dir.x > 0.0f ? 0.0f : 1.0f / 6.0f;
    const float foy = dir.y > 0.0f ? 2.0f / 6.0f : 3.0f / 6.0f;
    const float foz = dir.z > 0.0f ? 4.0f / 6.0f : 5.0f / 6.0f;
    const float3 wt = f3(dir.x * dir.x, dir.y * dir.y, dir.z * dir.z);
    unsigned int it = 0;
    while (step < kMaxTraceDistance && occlusion < 1.0f) {
        ++it;
        const float3 pos = f3(fmaf(dir.x, step, start.x), fmaf(dir.y, step, start.y), fmaf(dir.z, step, start.z));
        const float dx = C.cx - pos.x, dy = C.cy - pos.y, dz = C.cz - pos.z;
        // ceil(log2(dist / r)) as ceil(log2(dist^2 / r^2) / 2): no square root
        const float min_level = ceilf(0.5f * __log2f(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * C.inv_min_radius2));
        float cl = __log2f(diameter * C.inv_uvs);
        cl = fminf(fmaxf(fmaxf(start_level, cl), min_level), (float)(kClipLevels - 1));
        const float flo = floorf(cl);
        const int lo = (int)flo;
        const float fr = cl - flo;
        float4 s = sample_level(tex, C, pos, lo, fox, foy, foz, wt);
        if (fr > 0.0f) {
            const float4 h = sample_level(tex, C, pos, lo + 1, fox, foy, foz, wt);
            s = make_float4(fmaf(h.x - s.x, fr, s.x), fmaf(h.y - s.y, fr, s.y), fmaf(h.z - s.z, fr, s.z),
                            fmaf(h.w - s.w, fr, s.w));
        }
        vs = uvs * ex2_approx(cl);
        const float corr = __fdividef(seg, vs);
        // base clamped at 0 like the exact form: alpha rounded above 1 is opaque, not NaN -> 0
        const float opacity = __saturatef(1.0f - ex2_approx(corr * __log2f(fmaxf(1.0f - s.w, 0.0f))));
        const float k = __saturatef(1.0f - result.w);
        result = make_float4(fmaf(k * s.x, corr, result.x), fmaf(k * s.y, corr, result.y),
                             fmaf(k * s.z, corr, result.z), fmaf(k, opacity, result.w));
        occlusion = fmaf(1.0f - occlusion, __fdividef(opacity, fmaf(step + vs, C.decay, 1.0f)), occlusion);
        const float prev = step;
        step = fmaf(fmaxf(diameter, uvs), step_factor, step);
        seg = step - prev;
        diameter = step * coef;
    }
    steps += it;
    return make_float4(result.x, result.y, result.z, 1.0f - occlusion);
}

// 30-bit Morton key of the sample position in level-0 voxels around the volume centre.
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t morton_key(const vct_surface_sample* __restrict__ s, const FastConsts& C) {
    const float* p = s->position;
    const float q = 0.5f * C.inv_uvs;  // two level-0 voxels per cell
    int x = __float2int_rd((p[0] - C.cx) * q) + 512, y = __float2int_rd((p[1] - C.cy) * q) + 512,
        z = __float2int_rd((p[2] - C.cz) * q) + 512;
    x = min(max(x, 0), 1023);
    y = min(max(y, 0), 1023);
    z = min(max(z, 0), 1023);
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

__global__ void k_morton_keys(const vct_surface_sample* __restrict__ s, int64_t n, FastConsts C,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = morton_key(s + i, C);
        vals[i] = (uint32_t)i;
    }
}

// The shader traces a specular cone where depth != 1 and the sample has a
// specular colour and metalness.
__device__ __forceinline__ bool traces_specular(const vct_surface_sample* __restrict__ s) {
    const float4* p = reinterpret_cast<const float4*>(s);
    const float4 a = __ldg(p + 0), d = __ldg(p + 3);
    return a.w != 1.0f && (d.x > 1e-6f || d.y > 1e-6f || d.z > 1e-6f) && d.w > 1e-6f;
}

// Specular classification of the Morton-ordered samples (the shader traces
// a specular cone where depth != 1 and the sample has a specular colour and
// metalness): key 0 for specular samples, 256 otherwise, and their count.
// One radix pass on bit 8 then lists the specular samples in Morton order.
__global__ void k_spec_keys(const __grid_constant__ FastArgs A, const uint32_t* __restrict__ order,
                            uint32_t* __restrict__ spec_key, unsigned int* __restrict__ spec_count) {
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < A.n;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = base + lane;
        bool spec = false;
        if (pos < A.n && A.C.need_specular) spec = traces_specular(A.samples + __ldg(order + pos));
        if (pos < A.n) spec_key[pos] = spec ? 0u : 256u;
        const unsigned bal = __ballot_sync(0xffffffffu, spec);
        if (lane == 0 && bal) atomicAdd(spec_count, (unsigned)__popc(bal));
    }
}

constexpr int kWarpsPerBlock = 8;

// Run the specular cones on a second stream beside the diffuse kernel.
constexpr bool kTraceSideStream = true;
// Deal the specular cones to the warps by a ticket (kSpecConesPerTicket at a
// time) instead of a static grid stride.
constexpr bool kTraceTickets = true;
constexpr int kSpecConesPerTicket = 4;
constexpr bool kDiffuseTickets = false;

// The diffuse cones, dealt to the lanes of a warp (trace_deal.cuh), each
// marched by trace_cone_fast.
struct FastDiffuseMarch {
    cudaTextureObject_t tex;
    const FastConsts* C;
    __device__ __forceinline__ float4 operator()(float3 start, float3 dir, float start_level,
                                                 unsigned long long& steps) const {
        return trace_cone_fast(tex, *C, start, dir, C->coef_diffuse, start_level, C->sf_diffuse, steps);
    }
};

__global__ void __launch_bounds__(256) k_trace_diffuse(const __grid_constant__ FastArgs A, const uint32_t* __restrict__ order,
                                                       unsigned int* __restrict__ ticket) {
    DealArgs D{&A.P, A.samples, A.n, order, 0u, (uint32_t)A.n, A.dout, A.sout, A.C.ncones, A.C.need_diffuse != 0,
               A.C.need_specular != 0};
    unsigned long long steps = 0;
    // (a ticket for the diffuse items measured no faster than the static stride: 8.69 against 8.66 ms per step)
    deal_diffuse<kWarpsPerBlock, kDiffuseTickets>(D, FastDiffuseMarch{A.tex, &A.C}, steps, ticket);
    add_steps(A.steps, steps);
}

// One step of a cone: the sample's contribution (rgb * corr, opacity) and
// its transmittance factor 1 - opacity / (1 + (step + vs) * decay).
struct ConeStep {
    float r, g, b, a, t;
};

__device__ __forceinline__ ConeStep cone_step(cudaTextureObject_t tex, const FastConsts& C, float3 start, float3 dir,
                                              float fox, float foy, float foz, float3 wt, float start_level, float st,
                                              float dm, float sg) {
    const float3 pos = f3(fmaf(dir.x, st, start.x), fmaf(dir.y, st, start.y), fmaf(dir.z, st, start.z));
    const float dx = C.cx - pos.x, dy = C.cy - pos.y, dz = C.cz - pos.z;
    // ceil(log2(dist / r)) as ceil(log2(dist^2 / r^2) / 2): no square root
    const float min_level = ceilf(0.5f * __log2f(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * C.inv_min_radius2));
    float cl = __log2f(dm * C.inv_uvs);
    cl = fminf(fmaxf(fmaxf(start_level, cl), min_level), (float)(kClipLevels - 1));
    const float flo = floorf(cl);
    const int lo = (int)flo;
    const float fr = cl - flo;
    float4 smp = sample_level(tex, C, pos, lo, fox, foy, foz, wt);
    if (fr > 0.0f) {
        const float4 h = sample_level(tex, C, pos, lo + 1, fox, foy, foz, wt);
        smp = make_float4(fmaf(h.x - smp.x, fr, smp.x), fmaf(h.y - smp.y, fr, smp.y), fmaf(h.z - smp.z, fr, smp.z),
                          fmaf(h.w - smp.w, fr, smp.w));
    }
    const float vs = C.uvs * ex2_approx(cl);
    const float corr = __fdividef(sg, vs);
    const float opacity = __saturatef(1.0f - ex2_approx(corr * __log2f(fmaxf(1.0f - smp.w, 0.0f))));
    return ConeStep{smp.x * corr, smp.y * corr, smp.z * corr, opacity,
                    1.0f - __fdividef(opacity, fmaf(st + vs, C.decay, 1.0f))};
}

// `p` followed by `q` under front-to-back compositing: rgb and alpha by the
// "over" operator, transmittance by product.
__device__ __forceinline__ ConeStep over(const ConeStep& p, const ConeStep& q) {
    const float k = 1.0f - p.a;
    return ConeStep{fmaf(k, q.r, p.r), fmaf(k, q.g, p.g), fmaf(k, q.b, p.b), fmaf(k, q.a, p.a), p.t * q.t};
}

// One cone marched by a whole warp, 32 * S steps per round: lane j takes
// steps S j .. S j + S - 1 of the round.  The step schedule (step, diameter,
// segment length) depends only on the step index, not on the samples, and
// has a closed form (below), so every lane finds its own steps directly.  The
// front-to-back composite result += (1 - result.a) * src is the associative
// "over" operator and 1 - occlusion is the product of (1 - x_k): each lane
// composes its S steps, a warp scan composes the lanes.  The march stops at
// the first step whose occlusion reaches 1 or whose distance reaches
// maxDistance, like the loop.  Transmittance only falls, so the first lane
// whose composite reaches occlusion 1 holds that step; it marches its steps
// again from the state before them to stop exactly there (once per cone).
template <int S>
__device__ __forceinline__ float4 trace_cone_warp(cudaTextureObject_t tex, const FastConsts& C, float3 start,
                                                  float3 dir, float coef, float start_level, float step_factor,
                                                  unsigned long long& steps) {
    const int lane = threadIdx.x & 31;
    const float uvs = C.uvs;
    const float vs0 = uvs * exp2f(start_level);
    const float off = vs0 * C.start_off * 0.5f;
    start = f3(fmaf(dir.x, off, start.x), fmaf(dir.y, off, start.y), fmaf(dir.z, off, start.z));
    const float fox = dir.x > 0.0f ? 0.0f : 1.0f / 6.0f;
    const float foy = dir.y > 0.0f ? 2.0f / 6.0f : 3.0f / 6.0f;
    const float foz = dir.z > 0.0f ? 4.0f / 6.0f : 5.0f / 6.0f;
    const float3 wt = f3(dir.x * dir.x, dir.y * dir.y, dir.z * dir.z);
    const ConeStep id{0.f, 0.f, 0.f, 0.f, 1.0f};
    ConeStep carried = id;
    float st = 0.0f, dm = uvs, sg = vs0;  // schedule at the round's first step
    // The step schedule st += max(st * coef, uvs) * step_factor in closed form:
    // linear steps of u = uvs * step_factor while st * coef <= uvs, then
    // geometric growth by r = 1 + coef * step_factor.  From a round's start
    // st_0, with K = the number of linear steps left,
    //   st_j = st_0 + j u (j <= K),   st_j = (st_0 + K u) r^(j - K) (j >= K).
    const float u = uvs * step_factor, lr = __log2f(fmaf(coef, step_factor, 1.0f)), T = uvs / coef;
    unsigned long long it = 0;
    for (;;) {
        const float K = st <= T ? floorf((T - st) / u) + 1.0f : 0.0f;
        const float sK = fmaf(K, u, st);
        auto st_at = [&](float jf) { return jf <= K ? fmaf(jf, u, st) : sK * ex2_approx((jf - K) * lr); };
        const float j0 = (float)(S * lane);
        // march this lane's steps: composite, count of valid steps
        ConeStep x = id;
        int nvalid = 0;
        {
            float prev = lane == 0 ? 0.0f : st_at(j0 - 1.0f);
#pragma unroll
            for (int k = 0; k < S; ++k) {
                const float sk = st_at(j0 + (float)k);
                if (sk < kMaxTraceDistance) {
                    const bool first = lane == 0 && k == 0;
                    x = over(x, cone_step(tex, C, start, dir, fox, foy, foz, wt, start_level, sk,
                                          first ? dm : sk * coef, first ? sg : sk - prev));
                    ++nvalid;
                }
                prev = sk;
            }
        }
        const float s_last = st_at(32.0f * S - 1.0f), s_next = st_at(32.0f * S);
        // inclusive warp scan of the lanes' composites
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            ConeStep p;
            p.r = __shfl_up_sync(0xffffffffu, x.r, o);
            p.g = __shfl_up_sync(0xffffffffu, x.g, o);
            p.b = __shfl_up_sync(0xffffffffu, x.b, o);
            p.a = __shfl_up_sync(0xffffffffu, x.a, o);
            p.t = __shfl_up_sync(0xffffffffu, x.t, o);
            if (lane >= o) x = over(p, x);
        }
        const ConeStep after = over(carried, x);
        const unsigned tmask = __ballot_sync(0xffffffffu, nvalid > 0 && (1.0f - after.t) >= 1.0f);
        if (tmask) {  // occlusion reaches 1 within lane L's steps: stop after that step
            const int L = __ffs(tmask) - 1;
            ConeStep before;
            before.r = __shfl_up_sync(0xffffffffu, x.r, 1);
            before.g = __shfl_up_sync(0xffffffffu, x.g, 1);
            before.b = __shfl_up_sync(0xffffffffu, x.b, 1);
            before.a = __shfl_up_sync(0xffffffffu, x.a, 1);
            before.t = __shfl_up_sync(0xffffffffu, x.t, 1);
            int done = 0;
            if (lane == L) {
                ConeStep y = lane == 0 ? carried : over(carried, before);
                float prev = lane == 0 ? 0.0f : st_at(j0 - 1.0f);
                for (int k = 0; k < S; ++k) {
                    const float sk = st_at(j0 + (float)k);
                    const bool first = lane == 0 && k == 0;
                    y = over(y, cone_step(tex, C, start, dir, fox, foy, foz, wt, start_level, sk,
                                          first ? dm : sk * coef, first ? sg : sk - prev));
                    prev = sk;
                    done = k + 1;
                    if ((1.0f - y.t) >= 1.0f) break;
                }
                carried = y;
            }
            carried.r = __shfl_sync(0xffffffffu, carried.r, L);
            carried.g = __shfl_sync(0xffffffffu, carried.g, L);
            carried.b = __shfl_sync(0xffffffffu, carried.b, L);
            carried.t = __shfl_sync(0xffffffffu, carried.t, L);
            it += (unsigned long long)(S * L + __shfl_sync(0xffffffffu, done, L));
            break;
        }
        // invalid steps are the identity: the round's total is lane 31's prefix
        carried.r = __shfl_sync(0xffffffffu, after.r, 31);
        carried.g = __shfl_sync(0xffffffffu, after.g, 31);
        carried.b = __shfl_sync(0xffffffffu, after.b, 31);
        carried.a = __shfl_sync(0xffffffffu, after.a, 31);
        carried.t = __shfl_sync(0xffffffffu, after.t, 31);
        int nv = nvalid;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nv += __shfl_xor_sync(0xffffffffu, nv, o);
        it += (unsigned long long)nv;
        if (nv < 32 * S) break;  // maxDistance reached within the round
        st = s_next;
        sg = s_next - s_last;
        dm = s_next * coef;
    }
    if (lane == 0) steps += it;
    return make_float4(carried.r, carried.g, carried.b, carried.t);
}

// Consecutive steps of one specular cone per lane.
constexpr int kSpecStepsPerLane = 2;

// Sample idx's specular cone on the calling warp; lane 0 writes its output.
__device__ __forceinline__ void specular_cone_warp(const FastArgs& A, uint32_t idx, unsigned long long& steps) {
    const TraceParams& P = A.P;
    const FastConsts& C = A.C;
    const GSample g = load_sample(A.samples + idx, P.eye);
    const float min_level = calc_min_level(P.d, g.wp);
    const float vs = C.uvs * exp2f(min_level);
    const float3 start = g.wp + g.normal * (vs * C.start_off);
    const float3 sdir = reflect3(f3(-g.view.x, -g.view.y, -g.view.z), g.normal);
    const float ap = fmaxf(g.roughness, kMinSpecularAperture);
    const float coef = 2.0f * tanf(ap * 0.5f);
    const float4 r = trace_cone_warp<kSpecStepsPerLane>(A.tex, C, start, sdir, coef, min_level, C.uvs, steps);
    if ((threadIdx.x & 31) == 0) {
        const float isi = P.d.indirect_specular_intensity;
        reinterpret_cast<float4*>(A.sout)[idx] = make_float4(r.x * g.specular_color.x * isi,
                                                             r.y * g.specular_color.y * isi,
                                                             r.z * g.specular_color.z * isi, 1.0f);
    }
}

// One warp per specular cone of the list (the list is kept in Morton order).
__global__ void __launch_bounds__(256, 4) k_trace_specular_warp(const __grid_constant__ FastArgs A, const uint32_t* __restrict__ list,
                                                             const unsigned int* __restrict__ spec_count,
                                                             unsigned int* __restrict__ ticket) {
    const int lane = threadIdx.x & 31;
    const int64_t m = *spec_count;
    unsigned long long steps = 0;
    if (kTraceTickets) {
        // cones dealt to the warps as they free up: cone lengths differ by an order of magnitude
        for (;;) {
            uint32_t c0 = 0;
            if (lane == 0) c0 = atomicAdd(ticket, (unsigned)kSpecConesPerTicket);
            c0 = __shfl_sync(0xffffffffu, c0, 0);
            if ((int64_t)c0 >= m) break;
            const int64_t c1 = (int64_t)c0 + kSpecConesPerTicket < m ? (int64_t)c0 + kSpecConesPerTicket : m;
            for (int64_t c = c0; c < c1; ++c) specular_cone_warp(A, __ldg(list + c), steps);
        }
    } else {
        const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
        for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < m; c += nwarps)
            specular_cone_warp(A, __ldg(list + c), steps);
    }
    if (A.steps) {
        for (int o = 16; o > 0; o >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, o);
        if (lane == 0 && steps) atomicAdd(A.steps, steps);
    }
}

// ------------------------------------------------------------ batched form
// One trace over many jobs (clipmaps and sample sets) through a work queue:
// a table of job records and a global, padded index space in which job j
// owns the 32-aligned segment [bases[j], bases[j + 1]) (its count of samples
// rounded up to a multiple of 32; the rest is padding).  One radix sort of
// keys (job, Morton code of the sample, padding last) gives a coherent order
// in which each job keeps its segment, so every 32-position warp item of the
// diffuse kernel and every specular cone names one job.  The table travels as
// a kernel parameter (constant bank, like the single trace's arguments), so
// it holds up to kBatchJobs jobs per launch; longer lists run in chunks.
struct BatchJob {
    FastArgs A;
    uint32_t base, count;
};
constexpr int kBatchJobs = 64;
struct BatchTable {
    int njobs;
    uint32_t bases[kBatchJobs + 1];
    BatchJob jobs[kBatchJobs];
};
// kernel parameters may take 32,764 bytes (CUDA 12.1+, compute capability 7.0+); the kernels add at most 24
static_assert(sizeof(BatchTable) + 24 <= 32764, "the batch table must fit the kernel parameter space");

// Lane 0's value on every lane.  The batched kernels pass their job index
// through it: with a job index the compiler cannot prove warp-uniform, the
// job's texture handle is divergent and every fetch loops over the distinct
// handles of the warp (1.4 KB of register spills per thread in the specular
// kernel, and 2.4x its time).
__device__ __forceinline__ int warp_uniform(int v) { return __shfl_sync(0xffffffffu, v, 0); }

// The job whose segment holds global position g.
__device__ __forceinline__ int batch_job_of(const BatchTable& T, uint32_t g) {
    int lo = 0, hi = T.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (T.bases[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_batch_keys(const __grid_constant__ BatchTable T, uint32_t total,
                             unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int j = batch_job_of(T, g);
        const BatchJob& J = T.jobs[j];
        const uint32_t i = g - J.base;
        const uint32_t key = i < J.count ? morton_key(J.A.samples + i, J.A.C) : (1u << 30);
        keys[g] = ((unsigned long long)j << 31) | key;
        vals[g] = g;
    }
}

__global__ void k_batch_spec_keys(const __grid_constant__ BatchTable T, uint32_t total,
                                  const uint32_t* __restrict__ order, uint32_t* __restrict__ spec_key,
                                  unsigned int* __restrict__ spec_count) {
    const int lane = threadIdx.x & 31;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x - lane; b < total; b += gridDim.x * blockDim.x) {
        const uint32_t pos = b + lane;
        bool spec = false;
        if (pos < total) {
            const uint32_t g = __ldg(order + pos);
            const BatchJob& J = T.jobs[batch_job_of(T, g)];
            const uint32_t i = g - J.base;
            spec = i < J.count && J.A.C.need_specular && traces_specular(J.A.samples + i);
            spec_key[pos] = spec ? 0u : 256u;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, spec);
        if (lane == 0 && bal) atomicAdd(spec_count, (unsigned)__popc(bal));
    }
}

__global__ void __launch_bounds__(256) k_batch_diffuse(const __grid_constant__ BatchTable T, uint32_t total,
                                                       const uint32_t* __restrict__ order) {
    const int64_t nwarps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t base = ((int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5)) * 32; base < total;
         base += nwarps * 32) {
        const BatchJob& J = T.jobs[warp_uniform(batch_job_of(T, (uint32_t)base))];  // 32-aligned segments: one job
        const FastArgs& A = J.A;
        DealArgs D{&A.P, A.samples, (int64_t)total, order, J.base, J.count, A.dout, A.sout, A.C.ncones,
                   A.C.need_diffuse != 0, A.C.need_specular != 0};
        unsigned long long steps = 0;
        deal_diffuse_warp<kWarpsPerBlock>(D, FastDiffuseMarch{A.tex, &A.C}, base, steps);
        add_steps(A.steps, steps);
    }
}

__global__ void __launch_bounds__(256, 4) k_batch_specular(const __grid_constant__ BatchTable T,
                                                           const uint32_t* __restrict__ list,
                                                           const unsigned int* __restrict__ spec_count,
                                                           unsigned int* __restrict__ ticket) {
    const int64_t m = *spec_count;
    const int lane = threadIdx.x & 31;
    // cones dealt to the warps by a ticket, as in the single trace
    for (;;) {
        uint32_t c0 = 0;
        if (lane == 0) c0 = atomicAdd(ticket, (unsigned)kSpecConesPerTicket);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        if ((int64_t)c0 >= m) break;
        const int64_t c1 = (int64_t)c0 + kSpecConesPerTicket < m ? (int64_t)c0 + kSpecConesPerTicket : m;
        for (int64_t c = c0; c < c1; ++c) {
            const uint32_t g = __ldg(list + c);
            const BatchJob& J = T.jobs[warp_uniform(batch_job_of(T, g))];
            unsigned long long steps = 0;
            specular_cone_warp(J.A, g - J.base, steps);
            if (J.A.steps && lane == 0 && steps) atomicAdd(J.A.steps, steps);
        }
    }
}

// ------------------------------------------------------------- gather probe
// The trace's speed of light: one warp per synthetic cone, consecutive steps
// on consecutive lanes half a level-0 voxel apart (the specular kernel's
// access pattern), and at every step exactly the fetches a cone sample needs
// -- three face taps at two adjacent levels through sample_level -- with no
// compositing, lighting or scans.  Cones start within two level-0 voxels of
// the volume centre with hashed directions and cycle through the level
// pairs, so the taps are served by L1/TEX: the rate is the texture pipe's,
// an upper bound for the trace (which always does at least three of the six
// fetches and all of its other work on top).
__device__ __forceinline__ uint32_t probe_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__global__ void __launch_bounds__(256) k_gather_probe(const __grid_constant__ FastArgs A, int64_t cones, int steps,
                                                      float* __restrict__ out) {
    const FastConsts& C = A.C;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float ext0 = 2.0f * C.uvs;
    float acc = 0.0f;
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < cones; c += nwarps) {
        const uint32_t h0 = probe_hash((uint32_t)c * 3u + 1u), h1 = probe_hash((uint32_t)c * 3u + 2u),
                       h2 = probe_hash((uint32_t)c * 3u + 3u);
        const float3 start = f3(C.cx + ((float)(h0 & 0xffffu) * (1.0f / 65536.0f) - 0.5f) * ext0,
                                C.cy + ((float)(h0 >> 16) * (1.0f / 65536.0f) - 0.5f) * ext0,
                                C.cz + ((float)(h1 & 0xffffu) * (1.0f / 65536.0f) - 0.5f) * ext0);
        float3 dir = f3((float)(h1 >> 16) - 32768.0f, (float)(h2 & 0xffffu) - 32768.0f, (float)(h2 >> 16) - 32768.0f);
        const float inv = rsqrtf(fmaxf(dot3(dir, dir), 1.0f));
        dir = f3(dir.x * inv, dir.y * inv, dir.z * inv);
        const int lo = (int)(c % (kClipLevels - 1));
        const float fox = dir.x > 0.0f ? 0.0f : 1.0f / 6.0f;
        const float foy = dir.y > 0.0f ? 2.0f / 6.0f : 3.0f / 6.0f;
        const float foz = dir.z > 0.0f ? 4.0f / 6.0f : 5.0f / 6.0f;
        const float3 wt = f3(dir.x * dir.x, dir.y * dir.y, dir.z * dir.z);
        const float step = 0.5f * C.uvs;
        for (int k = lane; k < steps; k += 32) {
            const float d = step * (float)k;
            const float3 pos = f3(fmaf(dir.x, d, start.x), fmaf(dir.y, d, start.y), fmaf(dir.z, d, start.z));
            const float4 a = sample_level(A.tex, C, pos, lo, fox, foy, foz, wt);
            const float4 b = sample_level(A.tex, C, pos, lo + 1, fox, foy, foz, wt);
            acc += (a.x + a.w) + (b.y + b.w);
        }
    }
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// ------------------------------------------------------------- scratch layout
struct FastScratch {
    uint32_t *keys_in, *keys_out, *vals_in, *order, *spec_key, *spec_key_out, *spec_list;
    unsigned int* spec_count;
    void* temp;
    size_t temp_bytes;
    size_t total;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static int plan_scratch(int64_t n, void* base, FastScratch& s) {
    size_t t1 = 0, t2 = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, t1, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, 30);
    if (e != cudaSuccess) return cuda_fail(e, "cub::DeviceRadixSort::SortPairs (size query)");
    e = cub::DeviceRadixSort::SortPairs(nullptr, t2, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                        (uint32_t*)nullptr, (int)n, 0, 9);
    if (e != cudaSuccess) return cuda_fail(e, "cub::DeviceRadixSort::SortPairs (size query)");
    const size_t arr = align256(sizeof(uint32_t) * (size_t)n);
    char* p = (char*)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* q = p ? p + off : nullptr;
        off += align256(bytes);
        return q;
    };
    s.keys_in = (uint32_t*)take(arr);
    s.keys_out = (uint32_t*)take(arr);
    s.vals_in = (uint32_t*)take(arr);
    s.order = (uint32_t*)take(arr);
    s.spec_key = (uint32_t*)take(arr);
    s.spec_key_out = (uint32_t*)take(arr);
    s.spec_list = (uint32_t*)take(arr);
    s.spec_count = (unsigned int*)take(256);
    s.temp_bytes = t1 > t2 ? t1 : t2;
    s.temp = take(s.temp_bytes);
    s.total = off;
    return VCT_OK;
}

static void fill_fast_consts(FastConsts& C, const vct_cone_tracing_desc& d, float diffuse_aperture) {
    C.uvs = d.voxel_size;
    C.inv_uvs = 1.0f / d.voxel_size;
    C.min_radius = d.voxel_size * d.volume_dimension * 0.5f;
    C.inv_min_radius = 1.0f / C.min_radius;
    C.inv_min_radius2 = C.inv_min_radius * C.inv_min_radius;
    C.decay = d.occlusion_decay;
    C.start_off = d.trace_start_offset;
    const bool c32 = d.enable_32_cones != 0;
    C.ncones = c32 ? 32 : 16;
    C.aperture_diffuse = diffuse_aperture;
    C.coef_diffuse = 2.0f * tanf(C.aperture_diffuse * 0.5f);
    C.sf_diffuse = d.min_trace_step_factor > kMinTraceStepFactor ? d.min_trace_step_factor : kMinTraceStepFactor;
    C.cx = d.volume_center[0];
    C.cy = d.volume_center[1];
    C.cz = d.volume_center[2];
    const float dim = d.volume_dimension;
    for (int l = 0; l < kClipLevels; ++l) C.inv_ext[l] = 1.0f / (d.voxel_size * exp2f((float)l) * dim);
    // sx = ((f*dim + 1)/(dim+2))/6, sy = (((f*dim + 1)/(dim+2)) + l)/6, sz = (f*dim + 1)/(dim+2)
    C.ax = dim / ((dim + 2.0f) * 6.0f);
    C.bx = 1.0f / ((dim + 2.0f) * 6.0f);
    C.ay = C.ax;
    for (int l = 0; l < kClipLevels; ++l) C.by[l] = (1.0f / (dim + 2.0f) + (float)l) / 6.0f;
    C.az = dim / (dim + 2.0f);
    C.bz = 1.0f / (dim + 2.0f);
    const uint32_t mode = d.rendering_mode;
    C.need_diffuse = (mode == 4 || mode == 5 || mode == 7 || mode > 8 || mode == 8) ? 1 : 0;
    C.need_specular = (mode == 6 || mode >= 8) ? 1 : 0;
}

}  // namespace vct

using namespace vct;

namespace {

// The calling thread's second stream for the fast trace (non-blocking, with a
// fork and a join event), created on first use on each device; the specular
// cones run on it beside the diffuse kernel.  Null when it cannot be made
// (the trace then runs serially on the caller's stream).
struct TraceSide {
    int device = -1;
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~TraceSide() {
        if (s) cudaStreamDestroy(s);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
    }
};

TraceSide* trace_side() {
    static thread_local TraceSide side[8];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 8) return nullptr;
    TraceSide& t = side[dev];
    if (!t.s) {
        if (cudaStreamCreateWithFlags(&t.s, cudaStreamNonBlocking) != cudaSuccess) {
            t.s = nullptr;
            return nullptr;
        }
        if (cudaEventCreateWithFlags(&t.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&t.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaStreamDestroy(t.s);
            t.s = nullptr;
            return nullptr;
        }
        t.device = dev;
    }
    return &t;
}

}  // namespace

extern "C" int64_t vct_cone_trace_fast_scratch_bytes(int64_t n) {
    if (n < 0 || n > 0x7fffffffLL) return -1;
    FastScratch s;
    if (plan_scratch(n < 1 ? 1 : n, nullptr, s) != VCT_OK) return -1;
    return (int64_t)s.total;
}

extern "C" int vct_cone_trace_fast(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                   vct_texture_s* radiance, const vct_shadow_map* shadow,
                                   const vct_directional_light_desc* light,
                                   const vct_directional_light_shadow_desc* light_shadow,
                                   const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                   unsigned long long* cone_steps, void* scratch, size_t scratch_bytes,
                                   void* stream) {
    return vct_cone_trace_fast_opt(desc, cam, radiance, shadow, light, light_shadow, samples, n, dout, sout,
                                   cone_steps, nullptr, scratch, scratch_bytes, stream);
}

namespace {

// Launch shape of the fast trace: the grids of the diffuse and specular
// kernels in blocks (of 256 threads) per SM.  Result-neutral: both kernels
// are grid-stride loops in which a sample's diffuse item and a specular cone
// get the same arithmetic whichever warp takes them, and the step counter is
// an integer sum.
struct FastShape {
    int diffuse_per_sm = 8, specular_per_sm = 64;
};

int sm_count() {
    static int counts[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!counts[dev]) {
        int c = 0;
        if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c <= 0) c = 152;
        counts[dev] = c;
    }
    return counts[dev];
}

// Shapes chosen by vct_cone_trace_fast_autotune, per (device, log2 R).
std::mutex g_shape_mutex;
FastShape g_shapes[8][11];
bool g_tuned[8][11];

int log2_res(int R) { return 31 - __builtin_clz((unsigned)R); }

FastShape fast_shape(int R) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 8) return FastShape{};
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    const int l = log2_res(R);
    return g_tuned[dev][l] ? g_shapes[dev][l] : FastShape{};
}

// The trace pipeline after argument checks: Morton keys and sort, specular
// classification and partition, the diffuse and specular kernels.
int launch_fast(const FastArgs& A, const FastScratch& S, int64_t n, FastShape sh, cudaStream_t st) {
    const int sms = sm_count();
    const int block = 256;
    int64_t g = (n + block - 1) / block;
    const int grid_keys = (int)(g > (int64_t)sms * 32 ? (int64_t)sms * 32 : g);
    k_morton_keys<<<grid_keys, block, 0, st>>>(A.samples, n, A.C, S.keys_in, S.vals_in);
    VCT_LAUNCH_CHECK();
    size_t tb = S.temp_bytes;
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(S.temp, tb, S.keys_in, S.keys_out, S.vals_in, S.order, (int)n, 0, 30, st));
    // the specular count and the tickets of the specular cones and the diffuse items
    VCT_CUDA_TRY(cudaMemsetAsync(S.spec_count, 0, 3 * sizeof(unsigned int), st));
    int64_t gd = (n + 255) / 256;
    const int64_t cap_d = (int64_t)sms * sh.diffuse_per_sm;
    const int grid_d = (int)(gd > cap_d ? cap_d : gd);
    if (!A.C.need_specular) {
        k_trace_diffuse<<<grid_d, 256, 0, st>>>(A, S.order, S.spec_count + 2);
        VCT_LAUNCH_CHECK();
        return VCT_OK;
    }
    const int grid_k = (int)(gd > (int64_t)sms * 16 ? (int64_t)sms * 16 : gd);
    // the specular classification, partition and cones on the second stream,
    // beside the diffuse kernel (they share only the sorted order, read-only)
    TraceSide* side = kTraceSideStream ? trace_side() : nullptr;
    cudaStream_t ss = side ? side->s : st;
    if (side) {
        VCT_CUDA_TRY(cudaEventRecord(side->fork, st));
        VCT_CUDA_TRY(cudaStreamWaitEvent(ss, side->fork, 0));
    }
    k_spec_keys<<<grid_k, 256, 0, ss>>>(A, S.order, S.spec_key, S.spec_count);
    VCT_LAUNCH_CHECK();
    tb = S.temp_bytes;
    // stable partition (one radix pass on bit 8): specular samples first, Morton order kept
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(S.temp, tb, S.spec_key, S.spec_key_out, S.order, S.spec_list, (int)n,
                                                 8, 9, ss));
    int64_t gw = (n * 32 + 255) / 256;
    const int64_t cap_s = (int64_t)sms * sh.specular_per_sm;
    const int grid_s = (int)(gw > cap_s ? cap_s : gw);
    k_trace_specular_warp<<<grid_s, 256, 0, ss>>>(A, S.spec_list, S.spec_count, S.spec_count + 1);
    VCT_LAUNCH_CHECK();
    k_trace_diffuse<<<grid_d, 256, 0, st>>>(A, S.order, S.spec_count + 2);
    VCT_LAUNCH_CHECK();
    if (side) {
        VCT_CUDA_TRY(cudaEventRecord(side->join, ss));
        VCT_CUDA_TRY(cudaStreamWaitEvent(st, side->join, 0));
    }
    return VCT_OK;
}

// Argument checks and the kernels' argument block of one fast trace.
int prepare_fast(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture_s* radiance,
                 const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                 const vct_directional_light_shadow_desc* light_shadow, const vct_surface_sample* samples, int64_t n,
                 float* dout, float* sout, unsigned long long* cone_steps, const vct_trace_options* options,
                 void* scratch, size_t scratch_bytes, FastArgs& A, FastScratch& S) {
    VCT_CHECK_ARG(samples && dout && sout, "vct_cone_trace_fast: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_cone_trace_fast: sample/output buffers must be 16-byte aligned");
    VCT_CHECK_ARG(scratch && ((uintptr_t)scratch & 255) == 0, "vct_cone_trace_fast: scratch must be 256-byte aligned");
    int rc = fill_trace_params(A.P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    if ((rc = apply_trace_options(A.P, options)) != VCT_OK) return rc;
    VCT_CHECK_ARG((float)texture_resolution(radiance) == desc->volume_dimension,
                  "vct_cone_trace_fast: volume dimension differs from the texture's clipmap resolution");
    rc = plan_scratch(n, scratch, S);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(scratch_bytes >= S.total, "vct_cone_trace_fast: scratch buffer too small");
    fill_fast_consts(A.C, *desc, A.P.diffuse_aperture);
    A.tex = texture_object(radiance);
    A.samples = samples;
    A.n = n;
    A.dout = dout;
    A.sout = sout;
    A.steps = cone_steps;
    return VCT_OK;
}

}  // namespace

extern "C" int vct_cone_trace_fast_opt(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                       vct_texture_s* radiance, const vct_shadow_map* shadow,
                                       const vct_directional_light_desc* light,
                                       const vct_directional_light_shadow_desc* light_shadow,
                                       const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                       unsigned long long* cone_steps, const vct_trace_options* options,
                                       void* scratch, size_t scratch_bytes, void* stream) {
    vct::NvtxRange nvtx_range("vct_cone_trace_fast");
    VCT_CHECK_ARG(radiance, "vct_cone_trace_fast: null radiance texture");
    VCT_CHECK_ARG(n >= 0 && n <= 0x7fffffffLL, "vct_cone_trace_fast: sample count out of range");
    if (n == 0) return VCT_OK;
    FastArgs A;
    FastScratch S;
    int rc = prepare_fast(desc, cam, radiance, shadow, light, light_shadow, samples, n, dout, sout, cone_steps,
                          options, scratch, scratch_bytes, A, S);
    if (rc != VCT_OK) return rc;
    return launch_fast(A, S, n, fast_shape(texture_resolution(radiance)), as_stream(stream));
}

extern "C" int vct_cone_trace_fast_autotune(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                            vct_texture_s* radiance, const vct_shadow_map* shadow,
                                            const vct_directional_light_desc* light,
                                            const vct_directional_light_shadow_desc* light_shadow,
                                            const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                            void* scratch, size_t scratch_bytes, vct_trace_tuning* out,
                                            void* stream) {
    vct::NvtxRange nvtx_range("vct_cone_trace_fast_autotune");
    VCT_CHECK_ARG(radiance && out, "vct_cone_trace_fast_autotune: null argument");
    VCT_CHECK_ARG(n > 0 && n <= 0x7fffffffLL, "vct_cone_trace_fast_autotune: sample count out of range");
    int dev = 0;
    VCT_CUDA_TRY(cudaGetDevice(&dev));
    VCT_CHECK_ARG(dev >= 0 && dev < 8, "vct_cone_trace_fast_autotune: device index above 7");
    FastArgs A;
    FastScratch S;
    int rc = prepare_fast(desc, cam, radiance, shadow, light, light_shadow, samples, n, dout, sout, nullptr,
                          nullptr, scratch, scratch_bytes, A, S);
    if (rc != VCT_OK) return rc;
    cudaStream_t st = as_stream(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    VCT_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(VCT_E_CUDA, "vct_cone_trace_fast_autotune: cudaEventCreate");
    }
    // median of three timed traces after one warm-up, per shape
    auto time_shape = [&](FastShape sh, float* ms) -> int {
        float t[3];
        for (int k = -1; k < 3; ++k) {
            if (k >= 0 && cudaEventRecord(e0, st) != cudaSuccess) return fail(VCT_E_CUDA, "cudaEventRecord");
            int r = launch_fast(A, S, n, sh, st);
            if (r != VCT_OK) return r;
            if (k >= 0) {
                if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&t[k], e0, e1) != cudaSuccess)
                    return fail(VCT_E_CUDA, "vct_cone_trace_fast_autotune: event timing");
            }
        }
        const float lo = fminf(t[0], fminf(t[1], t[2])), hi = fmaxf(t[0], fmaxf(t[1], t[2]));
        *ms = t[0] + t[1] + t[2] - lo - hi;
        return VCT_OK;
    };
    // the specular grid first (the larger kernel), then the diffuse grid with it
    const int spec_c[] = {16, 32, 64, 128}, diff_c[] = {4, 8, 16};
    FastShape best;
    float best_ms = 0.0f, default_ms = 0.0f;
    rc = time_shape(best, &default_ms);
    best_ms = default_ms;
    for (int i = 0; rc == VCT_OK && i < 4; ++i) {
        FastShape c = best;
        c.specular_per_sm = spec_c[i];
        if (c.specular_per_sm == best.specular_per_sm && c.diffuse_per_sm == best.diffuse_per_sm) continue;
        float ms = 0.0f;
        rc = time_shape(c, &ms);
        if (rc == VCT_OK && ms < best_ms) best = c, best_ms = ms;
    }
    for (int i = 0; rc == VCT_OK && A.C.need_diffuse && i < 3; ++i) {
        FastShape c = best;
        c.diffuse_per_sm = diff_c[i];
        if (c.diffuse_per_sm == best.diffuse_per_sm) continue;
        float ms = 0.0f;
        rc = time_shape(c, &ms);
        if (rc == VCT_OK && ms < best_ms) best = c, best_ms = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VCT_OK) return rc;
    {
        std::lock_guard<std::mutex> lock(g_shape_mutex);
        const int l = log2_res(texture_resolution(radiance));
        g_shapes[dev][l] = best;
        g_tuned[dev][l] = true;
    }
    out->diffuse_blocks_per_sm = best.diffuse_per_sm;
    out->specular_blocks_per_sm = best.specular_per_sm;
    out->trace_ms = best_ms;
    out->default_ms = default_ms;
    out->tuned = 1;
    out->reserved = 0;
    return VCT_OK;
}

extern "C" int vct_trace_tuning_get(int32_t R, vct_trace_tuning* out) {
    VCT_CHECK_ARG(out && valid_resolution(R), "vct_trace_tuning_get: bad argument");
    int dev = 0;
    VCT_CUDA_TRY(cudaGetDevice(&dev));
    const FastShape sh = fast_shape(R);
    out->diffuse_blocks_per_sm = sh.diffuse_per_sm;
    out->specular_blocks_per_sm = sh.specular_per_sm;
    out->trace_ms = 0.0f;
    out->default_ms = 0.0f;
    {
        std::lock_guard<std::mutex> lock(g_shape_mutex);
        out->tuned = dev >= 0 && dev < 8 && g_tuned[dev][log2_res(R)] ? 1 : 0;
    }
    out->reserved = 0;
    return VCT_OK;
}

extern "C" int vct_trace_tuning_reset(void) {
    std::lock_guard<std::mutex> lock(g_shape_mutex);
    for (auto& row : g_tuned)
        for (bool& t : row) t = false;
    return VCT_OK;
}

// ------------------------------------------------------------ batched form
namespace {

// Scratch of one chunk of kBatchJobs jobs; the whole call reuses the
// largest chunk's layout (chunks run one after the other on the stream).
struct BatchLayout {
    uint32_t positions;  // padded global positions of the largest chunk
    size_t keys_in, keys_out, vals_in, order, spec_key, spec_key_out, spec_list, spec_count, temp;
    size_t temp_bytes, total;
};

int64_t padded(int64_t n) { return (n + 31) & ~int64_t(31); }

int batch_layout(const vct_trace_job* jobs, int32_t njobs, BatchLayout& L) {
    int64_t most = 0;
    for (int c0 = 0; c0 < njobs; c0 += kBatchJobs) {
        int64_t pos = 0;
        for (int j = c0; j < njobs && j < c0 + kBatchJobs; ++j) {
            if (jobs[j].sample_count < 0 || jobs[j].sample_count > 0x7fffffffLL)
                return fail(VCT_E_BAD_ARG, "vct_cone_trace_fast_batch: a job's sample count is out of range");
            pos += padded(jobs[j].sample_count);
            if (pos > 0x7fffffffLL)
                return fail(VCT_E_BAD_ARG,
                            "vct_cone_trace_fast_batch: more than 2^31 - 1 samples (32-padded per job) in one chunk");
        }
        most = pos > most ? pos : most;
    }
    L.positions = (uint32_t)most;
    int jb = 0;
    while ((1 << jb) < kBatchJobs) ++jb;
    size_t t1 = 0, t2 = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, t1, (unsigned long long*)nullptr,
                                                    (unsigned long long*)nullptr, (uint32_t*)nullptr,
                                                    (uint32_t*)nullptr, (int)L.positions, 0, 31 + jb);
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(nullptr, t2, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                            (uint32_t*)nullptr, (int)L.positions, 8, 9);
    if (e != cudaSuccess) return cuda_fail(e, "cub::DeviceRadixSort::SortPairs (size query)");
    L.temp_bytes = t1 > t2 ? t1 : t2;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += align256(bytes);
        return at;
    };
    const size_t n = L.positions;
    L.keys_in = take(8 * n);
    L.keys_out = take(8 * n);
    L.vals_in = take(4 * n);
    L.order = take(4 * n);
    L.spec_key = take(4 * n);
    L.spec_key_out = take(4 * n);
    L.spec_list = take(4 * n);
    L.spec_count = take(2 * sizeof(unsigned int));
    L.temp = take(L.temp_bytes);
    L.total = off;
    return VCT_OK;
}

}  // namespace

extern "C" int64_t vct_cone_trace_fast_batch_scratch_bytes(const vct_trace_job* jobs, int32_t job_count) {
    if (job_count < 0 || (job_count > 0 && !jobs)) return -1;
    BatchLayout L;
    if (batch_layout(jobs, job_count, L) != VCT_OK) return -1;
    return (int64_t)L.total;
}

extern "C" int vct_cone_trace_fast_batch(const vct_trace_job* jobs, int32_t job_count, void* scratch,
                                         size_t scratch_bytes, void* stream) {
    vct::NvtxRange nvtx_range("vct_cone_trace_fast_batch");
    VCT_CHECK_ARG(job_count >= 0, "vct_cone_trace_fast_batch: negative job count");
    if (job_count == 0) return VCT_OK;
    VCT_CHECK_ARG(jobs, "vct_cone_trace_fast_batch: null job list");
    BatchLayout L;
    int rc = batch_layout(jobs, job_count, L);
    if (rc != VCT_OK) return rc;
    if (L.positions == 0) return VCT_OK;
    VCT_CHECK_ARG(scratch && ((uintptr_t)scratch & 255) == 0,
                  "vct_cone_trace_fast_batch: scratch must be 256-byte aligned");
    VCT_CHECK_ARG(scratch_bytes >= L.total, "vct_cone_trace_fast_batch: scratch buffer too small");
    // every job is checked before any work is enqueued
    for (int j = 0; j < job_count; ++j) {
        const vct_trace_job& t = jobs[j];
        VCT_CHECK_ARG(t.radiance, "vct_cone_trace_fast_batch: a job has no radiance texture");
        VCT_CHECK_ARG((float)texture_resolution(t.radiance) == t.desc.volume_dimension,
                      "vct_cone_trace_fast_batch: a job's volume dimension differs from its texture's resolution");
        if (t.sample_count > 0) {
            VCT_CHECK_ARG(t.samples && t.diffuse_out && t.specular_out,
                          "vct_cone_trace_fast_batch: a job has a null sample or output buffer");
            VCT_CHECK_ARG((((uintptr_t)t.samples | (uintptr_t)t.diffuse_out | (uintptr_t)t.specular_out) & 15) == 0,
                          "vct_cone_trace_fast_batch: sample/output buffers must be 16-byte aligned");
        }
    }
    cudaStream_t st = as_stream(stream);
    char* b = static_cast<char*>(scratch);
    auto* keys_in = reinterpret_cast<unsigned long long*>(b + L.keys_in);
    auto* keys_out = reinterpret_cast<unsigned long long*>(b + L.keys_out);
    uint32_t* vals_in = reinterpret_cast<uint32_t*>(b + L.vals_in);
    uint32_t* order = reinterpret_cast<uint32_t*>(b + L.order);
    uint32_t* spec_key = reinterpret_cast<uint32_t*>(b + L.spec_key);
    uint32_t* spec_key_out = reinterpret_cast<uint32_t*>(b + L.spec_key_out);
    uint32_t* spec_list = reinterpret_cast<uint32_t*>(b + L.spec_list);
    unsigned int* spec_count = reinterpret_cast<unsigned int*>(b + L.spec_count);
    int jb = 0;
    while ((1 << jb) < kBatchJobs) ++jb;
    std::vector<BatchTable> tables((job_count + kBatchJobs - 1) / kBatchJobs);
    for (size_t c = 0; c < tables.size(); ++c) {
        BatchTable& T = tables[c];
        memset(&T, 0, sizeof(T));
        const int c0 = (int)c * kBatchJobs;
        T.njobs = job_count - c0 < kBatchJobs ? job_count - c0 : kBatchJobs;
        uint32_t pos = 0;
        for (int k = 0; k < T.njobs; ++k) {
            const vct_trace_job& t = jobs[c0 + k];
            BatchJob& B = T.jobs[k];
            vct_cam_matrix cam;
            memset(&cam, 0, sizeof(cam));
            for (int a = 0; a < 3; ++a) cam.eye_pos[a] = t.eye[a];
            rc = fill_trace_params(B.A.P, &t.desc, &cam, t.shadow.depth ? &t.shadow : nullptr, &t.light,
                                   &t.light_shadow);
            if (rc != VCT_OK) return rc;
            fill_fast_consts(B.A.C, t.desc, B.A.P.diffuse_aperture);
            B.A.tex = texture_object(t.radiance);
            B.A.samples = t.samples;
            B.A.n = t.sample_count;
            B.A.dout = t.diffuse_out;
            B.A.sout = t.specular_out;
            B.A.steps = t.cone_steps;
            B.base = pos;
            B.count = (uint32_t)t.sample_count;
            T.bases[k] = pos;
            pos += (uint32_t)padded(t.sample_count);
        }
        T.bases[T.njobs] = pos;
        if (pos == 0) continue;
        const int64_t n = pos;
        const int g256 = (int)((n + 255) / 256 > 152 * 32 ? 152 * 32 : (n + 255) / 256);
        k_batch_keys<<<g256, 256, 0, st>>>(T, pos, keys_in, vals_in);
        VCT_LAUNCH_CHECK();
        size_t tb = L.temp_bytes;
        VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(b + L.temp, tb, keys_in, keys_out, vals_in, order, (int)n, 0,
                                                     31 + jb, st));
        VCT_CUDA_TRY(cudaMemsetAsync(spec_count, 0, 2 * sizeof(unsigned int), st));  // count and cone ticket
        k_batch_spec_keys<<<(g256 > 152 * 16 ? 152 * 16 : g256), 256, 0, st>>>(T, pos, order, spec_key, spec_count);
        VCT_LAUNCH_CHECK();
        tb = L.temp_bytes;
        // stable partition (one radix pass on bit 8): specular positions first, the coherent order kept
        VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(b + L.temp, tb, spec_key, spec_key_out, order, spec_list,
                                                     (int)n, 8, 9, st));
        k_batch_diffuse<<<(g256 > 152 * 8 ? 152 * 8 : g256), 256, 0, st>>>(T, pos, order);
        VCT_LAUNCH_CHECK();
        const int64_t gw = (n * 32 + 255) / 256;
        k_batch_specular<<<(int)(gw > 152 * 64 ? 152 * 64 : gw), 256, 0, st>>>(T, spec_list, spec_count,
                                                                                spec_count + 1);
        VCT_LAUNCH_CHECK();
    }
    return VCT_OK;
}

extern "C" int vct_gather_probe(const vct_cone_tracing_desc* desc, vct_texture_s* radiance, int64_t cones,
                                int32_t steps_per_cone, double* samples_per_second, void* stream) {
    VCT_CHECK_ARG(desc && radiance && samples_per_second, "vct_gather_probe: null argument");
    VCT_CHECK_ARG(cones > 0 && cones <= (1LL << 30) && steps_per_cone > 0 && steps_per_cone <= (1 << 20),
                  "vct_gather_probe: cone or step count out of range");
    VCT_CHECK_ARG((float)texture_resolution(radiance) == desc->volume_dimension,
                  "vct_gather_probe: volume dimension differs from the texture's clipmap resolution");
    FastArgs A;
    memset(&A, 0, sizeof(A));
    fill_fast_consts(A.C, *desc, desc->enable_32_cones ? kAperture32 : kAperture16);
    A.tex = texture_object(radiance);
    cudaStream_t st = as_stream(stream);
    const int block = 256, grid = 152 * 8;
    float* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = VCT_OK;
    float ms = 0.0f;
    cudaError_t err = cudaMalloc(&out, sizeof(float) * (size_t)grid * block);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err == cudaSuccess) {
        k_gather_probe<<<grid, block, 0, st>>>(A, cones, steps_per_cone, out);  // warm-up
        err = cudaEventRecord(e0, st);
    }
    if (err == cudaSuccess) {
        k_gather_probe<<<grid, block, 0, st>>>(A, cones, steps_per_cone, out);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err != cudaSuccess) rc = cuda_fail(err, "vct_gather_probe");
    else *samples_per_second = (double)cones * (double)steps_per_cone / ((double)ms * 1e-3);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    return rc;
}
