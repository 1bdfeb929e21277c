// trace_deal.cuh -- the diffuse half of voxelConeTracing.frag's main()
// (:143-190, 258-293) for one warp of 32 samples, shared by the texture form
// (trace_fast.cu) and the exact FP32 forms (trace_exact.cu), generic in how
// one cone is marched.
//
// The (sample, cone) pairs with cos >= 0 of the warp's 32 samples are dealt
// to the 32 lanes in rounds, cone-major (lane k of a round takes the k-th
// pair ordered by cone, then by sample), so no lane idles on a back-facing
// cone and neighbouring lanes march the same direction from neighbouring
// samples.  Every sample's cone results are summed by its owner lane in cone
// order -- the shader's order -- so the diffuse sum does not depend on the
// dealing.  The owner lane then finishes the sample (normalisation, AO,
// albedo, direct term, rendering-mode switch) and writes the diffuse output,
// and the specular output of samples that trace no specular cone.
#pragma once

#include "trace_common.cuh"

namespace vct {

struct DealArgs {
    const TraceParams* P;
    const vct_surface_sample* __restrict__ samples;
    int64_t n;                           // positions in `order`
    const uint32_t* __restrict__ order;  // the visiting order: order[pos] - order_base is a sample index
    uint32_t order_base;
    uint32_t count;                      // entries whose sample index is >= count are padding
    float* __restrict__ dout;
    float* __restrict__ sout;
    int ncones;
    bool need_diffuse;   // trace the diffuse cones (otherwise their sum stays (0, 0, 0, 1))
    bool need_specular;  // specular samples get their specular output from the specular kernel
};

// The 32 positions base .. base + 31 of the order on the calling warp.
// `march(start, dir, start_level, steps)` traces one diffuse cone from `start`
// and returns traceCone's (rgb, 1 - occlusion).  WARPS = warps per block.
template <int WARPS, class Marcher>
__device__ __forceinline__ void deal_diffuse_warp(const DealArgs& A, const Marcher& march, int64_t base,
                                                  unsigned long long& steps) {
    __shared__ float4 s_start[WARPS][32];
    __shared__ float4 s_norm[WARPS][32];
    __shared__ int s_cincl[WARPS][32];     // inclusive prefix of the pairs per cone
    __shared__ uint32_t s_cmask[WARPS][32];  // samples (lanes) that trace each cone
    __shared__ float4 s_res[WARPS][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const TraceParams& P = *A.P;
    const vct_cone_tracing_desc& d = P.d;
    const bool c32 = A.ncones == 32;
    {
        const int64_t pos = base + lane;
        bool valid = pos < A.n;
        const uint32_t idx = valid ? __ldg(A.order + pos) - A.order_base : 0u;
        valid = valid && idx < A.count;
        GSample g;
        float min_level = 0.0f;
        float3 start = f3(0.f, 0.f, 0.f);
        uint32_t mask = 0;
        if (valid) {
            g = load_sample(A.samples + idx, P.eye);
            valid = g.depth != 1.0f;
        }
        if (valid) {
            min_level = calc_min_level(d, g.wp);
            const float vs = d.voxel_size * exp2f(min_level);
            start = g.wp + g.normal * (vs * d.trace_start_offset);
            if (A.need_diffuse)
                for (int c = 0; c < A.ncones; ++c) {
                    const float3 dir = c32 ? f3(c_dirs32[c][0], c_dirs32[c][1], c_dirs32[c][2])
                                           : f3(c_dirs16[c][0], c_dirs16[c][1], c_dirs16[c][2]);
                    if (!(dot3(g.normal, dir) < 0.0f)) mask |= 1u << c;
                }
        }
        // cone c's pairs are the lanes of cmask[c]
        uint32_t my_cmask = 0;
        for (int c = 0; c < A.ncones; ++c) {
            const uint32_t cm = __ballot_sync(0xffffffffu, (mask >> c) & 1u);
            if (lane == c) my_cmask = cm;
        }
        int cincl = __popc(my_cmask);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, cincl, o);
            if (lane >= o) cincl += t;
        }
        const int total = __shfl_sync(0xffffffffu, cincl, 31);
        s_start[w][lane] = make_float4(start.x, start.y, start.z, min_level);
        s_norm[w][lane] = valid ? make_float4(g.normal.x, g.normal.y, g.normal.z, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        s_cincl[w][lane] = cincl;
        s_cmask[w][lane] = my_cmask;
        __syncwarp();
        float4 acc = make_float4(0.f, 0.f, 0.f, 1.f);
        const uint32_t below = (1u << lane) - 1u;
        uint32_t pending = mask;  // this lane's cones not yet added, added in cone order
        for (int r0 = 0; r0 < total; r0 += 32) {
            const int k = r0 + lane;
            float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < total) {
                int lo = 0, hi = 31;  // the cone whose inclusive prefix first exceeds k
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (s_cincl[w][mid] > k) hi = mid;
                    else lo = mid + 1;
                }
                const int cone = lo;
                const uint32_t cm = s_cmask[w][cone];
                const int j = k - (s_cincl[w][cone] - __popc(cm));
                const int sl = (int)__fns(cm, 0, j + 1);  // the sample's lane
                const float3 dir = c32 ? f3(c_dirs32[cone][0], c_dirs32[cone][1], c_dirs32[cone][2])
                                       : f3(c_dirs16[cone][0], c_dirs16[cone][1], c_dirs16[cone][2]);
                const float4 st = s_start[w][sl];
                const float4 nn = s_norm[w][sl];
                const float cos_t = nn.x * dir.x + nn.y * dir.y + nn.z * dir.z;
                const float4 r = march(f3(st.x, st.y, st.z), dir, st.w, steps);
                res = make_float4(r.x * cos_t, r.y * cos_t, r.z * cos_t, r.w * cos_t);
            }
            s_res[w][lane] = res;
            __syncwarp();
            // this lane's pairs in this round, lowest cone first: a pair's index
            // grows with its cone, so the sum runs in cone order (the shader's)
            while (pending) {
                const int c = __ffs(pending) - 1;
                const uint32_t cm = s_cmask[w][c];
                const int pidx = s_cincl[w][c] - __popc(cm) + __popc(cm & below);
                if (pidx >= r0 + 32) break;
                const float4 v = s_res[w][pidx - r0];
                acc = make_float4(acc.x + v.x, acc.y + v.y, acc.z + v.z, acc.w + v.w);
                pending &= pending - 1u;
            }
            __syncwarp();
        }
        if (valid) {
            const float inv_n = 1.0f / (float)A.ncones;
            float4 ind = make_float4(acc.x * inv_n, acc.y * inv_n, acc.z * inv_n, acc.w * inv_n);
            ind.w = ind.w * d.ambient_occlusion_factor;
            ind.x = ind.x * (g.diffuse_color.x * d.indirect_diffuse_intensity);
            ind.y = ind.y * (g.diffuse_color.y * d.indirect_diffuse_intensity);
            ind.z = ind.z * (g.diffuse_color.z * d.indirect_diffuse_intensity);
            const float3 direct = direct_term(P, g);
            const bool spec = A.need_specular && has_specular_cone(g);
            float4 dd[2];
            write_outputs(P, g, min_level, ind, f3(0.f, 0.f, 0.f), direct, reinterpret_cast<float*>(&dd[0]),
                          reinterpret_cast<float*>(&dd[1]));
            reinterpret_cast<float4*>(A.dout)[idx] = dd[0];
            if (!spec) reinterpret_cast<float4*>(A.sout)[idx] = dd[1];
        }
    }
}

// Every warp of the grid over the order, 32 positions at a time: with
// TICKET (`ticket` zeroed before the launch), the items go to the warps as
// they free up; without, by a static grid stride.
template <int WARPS, bool TICKET = false, class Marcher>
__device__ __forceinline__ void deal_diffuse(const DealArgs& A, const Marcher& march, unsigned long long& steps,
                                             unsigned int* ticket = nullptr) {
    if constexpr (TICKET) {
        const int lane = threadIdx.x & 31;
        for (;;) {
            uint32_t it = 0;
            if (lane == 0) it = atomicAdd(ticket, 1u);
            it = __shfl_sync(0xffffffffu, it, 0);
            const int64_t base = (int64_t)it * 32;
            if (base >= A.n) break;
            deal_diffuse_warp<WARPS>(A, march, base, steps);
        }
        return;
    }
    const int64_t nwarps = (int64_t)gridDim.x * WARPS;
    for (int64_t base = ((int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5)) * 32; base < A.n; base += nwarps * 32)
        deal_diffuse_warp<WARPS>(A, march, base, steps);
}

// Adds a warp's step count to the counter (one atomic per warp).
__device__ __forceinline__ void add_steps(unsigned long long* counter, unsigned long long steps) {
    if (!counter) return;
    for (int o = 16; o > 0; o >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, o);
    if ((threadIdx.x & 31) == 0 && steps) atomicAdd(counter, steps);
}

}  // namespace vct
