// svo_trace.cu -- OctreeVoxelConeTracing pass (voxelConeTracing_Octree.frag)
// over a sparse-voxel-octree node pool.
//
// Same cone loop as the clipmap tracer, sampling the pool by point location:
// sampleSVO normalises the position by a scene box (the shader hard-codes
// Sponza's), descends from uVolumeDimension to resolution 2^level and reads
// the node's RGBA8; two levels are mixed by fract(level).  One thread per
// G-buffer sample, FP32 in the shader's order (-fmad=false), so the results
// track the FP32 restatement; the pool descents are dependent loads served
// from L2 (a depth-8 pool of a few million nodes is L2-resident).
#include "trace_common.cuh"

namespace vct {

int fill_trace_params(TraceParams& P, const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                      const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow);

struct SvoScene {
    const uint2* __restrict__ pool;
    uint32_t nodes;
    float bmin[3], bmax[3];
};

__device__ inline float4 sample_svo(const SvoScene& S, const vct_cone_tracing_desc& d, float3 p, uint32_t level) {
    const float ex = S.bmax[0] - S.bmin[0], ey = S.bmax[1] - S.bmin[1], ez = S.bmax[2] - S.bmin[2];
    const float ev = fmaxf(ex, fmaxf(ey, ez)) * 0.5f;
    const float c[3] = {(S.bmin[0] + S.bmax[0]) * 0.5f, (S.bmin[1] + S.bmax[1]) * 0.5f, (S.bmin[2] + S.bmax[2]) * 0.5f};
    uint32_t resolution = (uint32_t)d.volume_dimension;
    const float pp[3] = {p.x, p.y, p.z};
    uint32_t fp[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float s = (pp[a] - c[a]) / ev;
        float u = ((s + 1.0f) * 0.5f) * (float)resolution;
        u = fmaxf(u, 0.0f);
        const uint32_t q = (uint32_t)fminf(u, 4294967040.0f);
        fp[a] = min(q, resolution);
    }
    const uint32_t target = 1u << level;
    uint32_t idx = 0, cur = 0;
    do {
        resolution >>= 1;
        const uint32_t cx = fp[0] >= resolution, cy = fp[1] >= resolution, cz = fp[2] >= resolution;
        idx = cur + (cz | (cx << 1) | (cy << 2));
        if (idx >= S.nodes) return make_float4(0.f, 0.f, 0.f, 0.f);  // malformed pool: never read past it
        cur = __ldg(&S.pool[idx].x) & 0x7fffffffu;
        fp[0] -= cx * resolution;
        fp[1] -= cy * resolution;
        fp[2] -= cz * resolution;
    } while (cur != 0u && resolution > target);
    const uint32_t v = __ldg(&S.pool[idx].y);
    return unpack_rgba8(v);
}

__device__ float4 svo_trace_cone(const SvoScene& S, const vct_cone_tracing_desc& d, float3 start, float3 dir,
                                 float aperture, float start_level, float step_factor, unsigned long long& steps) {
    float4 result = make_float4(0.f, 0.f, 0.f, 0.f);
    const float uvs = d.voxel_size;
    const float cone_coef = 2.0f * tanf(aperture * 0.5f);
    float cur_level = start_level;
    float vs = uvs * exp2f(cur_level);
    start = start + dir * (vs * d.trace_start_offset * 0.5f);
    float step = 0.0f, diameter = fmaxf(step * cone_coef, uvs), occlusion = 0.0f, seg = vs;
    const float min_radius = uvs * d.volume_dimension * 0.5f;
    const float3 center = f3(d.volume_center[0], d.volume_center[1], d.volume_center[2]);
    while (step < kMaxTraceDistance && occlusion < 1.0f) {
        ++steps;
        const float3 pos = start + dir * step;
        const float dist = sqrtf(dot3(center - pos, center - pos));
        const float min_level = ceilf(log2f(dist / min_radius));
        cur_level = log2f(diameter / uvs);
        cur_level = fminf(fmaxf(fmaxf(start_level, cur_level), min_level), (float)(kClipLevels - 1));
        const uint32_t lo = (uint32_t)floorf(cur_level), hi = (uint32_t)ceilf(cur_level);
        const float4 a = sample_svo(S, d, pos, lo), b = sample_svo(S, d, pos, hi);
        const float fr = fractf(cur_level);
        const float4 s = make_float4(a.x * (1.0f - fr) + b.x * fr, a.y * (1.0f - fr) + b.y * fr,
                                     a.z * (1.0f - fr) + b.z * fr, a.w * (1.0f - fr) + b.w * fr);
        vs = uvs * exp2f(cur_level);
        const float correction = seg / vs;
        const float rx = s.x * correction, ry = s.y * correction, rz = s.z * correction;
        // alpha rounded above 1 (a pow of a negative base, undefined in GLSL) is taken as 1
        const float opacity = clampf(1.0f - powf(fmaxf(1.0f - s.w, 0.0f), correction), 0.0f, 1.0f);
        const float k = clampf(1.0f - result.w, 0.0f, 1.0f);
        result = make_float4(result.x + k * rx, result.y + k * ry, result.z + k * rz, result.w + k * opacity);
        occlusion = occlusion + (1.0f - occlusion) * opacity / (1.0f + (step + vs) * d.occlusion_decay);
        const float prev = step;
        step = step + fmaxf(diameter, uvs) * step_factor;
        seg = step - prev;
        diameter = step * cone_coef;
    }
    return make_float4(clampf(result.x, 0.f, 1.f), clampf(result.y, 0.f, 1.f), clampf(result.z, 0.f, 1.f),
                       clampf(1.0f - occlusion, 0.f, 1.f));
}

__global__ void __launch_bounds__(128) k_svo_trace(TraceParams P, SvoScene S, const vct_surface_sample* __restrict__ samples,
                                                   int64_t n, const uint32_t* __restrict__ order,
                                                   float* __restrict__ dout, float* __restrict__ sout,
                                                   unsigned long long* __restrict__ step_counter,
                                                   unsigned int* __restrict__ ticket) {
    unsigned long long steps = 0;
    const vct_cone_tracing_desc& d = P.d;
    const int lane = threadIdx.x & 31;
    // 32 consecutive samples of the coherent order per warp, dealt by a ticket as warps free up
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(ticket, 32u);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if ((int64_t)t0 >= n) break;
        const int64_t t = (int64_t)t0 + lane;
        if (t >= n) continue;
        const int64_t i = order ? (int64_t)__ldg(order + t) : t;
        GSample g = load_sample(samples + i, P.eye);
        if (g.depth == 1.0f) continue;
        const float min_level = calc_min_level(d, g.wp);
        const float vs = d.voxel_size * exp2f(min_level);
        const float3 start = g.wp + g.normal * (vs * d.trace_start_offset);
        float4 ind = make_float4(0.f, 0.f, 0.f, 1.f);
        float valid = 0.0f;
        const bool c32 = d.enable_32_cones != 0;
        const int nc = c32 ? 32 : 16;
        const float aperture = c32 ? kAperture32 : kAperture16;
        const float sf = fmaxf(kMinTraceStepFactor, d.min_trace_step_factor);
        for (int c = 0; c < nc; ++c) {
            const float3 dir = c32 ? f3(c_dirs32[c][0], c_dirs32[c][1], c_dirs32[c][2])
                                   : f3(c_dirs16[c][0], c_dirs16[c][1], c_dirs16[c][2]);
            const float cos_t = dot3(g.normal, dir);
            if (cos_t < 0.0f) continue;
            const float4 r = svo_trace_cone(S, d, start, dir, aperture, min_level, sf, steps);
            ind = make_float4(ind.x + r.x * cos_t, ind.y + r.y * cos_t, ind.z + r.z * cos_t, ind.w + r.w * cos_t);
            valid = valid + cos_t;
        }
        ind = make_float4(ind.x / valid, ind.y / valid, ind.z / valid, ind.w / valid);
        ind.w = ind.w * d.ambient_occlusion_factor;
        ind.x = ind.x * (g.diffuse_color.x * d.indirect_diffuse_intensity);
        ind.y = ind.y * (g.diffuse_color.y * d.indirect_diffuse_intensity);
        ind.z = ind.z * (g.diffuse_color.z * d.indirect_diffuse_intensity);
        ind = make_float4(clampf(ind.x, 0.f, 1.f), clampf(ind.y, 0.f, 1.f), clampf(ind.z, 0.f, 1.f), clampf(ind.w, 0.f, 1.f));
        float3 ispec = f3(0.f, 0.f, 0.f);
        if (has_specular_cone(g)) {
            const float3 sdir = normalize3(reflect3(f3(-g.view.x, -g.view.y, -g.view.z), g.normal));
            const float4 r = svo_trace_cone(S, d, start, sdir, fmaxf(g.roughness, kMinSpecularAperture), min_level,
                                            fmaxf(kMinTraceStepFactor, d.voxel_size), steps);
            const float isi = d.indirect_specular_intensity;
            ispec = f3(r.x * g.specular_color.x * isi, r.y * g.specular_color.y * isi, r.z * g.specular_color.z * isi);
        }
        float3 direct = direct_term(P, g);
        direct = f3(clampf(direct.x, 0.f, 1.f), clampf(direct.y, 0.f, 1.f), clampf(direct.z, 0.f, 1.f));
        float4 D = make_float4(0.f, 0.f, 0.f, 1.f), Sp = make_float4(0.f, 0.f, 0.f, 1.f);
        switch (d.rendering_mode) {
            case 0: D = make_float4(g.diffuse_color.x, g.diffuse_color.y, g.diffuse_color.z, 1.f); break;
            case 1: D = make_float4(g.specular_color.x, g.specular_color.y, g.specular_color.z, 1.f); break;
            case 2:
                D = make_float4(g.normal.x * 0.5f + 0.5f, g.normal.y * 0.5f + 0.5f, g.normal.z * 0.5f + 0.5f, 1.f);
                break;
            case 3: {
                const float colors[7][4] = {{1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {1, 1, 0, 1},
                                            {0, 1, 1, 1}, {1, 0, 1, 1}, {1, 1, 1, 1}};
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                for (int k = 0; k < 6; ++k)
                    if (min_level < (float)(k + 1)) {
                        const float fr = fractf(min_level);
                        for (int c = 0; c < 4; ++c) v[c] = colors[k][c] * (1.0f - fr) + colors[k + 1][c] * fr;
                        break;
                    }
                D = make_float4(v[0] * 0.5f, v[1] * 0.5f, v[2] * 0.5f, v[3] * 0.5f);
                break;
            }
            case 4:
                direct = direct * ind.w;
                D = make_float4(direct.x, direct.y, direct.z, 1.f);
                break;
            case 5: D = make_float4(D.x + ind.x, D.y + ind.y, D.z + ind.z, 1.f); break;
            case 6: Sp = make_float4(Sp.x + ispec.x, Sp.y + ispec.y, Sp.z + ispec.z, 1.f); break;
            case 7: D = make_float4(ind.w, ind.w, ind.w, 1.f); break;
            default:
                direct = direct * ind.w;
                D = make_float4(D.x + direct.x + ind.x, D.y + direct.y + ind.y, D.z + direct.z + ind.z, 1.f);
                Sp = make_float4(Sp.x + ispec.x, Sp.y + ispec.y, Sp.z + ispec.z, 1.f);
                break;
        }
        reinterpret_cast<float4*>(dout)[i] = D;
        reinterpret_cast<float4*>(sout)[i] = Sp;
    }
    if (step_counter) {
        for (int o = 16; o > 0; o >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, o);
        if ((threadIdx.x & 31) == 0 && steps) atomicAdd(step_counter, steps);
    }
}

}  // namespace vct

using namespace vct;

extern "C" int vct_svo_cone_trace(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const uint32_t* pool,
                                  int64_t node_count, const float bb_min[3], const float bb_max[3],
                                  const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                                  const vct_directional_light_shadow_desc* light_shadow,
                                  const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                  unsigned long long* cone_steps, void* stream) {
    VCT_CHECK_ARG(pool && node_count >= 8 && bb_min && bb_max, "vct_svo_cone_trace: bad node pool / scene box");
    VCT_CHECK_ARG(n >= 0, "vct_svo_cone_trace: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && dout && sout, "vct_svo_cone_trace: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_svo_cone_trace: buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    const uint32_t dim = (uint32_t)desc->volume_dimension;
    VCT_CHECK_ARG(dim >= 2 && (dim & (dim - 1)) == 0 && dim <= 4096,
                  "vct_svo_cone_trace: volume dimension must be a power of two (the pool's root resolution)");
    SvoScene S;
    S.pool = reinterpret_cast<const uint2*>(pool);
    VCT_CHECK_ARG(node_count < (1LL << 31), "vct_svo_cone_trace: node count out of range");
    S.nodes = (uint32_t)node_count;
    for (int a = 0; a < 3; ++a) {
        S.bmin[a] = bb_min[a];
        S.bmax[a] = bb_max[a];
    }
    // the samples walked in the coherent order (normal class, then Morton), as the clipmap trace does
    cudaStream_t st = as_stream(stream);
    SampleOrder so;
    rc = sample_coherent_order(samples, n, P.d, &so, st);
    if (rc != VCT_OK) return rc;
    int64_t blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    unsigned int* ticket = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&ticket, sizeof(unsigned int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) {
        k_svo_trace<<<(int)blocks, 128, 0, st>>>(P, S, samples, n, so.order, dout, sout, cone_steps, ticket);
        e = cudaGetLastError();
    }
    if (ticket) cudaFreeAsync(ticket, st);
    if (so.block) cudaFreeAsync(so.block, st);
    if (e != cudaSuccess) return cuda_fail(e, "k_svo_trace");
    return VCT_OK;
}
