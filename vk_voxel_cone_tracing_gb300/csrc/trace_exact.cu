// trace_exact.cu -- the plain FP32 drop-in of voxelConeTracing.frag.
//
// One thread per G-buffer sample, cones traced in the shader's order, the
// radiance clipmap read from the reference's linear RGBA8 atlas with a
// software trilinear filter (FP32 weights, REPEAT addressing) -- the same
// arithmetic, in the same order, as the FP32 restatement of the shader.
// Compiled with -fmad=false so no multiply-add is fused.
#include <cstring>

#include "trace_common.cuh"

namespace vct {

struct ExactAtlas {
    const uint32_t* __restrict__ p;
    AtlasDims A;
    __device__ __forceinline__ float4 fetch(int x, int y, int z) const { return unpack_rgba8(__ldg(p + A.index(x, y, z))); }
};

__device__ __forceinline__ int wrap_rep(int i, int n) {
    int m = i % n;
    return m < 0 ? m + n : m;
}

__device__ __forceinline__ float4 lerp4(float4 p, float4 q, float t) {
    return make_float4(p.x + (q.x - p.x) * t, p.y + (q.y - p.y) * t, p.z + (q.z - p.z) * t, p.w + (q.w - p.w) * t);
}

// Linear-filtered sampler3D fetch (Vulkan linear filter, REPEAT, one mip).
__device__ __forceinline__ float4 texture3d(const ExactAtlas& T, float ux, float uy, float uz) {
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
__device__ __forceinline__ float4 sample_clipmap(const ExactAtlas& T, const vct_cone_tracing_desc& d, float3 p,
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
__device__ float4 trace_cone(const ExactAtlas& T, const vct_cone_tracing_desc& d, float3 start, float3 dir,
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
        float4 hi = sample_clipmap(T, d, pos, upper, fo, wt);
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

__global__ void __launch_bounds__(128) k_cone_trace_exact(TraceParams P, ExactAtlas T,
                                                          const vct_surface_sample* __restrict__ samples, int64_t n,
                                                          float* __restrict__ dout, float* __restrict__ sout,
                                                          unsigned long long* __restrict__ step_counter) {
    unsigned long long steps = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        GSample g = load_sample(samples + i, P.eye);
        if (g.depth == 1.0f) continue;
        const vct_cone_tracing_desc& d = P.d;
        float min_level = calc_min_level(d, g.wp);
        float vs = d.voxel_size * exp2f(min_level);
        float3 start = g.wp + g.normal * (vs * d.trace_start_offset);
        float4 ind = make_float4(0.f, 0.f, 0.f, 1.f);
        const bool c32 = d.enable_32_cones != 0;
        const int nc = c32 ? 32 : 16;
        const float aperture = c32 ? kAperture32 : kAperture16;
        const float sf = fmaxf(kMinTraceStepFactor, d.min_trace_step_factor);
        for (int c = 0; c < nc; ++c) {
            float3 dir = c32 ? f3(c_dirs32[c][0], c_dirs32[c][1], c_dirs32[c][2])
                             : f3(c_dirs16[c][0], c_dirs16[c][1], c_dirs16[c][2]);
            float cos_t = dot3(g.normal, dir);
            if (cos_t < 0.0f) continue;
            float4 r = trace_cone(T, d, start, dir, aperture, kMaxTraceDistance, min_level, sf, steps);
            ind = make_float4(ind.x + r.x * cos_t, ind.y + r.y * cos_t, ind.z + r.z * cos_t, ind.w + r.w * cos_t);
        }
        ind = make_float4(ind.x / (float)nc, ind.y / (float)nc, ind.z / (float)nc, ind.w / (float)nc);
        ind.w = ind.w * d.ambient_occlusion_factor;
        ind.x = ind.x * (g.diffuse_color.x * d.indirect_diffuse_intensity);
        ind.y = ind.y * (g.diffuse_color.y * d.indirect_diffuse_intensity);
        ind.z = ind.z * (g.diffuse_color.z * d.indirect_diffuse_intensity);
        float3 ispec = f3(0.f, 0.f, 0.f);
        if (has_specular_cone(g)) {
            float3 sdir = reflect3(f3(-g.view.x, -g.view.y, -g.view.z), g.normal);
            float4 r = trace_cone(T, d, start, sdir, fmaxf(g.roughness, kMinSpecularAperture), kMaxTraceDistance,
                                  min_level, d.voxel_size, steps);
            const float isi = d.indirect_specular_intensity;
            ispec = f3(r.x * g.specular_color.x * isi, r.y * g.specular_color.y * isi, r.z * g.specular_color.z * isi);
        }
        float3 direct = direct_term(P, g);
        write_outputs(P, g, min_level, ind, ispec, direct, dout + 4 * i, sout + 4 * i);
    }
    if (step_counter) {
        // Warp-aggregated accumulation of the iteration count.
        for (int o = 16; o > 0; o >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, o);
        if ((threadIdx.x & 31) == 0 && steps) atomicAdd(step_counter, steps);
    }
}

}  // namespace vct

using namespace vct;

namespace vct {
int fill_trace_params(TraceParams& P, const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                      const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow) {
    VCT_CHECK_ARG(desc && cam && light, "cone trace: null descriptor");
    VCT_CHECK_ARG(desc->voxel_size > 0.0f && desc->volume_dimension >= 1.0f, "cone trace: bad voxel size / dimension");
    P.d = *desc;
    for (int a = 0; a < 3; ++a) P.eye[a] = cam->eye_pos[a];
    P.light = *light;
    if (shadow && shadow->depth) {
        VCT_CHECK_ARG(light_shadow, "cone trace: shadow map given without its light shadow desc");
        VCT_CHECK_ARG(shadow->width > 0 && shadow->height > 0 && shadow->width <= 32768 && shadow->height <= 32768,
                      "cone trace: bad shadow map size");
        P.shadow = shadow->depth;
        P.shadow_w = shadow->width;
        P.shadow_h = shadow->height;
        P.shadow_desc = *light_shadow;
    } else {
        P.shadow = nullptr;
        P.shadow_w = P.shadow_h = 0;
        memset(&P.shadow_desc, 0, sizeof(P.shadow_desc));
    }
    return VCT_OK;
}
}  // namespace vct

extern "C" int vct_cone_trace(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                              const uint32_t* radiance_atlas, int32_t R, const vct_shadow_map* shadow,
                              const vct_directional_light_desc* light,
                              const vct_directional_light_shadow_desc* light_shadow,
                              const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                              unsigned long long* cone_steps, void* stream) {
    VCT_CHECK_ARG(radiance_atlas && valid_resolution(R), "vct_cone_trace: bad radiance atlas / resolution");
    VCT_CHECK_ARG(n >= 0, "vct_cone_trace: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && dout && sout, "vct_cone_trace: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_cone_trace: sample/output buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    ExactAtlas T{radiance_atlas, AtlasDims(R)};
    int64_t blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_cone_trace_exact<<<(int)blocks, 128, 0, as_stream(stream)>>>(P, T, samples, n, dout, sout, cone_steps);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}
