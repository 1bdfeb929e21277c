// trace_exact.cu -- the plain FP32 drop-in of voxelConeTracing.frag.
//
// One thread per G-buffer sample, cones traced in the shader's order, the
// radiance clipmap read from the reference's linear RGBA8 atlas with a
// software trilinear filter (FP32 weights, REPEAT addressing) -- the same
// arithmetic, in the same order, as the FP32 restatement of the shader.
// Compiled with -fmad=false so no multiply-add is fused.
#include <cstring>

#include <cub/cub.cuh>

#include "trace_exact.cuh"

namespace vct {

template <class Atlas>
__global__ void __launch_bounds__(128) k_cone_trace_exact(TraceParams P, Atlas T,
                                                          const vct_surface_sample* __restrict__ samples, int64_t n,
                                                          const uint32_t* __restrict__ order,
                                                          float* __restrict__ dout, float* __restrict__ sout,
                                                          unsigned long long* __restrict__ step_counter) {
    unsigned long long steps = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = order ? (int64_t)__ldg(order + t) : t;
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

__device__ __forceinline__ uint32_t spread_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Key = normal class (6 bits: the octahedral map of the normal on an 8 x 8
// grid) above a 30-bit Morton code of the position (10 bits per axis, cells
// of two level-0 voxels: +-1024 voxels around the centre).  Samples with
// similar normals skip the same diffuse cones (cos < 0), so a warp's lanes
// agree on which cones to march; within a class, neighbouring points share
// texels.
__global__ void k_sample_keys(const vct_surface_sample* __restrict__ s, int64_t n, float cx, float cy, float cz,
                              float q, unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* p = s[i].position;
        const int x = min(max(__float2int_rd((p[0] - cx) * q) + 512, 0), 1023);
        const int y = min(max(__float2int_rd((p[1] - cy) * q) + 512, 0), 1023);
        const int z = min(max(__float2int_rd((p[2] - cz) * q) + 512, 0), 1023);
        const float* t = s[i].normal_texel;
        const float nx = t[0] * 2.0f - 1.0f, ny = t[1] * 2.0f - 1.0f, nz = t[2] * 2.0f - 1.0f;
        const float l1 = fabsf(nx) + fabsf(ny) + fabsf(nz);
        float ox = l1 > 0.0f ? nx / l1 : 0.0f, oy = l1 > 0.0f ? ny / l1 : 0.0f;
        if (nz < 0.0f) {
            const float ax = (1.0f - fabsf(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
            const float ay = (1.0f - fabsf(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
            ox = ax;
            oy = ay;
        }
        const int cu = min(max((int)((ox * 0.5f + 0.5f) * 8.0f), 0), 7);
        const int cv = min(max((int)((oy * 0.5f + 0.5f) * 8.0f), 0), 7);
        keys[i] = ((unsigned long long)(cv * 8 + cu) << 30) |
                  (spread_bits10(x) | (spread_bits10(y) << 1) | (spread_bits10(z) << 2));
        vals[i] = (uint32_t)i;
    }
}

int sample_coherent_order(const vct_surface_sample* samples, int64_t n, const vct_cone_tracing_desc& d,
                          SampleOrder* out, cudaStream_t st) {
    out->order = nullptr;
    out->block = nullptr;
    if (n <= 1 || n >= (1LL << 31)) return VCT_OK;
    size_t temp = 0;
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, temp, (unsigned long long*)nullptr,
                                                 (unsigned long long*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                 (int)n, 0, 36, st));
    const size_t arr4 = (4 * (size_t)n + 255) & ~(size_t)255, arr8 = (8 * (size_t)n + 255) & ~(size_t)255;
    char* b = nullptr;
    VCT_CUDA_TRY(cudaMallocAsync((void**)&b, 2 * arr8 + 2 * arr4 + temp, st));
    unsigned long long *keys = (unsigned long long*)b, *keys_out = (unsigned long long*)(b + arr8);
    uint32_t *vals = (uint32_t*)(b + 2 * arr8), *order = (uint32_t*)(b + 2 * arr8 + arr4);
    int64_t g = (n + 255) / 256;
    k_sample_keys<<<(int)(g > 152 * 32 ? 152 * 32 : g), 256, 0, st>>>(samples, n, d.volume_center[0],
                                                                        d.volume_center[1], d.volume_center[2],
                                                                        0.5f / d.voxel_size, keys, vals);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(b + 2 * arr8 + 2 * arr4, temp, keys, keys_out, vals, order, (int)n, 0, 36,
                                            st);
    if (e != cudaSuccess) {
        cudaFreeAsync(b, st);
        return cuda_fail(e, "sample_coherent_order");
    }
    out->order = order;
    out->block = b;
    return VCT_OK;
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

// One thread per sample, the samples walked in the coherent order (normal class, then Morton).
template <class Atlas>
static int launch_exact(const TraceParams& P, const Atlas& T, const vct_surface_sample* samples, int64_t n,
                        float* dout, float* sout, unsigned long long* cone_steps, cudaStream_t st) {
    SampleOrder so;
    int rc = sample_coherent_order(samples, n, P.d, &so, st);
    if (rc != VCT_OK) return rc;
    int64_t blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_cone_trace_exact<<<(int)blocks, 128, 0, st>>>(P, T, samples, n, so.order, dout, sout, cone_steps);
    cudaError_t e = cudaGetLastError();
    if (so.block) cudaFreeAsync(so.block, st);
    if (e != cudaSuccess) return cuda_fail(e, "k_cone_trace_exact");
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
    return launch_exact(P, T, samples, n, dout, sout, cone_steps, as_stream(stream));
}

extern "C" int vct_cone_trace_f32(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const float* atlas4,
                                  int32_t R, const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                                  const vct_directional_light_shadow_desc* light_shadow,
                                  const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                  unsigned long long* cone_steps, void* stream) {
    VCT_CHECK_ARG(atlas4 && valid_resolution(R), "vct_cone_trace_f32: bad atlas / resolution");
    VCT_CHECK_ARG(((uintptr_t)atlas4 & 15) == 0, "vct_cone_trace_f32: the atlas must be 16-byte aligned");
    VCT_CHECK_ARG(n >= 0, "vct_cone_trace_f32: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && dout && sout, "vct_cone_trace_f32: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_cone_trace_f32: sample/output buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    F4Atlas T{reinterpret_cast<const float4*>(atlas4), AtlasDims(R)};
    return launch_exact(P, T, samples, n, dout, sout, cone_steps, as_stream(stream));
}
