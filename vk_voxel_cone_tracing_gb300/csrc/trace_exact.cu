// trace_exact.cu -- the plain FP32 drop-in of voxelConeTracing.frag.
//
// The radiance clipmap is read from the reference's linear RGBA8 atlas (or a
// float RGBA atlas: the differentiable form) with a software trilinear
// filter (FP32 weights, REPEAT addressing) -- the same arithmetic, in the
// same order, as the FP32 restatement of the shader.  Compiled with
// -fmad=false so no multiply-add is fused.  The work is laid out like the
// texture form's: samples in a coherent order (normal class, then Morton),
// the diffuse cones of 32 samples dealt to the lanes of a warp
// (trace_deal.cuh), each cone marched by trace_cone; the specular cones one
// per lane over a list grouped by aperture (so a warp's cones march nearly
// the same number of steps).  The specular cone is traced wherever the
// shader traces it (every rendering mode), the diffuse cones likewise.
#include <cstring>
#include <type_traits>

#include <cub/cub.cuh>

#include "trace_deal.cuh"
#include "trace_exact.cuh"

namespace vct {

constexpr int kExactWarps = 4;  // warps per block of the diffuse kernel

// Tickets (work to warps as they free up) for the texture and float reads;
// the linear RGBA8 atlas's loads run faster with the static deal.
template <class Atlas>
constexpr bool kExactTickets = !std::is_same<Atlas, ExactAtlas>::value;

template <class Atlas>
struct ExactDiffuseMarch {
    Atlas T;
    const vct_cone_tracing_desc* d;
    float aperture, step_factor;
    __device__ __forceinline__ float4 operator()(float3 start, float3 dir, float start_level,
                                                 unsigned long long& steps) const {
        return trace_cone(T, *d, start, dir, aperture, kMaxTraceDistance, start_level, step_factor, steps);
    }
};

template <class Atlas>
__global__ void __launch_bounds__(32 * kExactWarps) k_exact_diffuse(TraceParams P, Atlas T,
                                                                    const vct_surface_sample* __restrict__ samples,
                                                                    int64_t n, const uint32_t* __restrict__ order,
                                                                    float* __restrict__ dout, float* __restrict__ sout,
                                                                    unsigned long long* __restrict__ step_counter,
                                                                    unsigned int* __restrict__ ticket) {
    const bool c32 = P.d.enable_32_cones != 0;
    DealArgs D{&P, samples, n, order, 0u, (uint32_t)n, dout, sout, c32 ? 32 : 16, true, true};
    const ExactDiffuseMarch<Atlas> march{T, &P.d, P.diffuse_aperture,
                                         fmaxf(kMinTraceStepFactor, P.d.min_trace_step_factor)};
    unsigned long long steps = 0;
    deal_diffuse<kExactWarps, kExactTickets<Atlas>>(D, march, steps, ticket);
    add_steps(step_counter, steps);
}

// One lane per specular cone of the list.  The list is grouped by aperture
// (then kept in the coherent order), and a cone's step count depends only on
// its aperture (and the occlusion stop), so a warp's cones march in step.
template <class Atlas>
__global__ void __launch_bounds__(128) k_exact_specular(TraceParams P, Atlas T,
                                                        const vct_surface_sample* __restrict__ samples,
                                                        const uint32_t* __restrict__ list,
                                                        const unsigned int* __restrict__ spec_count,
                                                        float* __restrict__ sout,
                                                        unsigned long long* __restrict__ step_counter,
                                                        unsigned int* __restrict__ ticket) {
    const vct_cone_tracing_desc& d = P.d;
    const int64_t m = *spec_count;
    const int lane = threadIdx.x & 31;
    unsigned long long steps = 0;
    // with tickets, 32 consecutive cones of the list to the warp at a time as warps free up; without, a
    // static grid stride
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t c_static = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - stride;
    for (;;) {
        int64_t c;
        if constexpr (kExactTickets<Atlas>) {
            uint32_t c0 = 0;
            if (lane == 0) c0 = atomicAdd(ticket, 32u);
            c0 = __shfl_sync(0xffffffffu, c0, 0);
            if ((int64_t)c0 >= m) break;
            c = (int64_t)c0 + lane;
            if (c >= m) continue;
        } else {
            c_static += stride;
            if (c_static >= m) break;
            c = c_static;
        }
        const uint32_t idx = __ldg(list + c);
        const GSample g = load_sample(samples + idx, P.eye);
        const float min_level = calc_min_level(d, g.wp);
        const float vs = d.voxel_size * exp2f(min_level);
        const float3 start = g.wp + g.normal * (vs * d.trace_start_offset);
        const float3 sdir = reflect3(f3(-g.view.x, -g.view.y, -g.view.z), g.normal);
        const float4 r = trace_cone(T, d, start, sdir, fmaxf(g.roughness, kMinSpecularAperture), kMaxTraceDistance,
                                    min_level, d.voxel_size, steps);
        const float isi = d.indirect_specular_intensity;
        const uint32_t mode = d.rendering_mode;
        float4 S = make_float4(0.f, 0.f, 0.f, 1.f);  // write_outputs' specular output
        if (mode == 6 || mode >= 8)
            S = make_float4(0.f + r.x * g.specular_color.x * isi, 0.f + r.y * g.specular_color.y * isi,
                            0.f + r.z * g.specular_color.z * isi, 1.f);
        reinterpret_cast<float4*>(sout)[idx] = S;
    }
    add_steps(step_counter, steps);
}

// The specular list's groups: kSpecApertureBuckets log-spaced buckets of the
// aperture max(roughness, 0.05) over [0.05, 1] (a cone's step count is about
// proportional to 1 / aperture, so a bucket's cones march within ~10 % of the
// same number of steps).  Measured against 256 linear buckets, against 128
// log buckets and against also splitting by the cone's direction: within a
// few per cent, this one the fastest on random normals.
constexpr int kSpecApertureBuckets = 32;
constexpr int kSpecKeyBits = 6;  // keys < 32: specular; 32: not specular

// Specular classification of the ordered samples (the shader traces a
// specular cone where depth != 1 and the sample has a specular colour and
// metalness): specular samples get their aperture bucket as the key, the
// others kSpecApertureBuckets; their count.  A stable radix sort of the keys
// then lists the specular samples grouped, each group in the coherent order.
__global__ void k_exact_spec_keys(const vct_surface_sample* __restrict__ samples, int64_t n,
                                  const uint32_t* __restrict__ order, uint32_t* __restrict__ spec_key,
                                  unsigned int* __restrict__ spec_count) {
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = base + lane;
        bool spec = false;
        if (pos < n) {
            const float4* q = reinterpret_cast<const float4*>(samples + __ldg(order + pos));
            const float4 a = __ldg(q + 0), c = __ldg(q + 2), d = __ldg(q + 3);
            spec = a.w != 1.0f && (d.x > 1e-6f || d.y > 1e-6f || d.z > 1e-6f) && d.w > 1e-6f;
            uint32_t key = (uint32_t)kSpecApertureBuckets;
            if (spec) {
                const float ap = fminf(fmaxf(c.w, kMinSpecularAperture), 1.0f);  // NaN -> the minimum
                const float lb = __log2f(ap * (1.0f / kMinSpecularAperture)) * (1.0f / 4.321928f);  // log_20
                key = (uint32_t)min(max((int)(lb * (float)kSpecApertureBuckets), 0), kSpecApertureBuckets - 1);
            }
            spec_key[pos] = key;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, spec);
        if (lane == 0 && bal) atomicAdd(spec_count, (unsigned)__popc(bal));
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
    P.diffuse_aperture = desc->enable_32_cones ? kAperture32 : kAperture16;
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

int exact_plan(const vct_surface_sample* samples, int64_t n, const vct_cone_tracing_desc& d, ExactPlan* plan,
               cudaStream_t st) {
    plan->order = nullptr;
    plan->spec_list = nullptr;
    plan->spec_count = nullptr;
    plan->block = nullptr;
    plan->order_block = nullptr;
    SampleOrder so;
    int rc = sample_coherent_order(samples, n, d, &so, st);
    if (rc != VCT_OK) return rc;
    size_t temp = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, temp, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, kSpecKeyBits,
                                                    st);
    const size_t arr4 = (4 * (size_t)n + 255) & ~(size_t)255;
    char* b = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b, 4 * arr4 + 256 + temp, st);
    if (e != cudaSuccess) {
        if (so.block) cudaFreeAsync(so.block, st);
        return cuda_fail(e, "cone trace scratch");
    }
    uint32_t* identity = (uint32_t*)b;  // the order of a single sample (the coherent order needs n >= 2)
    uint32_t* spec_key = (uint32_t*)(b + arr4);
    uint32_t* spec_key_out = (uint32_t*)(b + 2 * arr4);
    plan->spec_list = (uint32_t*)(b + 3 * arr4);
    plan->spec_count = (unsigned int*)(b + 4 * arr4);
    void* sort_temp = b + 4 * arr4 + 256;
    plan->block = b;
    plan->order_block = so.block;
    plan->order = so.order;
    if (!plan->order) {
        const uint32_t zero = 0;
        e = cudaMemcpyAsync(identity, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
        plan->order = identity;
    }
    // the specular count and the tickets of the specular and diffuse kernels
    if (e == cudaSuccess) e = cudaMemsetAsync(plan->spec_count, 0, 3 * sizeof(unsigned int), st);
    const int64_t gb = (n + 255) / 256;
    if (e == cudaSuccess) {
        k_exact_spec_keys<<<(int)(gb > 152 * 16 ? 152 * 16 : gb), 256, 0, st>>>(samples, n, plan->order, spec_key,
                                                                               plan->spec_count);
        e = cudaGetLastError();
    }
    // stable radix sort of the group keys: the specular samples first, by group, the order kept within
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(sort_temp, temp, spec_key, spec_key_out, plan->order, plan->spec_list,
                                            (int)n, 0, kSpecKeyBits, st);
    if (e != cudaSuccess) {
        exact_plan_free(plan, st);
        return cuda_fail(e, "exact trace plan");
    }
    return VCT_OK;
}

void exact_plan_free(ExactPlan* plan, cudaStream_t st) {
    if (plan->block) cudaFreeAsync(plan->block, st);
    if (plan->order_block) cudaFreeAsync(plan->order_block, st);
    plan->block = plan->order_block = nullptr;
}

int apply_trace_options(TraceParams& P, const vct_trace_options* o) {
    if (!o) return VCT_OK;
    VCT_CHECK_ARG(o->reserved[0] == 0.0f && o->reserved[1] == 0.0f && o->reserved[2] == 0.0f,
                  "cone trace options: reserved fields must be zero");
    VCT_CHECK_ARG(o->diffuse_aperture == 0.0f || (o->diffuse_aperture > 0.0f && o->diffuse_aperture < 3.14159265f),
                  "cone trace options: the diffuse aperture must be 0 or lie in (0, pi)");
    if (o->diffuse_aperture != 0.0f) P.diffuse_aperture = o->diffuse_aperture;
    return VCT_OK;
}

// The plan (coherent order, aperture-grouped specular list), then the
// diffuse and specular kernels.  Scratch is stream-ordered (cudaMallocAsync,
// freed after the kernels).  Counts of 2^30 samples or more run in chunks
// (the orders are 32-bit).
template <class Atlas>
static int launch_exact(const TraceParams& P, const Atlas& T, const vct_surface_sample* samples, int64_t n,
                        float* dout, float* sout, unsigned long long* cone_steps, cudaStream_t st) {
    constexpr int64_t kChunk = 1LL << 30;
    for (int64_t off = 0; off < n; off += kChunk) {
        const int64_t m = n - off < kChunk ? n - off : kChunk;
        const vct_surface_sample* smp = samples + off;
        ExactPlan plan;
        int rc = exact_plan(smp, m, P.d, &plan, st);
        if (rc != VCT_OK) return rc;
        unsigned int* spec_ticket = plan.spec_count + 1;
        unsigned int* diff_ticket = plan.spec_count + 2;
        const int64_t gdw = (m + 32 * kExactWarps - 1) / (32 * kExactWarps);
        k_exact_diffuse<<<(int)(gdw > 152 * 16 ? 152 * 16 : gdw), 32 * kExactWarps, 0, st>>>(
            P, T, smp, m, plan.order, dout + 4 * off, sout + 4 * off, cone_steps, diff_ticket);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) {
            const int64_t gl = (m + 127) / 128;
            k_exact_specular<<<(int)(gl > 152 * 16 ? 152 * 16 : gl), 128, 0, st>>>(
                P, T, smp, plan.spec_list, plan.spec_count, sout + 4 * off, cone_steps, spec_ticket);
            e = cudaGetLastError();
        }
        exact_plan_free(&plan, st);
        if (e != cudaSuccess) return cuda_fail(e, "exact cone trace");
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
    return vct_cone_trace_opt(desc, cam, radiance_atlas, R, shadow, light, light_shadow, samples, n, dout, sout,
                              cone_steps, nullptr, stream);
}

extern "C" int vct_cone_trace_opt(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                  const uint32_t* radiance_atlas, int32_t R, const vct_shadow_map* shadow,
                                  const vct_directional_light_desc* light,
                                  const vct_directional_light_shadow_desc* light_shadow,
                                  const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                  unsigned long long* cone_steps, const vct_trace_options* options, void* stream) {
    VCT_CHECK_ARG(radiance_atlas && valid_resolution(R), "vct_cone_trace: bad radiance atlas / resolution");
    VCT_CHECK_ARG(n >= 0, "vct_cone_trace: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && dout && sout, "vct_cone_trace: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_cone_trace: sample/output buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    if ((rc = apply_trace_options(P, options)) != VCT_OK) return rc;
    ExactAtlas T{radiance_atlas, AtlasDims(R)};
    return launch_exact(P, T, samples, n, dout, sout, cone_steps, as_stream(stream));
}

extern "C" int vct_cone_trace_tex(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                  vct_texture_s* radiance, const vct_shadow_map* shadow,
                                  const vct_directional_light_desc* light,
                                  const vct_directional_light_shadow_desc* light_shadow,
                                  const vct_surface_sample* samples, int64_t n, float* dout, float* sout,
                                  unsigned long long* cone_steps, const vct_trace_options* options, void* stream) {
    vct::NvtxRange nvtx_range("vct_cone_trace_tex");
    VCT_CHECK_ARG(radiance && texture_format(radiance) == VCT_TEX_RGBA8,
                  "vct_cone_trace_tex: the radiance texture must be RGBA8");
    VCT_CHECK_ARG(n >= 0, "vct_cone_trace_tex: negative sample count");
    if (n == 0) return VCT_OK;
    VCT_CHECK_ARG(samples && dout && sout, "vct_cone_trace_tex: null sample or output buffer");
    VCT_CHECK_ARG(((uintptr_t)samples & 15) == 0 && ((uintptr_t)dout & 15) == 0 && ((uintptr_t)sout & 15) == 0,
                  "vct_cone_trace_tex: sample/output buffers must be 16-byte aligned");
    TraceParams P;
    int rc = fill_trace_params(P, desc, cam, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    if ((rc = apply_trace_options(P, options)) != VCT_OK) return rc;
    VCT_CHECK_ARG((float)texture_resolution(radiance) == desc->volume_dimension,
                  "vct_cone_trace_tex: volume dimension differs from the texture's clipmap resolution");
    TexelAtlas T{texture_texel_object(radiance), AtlasDims(texture_resolution(radiance))};
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
