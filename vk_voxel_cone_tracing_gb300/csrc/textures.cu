// textures.cu -- hardware-filtered 3D texture of the radiance clipmap, and the
// FP16-storage atlas kernels (RGBA8 -> RGBA16F conversion, anisotropic
// downsample with FP32 arithmetic and RGBA16F storage).
//
// The fast cone tracer samples the atlas through a CUDA texture object: a 3D
// cudaArray with normalized coordinates, WRAP addressing and linear
// filtering -- the same sampler state as the reference's VoxelSampler
// (VFS/RenderPass/Clipmap/Voxelizer.cpp:279: REPEAT, LINEAR, one mip level).
#include <cuda_fp16.h>

#include "common.cuh"

struct vct_texture_s {
    int R = 0;
    int format = 0;
    cudaArray_t array = nullptr;
    cudaTextureObject_t tex = 0;
    cudaSurfaceObject_t surf = 0;  // the same array for direct texel stores
    cudaTextureObject_t texel = 0; // RGBA8: the same array read texel by texel (point filter,
                                   // unnormalised coordinates, unorm8 decoded to float)
};

namespace vct {

cudaTextureObject_t texture_object(const vct_texture_s* t) { return t->tex; }
cudaSurfaceObject_t texture_surface(const vct_texture_s* t) { return t->surf; }
cudaTextureObject_t texture_texel_object(const vct_texture_s* t) { return t->texel; }
int texture_resolution(const vct_texture_s* t) { return t->R; }
int texture_format(const vct_texture_s* t) { return t->format; }

// Zero every texel of a texture array through its surface (4- or 8-byte texels).
__global__ void k_surface_zero(cudaSurfaceObject_t s, int W, int H, int D, int texel_bytes) {
    const int64_t n = (int64_t)W * H * D;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % W);
        const int64_t r = i / W;
        const int y = (int)(r % H), z = (int)(r / H);
        if (texel_bytes == 4) surf3Dwrite(0u, s, x * 4, y, z);
        else surf3Dwrite(make_uint2(0u, 0u), s, x * 8, y, z);
    }
}

__device__ __forceinline__ uint16_t h_bits(float x) { return __half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ float h_val(uint16_t b) { return __half2float(__ushort_as_half(b)); }

// `mirror` (0 = none): an RGBA16F texture array of the same atlas; every
// texel written is stored into it as well, so it needs no copy afterwards.
// A block converts a 16 x 16 tile of one depth slice, each warp two
// neighbouring rows of 16 texels: a 32-byte sector of the array's
// block-linear layout holds two texels of two neighbouring rows, so every
// sector a warp writes is written whole (row-by-row warps wrote half sectors
// and paid a read-modify-write for each).
__global__ void __launch_bounds__(256) k_rgba8_to_rgba16f(const uint32_t* __restrict__ src, uint2* __restrict__ dst,
                                                          int W, int H, int D, cudaSurfaceObject_t mirror) {
    const int tx = (W + 15) >> 4, ty = (H + 15) >> 4;
    const int64_t tiles = (int64_t)tx * ty * D;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const int z = (int)(t / ((int64_t)tx * ty));
        const int r = (int)(t - (int64_t)z * tx * ty);
        const int x = ((r % tx) << 4) + (lane & 15), y = ((r / tx) << 4) + 2 * warp + (lane >> 4);
        if (x >= W || y >= H) continue;
        const int64_t i = ((int64_t)z * H + y) * W + x;
        float4 c = unpack_rgba8(__ldg(src + i));
        uint2 o;
        o.x = (uint32_t)h_bits(c.x) | ((uint32_t)h_bits(c.y) << 16);
        o.y = (uint32_t)h_bits(c.z) | ((uint32_t)h_bits(c.w) << 16);
        dst[i] = o;
        if (mirror) surf3Dwrite(o, mirror, x * 8, y, z);
    }
}

__device__ __forceinline__ int ds_wrap16(int p, int R) { return (p + R * (abs(p / R) + 1)) & (R - 1); }

}  // namespace vct
#include "mip_pairs.cuh"
namespace vct {

__device__ __forceinline__ float4 load_h4(const uint2* p, int64_t i) {
    uint2 v = p[i];
    return make_float4(h_val(v.x & 0xffff), h_val(v.x >> 16), h_val(v.y & 0xffff), h_val(v.y >> 16));
}
__device__ __forceinline__ uint2 store_h4(uint2* p, int64_t i, float4 c) {
    uint2 o;
    o.x = (uint32_t)h_bits(c.x) | ((uint32_t)h_bits(c.y) << 16);
    o.y = (uint32_t)h_bits(c.z) | ((uint32_t)h_bits(c.w) << 16);
    p[i] = o;
    return o;
}

// Same composite and band blend as the RGBA8 downsample (opacityDownSample.comp /
// radianceDownSample.comp), FP32 arithmetic, RGBA16F storage.
template <int MODE>
__global__ void k_downsample_f16(uint2* __restrict__ atlas, AtlasDims A, int3 pmin, int level, int band,
                                 cudaSurfaceObject_t mirror) {
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int g[3] = {(int)(t % half), (int)((t / half) % half), (int)(t / ((int64_t)half * half))};
        const int pm[3] = {pmin.x, pmin.y, pmin.z};
        int cur[3], wpos[3], ps[3];
        float dist[3];
        bool any_ge = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            cur[a] = (pm[a] >> 1) + g[a];
            wpos[a] = ds_wrap16(cur[a], A.R) + 1;
            ps[a] = ds_wrap16(cur[a] << 1, A.R) + 1;
            float center = (float)(pm[a] >> 1) + (float)(half >> 1);
            dist[a] = fabsf((float)cur[a] + 0.5f - center) - 0.5f;
            any_ge |= dist[a] >= (float)((half >> 1) - band);
        }
        wpos[1] += A.rb * level;
        ps[1] += A.rb * (level - 1);
        float lerp = 0.0f;
        if (any_ge)
            lerp = (fmaxf(dist[0], fmaxf(dist[1], dist[2])) - (float)((half >> 1) - band) + 1.0f) *
                   (1.0f / ((float)band + 1.0f));
        #pragma unroll
        for (int f = 0; f < 6; ++f) {
            float4 v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                v[i] = load_h4(atlas, A.index(ps[0] + (i & 1) + A.rb * f, ps[1] + ((i >> 1) & 1), ps[2] + ((i >> 2) & 1)));
            const int64_t wi = A.index(wpos[0] + A.rb * f, wpos[1], wpos[2]);
            float4 own = load_h4(atlas, wi);
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 a0 = v[ds_pair(f, k, 0)], a1 = v[ds_pair(f, k, 1)];
                const float tt = 1.0f - a0.w;
                if (MODE == 0) {
                    s.w += a0.w + tt * a1.w;
                } else {
                    s.x += a0.x + tt * a1.x;
                    s.y += a0.y + tt * a1.y;
                    s.z += a0.z + tt * a1.z;
                    s.w += a0.w + tt * a1.w;
                }
            }
            if (MODE == 0) {
                float a = s.w * 0.25f * (1.0f - lerp) + own.x * lerp;
                own.w = a;
                own.y = a;
                const uint2 o = store_h4(atlas, wi, own);
                if (mirror) surf3Dwrite(o, mirror, (wpos[0] + A.rb * f) * 8, wpos[1], wpos[2]);
            } else {
                float4 o = make_float4(s.x * 0.25f * (1.0f - lerp) + own.x * lerp, s.y * 0.25f * (1.0f - lerp) + own.y * lerp,
                                       s.z * 0.25f * (1.0f - lerp) + own.z * lerp, s.w * 0.25f * (1.0f - lerp) + own.w * lerp);
                const uint2 b = store_h4(atlas, wi, o);
                if (mirror) surf3Dwrite(b, mirror, (wpos[0] + A.rb * f) * 8, wpos[1], wpos[2]);
            }
        }
    }
}

static int grid_for16(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    return (int)(g > 152 * 64 ? 152 * 64 : (g < 1 ? 1 : g));
}

}  // namespace vct

using namespace vct;

extern "C" int vct_texture_create(int32_t R, int32_t format, vct_texture_s** out) {
    VCT_CHECK_ARG(out, "vct_texture_create: null output handle");
    *out = nullptr;
    VCT_CHECK_ARG(valid_resolution(R), "vct_texture_create: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(format == 0 || format == 1, "vct_texture_create: format must be VCT_TEX_RGBA8 or VCT_TEX_RGBA16F");
    AtlasDims A(R);
    auto* t = new vct_texture_s();
    t->R = R;
    t->format = format;
    cudaChannelFormatDesc ch = format == 0 ? cudaCreateChannelDesc<uchar4>() : cudaCreateChannelDescHalf4();
    cudaError_t e = cudaMalloc3DArray(&t->array, &ch, make_cudaExtent(A.W, A.H, A.D), cudaArraySurfaceLoadStore);
    if (e != cudaSuccess) {
        delete t;
        return cuda_fail(e, "cudaMalloc3DArray (radiance texture)");
    }
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = t->array;
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = format == 0 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
    td.normalizedCoords = 1;
    e = cudaCreateTextureObject(&t->tex, &rd, &td, nullptr);
    if (e == cudaSuccess && format == 0) {
        cudaTextureDesc tp = td;
        tp.filterMode = cudaFilterModePoint;
        tp.normalizedCoords = 0;
        e = cudaCreateTextureObject(&t->texel, &rd, &tp, nullptr);
    }
    if (e == cudaSuccess) e = cudaCreateSurfaceObject(&t->surf, &rd);
    if (e == cudaSuccess) {  // a defined starting content: all zero, like a fresh atlas
        k_surface_zero<<<grid_for16(A.texels(), 256), 256>>>(t->surf, A.W, A.H, A.D, format == 0 ? 4 : 8);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        if (t->surf) cudaDestroySurfaceObject(t->surf);
        if (t->texel) cudaDestroyTextureObject(t->texel);
        if (t->tex) cudaDestroyTextureObject(t->tex);
        cudaFreeArray(t->array);
        delete t;
        return cuda_fail(e, "vct_texture_create (texture/surface object or zero fill)");
    }
    *out = t;
    return VCT_OK;
}

extern "C" int vct_texture_update(vct_texture_s* t, const void* atlas, void* stream) {
    VCT_CHECK_ARG(t && atlas, "vct_texture_update: null argument");
    AtlasDims A(t->R);
    const size_t texel = t->format == 0 ? 4 : 8;
    cudaMemcpy3DParms p = {};
    p.srcPtr = make_cudaPitchedPtr(const_cast<void*>(atlas), A.W * texel, A.W, A.H);
    p.dstArray = t->array;
    p.extent = make_cudaExtent(A.W, A.H, A.D);
    p.kind = cudaMemcpyDeviceToDevice;
    VCT_CUDA_TRY(cudaMemcpy3DAsync(&p, as_stream(stream)));
    return VCT_OK;
}

extern "C" int vct_texture_read(const vct_texture_s* t, void* atlas, void* stream) {
    VCT_CHECK_ARG(t && atlas, "vct_texture_read: null argument");
    AtlasDims A(t->R);
    const size_t texel = t->format == 0 ? 4 : 8;
    cudaMemcpy3DParms p = {};
    p.srcArray = t->array;
    p.dstPtr = make_cudaPitchedPtr(atlas, A.W * texel, A.W, A.H);
    p.extent = make_cudaExtent(A.W, A.H, A.D);
    p.kind = cudaMemcpyDeviceToDevice;
    VCT_CUDA_TRY(cudaMemcpy3DAsync(&p, as_stream(stream)));
    return VCT_OK;
}

extern "C" int vct_texture_destroy(vct_texture_s* t) {
    if (!t) return VCT_OK;
    if (t->surf) cudaDestroySurfaceObject(t->surf);
    if (t->texel) cudaDestroyTextureObject(t->texel);
    cudaError_t e1 = cudaDestroyTextureObject(t->tex);
    cudaError_t e2 = cudaFreeArray(t->array);
    delete t;
    if (e1 != cudaSuccess) return cuda_fail(e1, "cudaDestroyTextureObject");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeArray");
    return VCT_OK;
}

static int fp16_mirror(const vct_texture_s* mirror, int R, const char* fn, cudaSurfaceObject_t* out) {
    *out = 0;
    if (!mirror) return VCT_OK;
    if (mirror->format != VCT_TEX_RGBA16F || mirror->R != R || !mirror->surf)
        return fail(VCT_E_BAD_ARG, std::string(fn) + ": the mirror must be an RGBA16F texture of the same resolution");
    *out = mirror->surf;
    return VCT_OK;
}

extern "C" int vct_atlas_rgba8_to_rgba16f(const uint32_t* src, uint16_t* dst, int32_t R, vct_texture_s* mirror,
                                          void* stream) {
    VCT_CHECK_ARG(src && dst && valid_resolution(R), "vct_atlas_rgba8_to_rgba16f: bad argument");
    VCT_CHECK_ARG(((uintptr_t)dst & 7) == 0, "vct_atlas_rgba8_to_rgba16f: destination must be 8-byte aligned");
    cudaSurfaceObject_t surf;
    int rc = fp16_mirror(mirror, R, "vct_atlas_rgba8_to_rgba16f", &surf);
    if (rc != VCT_OK) return rc;
    AtlasDims A(R);
    const int64_t tiles = (int64_t)((A.W + 15) >> 4) * ((A.H + 15) >> 4) * A.D;
    k_rgba8_to_rgba16f<<<(int)(tiles < 152 * 64 ? tiles : 152 * 64), 256, 0, as_stream(stream)>>>(
        src, reinterpret_cast<uint2*>(dst), A.W, A.H, A.D, surf);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_downsample_rgba16f(uint16_t* atlas, const vct_downsample_desc* d, int32_t mode,
                                      vct_texture_s* mirror, void* stream) {
    VCT_CHECK_ARG(atlas && d, "vct_downsample_rgba16f: null argument");
    VCT_CHECK_ARG(((uintptr_t)atlas & 7) == 0, "vct_downsample_rgba16f: atlas must be 8-byte aligned");
    VCT_CHECK_ARG(valid_resolution(d->clipmap_resolution), "vct_downsample_rgba16f: bad resolution");
    VCT_CHECK_ARG(d->clip_level >= 1 && d->clip_level < VCT_CLIP_LEVEL_COUNT, "vct_downsample_rgba16f: clip level must be 1..5");
    VCT_CHECK_ARG(mode == 0 || mode == 1, "vct_downsample_rgba16f: bad mode");
    VCT_CHECK_ARG(d->downsample_region_size >= 0 && d->downsample_region_size <= 4096, "vct_downsample_rgba16f: bad band");
    AtlasDims A(d->clipmap_resolution);
    const int half = A.R >> 1;
    const int64_t n = (int64_t)half * half * half;
    int3 pm = make_int3(d->prev_region_min_corner[0], d->prev_region_min_corner[1], d->prev_region_min_corner[2]);
    uint2* a = reinterpret_cast<uint2*>(atlas);
    cudaSurfaceObject_t surf;
    int rc = fp16_mirror(mirror, A.R, "vct_downsample_rgba16f", &surf);
    if (rc != VCT_OK) return rc;
    if (mode == 0)
        k_downsample_f16<0><<<grid_for16(n, 128), 128, 0, as_stream(stream)>>>(a, A, pm, d->clip_level,
                                                                              d->downsample_region_size, surf);
    else
        k_downsample_f16<1><<<grid_for16(n, 128), 128, 0, as_stream(stream)>>>(a, A, pm, d->clip_level,
                                                                              d->downsample_region_size, surf);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}
