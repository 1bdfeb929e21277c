// common.cuh -- shared device/host helpers of the GB300 voxel cone tracing core.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>

#include "../../include/vct_capi.h"

// Device scratch arena of the raster / SVO passes (vct_workspace), a
// second buffer that outlives a pass within one frame (the frame's
// touched-texel bitmap), and a side stream with two events and a workspace
// of its own, on which a frame runs the passes that are independent of the
// main stream's work beside them (created on first use, on the device
// current then).
struct vct_workspace_s {
    void* ptr = nullptr;
    size_t bytes = 0;
    void* aux = nullptr;
    size_t aux_bytes = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    int side_device = -1;
    vct_workspace_s* side_ws = nullptr;  // the scratch of the passes run on the side stream
};

namespace vct {

// Grow `ws` to at least `bytes` (synchronises the device before freeing).
int workspace_reserve(vct_workspace_s* ws, size_t bytes);

// Radiance texture accessors (textures.cu).
cudaTextureObject_t texture_object(const vct_texture_s* t);
cudaSurfaceObject_t texture_surface(const vct_texture_s* t);
// RGBA8 only (0 otherwise): point filter, unnormalised coordinates, texels read as normalised floats.
cudaTextureObject_t texture_texel_object(const vct_texture_s* t);
int texture_resolution(const vct_texture_s* t);
int texture_format(const vct_texture_s* t);

// Copy-alpha of one level, and copy-alpha + radiance mip of one level >= 1,
// optionally mirroring every texel they write into a texture array's surface
// (clipmap_passes.cu).
// `touched` (may be null): a bitmap over the atlas's texel indices; a texel
// whose bit is clear is read as zero rgb (the frame's radiance clear folded
// into these passes).
// `opa_r8`: the opacity atlas is the one-byte-per-texel form (alpha only).
int copy_alpha_pass(uint32_t* dst, const void* src, const vct_copy_alpha_desc* d, cudaSurfaceObject_t mirror,
                    const uint32_t* touched, cudaStream_t st, bool src_r8);
int copy_alpha_downsample_pass(uint32_t* radiance, const void* opacity, const vct_downsample_desc* d,
                               cudaSurfaceObject_t mirror, const uint32_t* touched, cudaStream_t st, bool opa_r8);
// The one-byte opacity form's mips 1..5 and border wrap (clipmap_passes.cu).
int opacity_r8_mips(uint8_t* atlas, const vct_clipmap_region regions[6], int R, cudaStream_t st);
int wrap_border_r8(uint8_t* atlas, int R, cudaStream_t st);

// The frame's rasterised passes with the deterministic injection, up to the
// fold (raster.cu): opacity clear + voxelisation + mips + border, shadow
// depth, clear of the due radiance levels and the injection.
// The radiance levels due are not cleared: the fold starts their texels from
// zero and marks each texel it writes in *touched (a bitmap over the atlas's
// texel indices, in the workspace's second buffer), and the copy-alpha / mip
// passes read unmarked texels as zero rgb -- the cleared result.
// With nslabs >= 0 the opacity atlas is updated toroidally: only the listed
// slabs are cleared and revoxelised (levels with a whole-region slab in
// full), and only the revoxelised levels' opacity mips are rebuilt.
int frame_raster_passes(const vct_scene* scene, const vct_frame_desc* f, const vct_clipmap_region regions[6],
                        uint32_t due, const vct_clipmap_region* slabs, const int32_t* slab_levels, int nslabs,
                        uint32_t* opacity, uint32_t* radiance, float* shadow_depth, vct_workspace_s* ws,
                        const uint32_t** touched, cudaStream_t st);

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define VCT_CHECK_ARG(cond, msg)                              \
    do {                                                       \
        if (!(cond)) return ::vct::fail(VCT_E_BAD_ARG, (msg)); \
    } while (0)
#define VCT_CUDA_TRY(expr)                                   \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return ::vct::cuda_fail(e_, #expr); \
    } while (0)
#define VCT_LAUNCH_CHECK() VCT_CUDA_TRY(cudaGetLastError())

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// An NVTX range over a pass's host-side submission (visible to profilers that
// attach an NVTX tool; a few nanoseconds otherwise).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ------------------------------------------------------------- geometry
// The reference atlas: width (R+2)*6, height (R+2)*6, depth R+2.
struct AtlasDims {
    int R, rb, W, H, D;
    __host__ __device__ explicit AtlasDims(int res) : R(res), rb(res + 2), W((res + 2) * 6), H((res + 2) * 6), D(res + 2) {}
    __host__ __device__ int64_t index(int x, int y, int z) const { return ((int64_t)z * H + y) * W + x; }
    __host__ __device__ int64_t texels() const { return (int64_t)W * H * D; }
};

inline bool valid_resolution(int R) { return R >= 8 && R <= 1024 && (R & (R - 1)) == 0; }

// ------------------------------------------------------------- unorm8
// Byte b -> the IEEE quotient b / 255 (the unorm8 decode), computed as one
// multiply by RN(1/255) followed by one Markstein correction step
// (P. Markstein, "IA-64 and Elementary Functions", 2000): q0 = b * r,
// e = b - 255 * q0 (exact through the fused multiply-add), q = q0 + e * r.
// Equal to the correctly rounded quotient for all 256 bytes (checked
// exhaustively in exact rational arithmetic by the test suite); a plain
// b * RN(1/255) is one ulp off for 126 of them.
__device__ __forceinline__ float unorm8_decode(uint32_t b) {
    const float x = (float)b;
    const float r = __uint_as_float(0x3b808081u);  // RN(1/255)
    const float q0 = __fmul_rn(x, r);
    const float e = __fmaf_rn(-q0, 255.0f, x);
    return __fmaf_rn(e, r, q0);
}
__device__ __forceinline__ float unorm8_load(uint32_t v, int c) { return unorm8_decode((v >> (8 * c)) & 0xffu); }
__device__ __forceinline__ float4 unpack_rgba8(uint32_t v) {
    return make_float4(unorm8_decode(v & 0xffu), unorm8_decode((v >> 8) & 0xffu), unorm8_decode((v >> 16) & 0xffu),
                       unorm8_decode(v >> 24));
}
// Pinned store rule: round-half-up of clamp(x, 0, 1) * 255.
__device__ __forceinline__ uint32_t unorm8_store(float x) {
    float c = fminf(fmaxf(x, 0.0f), 1.0f);
    return (uint32_t)floorf(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
}
__device__ __forceinline__ uint32_t pack_rgba8(float4 c) {
    return unorm8_store(c.x) | (unorm8_store(c.y) << 8) | (unorm8_store(c.z) << 16) | (unorm8_store(c.w) << 24);
}

// GLSL mix(x, y, a) = x * (1 - a) + y * a, without contraction.
__device__ __forceinline__ float mix_rn(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}

}  // namespace vct
