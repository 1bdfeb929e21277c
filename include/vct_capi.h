/*
 * vct_capi.h -- C ABI of the GB300-native voxel cone tracing core.
 *
 * Every entry point is a drop-in for one pass (or one helper recorder) of
 * Snowapril/vk_voxel_cone_tracing.  The reference records Vulkan commands into
 * a VkCommandBuffer; here each call enqueues CUDA kernels on the caller's
 * stream (`stream` is a cudaStream_t passed as void*, NULL = legacy default
 * stream).  All buffer pointers are DEVICE pointers unless the parameter name
 * ends in `_host`.  Nothing is allocated behind the caller's back except where
 * a function says so: texture objects (`vct_texture_*`), and stream-ordered
 * scratch (cudaMallocAsync on the call's stream, freed on it with
 * cudaFreeAsync before the call returns) in the per-sample traces
 * (vct_cone_trace, vct_cone_trace_f32, vct_cone_trace_backward,
 * vct_svo_cone_trace: the samples' processing order) and vct_sq_error.
 * vct_gather_probe allocates and frees a small device buffer and two events,
 * vct_cone_trace_fast_autotune two events.  vct_cone_trace_fast (and the
 * calls built on it) creates, on its first call in a thread on a device, one
 * non-blocking stream and two events for that thread, kept until the thread
 * ends: the specular cones run on it beside the diffuse kernel, joined back
 * to the caller's stream before the call returns.  A raster workspace
 * (vct_workspace) likewise creates a side stream, two events and a second
 * workspace on first use by vct_clipmap_frame.
 * vct_cone_trace_fast_noalloc never calls cudaMalloc: its scratch is a static
 * device array that the runtime commits when the array's module loads (see
 * that function).
 *
 * Parameter structs keep the reference's byte layouts (std140 / push-constant
 * layouts of the GLSL blocks); the static asserts at the end of this header
 * pin their sizes.  Images keep the reference's 3D atlas layout:
 *   width  = (R + 2) * 6 faces, height = (R + 2) * 6 clip levels, depth = R + 2,
 *   texel (x, y, z) at linear index (z * height + y) * width + x,
 *   RGBA8 texels as uint32 little-endian (R in the low byte), exactly the
 *   R32_UINT alias the reference uses for its atomic averages
 *   (VFS/RenderPass/Clipmap/Voxelizer.cpp:249-287).
 *
 * Status codes: every function returns VCT_OK or a negative VCT_E_* code;
 * vct_last_error() returns a message for the calling thread's last failure.
 */
#ifndef VCT_CAPI_H
#define VCT_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define VCT_OK 0
#define VCT_E_BAD_ARG -1      /* null pointer, size out of range, bad enum */
#define VCT_E_CUDA -2         /* a CUDA runtime call failed (message kept) */
#define VCT_E_OVERFLOW -3     /* fragment list / node pool capacity exceeded */
#define VCT_E_TIMEOUT -4      /* a bounded device-side wait gave up */
#define VCT_E_UNSUPPORTED -5  /* configuration this build does not handle */

/* Engine constants, VFS/Util/EngineConfig.h:19-33. */
#define VCT_FACE_COUNT 6
#define VCT_CLIP_LEVEL_COUNT 6
#define VCT_VOXEL_BORDER 2       /* DEFAULT_VOXEL_BORDER: one texel per side */
#define VCT_BORDER_WIDTH 1       /* BORDER_WIDTH specialisation constant     */
#define VCT_DOWNSAMPLE_REGION_SIZE 10
#define VCT_VOXEL_EXTENT_L0 16
#define VCT_MIN_OCTREE_NODE_NUM 1000000u
#define VCT_MAX_OCTREE_NODE_NUM 500000000u

/* ------------------------------------------------------- reference structs */

/* ClipmapRegion, VFS/RenderPass/Clipmap/ClipmapRegion.h:10-19. */
typedef struct vct_clipmap_region {
    int32_t min_corner[3];
    uint32_t extent[3];
    float voxel_size;
} vct_clipmap_region;

/* Voxelizer::VoxelizationDesc, VFS/RenderPass/Clipmap/Voxelizer.h:69-78 (64 B: four vec3 + scalar pairs). */
typedef struct vct_voxelization_desc {
    float region_min_corner[3];
    uint32_t clip_level;
    float region_max_corner[3];
    float clip_max_extent;
    float prev_region_min_corner[3];
    float voxel_size;
    float prev_region_max_corner[3];
    int32_t clipmap_resolution;
} vct_voxelization_desc;

/* DownSampler::DownSampleDesc, VFS/RenderPass/Clipmap/DownSampler.h:49-55 (24 B). */
typedef struct vct_downsample_desc {
    int32_t prev_region_min_corner[3];
    int32_t clip_level;
    int32_t clipmap_resolution;
    int32_t downsample_region_size;
} vct_downsample_desc;

/* ClipmapCleaner::ImageCleaningDesc, VFS/RenderPass/Clipmap/ClipmapCleaner.h:40-47 (36 B). */
typedef struct vct_image_cleaning_desc {
    int32_t region_min_corner[3];
    int32_t clip_level;
    uint32_t clip_max_extent[3];
    int32_t clipmap_resolution;
    uint32_t face_count;
} vct_image_cleaning_desc;

/* CopyAlpha::CopyAlphaDesc, VFS/RenderPass/Clipmap/CopyAlpha.h:30-35 (12 B). */
typedef struct vct_copy_alpha_desc {
    int32_t clip_level;
    int32_t clipmap_resolution;
    int32_t face_count;
} vct_copy_alpha_desc;

/* BorderWrapper::BorderWrappingDesc, VFS/RenderPass/Clipmap/BorderWrapper.h:39-44 (16 B). */
typedef struct vct_border_wrapping_desc {
    uint32_t clipmap_resolution;
    uint32_t clip_border_width;
    uint32_t face_count;
    uint32_t clip_region_count;
} vct_border_wrapping_desc;

/* VoxelConeTracingPass::VoxelConeTracingDesc,
 * VFS/RenderPass/Clipmap/VoxelConeTracingPass.h:46-59 (52 B); the push
 * constant block of VFS/Shaders/voxelConeTracing.frag:56-69. */
typedef struct vct_cone_tracing_desc {
    float volume_center[3];
    uint32_t rendering_mode;
    float voxel_size;
    float volume_dimension;
    float trace_start_offset;
    float indirect_diffuse_intensity;
    float ambient_occlusion_factor;
    float min_trace_step_factor;
    float indirect_specular_intensity;
    float occlusion_decay;
    int32_t enable_32_cones;
} vct_cone_tracing_desc;

/* Rendering modes, VFS/Shaders/voxelConeTracing.frag:47-55. */
#define VCT_MODE_DIFFUSE_ONLY 0
#define VCT_MODE_SPECULAR_ONLY 1
#define VCT_MODE_NORMAL_ONLY 2
#define VCT_MODE_MIN_LEVEL_ONLY 3
#define VCT_MODE_DIRECT_CONTRIBUTION_ONLY 4
#define VCT_MODE_INDIRECT_DIFFUSE_ONLY 5
#define VCT_MODE_INDIRECT_SPECULAR_ONLY 6
#define VCT_MODE_AMBIENT_OCCLUSION_ONLY 7
#define VCT_MODE_GI_OUTPUT 8

/* CamMatrix uniform block, VFS/Shaders/voxelConeTracing.frag:18-24 (144 B).
 * Matrices are column-major like glm / GLSL. */
typedef struct vct_cam_matrix {
    float view_proj[16];
    float view_proj_inv[16];
    float eye_pos[3];
    int32_t padding;
} vct_cam_matrix;

/* DirectionalLightDesc, VFS/Shaders/light.glsl:8-13 (32 B). */
typedef struct vct_directional_light_desc {
    float direction[3];
    float intensity;
    float color[3];
    int32_t padding;
} vct_directional_light_desc;

/* DirectionalLightShadowDesc, VFS/Shaders/light.glsl:15-20 (136 B as the C++
 * side of the reference lays it out: glm::mat4 view, proj; float zNear, zFar). */
typedef struct vct_directional_light_shadow_desc {
    float view[16];
    float proj[16];
    float z_near;
    float z_far;
} vct_directional_light_shadow_desc;

/* GltfShadeMaterial, VFS/Shaders/gltf.glsl:8-26 (80 B). */
typedef struct vct_gltf_shade_material {
    float pbr_base_color_factor[4];
    int32_t pbr_base_color_texture;
    float pbr_metallic_factor;
    float pbr_roughness_factor;
    int32_t pbr_metallic_roughness_texture;
    int32_t emissive_texture;
    int32_t alpha_mode;
    float alpha_cutoff;
    int32_t double_sided;
    float emissive_factor[3];
    int32_t normal_texture;
    float normal_texture_scale;
    int32_t occlusion_texture;
    float occlusion_texture_strength;
    int32_t padding;
} vct_gltf_shade_material;

/* One G-buffer texel set of the cone-tracing pass (80 B).  Replaces the
 * G-buffer images the pass samples (VFS/RenderPass/GBufferPass.cpp:179-194,
 * VFS/Shaders/voxelConeTracing.frag:145-163): the world position that
 * worldPosFromDepth() would reconstruct, the depth test value (1.0 = sky,
 * the fragment is discarded and its outputs are left untouched), and the
 * texel values of the diffuse (RGBA8: albedo, perceptual roughness),
 * normal (RGBA16F: n * 0.5 + 0.5), specular (RGBA8: F0, metallic) and
 * emission (RGBA16F) attachments, already converted to float. */
typedef struct vct_surface_sample {
    float position[3];
    float depth;
    float normal_texel[3];
    float pad0;
    float diffuse_texel[4];
    float specular_texel[4];
    float emission_texel[3];
    float pad1;
} vct_surface_sample;

/* Shadow map binding: a D32_SFLOAT depth image (row-major, width x height)
 * sampled with linear filtering and CLAMP_TO_BORDER opaque black
 * (VFS/RenderPass/Clipmap/VoxelConeTracingPass.cpp:294). */
typedef struct vct_shadow_map {
    const float* depth;
    int32_t width;
    int32_t height;
} vct_shadow_map;

/* ------------------------------------------------------------ helpers */

/* Message of the last failing call on this thread ("" if none). */
const char* vct_last_error(void);

/* Library version string and the device architecture it was built for. */
const char* vct_version(void);

/* Number of texels (uint32 words) of one RGBA8 clipmap atlas of resolution R. */
int64_t vct_atlas_texels(int32_t clipmap_resolution);

/* Per-level clip regions, VoxelizationPass::createVoxelClipmap +
 * calculateChangeDelta (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:335-357,
 * 438-448) fed by Application::updateClipRegionBoundingBox
 * (VFS/Application.cpp:116-128).  Host-side; writes 6 regions. */
int vct_clip_regions(const float camera_pos_host[3], int32_t clipmap_resolution,
                     int32_t voxel_extent_l0, vct_clipmap_region regions_host[6]);

/* VoxelizationPass::fillRevoxelizationRegions + calculateChangeDelta
 * (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:438-494), the toroidal mode
 * the reference leaves switched off (:79-92): moves each persistent region
 * (in/out) by the camera-snapped delta of its own corner and lists the newly
 * covered slabs (at most 3 per level, or the whole region when a delta
 * reaches the extent) with their levels.  Host only. */
int vct_update_clip_regions(vct_clipmap_region regions_inout_host[6], const float camera_pos_host[3], int32_t R,
                            int32_t extent_l0, vct_clipmap_region slabs_out_host[18], int32_t slab_level_out_host[18],
                            int32_t* slab_count_host);

/* ------------------------------------------------------- clipmap passes */

struct vct_texture_s; /* the radiance texture handle (see vct_texture_create) */

/* ClipmapCleaner::cmdClear{Opacity,Radiance}ClipRegion
 * (VFS/RenderPass/Clipmap/ClipmapCleaner.cpp:93-133, clipmapCleaning.comp):
 * zero `face_count` faces of a toroidal region of one level. */
int vct_clear_region(uint32_t* atlas, const vct_image_cleaning_desc* desc, void* stream);

/* CopyAlpha::cmdImageCopyAlpha (VFS/RenderPass/Clipmap/CopyAlpha.cpp:92-146,
 * copyAlphaImage.comp): dst.a := src.a over the R^3 interior of one level. */
int vct_copy_alpha(uint32_t* dst_atlas, const uint32_t* src_atlas,
                   const vct_copy_alpha_desc* desc, void* stream);

/* DownSampler::cmdDownSample{Opacity,Radiance}
 * (VFS/RenderPass/Clipmap/DownSampler.cpp:115-168, opacityDownSample.comp,
 * radianceDownSample.comp): one anisotropic 2x2x2 level, in place. */
#define VCT_DOWNSAMPLE_OPACITY 0
#define VCT_DOWNSAMPLE_RADIANCE 1
int vct_downsample(uint32_t* atlas, const vct_downsample_desc* desc, int32_t mode,
                   void* stream);

/* All levels 1..5 of one atlas in sequence, each from its predecessor, with
 * the same per-level descs the reference uploads; `regions` are the 6 clip
 * regions (host memory). */
int vct_downsample_all(uint32_t* atlas, const vct_clipmap_region regions_host[6],
                       int32_t clipmap_resolution, int32_t mode, void* stream);

/* vct_copy_alpha(radiance, opacity, level l) followed by
 * vct_downsample(radiance, desc, VCT_DOWNSAMPLE_RADIANCE) for the same level
 * l >= 1 (RadianceInjectionPass's CopyAlpha then DownSampler::cmdDownSampleRadiance,
 * RadianceInjectionPass.cpp:134-159), fused into one pass over the level; the
 * result is bit-identical to the two calls in sequence.  `mirror` (may be
 * NULL): an RGBA8 texture of the same resolution that receives every texel
 * the pass writes.  No single-pass counterpart in the reference. */
int vct_copy_alpha_downsample(uint32_t* radiance_atlas, const uint32_t* opacity_atlas,
                              const vct_downsample_desc* desc, struct vct_texture_s* mirror, void* stream);

/* BorderWrapper::cmdWrappingOpacityBorder (VFS/RenderPass/Clipmap/BorderWrapper.cpp:123-151,
 * borderWrapping.comp): copy toroidal neighbours into border texels. */
int vct_wrap_border(uint32_t* atlas, const vct_border_wrapping_desc* desc, void* stream);

/* VoxelConeTracingPass::onUpdate (VFS/RenderPass/Clipmap/VoxelConeTracingPass.cpp:75-106)
 * executing voxelConeTracing.frag per G-buffer sample.  `radiance_atlas` is
 * the RGBA8 atlas in the layout above; outputs are RGBA32F (4 floats per
 * sample) like the pass's two attachments.  `cone_steps` (optional, may be
 * NULL) receives += the number of traceCone loop iterations executed.
 * Exact form: FP32 arithmetic, trilinear weights in FP32 (no 8-bit filter
 * weights), reads the linear atlas.  One thread per sample; the samples are
 * walked in a coherent order (normal class, then Morton code of the
 * position; stream-ordered scratch of 24 B per sample), which changes no
 * output. */
int vct_cone_trace(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                   const uint32_t* radiance_atlas, int32_t clipmap_resolution,
                   const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                   const vct_directional_light_shadow_desc* light_shadow,
                   const vct_surface_sample* samples, int64_t sample_count,
                   float* diffuse_out, float* specular_out,
                   unsigned long long* cone_steps, void* stream);

/* ------------------------------------------------ differentiable form */

/* The FP32 trace over a float RGBA atlas (16 B per texel, the reference's
 * layout; the FP16 form widened): the same march and epilogue as
 * vct_cone_trace with the texels read as floats.  The forward of
 * vct_cone_trace_backward. */
int vct_cone_trace_f32(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const float* atlas4, int32_t R,
                       const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                       const vct_directional_light_shadow_desc* light_shadow,
                       const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                       float* specular_out, unsigned long long* cone_steps, void* stream);

/* The adjoint of vct_cone_trace_f32 with respect to the atlas: adds
 * dL/d(texel) to grad_atlas4 (same layout, float RGBA; not cleared here)
 * given dL/d(diffuse_out) and dL/d(specular_out) (sample_count x 4 floats
 * each).  The number of march steps (the occlusion stop) and the clamps are
 * held at their forward values.  Synchronises `stream`; VCT_E_OVERFLOW if a
 * cone marches more than 8192 steps.  Its stream-ordered scratch includes the
 * march records of the first 128 steps of each resident warp's cones
 * (192 KiB per warp: about 480 MB on a 152-SM GPU). */
int vct_cone_trace_backward(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const float* atlas4,
                            int32_t R, const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                            const vct_directional_light_shadow_desc* light_shadow,
                            const vct_surface_sample* samples, int64_t sample_count, const float* grad_diffuse,
                            const float* grad_specular, float* grad_atlas4, void* stream);

/* DownSampler::cmdDownSampleRadiance / Opacity of one level on a float RGBA
 * atlas (no 8-bit store; the RGBA8 pass's arithmetic otherwise), and its
 * adjoint: grad_atlas4 enters holding dL/d(atlas after the level's pass) and
 * leaves holding dL/d(atlas before it); atlas4 holds the forward's final
 * values.  Run the adjoint from level 5 down to 1 to reach level 0. */
int vct_downsample_f32(float* atlas4, const vct_downsample_desc* desc, int32_t mode, void* stream);
int vct_downsample_backward(const float* atlas4, float* grad_atlas4, const vct_downsample_desc* desc, int32_t mode,
                            void* stream);

/* Inverse radiance fitting (build-only; the reference renders forward only).
 * vct_sq_error: the squared error of `n` float4 outputs against targets,
 * grad4 = 2 (out - target) scale and *loss (one device double) = scale *
 * sum (out - target)^2, reduced in a fixed order (deterministic).
 * vct_adam_step: one Adam step (Kingma & Ba, ICLR 2015) over n floats of a
 * float RGBA volume with bias correction at `step` (1-based):
 *   m = b1 m + (1 - b1) g,  v = b2 v + (1 - b2) g^2,
 *   p = clamp(p - lr (m c1) / (sqrt(v c2) + eps)),  c1 = 1/(1 - b1^t), c2 = 1/(1 - b2^t),
 * each operation rounded once (no fused multiply-add), RGB clamped to
 * [rgb_lo, rgb_hi] and A to [alpha_lo, alpha_hi]; zero_grad != 0 clears g.
 * n is a multiple of 4; all buffers 16-byte aligned. */
typedef struct vct_adam_desc {
    float lr, beta1, beta2, eps;
    int32_t step, zero_grad;
    float rgb_lo, rgb_hi, alpha_lo, alpha_hi;
} vct_adam_desc;

int vct_sq_error(const float* out4, const float* target4, int64_t n, float scale, float* grad4, double* loss,
                 void* stream);
int vct_adam_step(float* param, float* grad, float* m, float* v, int64_t n, const vct_adam_desc* desc,
                  void* stream);

/* ------------------------------------------- texture-sampled (fast) form */

/* A hardware-filtered copy of a radiance atlas: a 3D CUDA array with
 * normalized coordinates, WRAP addressing and linear filtering (the
 * reference's VoxelSampler, VFS/RenderPass/Clipmap/Voxelizer.cpp:279).
 * vct_texture_create allocates the array (W x H x D texels of 4 or 8 B) and
 * zeroes it (synchronises the device); vct_texture_update copies a linear
 * atlas of the texture's format into it; vct_texture_read copies it back
 * into a linear atlas.  An RGBA8 texture can also be kept current without
 * copies: the frame (vct_frame_desc.radiance_texture) and
 * vct_copy_alpha_downsample write every texel they produce into it too. */
typedef struct vct_texture_s* vct_texture;
#define VCT_TEX_RGBA8 0
#define VCT_TEX_RGBA16F 1
int vct_texture_create(int32_t clipmap_resolution, int32_t format, vct_texture* out);
int vct_texture_update(vct_texture tex, const void* atlas, void* stream);
int vct_texture_read(const struct vct_texture_s* tex, void* atlas, void* stream);
int vct_texture_destroy(vct_texture tex);

/* FP16-storage form of the radiance clipmap (4 halves per texel, same
 * layout): conversion of an RGBA8 atlas, and the anisotropic downsample of
 * radianceDownSample.comp / opacityDownSample.comp with FP32 arithmetic and
 * RGBA16F storage (no 8-bit quantisation of the mips).  `mirror` (may be
 * NULL) is an RGBA16F texture of the same resolution: every texel written is
 * stored into it too, so a conversion followed by the level mips leaves it
 * equal to the FP16 atlas without a vct_texture_update. */
int vct_atlas_rgba8_to_rgba16f(const uint32_t* src, uint16_t* dst, int32_t clipmap_resolution,
                               struct vct_texture_s* mirror, void* stream);
int vct_downsample_rgba16f(uint16_t* atlas, const vct_downsample_desc* desc, int32_t mode,
                           struct vct_texture_s* mirror, void* stream);

/* Bytes of caller-provided scratch vct_cone_trace_fast needs for
 * `sample_count` samples (-1 if the count is out of range). */
int64_t vct_cone_trace_fast_scratch_bytes(int64_t sample_count);

/* VoxelConeTracingPass::onUpdate (VFS/RenderPass/Clipmap/VoxelConeTracingPass.cpp:75-106),
 * GB300 form: samples visited in Morton order, diffuse cones compacted per
 * warp, specular cones one per warp (on the calling thread's second stream,
 * joined back to `stream`), the clipmap sampled through `radiance` (hardware
 * trilinear filter), FP32 compositing.  Same inputs and outputs as
 * vct_cone_trace; `scratch` is 256-byte aligned device memory of at least
 * vct_cone_trace_fast_scratch_bytes(sample_count) bytes, in use until the
 * work the call enqueues on `stream` completes. */
int vct_cone_trace_fast(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture radiance,
                        const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                        const vct_directional_light_shadow_desc* light_shadow,
                        const vct_surface_sample* samples, int64_t sample_count,
                        float* diffuse_out, float* specular_out, unsigned long long* cone_steps,
                        void* scratch, size_t scratch_bytes, void* stream);

/* Options of the _opt trace entry points; no counterpart in the reference,
 * whose shader fixes its cone tables.  diffuse_aperture: the full cone angle,
 * in radians, of every diffuse cone, in place of the shader's constant
 * (0.872665 for the 16-cone set, 0.628319 for the 32-cone set,
 * voxelConeTracing.frag:78-135); 0 keeps the constant, otherwise it must lie
 * in (0, pi).  The cone directions stay the shader's.  reserved: zero. */
typedef struct vct_trace_options {
    float diffuse_aperture;
    float reserved[3];
} vct_trace_options;

/* vct_cone_trace / vct_cone_trace_fast with options (NULL = none): the same
 * passes, for workloads such as one of 16 fixed 30-degree cones
 * (diffuse_aperture = 0.523599). */
int vct_cone_trace_opt(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const uint32_t* radiance_atlas,
                       int32_t R, const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                       const vct_directional_light_shadow_desc* light_shadow, const vct_surface_sample* samples,
                       int64_t sample_count, float* diffuse_out, float* specular_out, unsigned long long* cone_steps,
                       const vct_trace_options* options, void* stream);
int vct_cone_trace_fast_opt(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture radiance,
                            const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                            const vct_directional_light_shadow_desc* light_shadow,
                            const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                            float* specular_out, unsigned long long* cone_steps, const vct_trace_options* options,
                            void* scratch, size_t scratch_bytes, void* stream);

/* The exact FP32 trace (vct_cone_trace_opt's arithmetic, in its order, and
 * its results bit for bit) reading the RGBA8 atlas's texels through a radiance
 * texture that holds them (vct_texture_update, or the texture a frame keeps
 * current): each texel is one point-sampled texture fetch that the texture
 * unit decodes exactly, instead of address arithmetic, a 4-byte load and a
 * software unorm8 decode.  No counterpart in the reference beyond
 * VoxelConeTracingPass::onUpdate (VoxelConeTracingPass.cpp:75-106). */
int vct_cone_trace_tex(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture radiance,
                       const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                       const vct_directional_light_shadow_desc* light_shadow, const vct_surface_sample* samples,
                       int64_t sample_count, float* diffuse_out, float* specular_out, unsigned long long* cone_steps,
                       const vct_trace_options* options, void* stream);

/* Launch shape of vct_cone_trace_fast: the diffuse and specular kernels'
 * grids in blocks (of 256 threads) per SM.  Every shape gives the same
 * results bit for bit (grid-stride loops; no per-warp state crosses work
 * items), so tuning changes only the time. */
typedef struct vct_trace_tuning {
    int32_t diffuse_blocks_per_sm;  /* default 8 */
    int32_t specular_blocks_per_sm; /* default 64 */
    float trace_ms;                 /* autotune: the chosen shape's median time on the tuning inputs */
    float default_ms;               /* autotune: the default shape's */
    int32_t tuned;                  /* 1 when the shape comes from vct_cone_trace_fast_autotune */
    int32_t reserved;
} vct_trace_tuning;

/* Autotuner of the fast trace (no counterpart in the reference): times the
 * trace of the given inputs (its arguments are vct_cone_trace_fast's; the
 * outputs receive the trace's results) under the default shape and a few
 * others -- specular grids of 16/32/64/128 blocks per SM, then diffuse grids of
 * 4/8/16 with the best of those -- with CUDA events on `stream` (median of
 * three after a warm-up; the call synchronises), and keeps the fastest for
 * this device and the texture's clipmap resolution: later vct_cone_trace_fast
 * calls there launch with it.  A context created with VCT_CONTEXT_AUTOTUNE
 * runs it on its first trace. */
int vct_cone_trace_fast_autotune(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture radiance,
                                 const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                                 const vct_directional_light_shadow_desc* light_shadow,
                                 const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                                 float* specular_out, void* scratch, size_t scratch_bytes, vct_trace_tuning* out,
                                 void* stream);
/* The shape vct_cone_trace_fast uses at resolution R on the current device. */
int vct_trace_tuning_get(int32_t R, vct_trace_tuning* out);
/* Forget every tuned shape (back to the defaults). */
int vct_trace_tuning_reset(void);

/* One trace of a batch: the arguments of vct_cone_trace_fast for one
 * clipmap (its radiance texture, desc, camera eye, lighting) and one sample
 * set with its outputs.  Host struct; the pointers are device pointers. */
typedef struct vct_trace_job {
    vct_cone_tracing_desc desc;
    float eye[3];
    vct_texture radiance;
    vct_shadow_map shadow;      /* depth NULL: visibility 1 */
    vct_directional_light_desc light;
    vct_directional_light_shadow_desc light_shadow;
    const vct_surface_sample* samples;
    int64_t sample_count;
    float* diffuse_out;
    float* specular_out;
    unsigned long long* cone_steps; /* may be NULL; added to */
} vct_trace_job;

/* The batched form of the cone-tracing pass (no counterpart in the
 * reference, which traces one view of one scene per pass): every job of
 * `jobs` in one launch per stage over a device work queue.  The jobs'
 * samples share one coherent order in which each job holds a 32-aligned
 * segment, so each warp-sized item of the diffuse kernel and each specular
 * cone names one job, whose record (texture, constants, lighting, outputs)
 * the kernels read from a job table passed as a kernel parameter (constant
 * memory).  A table holds 64 jobs: longer lists run as consecutive launches
 * of 64 jobs each on `stream`.  Every job's outputs equal, bit for bit,
 * those of vct_cone_trace_fast on that job alone.  Scratch: caller provided,
 * 256-byte aligned, vct_cone_trace_fast_batch_scratch_bytes bytes (negative:
 * a bad count, or more than 2^31 - 1 samples in one group of 64 jobs after
 * each job's count is rounded up to a multiple of 32). */
int64_t vct_cone_trace_fast_batch_scratch_bytes(const vct_trace_job* jobs_host, int32_t job_count);
int vct_cone_trace_fast_batch(const vct_trace_job* jobs_host, int32_t job_count, void* scratch, size_t scratch_bytes,
                              void* stream);

/* Calibration probe for the trace's roofline; no counterpart in the
 * reference.  Times (CUDA events on `stream`, after one warm-up launch) a
 * kernel that marches `cones` synthetic cones of `steps_per_cone` steps, one
 * warp per cone with consecutive steps on consecutive lanes, and performs at
 * every step exactly the texture fetches of one cone sample (three face taps
 * at two adjacent levels) and nothing else.  *samples_per_second receives
 * the measured cone-sample rate: the gather speed of light that
 * vct_cone_trace_fast's rate is compared with.  Allocates and frees a small
 * device buffer and creates and destroys two CUDA events; synchronises
 * `stream`. */
int vct_gather_probe(const vct_cone_tracing_desc* desc, vct_texture radiance, int64_t cones, int32_t steps_per_cone,
                     double* samples_per_second, void* stream);

/* ------------------------------------------------ scene and raster passes */

/* Scene in the reference's vertex-input layout (VFS/SceneManager.cpp:124-204,
 * VFS/GLTFScene.cpp:457-490): separate fp32 position / normal streams, uint32
 * indices, a material index per triangle (the per-draw push constant
 * uMaterialIndex), GltfShadeMaterial records, 1x1 RGBA8 textures indexed by
 * the materials' texture ids, and optional per-instance NodeMatrix {model,
 * itModel} (column-major, 32 floats) selected per triangle.  Device pointers. */
typedef struct vct_scene {
    const float* positions;
    const float* normals;
    const uint32_t* indices;
    int64_t vertex_count;
    int64_t triangle_count;
    const uint32_t* triangle_material;
    const vct_gltf_shade_material* materials;
    int32_t material_count;
    const uint32_t* textures;
    int32_t texture_count;
    const float* node_matrices;
    const uint32_t* triangle_instance;
    int32_t instance_count;
} vct_scene;

/* Device scratch arena for the raster passes (tile counts, prefix sums,
 * injection records, sort buffers).  Created by the caller; the passes grow
 * it with cudaMalloc when it is too small (synchronising the device first). */
typedef struct vct_workspace_s* vct_workspace;
int vct_workspace_create(size_t initial_bytes, vct_workspace* out);
int vct_workspace_destroy(vct_workspace ws);
int64_t vct_workspace_bytes(vct_workspace ws);

/* Host math of Voxelizer::setViewProjection (VFS/RenderPass/Clipmap/Voxelizer.cpp:394-423):
 * the three dominant-axis view-projection matrices of a region (48 floats). */
int vct_voxelization_view_proj(const vct_clipmap_region* region, float out_host[48]);
/* Voxelizer::cmdVoxelize's VoxelizationDesc for one level (Voxelizer.cpp:330-354). */
int vct_voxelization_desc_for(const vct_clipmap_region regions_host[6], int32_t level, int32_t clipmap_resolution,
                              vct_voxelization_desc* out_host);
/* DirectionalLight::setTransform (VFS/DirectionalLight.cpp:21-47): view and
 * +-16 orthographic projection of a directional light. */
int vct_directional_light_shadow(const float origin_host[3], const float direction_host[3], float z_near,
                                 float z_far, vct_directional_light_shadow_desc* out_host);
/* Camera::updateCamera (VFS/Camera.cpp:110-117): view = lookAtLH(position,
 * position + direction, up), proj = perspectiveLH_ZO(radians(fovy), aspect,
 * 0.01, 5000), and the CamMatrix block {proj * view, inverse(view) *
 * inverse(proj), position} (glm's cofactor inverse, FP32). */
int vct_camera_matrix(const float position_host[3], const float direction_host[3], const float up_host[3],
                      float fovy_degrees, float aspect, vct_cam_matrix* out_host);

/* vkCmdClearColorImage of a whole atlas to 0 (VoxelizationPass.cpp:104-125). */
int vct_clear_atlas(uint32_t* atlas, int32_t clipmap_resolution, void* stream);

/* VoxelizationPass::onUpdate + msaaVoxelizer.{vert,geom,frag}
 * (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:190-212): rasterise every
 * triangle into each clip level of `level_mask` (bit l = level l) and store
 * 1.0 into the 6 face copies of each covered voxel.  Does not clear. */
int vct_voxelize_opacity(const vct_scene* scene, const vct_clipmap_region regions_host[6], int32_t clipmap_resolution,
                         uint32_t* opacity_atlas, uint32_t level_mask, vct_workspace ws, void* stream);

/* Conservative voxelisation mode (build-only; the reference rasterises with
 * MSAA): every voxel of each level's region in `level_mask` that a triangle
 * touches -- the triangle / box overlap test of Schwarz & Seidel 2010 in the
 * level's voxel units -- stored like vct_voxelize_opacity (1.0 into the 6
 * face copies at the voxel's toroidal texel).  Does not clear.  Materials
 * whose occlusion texel is below 0.1 are skipped, as msaaVoxelizer.frag
 * discards them. */
int vct_voxelize_opacity_conservative(const vct_scene* scene, const vct_clipmap_region regions_host[6],
                                      int32_t clipmap_resolution, uint32_t* opacity_atlas, uint32_t level_mask,
                                      void* stream);

/* ReflectiveShadowMapPass depth (VFS/RenderPass/ReflectiveShadowMapPass.cpp,
 * reflectiveShadowPass.vert:40-50): clear to 1.0, rasterise with depth test
 * LESS into a width x height D32 map. */
int vct_shadow_depth(const vct_scene* scene, const vct_directional_light_shadow_desc* light_shadow, float* depth,
                     int32_t width, int32_t height, vct_workspace ws, void* stream);

/* RadianceInjectionPass::onUpdate + msaaInjectRadiance.{vert,geom,frag}
 * (VFS/RenderPass/Clipmap/RadianceInjectionPass.cpp:134-159): light each
 * covered sample and fold it into the RGBA8 running average of its faces.
 * VCT_INJECT_DETERMINISTIC folds in the traversal order (triangle, level,
 * tile, pixel, sample) -- bit-exact against the CPU oracle;
 * VCT_INJECT_ATOMIC runs the reference's CAS loop (order-dependent). */
#define VCT_INJECT_DETERMINISTIC 0
#define VCT_INJECT_ATOMIC 1
int vct_inject_radiance(const vct_scene* scene, const vct_clipmap_region regions_host[6], int32_t clipmap_resolution,
                        const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                        const vct_directional_light_shadow_desc* light_shadow, uint32_t* radiance_atlas,
                        uint32_t level_mask, int32_t mode, vct_workspace ws, void* stream);

/* GBufferPass::onUpdate + gBufferPass.{vert,frag} (VFS/RenderPass/GBufferPass.cpp:80-160,
 * 329; depth test LESS against a 1.0 clear, no culling) feeding the
 * cone-tracing pass: rasterise the scene with the camera's view-projection
 * at one centre sample per pixel (triangles clipped to the near plane),
 * resolve each pixel's closest fragment (ties: the earlier triangle) into a
 * vct_surface_sample with the attachments' formats applied, and the world
 * position rebuilt from the depth as worldPosFromDepth does.  Writes
 * width * height records (row-major, row 0 = NDC y -1); pixels no triangle
 * covers get depth 1.  `out` is a device pointer, 16-byte aligned. */
int vct_gbuffer(const vct_scene* scene, const vct_cam_matrix* cam_host, int32_t width, int32_t height,
                vct_surface_sample* out, vct_workspace ws, void* stream);

/* ------------------------------------------- specular filter + present */

/* SpecularFilterPass push constants (VFS/Shaders/specularFilter.frag:18-24)
 * and their defaults (VFS/RenderPass/SpecularFilterPass.h:48-51): gamma 2.2,
 * exposure 0.1, tone map off, filter 1 = the Gaussian blur.  filter_method 0
 * (and any value but 1) selects the bilateral filter.  (The reference's GUI
 * labels the two methods the other way round.) */
typedef struct vct_specular_filter_desc {
    float tonemap_gamma;
    float tonemap_exposure;
    int32_t tonemap_enable;
    int32_t filter_method;
} vct_specular_filter_desc;
#define VCT_FILTER_BILATERAL 0
#define VCT_FILTER_GAUSSIAN 1

/* SpecularFilterPass::onUpdate + specularFilter.frag: out = diffuse +
 * filter(specular) (rgb; alpha = diffuse's), Uncharted2 tone map when
 * enabled.  Images are RGBA32F, row-major width x height float4, device
 * pointers, 16-byte aligned (the cone trace's diffuse / specular outputs over
 * the G-buffer's pixels, pre-filled with the pass's clear (0, 0, 0, 1) where
 * the trace discards).  `out` must not alias `specular`.  The Gaussian blur's
 * taps are all within 0.01 texel, so it runs as one 3 x 3 stencil; the
 * stencil is returned by vct_specular_filter_stencil (9 floats, row-major
 * dy = -1..1, dx = -1..1, already divided by the shader's 241). */
int vct_specular_filter(const vct_specular_filter_desc* desc_host, const float* diffuse_rgba,
                        const float* specular_rgba, int32_t width, int32_t height, float* out_rgba, void* stream);
int vct_specular_filter_stencil(float out_host[9]);

/* FinalPass into the B8G8R8A8_SRGB swapchain (VFS/SwapChain.cpp:400-412,
 * finalPass.frag), headless: clamp to [0, 1], sRGB-encode rgb, store UNORM8
 * (round half up); one uint32 per pixel with bytes B, G, R, A. */
int vct_present_srgb8(const float* rgba, int32_t width, int32_t height, uint32_t* out_bgra8, void* stream);

/* ------------------------------------------------------------ scene ingest */

/* Reverses the scanline filters of an inflated PNG image (filter byte + row
 * per scanline; None / Sub / Up / Average / Paeth, ISO/IEC 15948 section 9)
 * into `out_host` (rows x row_bytes).  bpp = bytes per pixel (at least 1).
 * Host memory; used by the glTF loader for the scene's images. */
int vct_png_unfilter(const uint8_t* filtered_host, int64_t row_bytes, int64_t rows, int32_t bpp, uint8_t* out_host);

/* The toroidal half of VoxelizationPass (VoxelizationPass.cpp:127-141,
 * 190-212): clear each slab at its corner wrapped into the level
 * (ClipmapCleaner), then voxelise, for every level with slabs, the fragments
 * that fall inside them -- with the level's full-region projection, so a
 * voxel comes out as the full pass at `regions` would make it.  A slab that
 * covers the whole region revoxelises its level in full.  Slabs and levels
 * as vct_update_clip_regions lists them (host arrays). */
int vct_voxelize_opacity_slabs(const vct_scene* scene, const vct_clipmap_region regions_host[6], int32_t R,
                               uint32_t* opacity_atlas, const vct_clipmap_region* slabs_host,
                               const int32_t* slab_levels_host, int32_t slab_count, vct_workspace ws, void* stream);

/* SparseVoxelizer::preVoxelize + cmdVoxelize (VFS/RenderPass/Octree/SparseVoxelizer.cpp:248-326)
 * with voxelizer.{vert,geom,frag}: count pass, host readback of the count
 * into *count_host, write pass of packed uint2 fragments in traversal order.
 * capacity == 0 only counts.  Fragments discarded by the light test keep a
 * zeroed slot (the reference increments its counter before that discard). */
int vct_svo_fragments(const vct_scene* scene, int32_t octree_level, const float bb_min_host[3],
                      const float bb_max_host[3], const vct_shadow_map* shadow,
                      const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow, uint32_t* fragments,
                      int64_t capacity, int64_t* count_host, vct_workspace ws, void* stream);

/* ------------------------------------------------ sparse voxel octree */

/* OctreeBuilder::initialize pool size: clamp(8 * fragments, 1e6, 5e8) nodes
 * (VFS/RenderPass/Octree/OctreeBuilder.cpp:110-113). */
int64_t vct_svo_pool_capacity(int64_t fragment_count);

/* OctreeBuilder::cmdBuild (VFS/RenderPass/Octree/OctreeBuilder.cpp:205-345):
 * per level init / flag / allocate / advance the window, RGBA8 leaf average,
 * isotropic mips, over a uint2 node pool {MSB flag | child block, RGBA8}.
 * VCT_SVO_DETERMINISTIC allocates child blocks in breadth-first index order
 * and folds leaf colours in fragment order (bit-exact against the oracle);
 * VCT_SVO_ATOMIC uses the reference's atomic allocation and CAS loops
 * (equal to the deterministic pool after vct_svo_canonicalize, except for
 * leaf colours averaged in a different order).  *node_count_host receives
 * the number of nodes in use. */
#define VCT_SVO_DETERMINISTIC 0
#define VCT_SVO_ATOMIC 1
int vct_svo_build(const uint32_t* fragments, int64_t fragment_count, int32_t octree_level, uint32_t* node_pool,
                  int64_t pool_capacity, int32_t mode, int64_t* node_count_host, vct_workspace ws, void* stream);

/* Relabel a node pool's child blocks into breadth-first order (the order a
 * scan allocation produces), so pools built with racy allocation compare
 * bit for bit.  `pool_out` must not alias `pool_in`. */
int vct_svo_canonicalize(const uint32_t* pool_in, int64_t node_count, int32_t octree_level, uint32_t* pool_out,
                         vct_workspace ws, void* stream);

/* OctreeVoxelConeTracing::onUpdate (VFS/RenderPass/Octree/OctreeVoxelConeTracing.cpp:74-104)
 * running voxelConeTracing_Octree.frag: the cone loop of vct_cone_trace
 * sampling the node pool by point location.  `bb_min/bb_max` is the scene box
 * the shader normalises positions with (it hard-codes Sponza's,
 * voxelConeTracing_Octree.frag:321-322); desc->volume_dimension is the pool's
 * root resolution (the pass passes 256). */
int vct_svo_cone_trace(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, const uint32_t* node_pool,
                       int64_t node_count, const float bb_min_host[3], const float bb_max_host[3],
                       const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                       const vct_directional_light_shadow_desc* light_shadow,
                       const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                       float* specular_out, unsigned long long* cone_steps, void* stream);

/* -------------------------------------------------- instances and batches */

/* An atlas in the reference's layout ((R+2)*6 x (R+2)*6 x (R+2) texels),
 * zeroed: RGBA8 (4 B per texel, VCT_TEX_RGBA8) or the packed FP16 form
 * (8 B, VCT_TEX_RGBA16F). */
int vct_atlas_alloc(int32_t R, int32_t format, void** out);
int vct_atlas_free(void* atlas);

/* One headless instance of the clipmap method: what Application::initialize
 * and buildClipmapMethodPasses create once (VFS/Application.cpp:406-522) --
 * opacity and radiance atlases, the light's depth map, the radiance texture,
 * the raster workspace, the trace scratch -- and the state the passes keep
 * between frames (frame index of the radiance cadence, clip regions). */
typedef struct vct_config {
    int32_t clipmap_resolution; /* R: power of two in [8, 1024] (the reference's DEFAULT_VOXEL_RESOLUTION) */
    int32_t shadow_width;       /* light depth map size; 0 x 0 = no shadow pass (visibility 1) */
    int32_t shadow_height;
    int32_t flags;              /* VCT_CONTEXT_* bits, 0 = the reference's behaviour */
    size_t workspace_bytes;     /* initial raster workspace (grows on demand) */
} vct_config;

/* vct_config.flags: AUTOTUNE -- the context's first trace runs
 * vct_cone_trace_fast_autotune unless its resolution is already tuned on the
 * device; OPACITY_R8 -- the context's opacity atlas is the one-byte form
 * (VCT_OPACITY_R8: frames with the full revoxelisation and the deterministic
 * injection only). */
#define VCT_CONTEXT_AUTOTUNE 1
#define VCT_CONTEXT_OPACITY_R8 2

typedef struct vct_context_s* vct_context;

typedef struct vct_context_buffers {
    uint32_t* opacity;                    /* RGBA8 atlases, device */
    uint32_t* radiance;
    float* shadow_depth;                  /* NULL without a shadow pass */
    struct vct_texture_s* radiance_texture;
    struct vct_workspace_s* workspace;
    vct_clipmap_region regions[6];        /* of the last frame */
    int32_t frame_index;                  /* of the next frame */
    int32_t reserved;
} vct_context_buffers;

int vct_create(const vct_config* cfg_host, vct_context* out);
int vct_destroy(vct_context ctx); /* synchronises the device */
int vct_context_buffers_get(const struct vct_context_s* ctx, vct_context_buffers* out_host);
/* Forget the frame history: the next frame is frame 0 (every radiance level
 * due) with a full revoxelisation.  The atlases keep their contents. */
int vct_context_reset(vct_context ctx);

/* Application::run's pre-passes on the instance (vct_clipmap_frame with its
 * buffers, deterministic injection, the radiance texture kept current); the
 * frame index advances by one per call.  revoxelization: VCT_REVOX_FULL or
 * VCT_REVOX_TOROIDAL (the first frame of an instance is always full). */
int vct_context_frame(vct_context ctx, const vct_scene* scene, const float camera_pos_host[3],
                      const vct_directional_light_desc* light_host,
                      const vct_directional_light_shadow_desc* light_shadow_host, int32_t revoxelization,
                      void* stream);

/* VoxelConeTracingPass::onUpdate on the instance: the fast trace of
 * `samples` against its radiance texture and depth map; volume_center,
 * voxel_size and volume_dimension of `desc` are replaced by the ones the
 * pass derives from the last frame's level-0 region
 * (VoxelConeTracingPass.cpp:86-102).  The trace scratch grows on demand. */
int vct_context_trace(vct_context ctx, const vct_cone_tracing_desc* desc_host, const vct_cam_matrix* cam_host,
                      const vct_directional_light_desc* light_host,
                      const vct_directional_light_shadow_desc* light_shadow_host,
                      const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                      float* specular_out, unsigned long long* cone_steps, void* stream);

/* One independent unit of a batch: a frame of `scene` on `context` and the
 * trace of `samples` (sample_count 0: frame only). */
typedef struct vct_batch_job {
    vct_context context;
    const vct_scene* scene;
    float camera_pos[3];
    int32_t revoxelization;
    int32_t reset;              /* nonzero: vct_context_reset first (an independent single-frame job) */
    int32_t reserved;
    vct_directional_light_desc light;
    vct_directional_light_shadow_desc light_shadow;
    const vct_cone_tracing_desc* trace_desc;
    const vct_cam_matrix* cam;
    const vct_surface_sample* samples;
    int64_t sample_count;
    float* diffuse_out;
    float* specular_out;
    unsigned long long* cone_steps;
} vct_batch_job;

/* Runs every job (frame + trace) on `streams` host threads, each with its
 * own CUDA stream, so that one job's host-side waits overlap the others' GPU
 * work; returns when all are done.  The contexts are dealt round-robin to the
 * threads in order of first appearance; the jobs of one context run in list
 * order on its thread. */
int vct_batch_submit(const vct_batch_job* jobs_host, int32_t job_count, int32_t streams);

/* ------------------------------------------------------------ one frame */

/* Per-frame inputs of the clipmap method (Application::run and the passes it
 * drives): camera position (clip regions), clipmap resolution, frame index
 * (radiance levels are refreshed every 2^level frames), injection mode,
 * directional light with its shadow projection, shadow-map size (0 = no
 * shadow pass: visibility 1), and the radiance texture to keep current. */
typedef struct vct_frame_desc {
    float camera_pos[3];
    int32_t clipmap_resolution;
    int32_t frame_index;
    int32_t inject_mode;
    int32_t shadow_width;
    int32_t shadow_height;
    vct_directional_light_desc light;
    vct_directional_light_shadow_desc light_shadow;
    struct vct_texture_s* radiance_texture; /* may be NULL: an RGBA8 texture of the same resolution that
                                               receives every radiance texel the frame's copy-alpha and
                                               mip passes write (the texture the fast trace samples) */
    int32_t revoxelization;                 /* VCT_REVOX_FULL (the reference as shipped) or VCT_REVOX_TOROIDAL */
    int32_t opacity_format;                 /* VCT_OPACITY_RGBA8 (the reference's atlas, 4 bytes per texel) or
                                               VCT_OPACITY_R8 (1 byte per texel, alpha only; FULL revoxelisation
                                               with the deterministic injection) */
    vct_clipmap_region* regions_state;      /* host, 6 regions: FULL writes the frame's regions here (may be
                                               NULL); TOROIDAL reads the previous frame's regions, moves them
                                               (vct_update_clip_regions) and writes them back (required) */
} vct_frame_desc;

/* Opacity revoxelisation of a frame.  FULL: clear the atlas and voxelise
 * every level at regions placed from the camera (VoxelizationPass.cpp:79-92,
 * _fullRevoxelization stays true).  TOROIDAL: the regions persist; only the
 * slabs the camera move uncovers are cleared and voxelised, and only the
 * levels that moved get new opacity mips (the reference's switched-off path,
 * VoxelizationPass.cpp:93-141, 167-178, 450-494).  The opacity atlas must
 * hold the previous frame's voxels of `regions_state`. */
#define VCT_REVOX_FULL 0
#define VCT_REVOX_TOROIDAL 1

/* Opacity atlas storage of a frame.  RGBA8: the reference's image
 * (Voxelizer.cpp:159), uint32 texels.  R8: the same texel order at one byte
 * per texel holding the alpha that copy-alpha, the mips and the border wrap
 * read (the RGBA8 atlas's alpha bytes, bit for bit), a quarter of the clear,
 * voxelisation, mip and copy-alpha traffic; the radiance atlas and texture
 * are unchanged.  The `opacity` argument of vct_clipmap_frame then points at
 * those bytes. */
#define VCT_OPACITY_RGBA8 0
#define VCT_OPACITY_R8 1

/* Application::run's pre-pass sequence (VFS/Application.cpp:142-201):
 * VoxelizationPass (clear, voxelise all levels, opacity mips, border wrap),
 * RSMPass depth, RadianceInjectionPass (clear due levels, inject, copy alpha,
 * radiance mips).  Writes the 6 clip regions to regions_out (may be NULL). */
int vct_clipmap_frame(const vct_scene* scene, const vct_frame_desc* frame, uint32_t* opacity_atlas,
                      uint32_t* radiance_atlas, float* shadow_depth, vct_clipmap_region regions_out_host[6],
                      vct_workspace ws, void* stream);

/* ------------------------------------------ allocation-free fast trace */

/* No counterpart in the reference.  vct_cone_trace_fast for callers that
 * cannot allocate device memory (hosts that own all GPU memory through their
 * own allocator, frame loops that must not call cudaMalloc): the same pass,
 * with its scratch in a static device array of VCT_NOALLOC_SCRATCH_BYTES that
 * the library holds on every GPU that loads it, for up to
 * VCT_NOALLOC_MAX_SAMPLES samples (larger counts are rejected with
 * VCT_E_BAD_ARG).  No call runs cudaMalloc, but the array must be resident:
 * under lazy module loading (the CUDA runtime's default) the runtime commits
 * its 48 MiB on a device at the first call there, so make one call on each
 * device before the host reserves its device memory and before any stream
 * capture.  Every call looks up the array's address on the current device
 * (cudaGetSymbolAddress).  Calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
#define VCT_NOALLOC_MAX_SAMPLES 1048576
#define VCT_NOALLOC_SCRATCH_BYTES (48u << 20)
int vct_cone_trace_fast_noalloc(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam, vct_texture radiance,
                                const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                                const vct_directional_light_shadow_desc* light_shadow,
                                const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                                float* specular_out, unsigned long long* cone_steps, void* stream);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
#define VCT_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define VCT_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif
VCT_STATIC_ASSERT(sizeof(vct_voxelization_desc) == 64, "VoxelizationDesc is 64 B");
VCT_STATIC_ASSERT(sizeof(vct_downsample_desc) == 24, "DownSampleDesc is 24 B");
VCT_STATIC_ASSERT(sizeof(vct_image_cleaning_desc) == 36, "ImageCleaningDesc is 36 B");
VCT_STATIC_ASSERT(sizeof(vct_copy_alpha_desc) == 12, "CopyAlphaDesc is 12 B");
VCT_STATIC_ASSERT(sizeof(vct_border_wrapping_desc) == 16, "BorderWrappingDesc is 16 B");
VCT_STATIC_ASSERT(sizeof(vct_cone_tracing_desc) == 52, "VoxelConeTracingDesc is 52 B");
VCT_STATIC_ASSERT(sizeof(vct_cam_matrix) == 144, "CamMatrix is 144 B");
VCT_STATIC_ASSERT(sizeof(vct_directional_light_desc) == 32, "DirectionalLightDesc is 32 B");
VCT_STATIC_ASSERT(sizeof(vct_directional_light_shadow_desc) == 136, "DirectionalLightShadowDesc is 136 B");
VCT_STATIC_ASSERT(sizeof(vct_specular_filter_desc) == 16, "SpecularFilterPassDesc is 16 B");
VCT_STATIC_ASSERT(sizeof(vct_config) == 24, "vct_config is 24 B");
VCT_STATIC_ASSERT(sizeof(vct_adam_desc) == 40, "vct_adam_desc is 40 B");
VCT_STATIC_ASSERT(sizeof(vct_context_buffers) == 216, "vct_context_buffers is 216 B");
VCT_STATIC_ASSERT(sizeof(vct_batch_job) == 264, "vct_batch_job is 264 B");
VCT_STATIC_ASSERT(sizeof(vct_gltf_shade_material) == 80, "GltfShadeMaterial is 80 B");
VCT_STATIC_ASSERT(sizeof(vct_surface_sample) == 80, "surface sample is 80 B");
VCT_STATIC_ASSERT(sizeof(vct_trace_options) == 16, "vct_trace_options is 16 B");
VCT_STATIC_ASSERT(sizeof(vct_trace_job) == 296, "vct_trace_job is 296 B");
VCT_STATIC_ASSERT(sizeof(vct_trace_tuning) == 24, "vct_trace_tuning is 24 B");

#endif /* VCT_CAPI_H */
