// frame.cu -- one frame of the 3D-clipmap method in the reference's pass order
// (Application::run, VFS/Application.cpp:142-201, with the passes built in
// Application::buildClipmapMethodPasses, :406-522):
//
//   VoxelizationPass       clear opacity, voxelise every level, opacity
//                          mips 1..5, opacity border wrap (or, in the
//                          toroidal mode, clear + voxelise the slabs the
//                          camera move uncovered and redo the moved levels' mips)
//   RSMPass                directional-light depth map
//   RadianceInjectionPass  for each level due this frame (frame % 2^level == 0):
//                          clear, inject; then copy-alpha and radiance mips
//                          (levels 1..5: vct_copy_alpha_downsample, one pass)
//
// Host-side orchestration only: every step is one of the C-ABI passes (or
// its internal form with a texture mirror), run on the caller's stream.
#include "common.cuh"

extern "C" int vct_clipmap_frame(const vct_scene* scene, const vct_frame_desc* f, uint32_t* opacity,
                                 uint32_t* radiance, float* shadow_depth, vct_clipmap_region regions_out[6],
                                 vct_workspace_s* ws, void* stream) {
    vct::NvtxRange range("vct_clipmap_frame");
    VCT_CHECK_ARG(scene && f && opacity && radiance && ws, "vct_clipmap_frame: null argument");
    VCT_CHECK_ARG(!f->shadow_width || shadow_depth, "vct_clipmap_frame: shadow map size given without a buffer");
    VCT_CHECK_ARG(f->inject_mode == VCT_INJECT_DETERMINISTIC || f->inject_mode == VCT_INJECT_ATOMIC,
                  "vct_clipmap_frame: bad injection mode");
    const int R = f->clipmap_resolution;
    VCT_CHECK_ARG(!f->radiance_texture || (vct::texture_format(f->radiance_texture) == VCT_TEX_RGBA8 &&
                                           vct::texture_resolution(f->radiance_texture) == R),
                  "vct_clipmap_frame: the radiance texture must be RGBA8 of the clipmap resolution");
    VCT_CHECK_ARG(f->revoxelization == VCT_REVOX_FULL || f->revoxelization == VCT_REVOX_TOROIDAL,
                  "vct_clipmap_frame: bad revoxelization mode");
    const bool toroidal = f->revoxelization == VCT_REVOX_TOROIDAL;
    VCT_CHECK_ARG(!toroidal || f->regions_state, "vct_clipmap_frame: the toroidal mode needs regions_state");
    VCT_CHECK_ARG(f->opacity_format == VCT_OPACITY_RGBA8 || f->opacity_format == VCT_OPACITY_R8,
                  "vct_clipmap_frame: bad opacity format");
    const bool r8 = f->opacity_format == VCT_OPACITY_R8;
    VCT_CHECK_ARG(!r8 || (!toroidal && f->inject_mode == VCT_INJECT_DETERMINISTIC),
                  "vct_clipmap_frame: the R8 opacity form needs the full revoxelisation and the deterministic injection");
    vct_clipmap_region regions[6];
    vct_clipmap_region slabs[18];
    int32_t slab_levels[18];
    int32_t nslabs = -1;  // full revoxelisation
    int rc;
    if (toroidal) {
        for (int l = 0; l < 6; ++l) regions[l] = f->regions_state[l];
        rc = vct_update_clip_regions(regions, f->camera_pos, R, VCT_VOXEL_EXTENT_L0, slabs, slab_levels, &nslabs);
    } else {
        rc = vct_clip_regions(f->camera_pos, R, VCT_VOXEL_EXTENT_L0, regions);
    }
    if (rc != VCT_OK) return rc;
    if (f->regions_state)
        for (int l = 0; l < 6; ++l) f->regions_state[l] = regions[l];
    if (regions_out)
        for (int l = 0; l < 6; ++l) regions_out[l] = regions[l];

    uint32_t due = 0;  // radiance levels refreshed this frame: cadence 2^level frames
    for (int l = 0; l < 6; ++l)
        if (f->frame_index % (1 << l) == 0) due |= 1u << l;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const uint32_t* touched = nullptr;  // deterministic mode: the due levels' clear happens in the passes below
    if (f->inject_mode == VCT_INJECT_DETERMINISTIC) {
        // VoxelizationPass, RSMPass and RadianceInjectionPass up to the fold,
        // with the opacity voxelisation and the injection's coverage count
        // sharing one coverage pass (same results as the passes below)
        if ((rc = vct::frame_raster_passes(scene, f, regions, due, slabs, slab_levels, nslabs, opacity, radiance,
                                           shadow_depth, ws, &touched, st)) != VCT_OK)
            return rc;
    } else {
        if (!toroidal) {
            // VoxelizationPass (full revoxelisation every frame, VoxelizationPass.cpp:79-125)
            if ((rc = vct_clear_atlas(opacity, R, stream)) != VCT_OK) return rc;
            if ((rc = vct_voxelize_opacity(scene, regions, R, opacity, 0x3Fu, ws, stream)) != VCT_OK) return rc;
            if ((rc = vct_downsample_all(opacity, regions, R, VCT_DOWNSAMPLE_OPACITY, stream)) != VCT_OK) return rc;
        } else {
            // the toroidal path: slabs cleared and voxelised, mips of the levels that moved
            if ((rc = vct_voxelize_opacity_slabs(scene, regions, R, opacity, slabs, slab_levels, nslabs, ws,
                                                 stream)) != VCT_OK)
                return rc;
            uint32_t moved = 0;
            for (int i = 0; i < nslabs; ++i) moved |= 1u << slab_levels[i];
            for (int l = 1; l < 6; ++l) {
                if (!((moved >> l) & 1u)) continue;
                vct_downsample_desc d;
                for (int a = 0; a < 3; ++a) d.prev_region_min_corner[a] = regions[l - 1].min_corner[a];
                d.clip_level = l;
                d.clipmap_resolution = R;
                d.downsample_region_size = VCT_DOWNSAMPLE_REGION_SIZE;
                if ((rc = vct_downsample(opacity, &d, VCT_DOWNSAMPLE_OPACITY, stream)) != VCT_OK) return rc;
            }
        }
        vct_border_wrapping_desc bw = {(uint32_t)R, VCT_VOXEL_BORDER, VCT_FACE_COUNT, VCT_CLIP_LEVEL_COUNT};
        if ((rc = vct_wrap_border(opacity, &bw, stream)) != VCT_OK) return rc;
        // RSMPass: the depth map the injection's visibility samples
        vct_shadow_map sm = {nullptr, 0, 0};
        if (f->shadow_width > 0) {
            if ((rc = vct_shadow_depth(scene, &f->light_shadow, shadow_depth, f->shadow_width, f->shadow_height, ws,
                                       stream)) != VCT_OK)
                return rc;
            sm.depth = shadow_depth;
            sm.width = f->shadow_width;
            sm.height = f->shadow_height;
        }
        // RadianceInjectionPass (RadianceInjectionPass.cpp:64-159)
        for (int l = 0; l < 6; ++l) {
            if (!((due >> l) & 1u)) continue;
            vct_image_cleaning_desc c = {{0, 0, 0}, l, {(uint32_t)R, (uint32_t)R, (uint32_t)R}, R, VCT_FACE_COUNT};
            if ((rc = vct_clear_region(radiance, &c, stream)) != VCT_OK) return rc;
        }
        if ((rc = vct_inject_radiance(scene, regions, R, &sm, &f->light, &f->light_shadow, radiance, due,
                                      f->inject_mode, ws, stream)) != VCT_OK)
            return rc;
    }
    // copy-alpha of every due level, then the radiance mips 1..5 of the due
    // levels; a due level's predecessor is always due (frame % 2^l == 0), so
    // level 0 takes the plain copy and levels 1..5 the fused copy + mip pass,
    // each after its predecessor is final -- the same result as all copies
    // first and the mips after.
    // Both passes also store their texels into the radiance texture when one
    // is given: together they rewrite every interior texel of every due
    // level, and radiance borders are never written, so the texture stays
    // equal to the atlas without a copy.
    const cudaSurfaceObject_t mirror = f->radiance_texture ? vct::texture_surface(f->radiance_texture) : 0;
    if (due & 1u) {
        vct_copy_alpha_desc ca = {0, R, VCT_FACE_COUNT};
        if ((rc = vct::copy_alpha_pass(radiance, opacity, &ca, mirror, touched, st, r8)) != VCT_OK) return rc;
    }
    for (int l = 1; l < 6; ++l) {
        if (!((due >> l) & 1u)) continue;
        vct_downsample_desc d;
        for (int a = 0; a < 3; ++a) d.prev_region_min_corner[a] = regions[l - 1].min_corner[a];
        d.clip_level = l;
        d.clipmap_resolution = R;
        d.downsample_region_size = VCT_DOWNSAMPLE_REGION_SIZE;
        if ((rc = vct::copy_alpha_downsample_pass(radiance, opacity, &d, mirror, touched, st, r8)) != VCT_OK)
            return rc;
    }
    return VCT_OK;
}
