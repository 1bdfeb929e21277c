// capi.cu -- error state, version, and the host-side pieces of the C ABI.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "common.cuh"

namespace vct {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    // a failed call that leaves the context usable (an allocation the device cannot satisfy, a bad
    // argument) also sets the runtime's last-error state: clear it so that the next launch check does
    // not report it again; a sticky error stays and is reported by every later call
    cudaGetLastError();
    return VCT_E_CUDA;
}

}  // namespace vct

using namespace vct;

extern "C" const char* vct_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* vct_version(void) { return "vct-gb300 0.1 (sm_103a)"; }

extern "C" int64_t vct_atlas_texels(int32_t R) {
    if (!valid_resolution(R)) return -1;
    return AtlasDims(R).texels();
}

// VoxelizationPass::createVoxelClipmap + calculateChangeDelta
// (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:335-357, 438-448) with the
// camera-centred boxes of Application::updateClipRegionBoundingBox
// (VFS/Application.cpp:116-128).  The reference keeps full revoxelisation on
// every frame (VoxelizationPass.cpp:79-92), so the regions are the ones
// computed at creation from the camera position.
extern "C" int vct_clip_regions(const float cam[3], int32_t R, int32_t extent_l0, vct_clipmap_region out[6]) {
    VCT_CHECK_ARG(cam && out, "vct_clip_regions: null argument");
    VCT_CHECK_ARG(valid_resolution(R), "vct_clip_regions: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(extent_l0 > 0 && extent_l0 < (1 << 20), "vct_clip_regions: level-0 extent out of range");
    static const int kMinChange[6] = {2, 2, 2, 2, 2, 1};
    for (int l = 0; l < 6; ++l) {
        vct_clipmap_region& r = out[l];
        for (int a = 0; a < 3; ++a) {
            r.min_corner[a] = -(R >> 1);
            r.extent[a] = (uint32_t)R;
        }
        r.voxel_size = (float)((uint32_t)extent_l0 * (1u << l)) / (float)R;
        const float half_size = (float)((extent_l0 >> 1) * (1 << l));
        const float min_change = r.voxel_size * (float)kMinChange[l];
        for (int a = 0; a < 3; ++a) {
            const float bb_min = cam[a] - half_size;
            const float delta_w = bb_min - (float)r.min_corner[a] * r.voxel_size;
            r.min_corner[a] += (int32_t)std::trunc(delta_w / min_change) * kMinChange[l];
        }
    }
    return VCT_OK;
}

// VoxelizationPass::fillRevoxelizationRegions (VFS/RenderPass/Clipmap/
// VoxelizationPass.cpp:450-494) with calculateChangeDelta (:438-448): the
// toroidal update of regions that persist from frame to frame.  Each level
// moves by the camera-snapped delta of ITS current corner (so a region lags
// the camera by up to one snap step, unlike vct_clip_regions' from-scratch
// placement), and the part of the new region that the old one did not cover
// is listed as slabs: the whole region when a delta reaches the extent,
// otherwise one slab per moved axis, |delta| thick, on the side the region
// moved to.
extern "C" int vct_update_clip_regions(vct_clipmap_region regions[6], const float cam[3], int32_t R, int32_t extent_l0,
                                       vct_clipmap_region slabs_out[18], int32_t slab_level_out[18],
                                       int32_t* slab_count) {
    VCT_CHECK_ARG(regions && cam && slabs_out && slab_level_out && slab_count, "vct_update_clip_regions: null argument");
    VCT_CHECK_ARG(valid_resolution(R), "vct_update_clip_regions: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(extent_l0 > 0 && extent_l0 < (1 << 20), "vct_update_clip_regions: level-0 extent out of range");
    static const int kMinChange[6] = {2, 2, 2, 2, 2, 1};
    int n = 0;
    for (int l = 0; l < 6; ++l) {
        vct_clipmap_region& r = regions[l];
        for (int a = 0; a < 3; ++a)
            VCT_CHECK_ARG(r.extent[a] == (uint32_t)R, "vct_update_clip_regions: regions must have the clipmap extent");
        const float half_size = (float)((extent_l0 >> 1) * (1 << l));
        const float min_change = r.voxel_size * (float)kMinChange[l];
        int32_t delta[3];
        bool full = false;
        for (int a = 0; a < 3; ++a) {
            const float bb_min = cam[a] - half_size;
            const float delta_w = bb_min - (float)r.min_corner[a] * r.voxel_size;
            delta[a] = (int32_t)std::trunc(delta_w / min_change) * kMinChange[l];
            r.min_corner[a] += delta[a];
            full = full || std::abs(delta[a]) >= (int32_t)r.extent[a];
        }
        if (full) {
            slabs_out[n] = r;
            slab_level_out[n++] = l;
            continue;
        }
        for (int a = 0; a < 3; ++a) {
            if (std::abs(delta[a]) < kMinChange[l]) continue;
            vct_clipmap_region s = r;
            s.extent[a] = (uint32_t)std::abs(delta[a]);
            if (delta[a] > 0) s.min_corner[a] = r.min_corner[a] + (int32_t)r.extent[a] - (int32_t)s.extent[a];
            slabs_out[n] = s;
            slab_level_out[n++] = l;
        }
    }
    *slab_count = n;
    return VCT_OK;
}
