// capi.cu -- error state, version, and the host-side pieces of the C ABI.
#include <cmath>
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
