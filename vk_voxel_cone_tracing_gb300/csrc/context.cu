// context.cu -- a headless clipmap VCT instance and the batched submission.
//
// vct_context owns what Application::initialize / buildClipmapMethodPasses
// create once for the clipmap method (VFS/Application.cpp:406-522): the
// opacity and radiance atlases (Voxelizer.cpp:157-191), the directional
// light's depth map, the radiance texture the trace samples, the raster
// workspace, the trace scratch, and the per-frame state the passes keep
// between frames (the frame index of the radiance cadence and, for the
// toroidal mode, the clip regions).  vct_context_frame and
// vct_context_trace run Application::run's pre-passes and the cone-tracing
// pass on those buffers.
//
// vct_batch_submit runs many independent units (a frame and a trace each)
// concurrently: contexts are dealt round-robin to `streams` host threads,
// each with its own CUDA stream, so that the host-side waits of one job
// (tile-plan and count readbacks) overlap the GPU work of the others.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

using namespace vct;

struct vct_context_s {
    vct_config cfg{};
    uint32_t* opacity = nullptr;
    uint32_t* radiance = nullptr;
    float* shadow = nullptr;
    vct_texture_s* texture = nullptr;
    vct_workspace_s* ws = nullptr;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    vct_clipmap_region regions[6]{};
    int32_t frame_index = 0;
    bool have_regions = false;
};

namespace {

size_t atlas_bytes(int R, int format) { return (size_t)AtlasDims(R).texels() * (format == VCT_TEX_RGBA16F ? 8 : 4); }

void release(vct_context_s* c) {
    if (!c) return;
    if (c->opacity) cudaFree(c->opacity);
    if (c->radiance) cudaFree(c->radiance);
    if (c->shadow) cudaFree(c->shadow);
    if (c->scratch) cudaFree(c->scratch);
    if (c->texture) vct_texture_destroy(c->texture);
    if (c->ws) vct_workspace_destroy(c->ws);
    delete c;
}

}  // namespace

extern "C" int vct_atlas_alloc(int32_t R, int32_t format, void** out) {
    VCT_CHECK_ARG(out, "vct_atlas_alloc: null output");
    *out = nullptr;
    VCT_CHECK_ARG(valid_resolution(R), "vct_atlas_alloc: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(format == VCT_TEX_RGBA8 || format == VCT_TEX_RGBA16F, "vct_atlas_alloc: bad format");
    const size_t bytes = atlas_bytes(R, format);
    VCT_CUDA_TRY(cudaMalloc(out, bytes));
    cudaError_t e = cudaMemset(*out, 0, bytes);  // vkCmdClearColorImage to 0 at creation
    if (e != cudaSuccess) {
        cudaFree(*out);
        *out = nullptr;
        return cuda_fail(e, "cudaMemset (atlas)");
    }
    return VCT_OK;
}

extern "C" int vct_atlas_free(void* atlas) {
    if (atlas) VCT_CUDA_TRY(cudaFree(atlas));
    return VCT_OK;
}

extern "C" int vct_create(const vct_config* cfg, vct_context_s** out) {
    VCT_CHECK_ARG(cfg && out, "vct_create: null argument");
    *out = nullptr;
    VCT_CHECK_ARG(valid_resolution(cfg->clipmap_resolution), "vct_create: resolution must be a power of two in [8,1024]");
    VCT_CHECK_ARG(cfg->shadow_width >= 0 && cfg->shadow_height >= 0 && cfg->shadow_width <= 16384 &&
                      cfg->shadow_height <= 16384 && ((cfg->shadow_width == 0) == (cfg->shadow_height == 0)),
                  "vct_create: bad shadow map size");
    VCT_CHECK_ARG((cfg->flags & ~(VCT_CONTEXT_AUTOTUNE | VCT_CONTEXT_OPACITY_R8)) == 0, "vct_create: unknown flags");
    auto* c = new vct_context_s();
    c->cfg = *cfg;
    const int R = cfg->clipmap_resolution;
    int rc = VCT_OK;
    if (cfg->flags & VCT_CONTEXT_OPACITY_R8) {  // one byte per texel, zeroed like a fresh atlas
        const size_t bytes = (size_t)AtlasDims(R).texels();
        cudaError_t e = cudaMalloc((void**)&c->opacity, bytes);
        if (e == cudaSuccess) e = cudaMemset(c->opacity, 0, bytes);
        if (e != cudaSuccess) {
            release(c);
            return cuda_fail(e, "cudaMalloc / cudaMemset (R8 opacity atlas)");
        }
    } else if ((rc = vct_atlas_alloc(R, VCT_TEX_RGBA8, (void**)&c->opacity)) != VCT_OK) {
        release(c);
        return rc;
    }
    if ((rc = vct_atlas_alloc(R, VCT_TEX_RGBA8, (void**)&c->radiance)) != VCT_OK ||
        (rc = vct_texture_create(R, VCT_TEX_RGBA8, &c->texture)) != VCT_OK ||
        (rc = vct_workspace_create(cfg->workspace_bytes, &c->ws)) != VCT_OK) {
        release(c);
        return rc;
    }
    if (cfg->shadow_width > 0) {
        cudaError_t e = cudaMalloc(&c->shadow, (size_t)cfg->shadow_width * cfg->shadow_height * 4);
        if (e != cudaSuccess) {
            release(c);
            return cuda_fail(e, "cudaMalloc (shadow map)");
        }
    }
    *out = c;
    return VCT_OK;
}

extern "C" int vct_destroy(vct_context_s* c) {
    if (!c) return VCT_OK;
    VCT_CUDA_TRY(cudaDeviceSynchronize());
    release(c);
    return VCT_OK;
}

extern "C" int vct_context_buffers_get(const vct_context_s* c, vct_context_buffers* out) {
    VCT_CHECK_ARG(c && out, "vct_context_buffers_get: null argument");
    out->opacity = c->opacity;
    out->radiance = c->radiance;
    out->shadow_depth = c->shadow;
    out->radiance_texture = c->texture;
    out->workspace = c->ws;
    for (int l = 0; l < 6; ++l) out->regions[l] = c->regions[l];
    out->frame_index = c->frame_index;
    return VCT_OK;
}

extern "C" int vct_context_reset(vct_context_s* c) {
    VCT_CHECK_ARG(c, "vct_context_reset: null context");
    c->frame_index = 0;
    c->have_regions = false;
    return VCT_OK;
}

extern "C" int vct_context_frame(vct_context_s* c, const vct_scene* scene, const float camera_pos[3],
                                 const vct_directional_light_desc* light,
                                 const vct_directional_light_shadow_desc* light_shadow, int32_t revoxelization,
                                 void* stream) {
    VCT_CHECK_ARG(c && scene && camera_pos && light && light_shadow, "vct_context_frame: null argument");
    vct_frame_desc f;
    memset(&f, 0, sizeof(f));
    for (int a = 0; a < 3; ++a) f.camera_pos[a] = camera_pos[a];
    f.clipmap_resolution = c->cfg.clipmap_resolution;
    f.frame_index = c->frame_index;
    f.inject_mode = VCT_INJECT_DETERMINISTIC;
    f.shadow_width = c->cfg.shadow_width;
    f.shadow_height = c->cfg.shadow_height;
    f.light = *light;
    f.light_shadow = *light_shadow;
    f.radiance_texture = c->texture;
    f.opacity_format = (c->cfg.flags & VCT_CONTEXT_OPACITY_R8) ? VCT_OPACITY_R8 : VCT_OPACITY_RGBA8;
    // the first frame of an instance is always a full revoxelisation
    f.revoxelization = (revoxelization == VCT_REVOX_TOROIDAL && c->have_regions) ? VCT_REVOX_TOROIDAL : VCT_REVOX_FULL;
    f.regions_state = c->regions;
    int rc = vct_clipmap_frame(scene, &f, c->opacity, c->radiance, c->shadow, nullptr, c->ws, stream);
    if (rc != VCT_OK) return rc;
    c->have_regions = true;
    ++c->frame_index;
    return VCT_OK;
}

extern "C" int vct_context_trace(vct_context_s* c, const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                 const vct_directional_light_desc* light,
                                 const vct_directional_light_shadow_desc* light_shadow,
                                 const vct_surface_sample* samples, int64_t sample_count, float* diffuse_out,
                                 float* specular_out, unsigned long long* cone_steps, void* stream) {
    VCT_CHECK_ARG(c && desc && cam && light && light_shadow, "vct_context_trace: null argument");
    VCT_CHECK_ARG(sample_count >= 0, "vct_context_trace: negative sample count");
    const int64_t need = vct_cone_trace_fast_scratch_bytes(sample_count);
    VCT_CHECK_ARG(need >= 0, "vct_context_trace: too many samples");
    if ((size_t)need > c->scratch_bytes) {
        if (c->scratch) {
            VCT_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
            VCT_CUDA_TRY(cudaFree(c->scratch));
            c->scratch = nullptr;
            c->scratch_bytes = 0;
        }
        VCT_CUDA_TRY(cudaMalloc(&c->scratch, (size_t)need));
        c->scratch_bytes = (size_t)need;
    }
    VCT_CHECK_ARG(c->have_regions, "vct_context_trace: no frame has run on this context");
    // VoxelConeTracingPass::onUpdate (VoxelConeTracingPass.cpp:86-102): the volume fields come from the
    // level-0 clip region of the last frame
    vct_cone_tracing_desc d = *desc;
    const vct_clipmap_region& r0 = c->regions[0];
    for (int a = 0; a < 3; ++a)
        d.volume_center[a] = (float)r0.min_corner[a] * r0.voxel_size + ((float)r0.extent[a] * r0.voxel_size) * 0.5f;
    d.voxel_size = r0.voxel_size;
    d.volume_dimension = (float)c->cfg.clipmap_resolution;
    vct_shadow_map sm = {c->shadow, c->cfg.shadow_width, c->cfg.shadow_height};
    if ((c->cfg.flags & VCT_CONTEXT_AUTOTUNE) && sample_count > 0) {
        vct_trace_tuning t;
        int rc = vct_trace_tuning_get(c->cfg.clipmap_resolution, &t);
        if (rc == VCT_OK && !t.tuned)
            rc = vct_cone_trace_fast_autotune(&d, cam, c->texture, c->shadow ? &sm : nullptr, light, light_shadow,
                                              samples, sample_count, diffuse_out, specular_out, c->scratch,
                                              c->scratch_bytes, &t, stream);
        if (rc != VCT_OK) return rc;
    }
    return vct_cone_trace_fast(&d, cam, c->texture, c->shadow ? &sm : nullptr, light, light_shadow, samples,
                               sample_count, diffuse_out, specular_out, cone_steps, c->scratch, c->scratch_bytes,
                               stream);
}

extern "C" int vct_batch_submit(const vct_batch_job* jobs, int32_t job_count, int32_t streams) {
    vct::NvtxRange nvtx_range("vct_batch_submit");
    VCT_CHECK_ARG(job_count >= 0 && (job_count == 0 || jobs), "vct_batch_submit: bad job list");
    VCT_CHECK_ARG(streams >= 1 && streams <= 64, "vct_batch_submit: streams must be 1..64");
    for (int i = 0; i < job_count; ++i)
        VCT_CHECK_ARG(jobs[i].context && jobs[i].scene && jobs[i].trace_desc && jobs[i].cam,
                      "vct_batch_submit: a job misses its context, scene, trace desc or camera");
    if (job_count == 0) return VCT_OK;
    // contexts -> threads, round-robin in order of first appearance
    std::vector<vct_context_s*> ctxs;
    std::vector<int> thread_of(job_count);
    for (int i = 0; i < job_count; ++i) {
        int k = 0;
        while (k < (int)ctxs.size() && ctxs[k] != jobs[i].context) ++k;
        if (k == (int)ctxs.size()) ctxs.push_back(jobs[i].context);
        thread_of[i] = k % streams;
    }
    const int nthreads = streams < (int)ctxs.size() ? streams : (int)ctxs.size();
    int device = 0;
    VCT_CUDA_TRY(cudaGetDevice(&device));
    std::vector<int> rcs(nthreads, VCT_OK);
    std::vector<std::string> msgs(nthreads);
    auto worker = [&](int t) {
        cudaStream_t st = nullptr;
        if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            rcs[t] = VCT_E_CUDA;
            msgs[t] = "vct_batch_submit: cannot create a stream";
            return;
        }
        int rc = VCT_OK;
        for (int i = 0; i < job_count && rc == VCT_OK; ++i) {
            if (thread_of[i] != t) continue;
            const vct_batch_job& j = jobs[i];
            if (j.reset) rc = vct_context_reset(j.context);
            if (rc == VCT_OK)
                rc = vct_context_frame(j.context, j.scene, j.camera_pos, &j.light, &j.light_shadow, j.revoxelization, st);
            if (rc == VCT_OK && j.sample_count > 0)
                rc = vct_context_trace(j.context, j.trace_desc, j.cam, &j.light, &j.light_shadow, j.samples,
                                       j.sample_count, j.diffuse_out, j.specular_out, j.cone_steps, st);
        }
        if (rc == VCT_OK) {
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) rc = cuda_fail(e, "vct_batch_submit: stream");
        }
        if (rc != VCT_OK) msgs[t] = vct_last_error();
        rcs[t] = rc;
        cudaStreamDestroy(st);
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
    for (int t = 0; t < nthreads; ++t)
        if (rcs[t] != VCT_OK) return fail(rcs[t], msgs[t]);
    return VCT_OK;
}
