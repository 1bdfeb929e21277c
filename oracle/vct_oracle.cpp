// vct_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points over the CPU restatement (clipmap_oracle.hpp, svo_oracle.hpp,
// raster_oracle.hpp, gbuffer_oracle.hpp, composite_oracle.hpp) and its FP64
// reference gradients (adjoint_oracle.hpp) for the Python test harness and bench.py's CPU-baseline
// leg (ctypes).  The CUDA product library never links or calls this file.
#include <omp.h>

#include "adjoint_oracle.hpp"
#include "clipmap_oracle.hpp"
#include "composite_oracle.hpp"
#include "gbuffer_oracle.hpp"
#include "raster_oracle.hpp"
#include "svo_oracle.hpp"

using namespace vcto;

extern "C" {

int vcto_num_threads(void) { return omp_get_max_threads(); }
void vcto_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

void vcto_clip_regions(const float cam[3], int R, int extent_l0, Region out[6]) { clip_regions(cam, R, extent_l0, out); }

void vcto_clear_region(uint32_t* atlas, int R, const int32_t region_min[3], const uint32_t extent[3], int level,
                       int face_count) {
    clear_region(atlas, R, region_min, extent, level, face_count);
}

void vcto_copy_alpha(uint32_t* dst, const uint32_t* src, int R, int level, int face_count) {
    copy_alpha(dst, src, R, level, face_count);
}

void vcto_wrap_border(uint32_t* atlas, int R, int border_width_desc, int face_count, int region_count) {
    wrap_border(atlas, R, border_width_desc, face_count, region_count);
}

void vcto_downsample(uint32_t* atlas, int R, const int prev_min[3], int level, int band, int mode) {
    downsample(atlas, R, prev_min, level, band, mode);
}

void vcto_downsample_f4(float* atlas4, int R, const int prev_min[3], int level, int band, int mode) {
    downsample_f4<double>(atlas4, R, prev_min, level, band, mode);
}

// Cone trace over an RGBA8 atlas.  precision: 32 = FP32 mirror, 64 = FP64.
// Samples [begin, end) are traced; outputs are 4 doubles per sample.
// Returns the number of traceCone loop iterations executed.
uint64_t vcto_cone_trace_opt(int precision, const TraceDesc* desc, const float eye[3], const uint32_t* atlas, int R,
                             const float* shadow, int sw, int sh, const ShadowDesc* sd, const LightDesc* light,
                             const SurfaceSample* samples, int64_t begin, int64_t end, double* out_d, double* out_s,
                             uint8_t* written, float diffuse_aperture) {
    Atlas A(R);
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t i = begin; i < end; ++i) {
        bool ok;
        if (precision == 64) {
            Rgba8Fetch<double> f{atlas, A};
            ClipmapTracer<double, Rgba8Fetch<double>> tr{*desc, f, A};
            double d[4], s[4];
            ok = trace_sample<double>(tr, eye, shadow, sw, sh, *sd, *light, samples[i], d, s, diffuse_aperture);
            if (ok)
                for (int c = 0; c < 4; ++c) {
                    out_d[4 * i + c] = d[c];
                    out_s[4 * i + c] = s[c];
                }
            total += tr.steps;
        } else {
            Rgba8Fetch<float> f{atlas, A};
            ClipmapTracer<float, Rgba8Fetch<float>> tr{*desc, f, A};
            float d[4], s[4];
            ok = trace_sample<float>(tr, eye, shadow, sw, sh, *sd, *light, samples[i], d, s, diffuse_aperture);
            if (ok)
                for (int c = 0; c < 4; ++c) {
                    out_d[4 * i + c] = d[c];
                    out_s[4 * i + c] = s[c];
                }
            total += tr.steps;
        }
        if (written) written[i] = ok ? 1 : 0;
    }
    return total;
}

uint64_t vcto_cone_trace(int precision, const TraceDesc* desc, const float eye[3], const uint32_t* atlas, int R,
                         const float* shadow, int sw, int sh, const ShadowDesc* sd, const LightDesc* light,
                         const SurfaceSample* samples, int64_t begin, int64_t end, double* out_d, double* out_s,
                         uint8_t* written) {
    return vcto_cone_trace_opt(precision, desc, eye, atlas, R, shadow, sw, sh, sd, light, samples, begin, end, out_d,
                               out_s, written, 0.0f);
}

// Cone trace over a float4 atlas (unquantised storage) in FP64: the error
// reference for the FP16-storage form.
uint64_t vcto_cone_trace_f4(const TraceDesc* desc, const float eye[3], const float* atlas4, int R, const float* shadow,
                            int sw, int sh, const ShadowDesc* sd, const LightDesc* light, const SurfaceSample* samples,
                            int64_t begin, int64_t end, double* out_d, double* out_s) {
    Atlas A(R);
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t i = begin; i < end; ++i) {
        Float4Fetch<double> f{atlas4, A};
        ClipmapTracer<double, Float4Fetch<double>> tr{*desc, f, A};
        double d[4], s[4];
        if (trace_sample<double>(tr, eye, shadow, sw, sh, *sd, *light, samples[i], d, s))
            for (int c = 0; c < 4; ++c) {
                out_d[4 * i + c] = d[c];
                out_s[4 * i + c] = s[c];
            }
        total += tr.steps;
    }
    return total;
}

// FP64 reference gradient of the float-atlas trace (adjoint_oracle.hpp):
// grad (4 doubles per texel, zeroed here) = d/d(atlas4) of
// sum_i gd_i . diffuse_i + gs_i . specular_i over samples [begin, end).
void vcto_cone_trace_grad_f4(const TraceDesc* desc, const float eye[3], const float* atlas4, int R,
                             const float* shadow, int sw, int sh, const ShadowDesc* sd, const LightDesc* light,
                             const SurfaceSample* samples, int64_t begin, int64_t end, const float* gd,
                             const float* gs, double* grad) {
    const int64_t n = 4 * Atlas(R).texels();
    for (int64_t k = 0; k < n; ++k) grad[k] = 0.0;
    cone_trace_grad_f4(*desc, eye, atlas4, R, shadow, sw, sh, *sd, *light, samples, begin, end, gd, gs, grad);
}

// FP64 reference adjoint of the float mips, levels first..5 (adjoint_oracle.hpp):
// G enters as dL/d(atlas after the chain) and leaves as dL/d(atlas before it).
void vcto_downsample_chain_grad_f4(const float* atlas4, int R, const int prev_min[15], int first, int band, int mode,
                                   double* G) {
    int pm[5][3];
    for (int l = 0; l < 5; ++l)
        for (int a = 0; a < 3; ++a) pm[l][a] = prev_min[3 * l + a];
    downsample_chain_grad_f4(atlas4, R, pm, first, band, mode, G);
}

// The benchmark's hash-random sparse atlas (same words as
// vk_voxel_cone_tracing_gb300.scene.procedural_atlas_words), OpenMP-parallel.
static inline uint64_t fmix32(uint64_t h) {
    const uint64_t m = 0xFFFFFFFFull;
    h ^= h >> 16;
    h = (h * 0x85EBCA6Bull) & m;
    h ^= h >> 13;
    h = (h * 0xC2B2AE35ull) & m;
    h ^= h >> 16;
    return h;
}
void vcto_procedural_atlas(uint32_t* out, int64_t n, uint32_t seed, double fill) {
    const uint64_t m = 0xFFFFFFFFull;
    const uint64_t thr = (uint64_t)(int64_t)(fill * 65536.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t h = fmix32((((uint64_t)i * 0x9E3779B1ull) & m) ^ (uint64_t)seed);
        uint64_t h2 = fmix32((h * 0x27D4EB2Full + 0x165667B1ull) & m);
        bool occ = (h & 0xFFFF) < thr;
        uint64_t alpha = 64 + ((h >> 16) % 192);
        out[i] = occ ? (uint32_t)((h2 & 0xFFFFFF) | (alpha << 24)) : 0u;
    }
}

// ---------------------------------------------------------- raster passes
void vcto_voxel_view_proj(const Region* region, float out[48]) {
    Mat4 m[3];
    voxel_view_proj(*region, m);
    for (int i = 0; i < 3; ++i) std::memcpy(out + 16 * i, m[i].m, 64);
}
void vcto_voxelization_desc(const Region regions[6], int level, int R, VoxDesc* out) {
    *out = voxelization_desc(regions, level, R);
}
void vcto_light_shadow_desc(const float origin[3], const float direction[3], float z_near, float z_far,
                            ShadowDesc* out) {
    light_shadow_desc(origin, direction, z_near, z_far, *out);
}
void vcto_voxelize_opacity(const SceneView* s, int R, const Region regions[6], uint32_t* atlas, int level_mask) {
    voxelize_opacity(*s, R, regions, atlas, level_mask);
}
void vcto_voxelize_conservative(const SceneView* s, int R, const Region regions[6], uint32_t* atlas, int level_mask) {
    voxelize_conservative(*s, R, regions, atlas, level_mask);
}
// One triangle / box overlap decision (voxel units of `region`), for tests of the test.
int vcto_cons_overlap(const float tri[9], const Region* region, int R, int i, int j, int k) {
    V3<float> p[3];
    for (int v = 0; v < 3; ++v) p[v] = V3<float>(tri[3 * v], tri[3 * v + 1], tri[3 * v + 2]);
    const ConsTri t = cons_setup(p, *region, R);
    return cons_overlap(t, i, j, k) ? 1 : 0;
}
void vcto_shadow_depth(const SceneView* s, const ShadowDesc* sd, float* depth, int W, int H) {
    shadow_depth(*s, *sd, depth, W, H);
}
void vcto_camera_matrix(const float pos[3], const float dir[3], const float up[3], float fovy_deg, float aspect,
                        CamMatrix* out) {
    *out = camera_matrix(pos, dir, up, fovy_deg, aspect);
}
void vcto_inverse4(const float m[16], float out[16]) {
    Mat4 a;
    std::memcpy(a.m, m, 64);
    const Mat4 r = inverse4(a);
    std::memcpy(out, r.m, 64);
}
void vcto_gbuffer(const SceneView* s, const CamMatrix* cam, int W, int H, SurfaceSample* out) {
    gbuffer(*s, *cam, W, H, out);
}
void vcto_gaussian_stencil(float w[9]) { gaussian_stencil(w); }
void vcto_specular_filter(const FilterDesc* fd, const float* diffuse, const float* specular, int W, int H,
                          float* out) {
    specular_filter(*fd, diffuse, specular, W, H, out);
}
void vcto_present_srgb8(const float* rgba, int64_t n, uint32_t* out) { present_srgb8(rgba, n, out); }
int vcto_update_clip_regions(Region regions[6], const float cam[3], int R, int extent_l0, Region slabs[18],
                             int32_t levels[18]) {
    return update_clip_regions(regions, cam, R, extent_l0, slabs, levels);
}
void vcto_voxelize_opacity_slabs(const SceneView* s, int R, const Region regions[6], uint32_t* atlas,
                                 const Region* slabs, const int32_t* levels, int n) {
    voxelize_opacity_slabs(*s, R, regions, atlas, slabs, levels, n);
}
void vcto_inject_radiance(const SceneView* s, int R, const Region regions[6], const float* shadow, int sw, int sh,
                          const ShadowDesc* sd, const LightDesc* light, uint32_t* radiance, int level_mask) {
    inject_radiance(*s, R, regions, shadow, sw, sh, *sd, *light, radiance, level_mask);
}
int64_t vcto_svo_fragments(const SceneView* s, int level, const float bb_min[3], const float bb_max[3],
                           const float* shadow, int sw, int sh, const ShadowDesc* sd, const LightDesc* light,
                           uint32_t* frags, int64_t capacity) {
    return svo_fragments(*s, level, bb_min, bb_max, shadow, sw, sh, *sd, *light, frags, capacity);
}
int vcto_svo_build(const uint32_t* frags, int64_t F, int level, uint32_t* pool, int64_t capacity,
                   int64_t* node_count) {
    int rc = svo_subdivide(frags, F, level, pool, capacity, node_count);
    if (rc != 0) return rc;
    svo_leaf_write(frags, F, level, pool);
    svo_mip_write(frags, F, level, pool);
    return 0;
}

uint64_t vcto_svo_trace(int precision, const TraceDesc* desc, const float eye[3], const uint32_t* pool,
                        const float bb_min[3], const float bb_max[3], const float* shadow, int sw, int sh,
                        const ShadowDesc* sd, const LightDesc* light, const SurfaceSample* samples, int64_t begin,
                        int64_t end, double* out_d, double* out_s) {
    SvoTraceScene S;
    S.pool = pool;
    for (int a = 0; a < 3; ++a) {
        S.bb_min[a] = bb_min[a];
        S.bb_max[a] = bb_max[a];
    }
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t i = begin; i < end; ++i) {
        if (precision == 64) {
            SvoTracer<double> tr{*desc, S};
            double d[4], s[4];
            if (trace_sample_svo<double>(tr, eye, shadow, sw, sh, *sd, *light, samples[i], d, s))
                for (int c = 0; c < 4; ++c) {
                    out_d[4 * i + c] = d[c];
                    out_s[4 * i + c] = s[c];
                }
            total += tr.steps;
        } else {
            SvoTracer<float> tr{*desc, S};
            float d[4], s[4];
            if (trace_sample_svo<float>(tr, eye, shadow, sw, sh, *sd, *light, samples[i], d, s))
                for (int c = 0; c < 4; ++c) {
                    out_d[4 * i + c] = d[c];
                    out_s[4 * i + c] = s[c];
                }
            total += tr.steps;
        }
    }
    return total;
}

}  // extern "C"
