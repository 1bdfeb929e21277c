// raster_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the rasterisation-driven passes of the reference:
//   * host matrices of Voxelizer::setViewProjection (Voxelizer.cpp:394-423) and
//     DirectionalLight::setTransform (DirectionalLight.cpp:21-47), written from
//     the published glm definitions (left-handed, depth 0..1: VFS/pch.h:33-35);
//   * the fixed-function rasteriser the GLSL runs under, pinned as described
//     below (the reference's result is implementation-defined: device-max MSAA
//     with sample shading 0.25, VoxelizationPass.cpp:408-417);
//   * msaaVoxelizer.frag (opacity), reflectiveShadowPass.vert (depth),
//     msaaInjectRadiance.frag (radiance injection, CAS running average),
//     voxelizer.frag (SVO voxel-fragment list).
//
// Pinned rasteriser (identical in the CUDA kernels):
//   * viewport transform x_fb = (W/2) x_ndc + W/2, y_fb = (H/2) y_ndc + H/2
//     (FP32), vertices snapped to 1/256 pixel (round to nearest even);
//   * samples: 8x MSAA at the Vulkan standard sample locations, or one sample
//     at the pixel centre for the depth-only shadow pass;
//   * coverage by exact 64-bit edge functions; a sample on an edge belongs to
//     the triangle for which the edge runs (dy > 0) or (dy == 0 and dx > 0)
//     after orienting the triangle counter-clockwise (one owner per shared
//     edge); zero-area triangles produce nothing; no culling;
//   * depth clip 0 <= z <= 1; barycentrics b_i = float(e_i) * (1 / float(area))
//     and attributes (b0 a0 + b1 a1) + b2 a2, all FP32 without fused multiply-add;
//   * the fragment shader runs at every covered sample (sample-rate shading);
//   * traversal order (the order of atomic-average folds and fragment-list
//     appends): triangles in index order, then clip levels, then 8x8-pixel
//     tiles of the bounding box row-major, pixels row-major, samples 0..N-1.
#pragma once

#include <vector>

#include "clipmap_oracle.hpp"

namespace vcto {

// ------------------------------------------------------------ glm matrices
struct Mat4 {
    float m[16];  // column-major: m[c*4 + r]
    float& at(int c, int r) { return m[c * 4 + r]; }
    float at(int c, int r) const { return m[c * 4 + r]; }
};

inline Mat4 mat_identity() {
    Mat4 a{};
    for (int i = 0; i < 4; ++i) a.at(i, i) = 1.0f;
    return a;
}

// glm::operator*(mat4, mat4): Result[i] = ((A0*B[i][0] + A1*B[i][1]) + A2*B[i][2]) + A3*B[i][3].
inline Mat4 mat_mul4(const Mat4& A, const Mat4& B) {
    Mat4 R{};
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 4; ++r) {
            float s = A.at(0, r) * B.at(i, 0);
            s = s + A.at(1, r) * B.at(i, 1);
            s = s + A.at(2, r) * B.at(i, 2);
            s = s + A.at(3, r) * B.at(i, 3);
            R.at(i, r) = s;
        }
    return R;
}

// glm::operator*(mat4, vec4): ((c0*x + c1*y) + (c2*z + c3*w)).
inline V4<float> mat_vec4(const Mat4& M, float x, float y, float z, float w) {
    V4<float> out;
    float r[4];
    for (int i = 0; i < 4; ++i) {
        float a = M.at(0, i) * x + M.at(1, i) * y;
        float b = M.at(2, i) * z + M.at(3, i) * w;
        r[i] = a + b;
    }
    out.x = r[0];
    out.y = r[1];
    out.z = r[2];
    out.w = r[3];
    return out;
}

inline V3<float> cross3(V3<float> a, V3<float> b) {
    return V3<float>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float dot3f(V3<float> a, V3<float> b) {
    float t0 = a.x * b.x, t1 = a.y * b.y, t2 = a.z * b.z;
    return (t0 + t1) + t2;
}
inline V3<float> normalize3f(V3<float> v) {
    float inv = 1.0f / std::sqrt(dot3f(v, v));
    return V3<float>(v.x * inv, v.y * inv, v.z * inv);
}

// glm::lookAtLH.
inline Mat4 look_at_lh(V3<float> eye, V3<float> center, V3<float> up) {
    V3<float> f = normalize3f(V3<float>(center.x - eye.x, center.y - eye.y, center.z - eye.z));
    V3<float> s = normalize3f(cross3(up, f));
    V3<float> u = cross3(f, s);
    Mat4 R = mat_identity();
    R.at(0, 0) = s.x;
    R.at(1, 0) = s.y;
    R.at(2, 0) = s.z;
    R.at(0, 1) = u.x;
    R.at(1, 1) = u.y;
    R.at(2, 1) = u.z;
    R.at(0, 2) = f.x;
    R.at(1, 2) = f.y;
    R.at(2, 2) = f.z;
    R.at(3, 0) = -dot3f(s, eye);
    R.at(3, 1) = -dot3f(u, eye);
    R.at(3, 2) = -dot3f(f, eye);
    return R;
}

// glm::orthoLH_ZO.
inline Mat4 ortho_lh_zo(float l, float r, float b, float t, float n, float f) {
    Mat4 R = mat_identity();
    R.at(0, 0) = 2.0f / (r - l);
    R.at(1, 1) = 2.0f / (t - b);
    R.at(2, 2) = 1.0f / (f - n);
    R.at(3, 0) = -(r + l) / (r - l);
    R.at(3, 1) = -(t + b) / (t - b);
    R.at(3, 2) = -n / (f - n);
    return R;
}

// Voxelizer::setViewProjection for the extended region (min - 1, extent + 2).
inline void voxel_view_proj(const Region& region, Mat4 out[3]) {
    int mn[3];
    float ext[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = region.min_corner[a] - 1;
        ext[a] = (float)(region.extent[a] + 2u);
    }
    const float vs = region.voxel_size;
    V3<float> rg(ext[0] * vs, ext[1] * vs, ext[2] * vs);
    V3<float> mcg((float)mn[0] * vs, (float)mn[1] * vs, (float)mn[2] * vs);
    V3<float> eye(mcg.x + 0.0f, mcg.y + 0.0f, mcg.z + rg.z);
    out[0] = mat_mul4(ortho_lh_zo(-rg.z, rg.z, -rg.y, rg.y, 0.1f, rg.x),
                      look_at_lh(eye, V3<float>(eye.x + 1.0f, eye.y + 0.0f, eye.z + 0.0f), V3<float>(0.f, 1.f, 0.f)));
    out[1] = mat_mul4(ortho_lh_zo(-rg.x, rg.x, -rg.z, rg.z, 0.1f, rg.y),
                      look_at_lh(eye, V3<float>(eye.x + 0.0f, eye.y + 1.0f, eye.z + 0.0f), V3<float>(0.f, 0.f, -1.f)));
    out[2] = mat_mul4(ortho_lh_zo(-rg.x, rg.x, -rg.y, rg.y, 0.1f, rg.z),
                      look_at_lh(mcg, V3<float>(mcg.x + 0.0f, mcg.y + 0.0f, mcg.z + 1.0f), V3<float>(0.f, 1.f, 0.f)));
}

// Voxelizer::cmdVoxelize's VoxelizationDesc (Voxelizer.cpp:330-354).
struct VoxDesc {
    float region_min[3];
    uint32_t clip_level;
    float region_max[3];
    float clip_max_extent;
    float prev_min[3];
    float voxel_size;
    float prev_max[3];
    int32_t clipmap_resolution;
};

inline VoxDesc voxelization_desc(const Region* regions, int level, int R) {
    VoxDesc d{};
    const Region& r = regions[level];
    for (int a = 0; a < 3; ++a) {
        d.region_min[a] = (float)r.min_corner[a] * r.voxel_size - 1e-6f;
        d.region_max[a] = (float)(r.min_corner[a] + (int32_t)r.extent[a]) * r.voxel_size + 1e-6f;
    }
    d.clip_level = (uint32_t)level;
    d.clip_max_extent = (float)r.extent[0] * r.voxel_size;
    d.voxel_size = r.voxel_size;
    if (level > 0) {
        const Region& p = regions[level - 1];
        for (int a = 0; a < 3; ++a) {
            d.prev_min[a] = (float)p.min_corner[a] * p.voxel_size;
            d.prev_max[a] = (float)(p.min_corner[a] + (int32_t)p.extent[a]) * p.voxel_size;
        }
    }
    d.clipmap_resolution = R;
    return d;
}

// DirectionalLight::setTransform (DirectionalLight.cpp:21-47): ortho half extent
// 16, near/far from the light (defaults 0.1 / 30).
inline void light_shadow_desc(const float origin[3], const float direction[3], float z_near, float z_far,
                              ShadowDesc& out) {
    V3<float> o(origin[0], origin[1], origin[2]);
    V3<float> d = normalize3f(V3<float>(direction[0], direction[1], direction[2]));
    Mat4 view = look_at_lh(o, V3<float>(o.x + d.x, o.y + d.y, o.z + d.z), V3<float>(0.f, 1.f, 0.f));
    Mat4 proj = ortho_lh_zo(-16.0f, 16.0f, -16.0f, 16.0f, z_near, z_far);
    std::memcpy(out.view, view.m, sizeof(view.m));
    std::memcpy(out.proj, proj.m, sizeof(proj.m));
    out.z_near = z_near;
    out.z_far = z_far;
}

// ------------------------------------------------------------------ scene
struct Material {  // GltfShadeMaterial (gltf.glsl:8-26)
    float base_color_factor[4];
    int32_t base_color_texture;
    float metallic_factor, roughness_factor;
    int32_t metallic_roughness_texture, emissive_texture, alpha_mode;
    float alpha_cutoff;
    int32_t double_sided;
    float emissive_factor[3];
    int32_t normal_texture;
    float normal_texture_scale;
    int32_t occlusion_texture;
    float occlusion_texture_strength;
    int32_t padding;
};

struct SceneView {
    const float* positions;
    const float* normals;
    const uint32_t* indices;
    int64_t vertex_count, triangle_count;
    const uint32_t* triangle_material;
    const Material* materials;
    int32_t material_count;
    const uint32_t* textures;  // 1x1 RGBA8 texels
    int32_t texture_count;
    const float* node_matrices;  // model (16) + itModel (16) per instance, column-major
    const uint32_t* triangle_instance;
    int32_t instance_count;
};

struct WorldTri {
    V3<float> p[3], n[3];
    uint32_t material;
};

inline WorldTri world_triangle(const SceneView& s, int64_t t) {
    WorldTri w;
    // instance and vertex indices clamped to the arrays, as the CUDA path does
    const uint32_t inst =
        s.triangle_instance ? std::min<uint32_t>(s.triangle_instance[t], (uint32_t)std::max(s.instance_count - 1, 0)) : 0u;
    const uint32_t vmax = (uint32_t)std::max<int64_t>(s.vertex_count - 1, 0);
    Mat4 model = mat_identity(), it = mat_identity();
    if (s.node_matrices) {
        std::memcpy(model.m, s.node_matrices + 32 * (int64_t)inst, 64);
        std::memcpy(it.m, s.node_matrices + 32 * (int64_t)inst + 16, 64);
    }
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = std::min(s.indices[3 * t + k], vmax);
        const float* p = s.positions + 3 * (int64_t)vi;
        const float* n = s.normals + 3 * (int64_t)vi;
        if (s.node_matrices) {
            V4<float> wp = mat_vec4(model, p[0], p[1], p[2], 1.0f);
            V4<float> wn = mat_vec4(it, n[0], n[1], n[2], 0.0f);
            w.p[k] = V3<float>(wp.x, wp.y, wp.z);
            w.n[k] = V3<float>(wn.x, wn.y, wn.z);
        } else {  // identity NodeMatrix: the product returns the inputs
            w.p[k] = V3<float>(p[0], p[1], p[2]);
            w.n[k] = V3<float>(n[0], n[1], n[2]);
        }
    }
    w.material = s.triangle_material ? s.triangle_material[t] : 0u;
    return w;
}

// getDominantAxis (msaaVoxelizer.geom:27-32).
inline int dominant_axis(const V3<float> p[3]) {
    V3<float> e1(p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z);
    V3<float> e2(p[2].x - p[0].x, p[2].y - p[0].y, p[2].z - p[0].z);
    V3<float> c = cross3(e1, e2);
    float nx = std::fabs(c.x), ny = std::fabs(c.y), nz = std::fabs(c.z);
    return (nx > ny && nx > nz) ? 0 : ((ny > nz) ? 1 : 2);
}

// Texel of a 1x1 texture (any filter / lod returns it), RGBA8 -> float.
inline V4<float> texture_1x1(const SceneView& s, int32_t id) {
    if (!s.textures || id < 0 || id >= s.texture_count) return V4<float>(0.f, 0.f, 0.f, 0.f);
    return unpack_unorm<float>(s.textures[id]);
}

// ------------------------------------------------------------- rasteriser
static const int kSampleLoc8[8][2] = {{144, 80}, {112, 176}, {208, 144}, {80, 48},
                                      {48, 208}, {16, 112}, {176, 240}, {240, 16}};  // 1/256 pixel

struct RasterSetup {
    int64_t X[3], Y[3];
    float z[3];
    int order[3];  // original vertex index of each oriented vertex
    int64_t area;
    float inv_area;
    int px0, py0, px1, py1;  // inclusive pixel bbox, clipped to the viewport
    bool owned[3];
    bool ok;
};

inline int64_t snap256(float v) { return (int64_t)std::nearbyint(v * 256.0f); }

inline int64_t floor_div256(int64_t v) { return v >= 0 ? v / 256 : -((-v + 255) / 256); }

// clip-space (w = 1) vertex xyz -> oriented, snapped screen triangle.
inline RasterSetup raster_setup(const V4<float> c[3], int W, int H) {
    RasterSetup r{};
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    int64_t X[3], Y[3];
    for (int k = 0; k < 3; ++k) {
        X[k] = snap256(hw * c[k].x + hw);
        Y[k] = snap256(hh * c[k].y + hh);
    }
    int64_t area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
    r.ok = area != 0;
    if (!r.ok) return r;
    int o[3] = {0, 1, 2};
    if (area < 0) {
        o[1] = 2;
        o[2] = 1;
        area = -area;
    }
    for (int k = 0; k < 3; ++k) {
        r.X[k] = X[o[k]];
        r.Y[k] = Y[o[k]];
        r.z[k] = c[o[k]].z;
        r.order[k] = o[k];
    }
    r.area = area;
    r.inv_area = 1.0f / (float)area;
    for (int i = 0; i < 3; ++i) {  // edge i runs from vertex i+1 to vertex i+2
        const int a = (i + 1) % 3, b = (i + 2) % 3;
        const int64_t dy = r.Y[b] - r.Y[a], dx = r.X[b] - r.X[a];
        r.owned[i] = dy > 0 || (dy == 0 && dx > 0);
    }
    int64_t mnx = std::min(r.X[0], std::min(r.X[1], r.X[2])), mxx = std::max(r.X[0], std::max(r.X[1], r.X[2]));
    int64_t mny = std::min(r.Y[0], std::min(r.Y[1], r.Y[2])), mxy = std::max(r.Y[0], std::max(r.Y[1], r.Y[2]));
    int64_t px0 = floor_div256(mnx), px1 = floor_div256(mxx), py0 = floor_div256(mny), py1 = floor_div256(mxy);
    px0 = std::max<int64_t>(px0, 0);
    py0 = std::max<int64_t>(py0, 0);
    px1 = std::min<int64_t>(px1, W - 1);
    py1 = std::min<int64_t>(py1, H - 1);
    if (px0 > px1 || py0 > py1) {
        r.ok = false;
        return r;
    }
    r.px0 = (int)px0;
    r.py0 = (int)py0;
    r.px1 = (int)px1;
    r.py1 = (int)py1;
    return r;
}

// Coverage of sample S (in 1/256 pixel): the exact edge tests only.
inline bool raster_cover(const RasterSetup& r, int64_t sx, int64_t sy, int64_t e[3]) {
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, c = (i + 2) % 3;
        e[i] = (r.X[c] - r.X[a]) * (sy - r.Y[a]) - (r.Y[c] - r.Y[a]) * (sx - r.X[a]);
        if (e[i] < 0 || (e[i] == 0 && !r.owned[i])) return false;
    }
    return true;
}

// Barycentrics of a covered sample in the ORIGINAL vertex order and its
// depth; false if the depth clip rejects it.
inline bool raster_interp(const RasterSetup& r, const int64_t e[3], float b[3], float& z) {
    float bo[3];
    for (int i = 0; i < 3; ++i) bo[i] = (float)e[i] * r.inv_area;
    z = (bo[0] * r.z[0] + bo[1] * r.z[1]) + bo[2] * r.z[2];
    if (!(z >= 0.0f && z <= 1.0f)) return false;
    for (int i = 0; i < 3; ++i) b[r.order[i]] = bo[i];
    return true;
}

inline bool raster_test(const RasterSetup& r, int64_t sx, int64_t sy, float b[3], float& z) {
    int64_t e[3];
    return raster_cover(r, sx, sy, e) && raster_interp(r, e, b, z);
}

inline V3<float> interp3(const float b[3], const V3<float> v[3]) {
    return V3<float>((b[0] * v[0].x + b[1] * v[1].x) + b[2] * v[2].x, (b[0] * v[0].y + b[1] * v[1].y) + b[2] * v[2].y,
                     (b[0] * v[0].z + b[1] * v[1].z) + b[2] * v[2].z);
}

// Visit every covered sample of a set-up triangle in the pinned order.
template <class F>
inline void raster_visit(const RasterSetup& r, int nsamples, F&& frag) {
    for (int ty = r.py0; ty <= r.py1; ty += 8)
        for (int tx = r.px0; tx <= r.px1; tx += 8)
            for (int py = ty; py <= std::min(ty + 7, r.py1); ++py)
                for (int px = tx; px <= std::min(tx + 7, r.px1); ++px)
                    for (int s = 0; s < nsamples; ++s) {
                        int64_t sx, sy;
                        if (nsamples == 1) {
                            sx = (int64_t)px * 256 + 128;
                            sy = (int64_t)py * 256 + 128;
                        } else {
                            sx = (int64_t)px * 256 + kSampleLoc8[s][0];
                            sy = (int64_t)py * 256 + kSampleLoc8[s][1];
                        }
                        float b[3];
                        float z;
                        if (raster_test(r, sx, sy, b, z)) frag(px, py, s, b, z);
                    }
}

// ------------------------------------------------------- clipmap raster
// msaaVoxelizer.frag / msaaInjectRadiance.frag calculateImageCoords: clamp all
// three axes by the region's x bounds (float(vec3) takes .x), toroidal coord.
inline I3 clip_image_coords(const VoxDesc& d, V3<float> wp) {
    const float c = d.voxel_size * 0.25f;
    const float lo = d.region_min[0] + c, hi = d.region_max[0] - c;
    float p[3] = {std::min(std::max(wp.x, lo), hi), std::min(std::max(wp.y, lo), hi), std::min(std::max(wp.z, lo), hi)};
    const int R = d.clipmap_resolution;
    int ic[3];
    for (int a = 0; a < 3; ++a) {
        float q = p[a] / d.clip_max_extent;
        float f = q - std::floor(q);
        ic[a] = ((int)(f * (float)R)) % R;
    }
    I3 out;
    out.x = ic[0] + 1;
    out.y = ic[1] + 1 + (R + 2) * (int)d.clip_level;
    out.z = ic[2] + 1;
    return out;
}

// Clip-space vertices of a world triangle in the level's per-axis view.
inline int clip_vertices(const WorldTri& w, const Mat4 vp[3], V4<float> c[3]) {
    const int axis = dominant_axis(w.p);
    for (int k = 0; k < 3; ++k) c[k] = mat_vec4(vp[axis], w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
    return axis;
}

// Fragment filter of the toroidal update: per level, keep everything
// (unrestricted) or only the union of the level's slabs (per axis an interval
// [lo, hi], empty when lo > hi).
struct SlabFilter {
    uint32_t restricted = 0;
    float lo[6][3], hi[6][3];
    bool keeps(int level, V3<float> p) const {
        if (!((restricted >> level) & 1u)) return true;
        return (p.x >= lo[level][0] && p.x <= hi[level][0]) || (p.y >= lo[level][1] && p.y <= hi[level][1]) ||
               (p.z >= lo[level][2] && p.z <= hi[level][2]);
    }
};

// VoxelizationPass::onUpdate + msaaVoxelizer.* over the levels in `level_mask`.
inline void voxelize_opacity(const SceneView& s, int R, const Region regions[6], uint32_t* atlas, int level_mask,
                             const SlabFilter* filter = nullptr) {
    Atlas A(R);
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        WorldTri w = world_triangle(s, t);
        const Material& mat = s.materials[w.material];
        for (int level = 0; level < 6; ++level) {
            if (!((level_mask >> level) & 1)) continue;
            VoxDesc d = voxelization_desc(regions, level, R);
            Mat4 vp[3];
            voxel_view_proj(regions[level], vp);
            V4<float> c[3];
            clip_vertices(w, vp, c);
            RasterSetup rs = raster_setup(c, R + 2, R + 2);
            if (!rs.ok) continue;
            raster_visit(rs, 8, [&](int, int, int, const float* b, float) {
                V3<float> wp = interp3(b, w.p);
                if (wp.x < d.region_min[0] || wp.y < d.region_min[1] || wp.z < d.region_min[2] ||
                    wp.x > d.region_max[0] || wp.y > d.region_max[1] || wp.z > d.region_max[2])
                    return;
                if (filter && !filter->keeps(level, wp)) return;
                if (mat.occlusion_texture > -1 && texture_1x1(s, mat.occlusion_texture).x < 0.1f) return;
                I3 ic = clip_image_coords(d, wp);
                for (int f = 0; f < 6; ++f) atlas[A.index(ic.x + (R + 2) * f, ic.y, ic.z)] = 0xFFFFFFFFu;
            });
        }
    }
}

// -------------------------------------------------- conservative voxels
// The conservative voxelisation mode (an extension beside the MSAA voxeliser
// the reference runs): every voxel of a level's region that the triangle
// touches, by the triangle / box overlap test of M. Schwarz and H.-P. Seidel,
// "Fast parallel surface and solid voxelization on GPUs" (SIGGRAPH Asia 2010,
// section 3.1): the box overlaps the triangle's plane (the plane's values at
// the box's two critical corners differ in sign or vanish) and, in each of
// the three axis projections, lies on the inner side of every edge line
// shifted outward by the box's extent.  FP32 throughout, no contraction, in
// the level's voxel units u = p * (1 / voxel_size) - min_corner, the voxel
// (i, j, k) being the box [i, i+1] x [j, j+1] x [k, k+1]; the voxel is stored
// (opacity 1.0 in all six faces) at its toroidal texel, as msaaVoxelizer.frag
// stores.  Materials with an occlusion texture below 0.1 are skipped, as there.
struct ConsTri {
    float u[3][3];     // vertices in voxel units
    float n[3];        // (u1 - u0) x (u2 - u0)
    float d1, d2;      // plane offsets at the critical corners
    float ne[3][3][2]; // [projection xy, yz, zx][edge][2] edge normals
    float de[3][3];    // [projection][edge] offsets
    int lo[3], hi[3];  // voxel bounds in [0, R)
    bool ok;
};

inline float fmax0(float x) { return x > 0.0f ? x : 0.0f; }

inline ConsTri cons_setup(const V3<float> p[3], const Region& rg, int R) {
    ConsTri t;
    const float inv = 1.0f / rg.voxel_size;
    for (int k = 0; k < 3; ++k) {
        const float w[3] = {p[k].x, p[k].y, p[k].z};
        for (int a = 0; a < 3; ++a) t.u[k][a] = w[a] * inv - (float)rg.min_corner[a];
    }
    t.ok = true;
    for (int a = 0; a < 3; ++a) {
        const float mn = std::min(std::min(t.u[0][a], t.u[1][a]), t.u[2][a]);
        const float mx = std::max(std::max(t.u[0][a], t.u[1][a]), t.u[2][a]);
        const float fl = std::floor(mn), fh = std::floor(mx);
        t.lo[a] = fl < 0.0f ? 0 : (fl > (float)(R - 1) ? R : (int)fl);
        t.hi[a] = fh > (float)(R - 1) ? R - 1 : (fh < 0.0f ? -1 : (int)fh);
        if (t.lo[a] > t.hi[a]) t.ok = false;
    }
    float e0[3], e1[3];
    for (int a = 0; a < 3; ++a) {
        e0[a] = t.u[1][a] - t.u[0][a];
        e1[a] = t.u[2][a] - t.u[0][a];
    }
    t.n[0] = e0[1] * e1[2] - e0[2] * e1[1];
    t.n[1] = e0[2] * e1[0] - e0[0] * e1[2];
    t.n[2] = e0[0] * e1[1] - e0[1] * e1[0];
    float c[3], c2[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = t.n[a] > 0.0f ? 1.0f : 0.0f;
        c2[a] = 1.0f - c[a];
    }
    t.d1 = t.n[0] * (c[0] - t.u[0][0]) + t.n[1] * (c[1] - t.u[0][1]) + t.n[2] * (c[2] - t.u[0][2]);
    t.d2 = t.n[0] * (c2[0] - t.u[0][0]) + t.n[1] * (c2[1] - t.u[0][1]) + t.n[2] * (c2[2] - t.u[0][2]);
    // projection q onto axes (a0, a1), oriented by the sign of the normal's third component
    static const int kAx[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    for (int q = 0; q < 3; ++q) {
        const int a0 = kAx[q][0], a1 = kAx[q][1], a2 = kAx[q][2];
        const float sg = t.n[a2] >= 0.0f ? 1.0f : -1.0f;
        for (int e = 0; e < 3; ++e) {
            const float* v0 = t.u[e];
            const float* v1 = t.u[(e + 1) % 3];
            const float n0 = -(v1[a1] - v0[a1]) * sg, n1 = (v1[a0] - v0[a0]) * sg;
            t.ne[q][e][0] = n0;
            t.ne[q][e][1] = n1;
            t.de[q][e] = -(n0 * v0[a0] + n1 * v0[a1]) + fmax0(n0) + fmax0(n1);
        }
    }
    return t;
}

// The three tests assume the box lies in the triangle's bounding box (the
// loop visits only those boxes); the first line makes the decision standalone.
inline bool cons_overlap(const ConsTri& t, int i, int j, int k) {
    if (i < t.lo[0] || i > t.hi[0] || j < t.lo[1] || j > t.hi[1] || k < t.lo[2] || k > t.hi[2]) return false;
    const float p[3] = {(float)i, (float)j, (float)k};
    const float np = t.n[0] * p[0] + t.n[1] * p[1] + t.n[2] * p[2];
    if ((np + t.d1) * (np + t.d2) > 0.0f) return false;
    static const int kAx[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    for (int q = 0; q < 3; ++q)
        for (int e = 0; e < 3; ++e)
            if (t.ne[q][e][0] * p[kAx[q][0]] + t.ne[q][e][1] * p[kAx[q][1]] + t.de[q][e] < 0.0f) return false;
    return true;
}

inline void voxelize_conservative(const SceneView& s, int R, const Region regions[6], uint32_t* atlas,
                                  int level_mask) {
    Atlas A(R);
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        WorldTri w = world_triangle(s, t);
        const Material& mat = s.materials[w.material];
        if (mat.occlusion_texture > -1 && texture_1x1(s, mat.occlusion_texture).x < 0.1f) continue;
        for (int level = 0; level < 6; ++level) {
            if (!((level_mask >> level) & 1)) continue;
            const Region& rg = regions[level];
            const ConsTri ct = cons_setup(w.p, rg, R);
            if (!ct.ok) continue;
            for (int k = ct.lo[2]; k <= ct.hi[2]; ++k)
                for (int j = ct.lo[1]; j <= ct.hi[1]; ++j)
                    for (int i = ct.lo[0]; i <= ct.hi[0]; ++i) {
                        if (!cons_overlap(ct, i, j, k)) continue;
                        const int x = (((rg.min_corner[0] + i) % R) + R) % R + 1;
                        const int y = (((rg.min_corner[1] + j) % R) + R) % R + 1 + (R + 2) * level;
                        const int z = (((rg.min_corner[2] + k) % R) + R) % R + 1;
                        for (int f = 0; f < 6; ++f) atlas[A.index(x + (R + 2) * f, y, z)] = 0xFFFFFFFFu;
                    }
        }
    }
}

// The toroidal update of the opacity atlas (VoxelizationPass.cpp:127-141,
// 190-212 with fillRevoxelizationRegions' slabs): clear each slab at its
// wrapped corner, then voxelise the levels with slabs keeping only the
// fragments inside them; a slab spanning the whole region keeps the whole
// level.  Slab bounds as Voxelizer::cmdVoxelize would set them for the slab.
inline void voxelize_opacity_slabs(const SceneView& s, int R, const Region regions[6], uint32_t* atlas,
                                   const Region* slabs, const int32_t* levels, int n) {
    SlabFilter F;
    uint32_t changed = 0, full = 0;
    for (int l = 0; l < 6; ++l)
        for (int a = 0; a < 3; ++a) {
            F.lo[l][a] = 3.0e38f;
            F.hi[l][a] = -3.0e38f;
        }
    for (int i = 0; i < n; ++i) {
        const Region& sl = slabs[i];
        const int l = levels[i];
        changed |= 1u << l;
        int thin = -1;
        for (int a = 0; a < 3; ++a)
            if (sl.extent[a] != (uint32_t)R) thin = a;
        if (thin < 0) {
            full |= 1u << l;
        } else {
            const float vs = sl.voxel_size;
            F.lo[l][thin] = std::min(F.lo[l][thin], (float)sl.min_corner[thin] * vs - 1e-6f);
            F.hi[l][thin] = std::max(F.hi[l][thin], (float)(sl.min_corner[thin] + (int32_t)sl.extent[thin]) * vs + 1e-6f);
        }
        int32_t mn[3];
        for (int a = 0; a < 3; ++a) mn[a] = ((sl.min_corner[a] % R) + R) % R;
        clear_region(atlas, R, mn, sl.extent, l, 6);
    }
    F.restricted = 0x3Fu & ~full;
    voxelize_opacity(s, R, regions, atlas, (int)changed, &F);
}

// RSM pass depth (reflectiveShadowPass.vert:40-50): gl_Position =
// (proj * view) * worldPos, one sample per pixel, depth test LESS, clear 1.0.
inline void shadow_depth(const SceneView& s, const ShadowDesc& sd, float* depth, int W, int H) {
    for (int64_t i = 0; i < (int64_t)W * H; ++i) depth[i] = 1.0f;
    Mat4 view, proj;
    std::memcpy(view.m, sd.view, 64);
    std::memcpy(proj.m, sd.proj, 64);
    Mat4 pv = mat_mul4(proj, view);
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        WorldTri w = world_triangle(s, t);
        V4<float> c[3];
        for (int k = 0; k < 3; ++k) c[k] = mat_vec4(pv, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
        RasterSetup rs = raster_setup(c, W, H);
        if (!rs.ok) continue;
        raster_visit(rs, 1, [&](int px, int py, int, const float*, float z) {
            float& d = depth[(int64_t)py * W + px];
            if (z < d) d = z;
        });
    }
}

// imageAtomicRGBA8Avg (msaaInjectRadiance.frag:185-201) executed without
// contention: the CAS succeeds first time iff the texel holds 0.
inline uint32_t rgba8_avg_fold(uint32_t cur, float vr, float vg, float vb, float va) {
    auto conv = [](float x, float y, float z, float w) {
        return (((uint32_t)w & 0xffu) << 24) | (((uint32_t)z & 0xffu) << 16) | (((uint32_t)y & 0xffu) << 8) |
               ((uint32_t)x & 0xffu);
    };
    if (cur == 0u) return conv(vr, vg, vb, va);
    float rx = (float)(cur & 0xffu), ry = (float)((cur >> 8) & 0xffu), rz = (float)((cur >> 16) & 0xffu),
          rw = (float)(cur >> 24);
    rx = rx * rw;
    ry = ry * rw;
    rz = rz * rw;
    float cx = rx + vr, cy = ry + vg, cz = rz + vb, cw = rw + va;
    cx = cx / cw;
    cy = cy / cw;
    cz = cz / cw;
    return conv(cx, cy, cz, cw);
}

// RadianceInjectionPass::onUpdate + msaaInjectRadiance.* (frag :68-155): one
// deterministic fold per covered sample in the pinned traversal order.
inline void inject_radiance(const SceneView& s, int R, const Region regions[6], const float* shadow, int sw, int sh,
                            const ShadowDesc& sd, const LightDesc& light, uint32_t* radiance, int level_mask) {
    Atlas A(R);
    const int rb = R + 2;
    V3<float> ldir = normalize3f(V3<float>(-light.direction[0], -light.direction[1], -light.direction[2]));
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        WorldTri w = world_triangle(s, t);
        const Material& mat = s.materials[w.material];
        for (int level = 0; level < 6; ++level) {
            if (!((level_mask >> level) & 1)) continue;
            VoxDesc d = voxelization_desc(regions, level, R);
            Mat4 vp[3];
            voxel_view_proj(regions[level], vp);
            V4<float> c[3];
            clip_vertices(w, vp, c);
            RasterSetup rs = raster_setup(c, rb, rb);
            if (!rs.ok) continue;
            raster_visit(rs, 8, [&](int, int, int, const float* b, float) {
                V3<float> wp = interp3(b, w.p);
                I3 ic = clip_image_coords(d, wp);
                if (mat.occlusion_texture > -1 && texture_1x1(s, mat.occlusion_texture).x < 0.1f) return;
                const bool emissive = mat.emissive_factor[0] > 0.0f || mat.emissive_factor[1] > 0.0f ||
                                      mat.emissive_factor[2] > 0.0f;
                if (emissive) {
                    float e[3] = {mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]};
                    if (mat.emissive_texture > -1) {
                        V4<float> tx = texture_1x1(s, mat.emissive_texture);
                        e[0] = e[0] + tx.x;
                        e[1] = e[1] + tx.y;
                        e[2] = e[2] + tx.z;
                    }
                    for (int k = 0; k < 3; ++k) e[k] = std::min(std::max(e[k], 0.0f), 1.0f) * 255.0f;
                    for (int f = 0; f < 6; ++f) {
                        uint32_t& cell = radiance[A.index(ic.x + rb * f, ic.y, ic.z)];
                        cell = rgba8_avg_fold(cell, e[0], e[1], e[2], 1.0f);
                    }
                    return;
                }
                V4<float> color(mat.base_color_factor[0], mat.base_color_factor[1], mat.base_color_factor[2],
                                mat.base_color_factor[3]);
                if (mat.base_color_texture > -1) {
                    V4<float> tx = texture_1x1(s, mat.base_color_texture);
                    color = V4<float>(color.x * tx.x, color.y * tx.y, color.z * tx.z, color.w * tx.w);
                }
                V3<float> nrm = normalize3f(interp3(b, w.n));
                float NdotL = std::min(std::max(dot3f(nrm, ldir), 0.001f), 1.0f);
                float vis = calc_visibility<float>(shadow, sw, sh, sd, wp);
                float lc[3];
                for (int k = 0; k < 3; ++k) lc[k] = 0.0f + NdotL * vis * light.color[k] * light.intensity;
                if (lc[0] == 0.0f && lc[1] == 0.0f && lc[2] == 0.0f) return;
                float rad[3] = {lc[0] * color.x * color.w, lc[1] * color.y * color.w, lc[2] * color.z * color.w};
                for (int k = 0; k < 3; ++k) rad[k] = std::min(std::max(rad[k], 0.0f), 1.0f);
                const int face[3] = {-nrm.x > 0.0f ? 0 : 1, -nrm.y > 0.0f ? 2 : 3, -nrm.z > 0.0f ? 4 : 5};
                const float wgt[3] = {std::fabs(nrm.x), std::fabs(nrm.y), std::fabs(nrm.z)};
                for (int k = 0; k < 3; ++k) {
                    uint32_t& cell = radiance[A.index(ic.x + rb * face[k], ic.y, ic.z)];
                    cell = rgba8_avg_fold(cell, rad[0] * wgt[k] * 255.0f, rad[1] * wgt[k] * 255.0f,
                                          rad[2] * wgt[k] * 255.0f, 1.0f);
                }
            });
        }
    }
}

// ------------------------------------------------------ SVO voxel fragments
// SparseVoxelizer (SparseVoxelizer.cpp:248-326) + voxelizer.{vert,geom,frag}:
// scene-bbox-normalised positions, dominant-axis projection to NDC with z = 1,
// res x res viewport.  The counter is incremented before the light discard, so
// a discarded fragment leaves its slot as the buffer held it (here: 0).
// Returns the fragment count (written slots + discarded slots).
inline int64_t svo_fragments(const SceneView& s, int octree_level, const float bb_min[3], const float bb_max[3],
                             const float* shadow, int sw, int sh, const ShadowDesc& sd, const LightDesc& light,
                             uint32_t* frags, int64_t capacity) {
    const int res = 1 << octree_level;
    V3<float> ext(bb_max[0] - bb_min[0], bb_max[1] - bb_min[1], bb_max[2] - bb_min[2]);
    const float ev = std::max(ext.x, std::max(ext.y, ext.z)) * 0.5f;
    V3<float> center((bb_min[0] + bb_max[0]) * 0.5f, (bb_min[1] + bb_max[1]) * 0.5f, (bb_min[2] + bb_max[2]) * 0.5f);
    V3<float> ldir = normalize3f(V3<float>(-light.direction[0], -light.direction[1], -light.direction[2]));
    int64_t cur = 0;
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        WorldTri w = world_triangle(s, t);
        const Material& mat = s.materials[w.material];
        V3<float> q[3], pos[3];
        for (int k = 0; k < 3; ++k) {
            q[k] = V3<float>((w.p[k].x - center.x) / ev, (w.p[k].y - center.y) / ev, (w.p[k].z - center.z) / ev);
            pos[k] = V3<float>((q[k].x + 1.0f) * 0.5f, (q[k].y + 1.0f) * 0.5f, (q[k].z + 1.0f) * 0.5f);
        }
        const int axis = dominant_axis(q);
        V4<float> c[3];
        for (int k = 0; k < 3; ++k) {
            float a = axis == 0 ? q[k].y : q[k].x;
            float bb = axis == 2 ? q[k].y : q[k].z;
            c[k] = V4<float>(a, bb, 1.0f, 1.0f);
        }
        RasterSetup rs = raster_setup(c, res, res);
        if (!rs.ok) continue;
        raster_visit(rs, 8, [&](int, int, int, const float* b, float) {
            if (mat.occlusion_texture > -1 && texture_1x1(s, mat.occlusion_texture).x < 0.1f) return;
            const int64_t slot = cur++;
            V3<float> fp = interp3(b, pos);
            float rad[4] = {1.0f, 1.0f, 1.0f, 1.0f};
            const bool emissive = mat.emissive_factor[0] > 0.0f || mat.emissive_factor[1] > 0.0f ||
                                  mat.emissive_factor[2] > 0.0f;
            if (emissive) {
                float e[3] = {mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]};
                if (mat.emissive_texture > -1) {
                    V4<float> tx = texture_1x1(s, mat.emissive_texture);
                    e[0] = e[0] + tx.x;
                    e[1] = e[1] + tx.y;
                    e[2] = e[2] + tx.z;
                }
                for (int k = 0; k < 3; ++k) rad[k] = std::min(std::max(e[k], 0.0f), 1.0f);
            } else {
                V4<float> color(0.f, 0.f, 0.f, 1.f);
                if (mat.base_color_texture > -1) {
                    V4<float> tx = texture_1x1(s, mat.base_color_texture);
                    color = V4<float>(tx.x * mat.base_color_factor[0], tx.y * mat.base_color_factor[1],
                                      tx.z * mat.base_color_factor[2], tx.w * mat.base_color_factor[3]);
                }
                V3<float> wp = interp3(b, w.p);
                V3<float> nrm = normalize3f(interp3(b, w.n));
                float NdotL = std::min(std::max(dot3f(nrm, ldir), 0.001f), 1.0f);
                float vis = calc_visibility<float>(shadow, sw, sh, sd, fp);
                (void)wp;
                float lc[3];
                for (int k = 0; k < 3; ++k) lc[k] = 0.0f + NdotL * vis * light.color[k] * light.intensity;
                if (lc[0] == 0.0f && lc[1] == 0.0f && lc[2] == 0.0f) return;
                float cc[3] = {color.x, color.y, color.z};
                for (int k = 0; k < 3; ++k) rad[k] = std::min(std::max(lc[k] * cc[k] * color.w, 0.0f), 1.0f);
                rad[3] = 1.0f;
            }
            uint32_t vx = (uint32_t)std::min(std::max(fp.x * (float)res, 0.0f), (float)res);
            uint32_t vy = (uint32_t)std::min(std::max(fp.y * (float)res, 0.0f), (float)res);
            uint32_t vz = (uint32_t)std::min(std::max(fp.z * (float)res, 0.0f), (float)res);
            uint32_t rgba = ((uint32_t)(rad[3] * 255.0f) & 0xffu) << 24 | ((uint32_t)(rad[2] * 255.0f) & 0xffu) << 16 |
                            ((uint32_t)(rad[1] * 255.0f) & 0xffu) << 8 | ((uint32_t)(rad[0] * 255.0f) & 0xffu);
            if (slot < capacity) {
                frags[2 * slot] = vx | (vy << 12) | ((vz & 0xffu) << 24);
                frags[2 * slot + 1] = ((vz >> 8) << 28) | (rgba & 0xfffffffu);
            }
        });
    }
    return cur;
}

}  // namespace vcto
