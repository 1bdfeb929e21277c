// gbuffer_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the camera and G-buffer producer of the reference:
//   * Camera::updateCamera (VFS/Camera.cpp:110-117): glm::lookAtLH,
//     glm::perspectiveLH_ZO(radians(fovy), aspect, 0.01, 5000) and the
//     CamMatrix block {P * V, inverse(V) * inverse(P), eye}; glm::inverse is
//     restated from glm 0.9.9's published cofactor algorithm
//     (glm/detail/func_matrix.inl, compute_inverse<4, 4>) in its evaluation
//     order; the result is pinned against glm itself by the golden vectors;
//   * GBufferPass (VFS/RenderPass/GBufferPass.cpp:80-160, 329; depth LESS
//     against a 1.0 clear, no culling) with gBufferPass.vert / .frag, under
//     the pinned rasteriser of raster_oracle.hpp at one centre sample per
//     pixel, after clipping each clip-space triangle to the near plane z >= 0
//     and the guard band |x|, |y| <= 16 w (Sutherland-Hodgman, fan from the
//     first vertex, at most 6 sub-triangles);
//   * the record the cone-tracing pass reads per pixel (vct_surface_sample):
//     world position from depth (voxelConeTracing.frag:305-311) and the
//     attachment texels after their formats (RGBA8 UNORM diffuse / specular,
//     RGBA16F normal / emission).
// Everything FP32 without contraction, in the order the CUDA path uses.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "clipmap_oracle.hpp"  // SurfaceSample
#include "raster_oracle.hpp"

namespace vcto {

// glm::radians then glm::perspectiveLH_ZO.
inline Mat4 perspective_lh_zo(float fovy, float aspect, float n, float f) {
    Mat4 R{};
    const float th = std::tan(fovy / 2.0f);
    R.at(0, 0) = 1.0f / (aspect * th);
    R.at(1, 1) = 1.0f / th;
    R.at(2, 2) = f / (f - n);
    R.at(2, 3) = 1.0f;
    R.at(3, 2) = -(f * n) / (f - n);
    return R;
}

// glm::inverse(mat4): adjugate from 2x2 minors of the lower rows, then a
// scale by 1 / det.  Written out entry by entry (m(c, r) = column c, row r).
inline Mat4 inverse4(const Mat4& M) {
    auto m = [&](int c, int r) { return M.at(c, r); };
    // minors of the row pair (r0, r1) over column pairs (2,3), (1,3), (1,2)
    auto minor = [&](int ca, int cb, int r0, int r1) { return m(ca, r0) * m(cb, r1) - m(cb, r0) * m(ca, r1); };
    const int rows[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
    float f23[6], f13[6], f12[6];
    for (int k = 0; k < 6; ++k) {
        f23[k] = minor(2, 3, rows[k][0], rows[k][1]);
        f13[k] = minor(1, 3, rows[k][0], rows[k][1]);
        f12[k] = minor(1, 2, rows[k][0], rows[k][1]);
    }
    // Fac_k as a 4-vector: (f23, f23, f13, f12)
    auto fac = [&](int k, int j) { return j < 2 ? f23[k] : (j == 2 ? f13[k] : f12[k]); };
    // Vec_r as a 4-vector: (m(1, r), m(0, r), m(0, r), m(0, r))
    auto vec = [&](int r, int j) { return j == 0 ? m(1, r) : m(0, r); };
    Mat4 I{};
    for (int j = 0; j < 4; ++j) {
        const float inv0 = (vec(1, j) * fac(0, j) - vec(2, j) * fac(1, j)) + vec(3, j) * fac(2, j);
        const float inv1 = (vec(0, j) * fac(0, j) - vec(2, j) * fac(3, j)) + vec(3, j) * fac(4, j);
        const float inv2 = (vec(0, j) * fac(1, j) - vec(1, j) * fac(3, j)) + vec(3, j) * fac(5, j);
        const float inv3 = (vec(0, j) * fac(2, j) - vec(1, j) * fac(4, j)) + vec(2, j) * fac(5, j);
        const float sa = (j & 1) ? -1.0f : 1.0f;  // SignA; SignB = -SignA
        I.at(0, j) = inv0 * sa;
        I.at(1, j) = inv1 * -sa;
        I.at(2, j) = inv2 * sa;
        I.at(3, j) = inv3 * -sa;
    }
    const float dot = (m(0, 0) * I.at(0, 0) + m(0, 1) * I.at(1, 0)) + (m(0, 2) * I.at(2, 0) + m(0, 3) * I.at(3, 0));
    const float s = 1.0f / dot;
    for (int i = 0; i < 16; ++i) I.m[i] = I.m[i] * s;
    return I;
}

struct CamMatrix {  // CamMatrix uniform block (144 B)
    float view_proj[16];
    float view_proj_inv[16];
    float eye[3];
    int32_t padding;
};

inline CamMatrix camera_matrix(const float pos[3], const float dir[3], const float up[3], float fovy_deg,
                               float aspect) {
    const V3<float> eye(pos[0], pos[1], pos[2]);
    const Mat4 view = look_at_lh(eye, V3<float>(eye.x + dir[0], eye.y + dir[1], eye.z + dir[2]),
                                 V3<float>(up[0], up[1], up[2]));
    const float fovy = fovy_deg * static_cast<float>(0.01745329251994329576923690768489);
    const Mat4 proj = perspective_lh_zo(fovy, aspect, 0.01f, 5000.0f);
    const Mat4 vp = mat_mul4(proj, view);
    const Mat4 vpi = mat_mul4(inverse4(view), inverse4(proj));
    CamMatrix c{};
    std::memcpy(c.view_proj, vp.m, 64);
    std::memcpy(c.view_proj_inv, vpi.m, 64);
    c.eye[0] = pos[0];
    c.eye[1] = pos[1];
    c.eye[2] = pos[2];
    return c;
}

// ------------------------------------------------------- homogeneous clip
struct ClipV {
    float x, y, z, w;
    float l[3];  // barycentrics in the original triangle
};

inline float clip_plane_dist(const ClipV& v, int plane) {
    const float g = 16.0f;
    if (plane == 0) return v.z;
    if (plane == 1) return v.x + g * v.w;
    if (plane == 2) return g * v.w - v.x;
    if (plane == 3) return v.y + g * v.w;
    return g * v.w - v.y;
}

// Clipped polygon of a clip-space triangle: returns the vertex count (0 or 3..8).
inline int clip_polygon(const V4<float> c[3], ClipV out[8]) {
    ClipV cur[8], nxt[8];
    int n = 3;
    for (int k = 0; k < 3; ++k) {
        cur[k] = ClipV{c[k].x, c[k].y, c[k].z, c[k].w, {0.0f, 0.0f, 0.0f}};
        cur[k].l[k] = 1.0f;
    }
    for (int plane = 0; plane < 5; ++plane) {
        bool inside = true;
        for (int k = 0; k < n; ++k) inside = inside && clip_plane_dist(cur[k], plane) >= 0.0f;
        if (inside) continue;
        int m = 0;
        for (int k = 0; k < n; ++k) {
            const ClipV& p = cur[k];
            const ClipV& q = cur[(k + 1) % n];
            const float dp = clip_plane_dist(p, plane), dq = clip_plane_dist(q, plane);
            if (dp >= 0.0f) nxt[m++] = p;
            if ((dp >= 0.0f) != (dq >= 0.0f)) {
                const float t = dp / (dp - dq);
                ClipV r;
                r.x = p.x + t * (q.x - p.x);
                r.y = p.y + t * (q.y - p.y);
                r.z = p.z + t * (q.z - p.z);
                r.w = p.w + t * (q.w - p.w);
                for (int i = 0; i < 3; ++i) r.l[i] = p.l[i] + t * (q.l[i] - p.l[i]);
                nxt[m++] = r;
            }
        }
        n = m;
        for (int k = 0; k < n; ++k) cur[k] = nxt[k];
        if (n < 3) return 0;
    }
    for (int k = 0; k < n; ++k) out[k] = cur[k];
    return n;
}

// ------------------------------------------------------------- G-buffer
inline float unorm8_texel(float x) {
    const float c = std::fmin(std::fmax(x, 0.0f), 1.0f);
    const uint32_t b = (uint32_t)std::floor(c * 255.0f + 0.5f);
    return (float)b / 255.0f;
}
inline float half_texel(float x) { return (float)(_Float16)x; }

inline void gbuffer(const SceneView& s, const CamMatrix& cam, int W, int H, SurfaceSample* out) {
    const int64_t npx = (int64_t)W * H;
    // visibility: closest fragment per pixel centre, first drawn on ties
    float* depth = new float[npx];
    int64_t* win_tri = new int64_t[npx];
    int* win_sub = new int[npx];
    float (*win_b)[3] = new float[npx][3];
    for (int64_t i = 0; i < npx; ++i) {
        depth[i] = 1.0f;
        win_tri[i] = -1;
    }
    Mat4 vp, vpi;
    std::memcpy(vp.m, cam.view_proj, 64);
    std::memcpy(vpi.m, cam.view_proj_inv, 64);
    for (int64_t t = 0; t < s.triangle_count; ++t) {
        const WorldTri w = world_triangle(s, t);
        const Material& mat = s.materials[w.material];
        V4<float> base(mat.base_color_factor[0], mat.base_color_factor[1], mat.base_color_factor[2],
                       mat.base_color_factor[3]);
        if (mat.base_color_texture > -1) {
            const V4<float> tx = texture_1x1(s, mat.base_color_texture);
            base = V4<float>(base.x * tx.x, base.y * tx.y, base.z * tx.z, base.w * tx.w);
        }
        if (mat.alpha_mode > 0 && base.w < mat.alpha_cutoff) continue;  // discard (1x1 textures: per material)
        V4<float> h[3];
        for (int k = 0; k < 3; ++k) h[k] = mat_vec4(vp, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
        ClipV poly[8];
        const int n = clip_polygon(h, poly);
        for (int sub = 0; sub + 2 < n; ++sub) {
            const ClipV* v[3] = {&poly[0], &poly[sub + 1], &poly[sub + 2]};
            V4<float> c[3];
            for (int k = 0; k < 3; ++k) c[k] = V4<float>(v[k]->x / v[k]->w, v[k]->y / v[k]->w, v[k]->z / v[k]->w, 1.0f);
            const RasterSetup rs = raster_setup(c, W, H);
            if (!rs.ok) continue;
            raster_visit(rs, 1, [&](int px, int py, int, const float* b, float z) {
                const int64_t i = (int64_t)py * W + px;
                if (z < depth[i]) {
                    depth[i] = z;
                    win_tri[i] = t;
                    win_sub[i] = sub;
                    for (int k = 0; k < 3; ++k) win_b[i][k] = b[k];
                }
            });
        }
    }
    // resolve
    for (int64_t i = 0; i < npx; ++i) {
        const int px = (int)(i % W), py = (int)(i / W);
        SurfaceSample& o = out[i];
        std::memset(&o, 0, sizeof(o));
        const float d = win_tri[i] >= 0 ? std::fabs(depth[i]) : 1.0f;  // -0 is recorded as +0
        o.diffuse_texel[3] = o.specular_texel[3] = 1.0f;  // the colour clear (0, 0, 0, 1)
        o.pad0 = o.pad1 = 1.0f;
        if (win_tri[i] >= 0) {
            const WorldTri w = world_triangle(s, win_tri[i]);
            V4<float> h[3];
            for (int k = 0; k < 3; ++k) h[k] = mat_vec4(vp, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
            ClipV poly[8];
            clip_polygon(h, poly);
            const int sub = win_sub[i];
            const ClipV* v[3] = {&poly[0], &poly[sub + 1], &poly[sub + 2]};
            // perspective-correct weights: b_k / w_k normalised, mapped to the original triangle
            float q[3];
            for (int k = 0; k < 3; ++k) q[k] = win_b[i][k] / v[k]->w;
            const float qs = (q[0] + q[1]) + q[2];
            for (int k = 0; k < 3; ++k) q[k] = q[k] / qs;
            float lam[3];
            for (int j = 0; j < 3; ++j) lam[j] = (q[0] * v[0]->l[j] + q[1] * v[1]->l[j]) + q[2] * v[2]->l[j];
            const V3<float> nrm = normalize3f(interp3(lam, w.n));
            const Material& mat = s.materials[w.material];
            float rough = mat.roughness_factor, metal = mat.metallic_factor;
            if (mat.metallic_roughness_texture > -1) {
                const V4<float> mr = texture_1x1(s, mat.metallic_roughness_texture);
                rough = rough * mr.y;
                metal = metal * mr.z;
            } else {
                rough = std::fmin(std::fmax(rough, 0.04f), 1.0f);
                metal = std::fmin(std::fmax(metal, 0.0f), 1.0f);
            }
            float base[3] = {mat.base_color_factor[0], mat.base_color_factor[1], mat.base_color_factor[2]};
            if (mat.base_color_texture > -1) {
                const V4<float> tx = texture_1x1(s, mat.base_color_texture);
                base[0] = base[0] * tx.x;
                base[1] = base[1] * tx.y;
                base[2] = base[2] * tx.z;
            }
            const float one_minus_f0 = 1.0f - 0.04f;
            for (int k = 0; k < 3; ++k) {
                const float diff = base[k] * one_minus_f0 * (1.0f - metal);
                const float spec = 0.04f * (1.0f - metal) + base[k] * metal;  // mix(f0, base, metallic)
                o.diffuse_texel[k] = unorm8_texel(diff);
                o.specular_texel[k] = unorm8_texel(spec);
            }
            o.diffuse_texel[3] = unorm8_texel(rough);
            o.specular_texel[3] = unorm8_texel(metal);
            const float nn[3] = {nrm.x, nrm.y, nrm.z};
            for (int k = 0; k < 3; ++k) o.normal_texel[k] = half_texel(nn[k] * 0.5f + 0.5f);
            float em[3] = {mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]};
            if (mat.emissive_texture > -1) {
                const V4<float> tx = texture_1x1(s, mat.emissive_texture);
                const float t3[3] = {tx.x, tx.y, tx.z};
                for (int k = 0; k < 3; ++k) em[k] = em[k] * std::pow(t3[k], 2.2f);
            }
            for (int k = 0; k < 3; ++k) o.emission_texel[k] = half_texel(em[k]);
        }
        // worldPosFromDepth at the pixel centre
        const float u = ((float)px + 0.5f) / (float)W, vv = ((float)py + 0.5f) / (float)H;
        const V4<float> wp = mat_vec4(vpi, u * 2.0f - 1.0f, vv * 2.0f - 1.0f, d, 1.0f);
        o.position[0] = wp.x / wp.w;
        o.position[1] = wp.y / wp.w;
        o.position[2] = wp.z / wp.w;
        o.depth = d;
    }
    delete[] depth;
    delete[] win_tri;
    delete[] win_sub;
    delete[] win_b;
}

}  // namespace vcto
