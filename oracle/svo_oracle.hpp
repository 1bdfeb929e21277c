// svo_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the sparse-voxel-octree build of the reference
// (OctreeBuilder::cmdBuild, VFS/RenderPass/Octree/OctreeBuilder.cpp:205-345)
// and its six compute shaders:
//   octreeNodeInit.comp:15-24, octreeNodeFlag.comp:20-47,
//   octreeNodeAlloc.comp:20-34, octreeNodeModifyArg.comp:22-27,
//   octreeNodeLeafWrite.comp:26-89, octreeNodeMipmapWrite.comp:26-96.
// Node pool: uint2 per node, x = MSB flag | child block index, y = RGBA8.
// Node allocation is the sequential order of the atomic counter when the
// flagged nodes of a window are visited in index order (the canonical
// breadth-first order); the reference's racy allocation differs from it only by
// a relabelling of child blocks.
#pragma once

#include <cstdint>
#include <vector>

#include "raster_oracle.hpp"

namespace vcto {

struct SvoPos {
    uint32_t x, y, z;
};

// Packed fragment -> position, halved (the shaders' ">> 1", octreeNodeFlag.comp:28-32).
inline SvoPos svo_frag_pos(const uint32_t* f) {
    SvoPos p;
    p.x = (f[0] & 0xfffu) >> 1;
    p.y = ((f[0] >> 12) & 0xfffu) >> 1;
    p.z = (((f[0] >> 24) & 0xffu) | ((f[1] >> 20) & 0xf00u)) >> 1;
    return p;
}

// The shared descent: returns idx; `res_out` receives the final resolution.
// stop(res) decides whether to continue after a step: the loop runs
// "do { ... } while (cur != 0 && res > limit)".
inline uint32_t svo_descend(const uint32_t* pool, SvoPos p, uint32_t resolution, uint32_t limit, uint32_t& res_out) {
    uint32_t idx = 0, cur = 0;
    do {
        resolution >>= 1;
        const uint32_t cx = p.x >= resolution, cy = p.y >= resolution, cz = p.z >= resolution;
        idx = cur + (cz | (cx << 1) | (cy << 2));
        cur = pool[2 * (uint64_t)idx] & 0x7fffffffu;
        p.x -= cx * resolution;
        p.y -= cy * resolution;
        p.z -= cz * resolution;
    } while (cur != 0u && resolution > limit);
    res_out = resolution;
    return idx;
}

// Top-down subdivision (cmdNodeSubdivision).  Returns 0, or -1 if the pool
// capacity would be exceeded (the reference writes out of bounds there).
inline int svo_subdivide(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool, int64_t capacity,
                         int64_t* node_count) {
    const uint32_t res = 1u << octree_level;
    uint64_t begin = 0, num = 8, counter = 0;
    if (capacity < 8) return -1;
    for (int i = 1; i <= octree_level; ++i) {
        if (begin + num > (uint64_t)capacity) return -1;
        for (uint64_t k = begin; k < begin + num; ++k) pool[2 * k] = pool[2 * k + 1] = 0u;  // Init
        for (int64_t f = 0; f < F; ++f) {                                                   // Flag
            uint32_t r;
            uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, 1u, r);
            pool[2 * (uint64_t)idx] |= 0x80000000u;
        }
        if (i != octree_level) {
            for (uint64_t k = begin; k < begin + num; ++k) {  // Alloc
                if (pool[2 * k] & 0x80000000u) {
                    const uint64_t c = counter++;
                    pool[2 * k] = (uint32_t)((c + 1) << 3) | 0x80000000u;
                    pool[2 * k + 1] = 0u;
                }
            }
            begin += num;  // ModifyArg
            num = counter * 8 + 8 - begin;
        }
    }
    *node_count = (int64_t)(counter * 8 + 8);
    return 0;
}

// octreeNodeLeafWrite.comp: RGBA8 running average of the 28-bit fragment
// colour (alpha 15 per fragment, wrapping at 256) into each reached leaf.
inline void svo_leaf_write(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool) {
    const uint32_t res = 1u << octree_level;
    for (int64_t f = 0; f < F; ++f) {
        uint32_t r;
        uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, 1u, r);
        if (r == 1u) {
            const uint32_t v = frags[2 * f + 1] & 0xfffffffu;
            uint32_t& cell = pool[2 * (uint64_t)idx + 1];
            cell = rgba8_avg_fold(cell, (float)(v & 0xffu), (float)((v >> 8) & 0xffu), (float)((v >> 16) & 0xffu),
                                  (float)(v >> 24));
        }
    }
}

// octreeNodeMipmapWrite.comp for targetLevel = 2..L: the descent stops when
// resolution <= targetLevel and writes only if resolution == targetLevel, so
// only power-of-two target levels below the root resolution produce mips.
inline void svo_mip_write(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool) {
    const uint32_t res = 1u << octree_level;
    for (int target = 2; target <= octree_level; ++target) {
        for (int64_t f = 0; f < F; ++f) {
            uint32_t r;
            uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, (uint32_t)target, r);
            if (r == (uint32_t)target) {
                const uint32_t child = pool[2 * (uint64_t)idx] & 0x7fffffffu;
                float s[4] = {0.f, 0.f, 0.f, 0.f};
                for (int j = 0; j < 8; ++j) {
                    const uint32_t v = pool[2 * ((uint64_t)child + j) + 1];
                    for (int c = 0; c < 4; ++c) s[c] = s[c] + (float)((v >> (8 * c)) & 0xffu) / 8.0f;
                }
                pool[2 * (uint64_t)idx + 1] = (((uint32_t)s[3] & 0xffu) << 24) | (((uint32_t)s[2] & 0xffu) << 16) |
                                              (((uint32_t)s[1] & 0xffu) << 8) | ((uint32_t)s[0] & 0xffu);
            }
        }
    }
}

}  // namespace vcto

namespace vcto {

// ------------------------------------------------------------ SVO cone trace
// voxelConeTracing_Octree.frag:148-461.  sampleSVO normalises the position by
// a fixed scene box (the shader hard-codes Sponza's, :321-322) and descends the
// pool with uVolumeDimension as the root resolution (256 in the pass,
// OctreeVoxelConeTracing.cpp:93) -- without the builder's ">> 1".
struct SvoTraceScene {
    const uint32_t* pool;
    float bb_min[3], bb_max[3];
};

template <class T>
struct SvoTracer {
    const TraceDesc& d;
    SvoTraceScene S;
    uint64_t steps = 0;

    V4<T> sample_svo(V3<T> p, uint32_t level) const {
        T ext[3] = {T(S.bb_max[0]) - T(S.bb_min[0]), T(S.bb_max[1]) - T(S.bb_min[1]), T(S.bb_max[2]) - T(S.bb_min[2])};
        T ev = std::max(ext[0], std::max(ext[1], ext[2])) * T(0.5);
        T c[3] = {(T(S.bb_min[0]) + T(S.bb_max[0])) * T(0.5), (T(S.bb_min[1]) + T(S.bb_max[1])) * T(0.5),
                  (T(S.bb_min[2]) + T(S.bb_max[2])) * T(0.5)};
        uint32_t resolution = (uint32_t)d.volume_dimension;
        T pp[3] = {p.x, p.y, p.z};
        uint32_t fp[3];
        for (int a = 0; a < 3; ++a) {
            T s = (pp[a] - c[a]) / ev;
            T u = ((s + T(1)) * T(0.5)) * T(resolution);
            u = std::max(u, T(0));  // float -> uint of a negative value: 0
            uint32_t q = (uint32_t)std::min(u, T(4294967040.0));
            fp[a] = std::min(q, resolution);
        }
        const uint32_t target = 1u << level;
        uint32_t idx = 0, cur = 0;
        do {
            resolution >>= 1;
            uint32_t cx = fp[0] >= resolution, cy = fp[1] >= resolution, cz = fp[2] >= resolution;
            idx = cur + (cz | (cx << 1) | (cy << 2));
            cur = S.pool[2 * (uint64_t)idx] & 0x7fffffffu;
            fp[0] -= cx * resolution;
            fp[1] -= cy * resolution;
            fp[2] -= cz * resolution;
        } while (cur != 0u && resolution > target);
        uint32_t v = S.pool[2 * (uint64_t)idx + 1];
        return V4<T>(T(v & 0xffu) / T(255), T((v >> 8) & 0xffu) / T(255), T((v >> 16) & 0xffu) / T(255),
                     T(v >> 24) / T(255));
    }

    V4<T> sample_svo_linear(V3<T> p, T level) const {
        uint32_t lo = (uint32_t)std::floor(level), hi = (uint32_t)std::ceil(level);
        V4<T> a = sample_svo(p, lo), b = sample_svo(p, hi);
        T f = fractv(level);
        return V4<T>(mixv(a.x, b.x, f), mixv(a.y, b.y, f), mixv(a.z, b.z, f), mixv(a.w, b.w, f));
    }

    V4<T> trace_cone(V3<T> start, V3<T> dir, T aperture, T max_dist, T start_level, T step_factor) {
        V4<T> result(T(0));
        const T uvs = T(d.voxel_size);
        const T cone_coef = T(2) * std::tan(aperture * T(0.5));
        T cur_level = start_level;
        T vs = uvs * std::exp2(cur_level);
        start = start + dir * (vs * T(d.trace_start_offset) * T(0.5));
        T step = T(0), diameter = std::max(step * cone_coef, uvs), occlusion = T(0), seg = vs;
        const T min_radius = uvs * T(d.volume_dimension) * T(0.5);
        const V3<T> center(T(d.volume_center[0]), T(d.volume_center[1]), T(d.volume_center[2]));
        while (step < max_dist && occlusion < T(1)) {
            ++steps;
            V3<T> pos = start + dir * step;
            T dist = length(center - pos);
            T min_level = std::ceil(std::log2(dist / min_radius));
            cur_level = std::log2(diameter / uvs);
            cur_level = std::min(std::max(std::max(start_level, cur_level), min_level), T(kClipLevels - 1));
            V4<T> s = sample_svo_linear(pos, cur_level);
            vs = uvs * std::exp2(cur_level);
            T correction = seg / vs;
            V3<T> radiance(s.x * correction, s.y * correction, s.z * correction);
            // base of pow clamped at 0, as in the clipmap tracer
            T opacity = clampv(T(1) - std::pow(std::max(T(1) - s.w, T(0)), correction), T(0), T(1));
            T k = clampv(T(1) - result.w, T(0), T(1));
            result = V4<T>(result.x + k * radiance.x, result.y + k * radiance.y, result.z + k * radiance.z,
                           result.w + k * opacity);
            occlusion = occlusion + (T(1) - occlusion) * opacity / (T(1) + (step + vs) * T(d.occlusion_decay));
            T prev = step;
            step = step + std::max(diameter, uvs) * step_factor;
            seg = step - prev;
            diameter = step * cone_coef;
        }
        return V4<T>(clampv(result.x, T(0), T(1)), clampv(result.y, T(0), T(1)), clampv(result.z, T(0), T(1)),
                     clampv(T(1) - occlusion, T(0), T(1)));
    }
};

// main() of voxelConeTracing_Octree.frag (:148-300).
template <class T>
inline bool trace_sample_svo(SvoTracer<T>& tr, const float eye[3], const float* shadow, int sw, int sh,
                             const ShadowDesc& sd, const LightDesc& light, const SurfaceSample& s, T out_d[4],
                             T out_s[4]) {
    const TraceDesc& d = tr.d;
    if (T(s.depth) == T(1)) return false;
    V3<T> wp(T(s.position[0]), T(s.position[1]), T(s.position[2]));
    V3<T> view = normalize(V3<T>(T(eye[0]), T(eye[1]), T(eye[2])) - wp);
    V3<T> diffuse_color(T(s.diffuse_texel[0]), T(s.diffuse_texel[1]), T(s.diffuse_texel[2]));
    T rough = T(s.diffuse_texel[3]);
    V3<T> normal = normalize(V3<T>(T(s.normal_texel[0]) * T(2) - T(1), T(s.normal_texel[1]) * T(2) - T(1),
                                   T(s.normal_texel[2]) * T(2) - T(1)));
    V3<T> spec(T(s.specular_texel[0]), T(s.specular_texel[1]), T(s.specular_texel[2]));
    T metallic = T(s.specular_texel[3]);
    V3<T> emission(T(s.emission_texel[0]), T(s.emission_texel[1]), T(s.emission_texel[2]));
    bool has_emission = emission.x > T(0) || emission.y > T(0) || emission.z > T(0);

    // calcMinLevel: same as the clipmap tracer
    const V3<T> center(T(d.volume_center[0]), T(d.volume_center[1]), T(d.volume_center[2]));
    T dist = length(center - wp);
    T min_radius = T(d.voxel_size) * T(d.volume_dimension) * T(0.5);
    T ml = std::max(std::log2(dist / min_radius), T(0));
    T radius = min_radius * std::exp2(std::ceil(ml));
    T f = dist / radius;
    T min_level = f > T(0.5) ? std::ceil(ml) + (f - T(0.5)) * (T(1) / (T(1) - T(0.5))) : std::ceil(ml);

    T vs = T(d.voxel_size) * std::exp2(min_level);
    V3<T> start = wp + normal * (vs * T(d.trace_start_offset));
    V4<T> ind(T(0), T(0), T(0), T(1));
    T valid = T(0);
    const bool c32 = d.enable_32_cones != 0;
    const int n = c32 ? 32 : 16;
    const T aperture = T(c32 ? kAperture32 : kAperture16);
    const T sf = std::max(T(kMinTraceStepFactor), T(d.min_trace_step_factor));
    for (int i = 0; i < n; ++i) {
        const float* dd = c32 ? kDirs32[i] : kDirs16[i];
        V3<T> dir{T(dd[0]), T(dd[1]), T(dd[2])};
        T cos_t = dot(normal, dir);
        if (cos_t < T(0)) continue;
        V4<T> c = tr.trace_cone(start, dir, aperture, T(kMaxTraceDistance), min_level, sf);
        ind = ind + c * cos_t;
        valid = valid + cos_t;
    }
    ind = V4<T>(ind.x / valid, ind.y / valid, ind.z / valid, ind.w / valid);
    ind.w = ind.w * T(d.ambient_occlusion_factor);
    const T idi = T(d.indirect_diffuse_intensity);
    ind.x = ind.x * (diffuse_color.x * idi);
    ind.y = ind.y * (diffuse_color.y * idi);
    ind.z = ind.z * (diffuse_color.z * idi);
    ind = V4<T>(clampv(ind.x, T(0), T(1)), clampv(ind.y, T(0), T(1)), clampv(ind.z, T(0), T(1)), clampv(ind.w, T(0), T(1)));

    V3<T> ispec(T(0));
    if ((spec.x > T(1e-6f) || spec.y > T(1e-6f) || spec.z > T(1e-6f)) && metallic > T(1e-6f)) {
        V3<T> sdir = normalize(reflect(-view, normal));
        V4<T> c = tr.trace_cone(start, sdir, std::max(rough, T(kMinSpecularAperture)), T(kMaxTraceDistance), min_level,
                                std::max(T(kMinTraceStepFactor), T(d.voxel_size)));
        const T isi = T(d.indirect_specular_intensity);
        ispec = V3<T>(c.x * spec.x * isi, c.y * spec.y * isi, c.z * spec.z * isi);
    }
    V3<T> direct(T(0));
    if (has_emission) {
        direct = emission;
    } else {
        T alpha_r = rough * rough;
        T reflectance = std::max(std::max(spec.x, spec.y), spec.z);
        V3<T> r90(clampv(reflectance * T(50), T(0), T(1)));
        V3<T> l = normalize(-V3<T>(T(light.direction[0]), T(light.direction[1]), T(light.direction[2])));
        V3<T> h = normalize(l + view);
        T NdotL = clampv(dot(normal, l), T(0.001f), T(1));
        T NdotV = clampv(std::fabs(dot(normal, view)), T(0.001f), T(1));
        T NdotH = clampv(dot(normal, h), T(0), T(1));
        T VdotH = clampv(dot(view, h), T(0), T(1));
        T vis = calc_visibility<T>(shadow, sw, sh, sd, wp);
        direct = microfacet_brdf<T>(NdotL, NdotV, NdotH, VdotH, spec, r90, alpha_r, diffuse_color) * vis;
    }
    direct = V3<T>(clampv(direct.x, T(0), T(1)), clampv(direct.y, T(0), T(1)), clampv(direct.z, T(0), T(1)));

    V4<T> D(T(0), T(0), T(0), T(1)), Sp(T(0), T(0), T(0), T(1));
    switch (d.rendering_mode) {
        case 0: D = V4<T>(diffuse_color.x, diffuse_color.y, diffuse_color.z, T(1)); break;
        case 1: D = V4<T>(spec.x, spec.y, spec.z, T(1)); break;
        case 2: D = V4<T>(normal.x * T(0.5) + T(0.5), normal.y * T(0.5) + T(0.5), normal.z * T(0.5) + T(0.5), T(1)); break;
        case 3: {
            static const float colors[7][4] = {{1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {1, 1, 0, 1},
                                               {0, 1, 1, 1}, {1, 0, 1, 1}, {1, 1, 1, 1}};
            V4<T> c(T(0));
            for (int k = 0; k < 6; ++k)
                if (min_level < T(k + 1)) {
                    T fr = fractv(min_level);
                    c = V4<T>(mixv(T(colors[k][0]), T(colors[k + 1][0]), fr), mixv(T(colors[k][1]), T(colors[k + 1][1]), fr),
                              mixv(T(colors[k][2]), T(colors[k + 1][2]), fr), mixv(T(colors[k][3]), T(colors[k + 1][3]), fr));
                    break;
                }
            D = c * T(0.5);
            break;
        }
        case 4: direct = direct * ind.w; D = V4<T>(direct.x, direct.y, direct.z, T(1)); break;
        case 5: D = V4<T>(D.x + ind.x, D.y + ind.y, D.z + ind.z, T(1)); break;
        case 6: Sp = V4<T>(Sp.x + ispec.x, Sp.y + ispec.y, Sp.z + ispec.z, T(1)); break;
        case 7: D = V4<T>(ind.w, ind.w, ind.w, T(1)); break;
        default:
            direct = direct * ind.w;
            D = V4<T>(D.x + direct.x + ind.x, D.y + direct.y + ind.y, D.z + direct.z + ind.z, T(1));
            Sp = V4<T>(Sp.x + ispec.x, Sp.y + ispec.y, Sp.z + ispec.z, T(1));
            break;
    }
    out_d[0] = D.x; out_d[1] = D.y; out_d[2] = D.z; out_d[3] = D.w;
    out_s[0] = Sp.x; out_s[1] = Sp.y; out_s[2] = Sp.z; out_s[3] = Sp.w;
    return true;
}

}  // namespace vcto
