// clipmap_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's 3D-clipmap compute passes and the clipmap
// cone tracer.  Each function names the reference file:line it restates.
// Loops are plain and sequential per output element (OpenMP across output
// elements only where every element is written by exactly one iteration), so
// the RGBA8 results are a deterministic function of the inputs.
// Parity of this shader arithmetic with the reference's GLSL is unpinned (the
// passes need Vulkan, unavailable on this machine); the host math it uses is
// pinned against the reference's glm by tests/golden.
#pragma once

#include <cstdlib>

#include "oracle_common.hpp"

namespace vcto {

// ----------------------------------------------------------------- regions
// VoxelizationPass::createVoxelClipmap + calculateChangeDelta
// (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:335-357, 438-448) with the
// camera boxes of Application::updateClipRegionBoundingBox
// (VFS/Application.cpp:116-128); _clipMinChange = {2,2,2,2,2,1}
// (VFS/RenderPass/Clipmap/VoxelizationPass.h:57).
struct Region {
    int32_t min_corner[3];
    uint32_t extent[3];
    float voxel_size;
};

inline void clip_regions(const float cam[3], int R, int extent_l0, Region out[6]) {
    static const int kMinChange[6] = {2, 2, 2, 2, 2, 1};
    for (int l = 0; l < 6; ++l) {
        Region& r = out[l];
        const int half = R >> 1;
        for (int a = 0; a < 3; ++a) {
            r.min_corner[a] = -half;
            r.extent[a] = (uint32_t)R;
        }
        r.voxel_size = (float)((uint32_t)extent_l0 * (1u << l)) / (float)R;
        const float half_size = (float)((extent_l0 >> 1) * (1 << l));
        const float min_change = r.voxel_size * (float)kMinChange[l];
        for (int a = 0; a < 3; ++a) {
            const float bb_min = cam[a] - half_size;
            const float delta_w = bb_min - (float)r.min_corner[a] * r.voxel_size;
            const int32_t d = (int32_t)std::trunc(delta_w / min_change) * kMinChange[l];
            r.min_corner[a] += d;
        }
    }
}

// VoxelizationPass::fillRevoxelizationRegions + calculateChangeDelta
// (VoxelizationPass.cpp:438-494): move persistent regions by the snapped
// delta of their own corner; list the uncovered slabs (whole region when a
// delta reaches the extent).  Returns the slab count.
inline int update_clip_regions(Region regions[6], const float cam[3], int R, int extent_l0, Region slabs[18],
                               int32_t levels[18]) {
    static const int kMinChange[6] = {2, 2, 2, 2, 2, 1};
    int n = 0;
    for (int l = 0; l < 6; ++l) {
        Region& r = regions[l];
        const float half_size = (float)((extent_l0 >> 1) * (1 << l));
        const float min_change = r.voxel_size * (float)kMinChange[l];
        int32_t d[3];
        for (int a = 0; a < 3; ++a) {
            const float bb_min = cam[a] - half_size;
            const float delta_w = bb_min - (float)r.min_corner[a] * r.voxel_size;
            d[a] = (int32_t)std::trunc(delta_w / min_change) * kMinChange[l];
            r.min_corner[a] += d[a];
        }
        if (std::abs(d[0]) >= (int)r.extent[0] || std::abs(d[1]) >= (int)r.extent[1] ||
            std::abs(d[2]) >= (int)r.extent[2]) {
            slabs[n] = r;
            levels[n++] = l;
            continue;
        }
        for (int a = 0; a < 3; ++a) {
            if (std::abs(d[a]) < kMinChange[l]) continue;
            Region sl = r;
            sl.extent[a] = (uint32_t)std::abs(d[a]);
            if (d[a] > 0) sl.min_corner[a] = r.min_corner[a] + (int32_t)r.extent[a] - (int32_t)sl.extent[a];
            slabs[n] = sl;
            levels[n++] = l;
        }
    }
    (void)R;
    return n;
}

// ------------------------------------------------------------------ clear
// clipmapCleaning.comp:17-31 driven by ClipmapCleaner.cpp:93-133.
inline void clear_region(uint32_t* atlas, int R, const int32_t region_min[3], const uint32_t extent[3],
                         int level, int face_count) {
    Atlas A(R);
    const int rb = R + 2;
    for (uint32_t gz = 0; gz < extent[2]; ++gz)
        for (uint32_t gy = 0; gy < extent[1]; ++gy)
            for (uint32_t gx = 0; gx < extent[0]; ++gx) {
                // GLSL '%' of a non-negative ivec3 by an int.
                int px = ((int)gx + region_min[0]) % R + 1;
                int py = ((int)gy + region_min[1]) % R + 1 + level * rb;
                int pz = ((int)gz + region_min[2]) % R + 1;
                for (int f = 0; f < face_count; ++f) atlas[A.index(px + rb * f, py, pz)] = 0u;
            }
}

// -------------------------------------------------------------- copy alpha
// copyAlphaImage.comp:16-30 driven by CopyAlpha.cpp:92-146 (R^3 invocations).
inline void copy_alpha(uint32_t* dst, const uint32_t* src, int R, int level, int face_count) {
    Atlas A(R);
    const int rb = R + 2;
    for (int z = 0; z < R; ++z)
        for (int y = 0; y < R; ++y)
            for (int x = 0; x < R; ++x)
                for (int f = 0; f < face_count; ++f) {
                    int64_t i = A.index(x + 1 + rb * f, y + 1 + level * rb, z + 1);
                    dst[i] = (dst[i] & 0x00ffffffu) | (src[i] & 0xff000000u);
                }
}

// ---------------------------------------------------------------- border
// borderWrapping.comp:14-37 driven by BorderWrapper.cpp:123-151: the
// dispatch is ((R+2) >> 3) groups of 8 per axis and only invocations with a
// zero component write (index R+1 is never written).
inline void wrap_border(uint32_t* atlas, int R, int border_width_desc, int face_count, int region_count) {
    Atlas A(R);
    const int rwb = R + border_width_desc;  // resolutionWithBorder
    const int n = ((R + 2) >> 3) * 8;
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                if (x >= rwb || y >= rwb || z >= rwb) continue;
                if (x < R + 1 && y < R + 1 && z < R + 1 && x > 0 && y > 0 && z > 0) continue;
                int rx = ((x + R - 1) & (R - 1)) + 1, ry = ((y + R - 1) & (R - 1)) + 1, rz = ((z + R - 1) & (R - 1)) + 1;
                int wx = x, wy = y, wz = z;
                for (int i = 0; i < region_count; ++i) {
                    for (int j = 0; j < face_count; ++j)
                        atlas[A.index(wx + rwb * j, wy, wz)] = atlas[A.index(rx + rwb * j, ry, rz)];
                    ry += rwb;
                    wy += rwb;
                }
            }
}

// ------------------------------------------------------------- downsample
// opacityDownSample.comp:28-138 and radianceDownSample.comp:28-139 driven by
// DownSampler.cpp:115-168.  The radiance shader declares lerpFactor inside an
// if-block and reads it outside (it does not compile as written); the
// restatement uses the opacity shader's scoping (default 0, set in the band).
static const int kOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
// Per face: the 4 (front, back) pairs of the directional composite.
static const int kPairs[6][4][2] = {
    {{0, 1}, {2, 3}, {4, 5}, {6, 7}},  // +x
    {{1, 0}, {3, 2}, {5, 4}, {7, 6}},  // -x
    {{0, 2}, {1, 3}, {4, 6}, {5, 7}},  // +y
    {{2, 0}, {3, 1}, {6, 4}, {7, 5}},  // -y
    {{0, 4}, {1, 5}, {2, 6}, {3, 7}},  // +z
    {{4, 0}, {5, 1}, {6, 2}, {7, 3}},  // -z
};

// calculateImageCoords of the downsample shaders: (p + R*(|p/R|+1)) & (R-1).
inline int ds_wrap(int p, int R) { return (p + R * (std::abs(p / R) + 1)) & (R - 1); }

// Lerp factor of the blend band (opacityDownSample.comp:55-64); FP32.
inline float ds_lerp(const int cur[3], const int prev_min[3], int R, int band) {
    const int half = R >> 1;
    float dist[3];
    bool any_ge = false;
    for (int a = 0; a < 3; ++a) {
        float center = (float)(prev_min[a] >> 1) + (float)(half >> 1);
        dist[a] = std::fabs((float)cur[a] + 0.5f - center) - 0.5f;
        if (dist[a] >= (float)((half >> 1) - band)) any_ge = true;
    }
    float lerp = 0.0f;
    float inv = 1.0f / ((float)band + 1.0f);
    if (any_ge) {
        lerp = std::max(dist[0], std::max(dist[1], dist[2])) - (float)((half >> 1) - band) + 1.0f;
        lerp = lerp * inv;
    }
    return lerp;
}

// One level l (1..5) of the RGBA8 atlas, in place.  mode 0 = opacity, 1 = radiance.
inline void downsample(uint32_t* atlas, int R, const int prev_min[3], int level, int band, int mode) {
    Atlas A(R);
    const int half = R >> 1;
    const int rb = R + 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int gz = 0; gz < half; ++gz)
        for (int gy = 0; gy < half; ++gy)
            for (int gx = 0; gx < half; ++gx) {
                const int g[3] = {gx, gy, gz};
                int cur[3], wpos[3], pstart[3];
                for (int a = 0; a < 3; ++a) {
                    cur[a] = (prev_min[a] >> 1) + g[a];
                    wpos[a] = ds_wrap(cur[a], R) + 1;
                    pstart[a] = ds_wrap(cur[a] << 1, R);
                }
                wpos[1] += rb * level;
                int pp[8][3];
                for (int i = 0; i < 8; ++i) {
                    for (int a = 0; a < 3; ++a) pp[i][a] = pstart[a] + kOff[i][a] + 1;
                    pp[i][1] += rb * (level - 1);
                }
                const float lerp = ds_lerp(cur, prev_min, R, band);
                for (int f = 0; f < 6; ++f) {
                    V4<float> v[8];
                    for (int i = 0; i < 8; ++i) v[i] = unpack_unorm<float>(atlas[A.index(pp[i][0] + rb * f, pp[i][1], pp[i][2])]);
                    const int64_t wi = A.index(wpos[0] + rb * f, wpos[1], wpos[2]);
                    V4<float> own = unpack_unorm<float>(atlas[wi]);
                    if (mode == 0) {
                        // (a0 + (1-a0)*a1 + a2 + (1-a2)*a3 + ...) evaluated left to right.
                        float s = 0.0f;
                        for (int k = 0; k < 4; ++k) {
                            const V4<float>& a0 = v[kPairs[f][k][0]];
                            const V4<float>& a1 = v[kPairs[f][k][1]];
                            const float t = (1.0f - a0.w) * a1.w;
                            s = (k == 0) ? (a0.w + t) : ((s + a0.w) + t);
                        }
                        float res = s * 0.25f;
                        float a = mixv(res, own.x, lerp);
                        own.w = a;
                        own.y = a;
                        atlas[wi] = pack_unorm(own);
                    } else {
                        V4<float> s(0.0f);
                        for (int k = 0; k < 4; ++k) {
                            const V4<float>& a0 = v[kPairs[f][k][0]];
                            const V4<float>& a1 = v[kPairs[f][k][1]];
                            const float t = 1.0f - a0.w;
                            V4<float> b(t * a1.x, t * a1.y, t * a1.z, t * a1.w);
                            if (k == 0) s = V4<float>(a0.x + b.x, a0.y + b.y, a0.z + b.z, a0.w + b.w);
                            else s = V4<float>((s.x + a0.x) + b.x, (s.y + a0.y) + b.y, (s.z + a0.z) + b.z, (s.w + a0.w) + b.w);
                        }
                        V4<float> res = s * 0.25f;
                        V4<float> out(mixv(res.x, own.x, lerp), mixv(res.y, own.y, lerp), mixv(res.z, own.z, lerp),
                                      mixv(res.w, own.w, lerp));
                        atlas[wi] = pack_unorm(out);
                    }
                }
            }
}


// The same level downsample on float4 storage (no 8-bit quantisation),
// arithmetic in T: the error reference of the FP16-storage mips.  The texel
// store is a parameter: F4Store rounds every written value to float (the
// float atlas); the reference gradient instantiates it with a store of
// ad::Var values (adjoint_oracle.hpp).
struct F4Store {
    float* atlas4;
    static constexpr bool kParallel = true;
    template <class T> V4<T> load(int64_t t) const {
        const float* p = atlas4 + 4 * t;
        return V4<T>(T(p[0]), T(p[1]), T(p[2]), T(p[3]));
    }
    template <class T> void put(int64_t t, int c, T v) { atlas4[4 * t + c] = (float)v; }
};

template <class T, class Store>
inline void downsample_f4_on(Store& st, int R, const int prev_min[3], int level, int band, int mode) {
    Atlas A(R);
    const int half = R >> 1;
    const int rb = R + 2;
#pragma omp parallel for collapse(2) schedule(static) if (Store::kParallel)
    for (int gz = 0; gz < half; ++gz)
        for (int gy = 0; gy < half; ++gy)
            for (int gx = 0; gx < half; ++gx) {
                const int g[3] = {gx, gy, gz};
                int cur[3], wpos[3], pstart[3];
                for (int a = 0; a < 3; ++a) {
                    cur[a] = (prev_min[a] >> 1) + g[a];
                    wpos[a] = ds_wrap(cur[a], R) + 1;
                    pstart[a] = ds_wrap(cur[a] << 1, R);
                }
                wpos[1] += rb * level;
                const T lerp = T(ds_lerp(cur, prev_min, R, band));
                for (int f = 0; f < 6; ++f) {
                    V4<T> v[8];
                    for (int i = 0; i < 8; ++i)
                        v[i] = st.template load<T>(A.index(pstart[0] + kOff[i][0] + 1 + rb * f,
                                                           pstart[1] + kOff[i][1] + 1 + rb * (level - 1),
                                                           pstart[2] + kOff[i][2] + 1));
                    const int64_t o = A.index(wpos[0] + rb * f, wpos[1], wpos[2]);
                    V4<T> s(T(0));
                    for (int k = 0; k < 4; ++k) {
                        const V4<T>& a0 = v[kPairs[f][k][0]];
                        const V4<T>& a1 = v[kPairs[f][k][1]];
                        const T t = T(1) - a0.w;
                        s = V4<T>(s.x + a0.x + t * a1.x, s.y + a0.y + t * a1.y, s.z + a0.z + t * a1.z, s.w + a0.w + t * a1.w);
                    }
                    const V4<T> own = st.template load<T>(o);
                    if (mode == 0) {
                        T a = mixv(s.w * T(0.25), own.x, lerp);
                        st.put(o, 3, a);
                        st.put(o, 1, a);
                    } else {
                        st.put(o, 0, mixv(s.x * T(0.25), own.x, lerp));
                        st.put(o, 1, mixv(s.y * T(0.25), own.y, lerp));
                        st.put(o, 2, mixv(s.z * T(0.25), own.z, lerp));
                        st.put(o, 3, mixv(s.w * T(0.25), own.w, lerp));
                    }
                }
            }
}

template <class T>
inline void downsample_f4(float* atlas4, int R, const int prev_min[3], int level, int band, int mode) {
    F4Store st{atlas4};
    downsample_f4_on<T>(st, R, prev_min, level, band, mode);
}

// ----------------------------------------------------------- texture fetch
// Linear-filtered sampler3D lookup with REPEAT addressing and no mip chain
// (VoxelSampler, Voxelizer.cpp:279; the atlas has one mip level).  Vulkan's
// linear filter: u' = u * W - 0.5, i0 = floor(u'), alpha = frac(u'), i1 = i0+1,
// both wrapped; weights in T (no 8-bit hardware weight quantisation).
template <class T, class Fetch>
inline V4<T> texture3d(const Fetch& fetch, const Atlas& A, V3<T> uvw) {
    T u = uvw.x * T(A.W) - T(0.5), v = uvw.y * T(A.H) - T(0.5), w = uvw.z * T(A.D) - T(0.5);
    T fu = std::floor(u), fv = std::floor(v), fw = std::floor(w);
    T a = u - fu, b = v - fv, c = w - fw;
    int i0 = wrap_repeat((int)fu, A.W), i1 = wrap_repeat((int)fu + 1, A.W);
    int j0 = wrap_repeat((int)fv, A.H), j1 = wrap_repeat((int)fv + 1, A.H);
    int k0 = wrap_repeat((int)fw, A.D), k1 = wrap_repeat((int)fw + 1, A.D);
    V4<T> t000 = fetch(i0, j0, k0), t100 = fetch(i1, j0, k0), t010 = fetch(i0, j1, k0), t110 = fetch(i1, j1, k0);
    V4<T> t001 = fetch(i0, j0, k1), t101 = fetch(i1, j0, k1), t011 = fetch(i0, j1, k1), t111 = fetch(i1, j1, k1);
    auto lerp4 = [](V4<T> p, V4<T> q, T t) {
        return V4<T>(p.x + (q.x - p.x) * t, p.y + (q.y - p.y) * t, p.z + (q.z - p.z) * t, p.w + (q.w - p.w) * t);
    };
    V4<T> x00 = lerp4(t000, t100, a), x10 = lerp4(t010, t110, a), x01 = lerp4(t001, t101, a), x11 = lerp4(t011, t111, a);
    V4<T> y0 = lerp4(x00, x10, b), y1 = lerp4(x01, x11, b);
    return lerp4(y0, y1, c);
}

template <class T> struct Rgba8Fetch {
    const uint32_t* atlas;
    Atlas A;
    V4<T> operator()(int x, int y, int z) const { return unpack_unorm<T>(atlas[A.index(x, y, z)]); }
};
template <class T> struct Float4Fetch {
    const float* atlas;  // 4 floats per texel
    Atlas A;
    V4<T> operator()(int x, int y, int z) const {
        const float* p = atlas + 4 * A.index(x, y, z);
        return V4<T>(T(p[0]), T(p[1]), T(p[2]), T(p[3]));
    }
};

// 2D depth lookup with linear filtering and CLAMP_TO_BORDER (opaque black -> 0)
// (shadow sampler, VoxelConeTracingPass.cpp:294, RadianceInjectionPass.cpp:210).
template <class T>
inline T shadow_tap(const float* depth, int W, int H, T s, T t) {
    T u = s * T(W) - T(0.5), v = t * T(H) - T(0.5);
    T fu = std::floor(u), fv = std::floor(v);
    T a = u - fu, b = v - fv;
    int i0 = (int)fu, j0 = (int)fv;
    auto at = [&](int i, int j) -> T {
        if (i < 0 || j < 0 || i >= W || j >= H) return T(0);
        return T(depth[(int64_t)j * W + i]);
    };
    T r0 = at(i0, j0) + (at(i0 + 1, j0) - at(i0, j0)) * a;
    T r1 = at(i0, j0 + 1) + (at(i0 + 1, j0 + 1) - at(i0, j0 + 1)) * a;
    return r0 + (r1 - r0) * b;
}

struct ShadowDesc {
    float view[16];
    float proj[16];
    float z_near, z_far;
};

// calcVisibility + calcShadowCoefficientPCF16 (shadow.glsl:8-36): the sampler
// has compare disabled, so the "PCF" is the mean of 16 bilinear raw depths.
template <class T>
inline T calc_visibility(const float* depth, int W, int H, const ShadowDesc& sd, V3<T> wp) {
    if (!depth) return T(1);
    V4<T> ls = mat_mul<T>(sd.view, V4<T>(wp.x, wp.y, wp.z, T(1)));
    T lz = ls.z / (T(sd.z_far) - T(sd.z_near));
    (void)lz;
    V4<T> pxy = mat_mul<T>(sd.proj, V4<T>(ls.x, ls.y, T(0), T(1)));
    T sx = pxy.x * T(0.5) + T(0.5), sy = pxy.y * T(0.5) + T(0.5);
    T scale_x = T(1) / T(W), scale_y = T(1) / T(H);
    T sum = T(0);
    for (int yi = 0; yi < 4; ++yi)
        for (int xi = 0; xi < 4; ++xi) {
            T ox = T(-1.5) + T(xi), oy = T(-1.5) + T(yi);
            sum += shadow_tap<T>(depth, W, H, sx + ox * scale_x * T(1), sy + oy * scale_y * T(1));
        }
    return sum * T(0.0625);
}

// ------------------------------------------------------------- cone trace
// voxelConeTracing.frag:71-135 (constants) and :143-414 (main, traceCone,
// sampleClipmap, sampleClipmapLinear, calcMinLevel).
static const float kDirs16[16][3] = {
    {0.57735f, 0.57735f, 0.57735f},       {0.57735f, -0.57735f, -0.57735f},     {-0.57735f, 0.57735f, -0.57735f},
    {-0.57735f, -0.57735f, 0.57735f},     {-0.903007f, -0.182696f, -0.388844f}, {-0.903007f, 0.182696f, 0.388844f},
    {0.903007f, -0.182696f, 0.388844f},   {0.903007f, 0.182696f, -0.388844f},   {-0.388844f, -0.903007f, -0.182696f},
    {0.388844f, -0.903007f, 0.182696f},   {0.388844f, 0.903007f, -0.182696f},   {-0.388844f, 0.903007f, 0.182696f},
    {-0.182696f, -0.388844f, -0.903007f}, {0.182696f, 0.388844f, -0.903007f},   {-0.182696f, 0.388844f, 0.903007f},
    {0.182696f, -0.388844f, 0.903007f}};
static const float kAperture16 = 0.872665f;
static const float kDirs32[32][3] = {
    {0.898904f, 0.435512f, 0.0479745f},   {0.898904f, -0.435512f, -0.0479745f}, {0.898904f, 0.0479745f, -0.435512f},
    {0.898904f, -0.0479745f, 0.435512f},  {-0.898904f, 0.435512f, -0.0479745f}, {-0.898904f, -0.435512f, 0.0479745f},
    {-0.898904f, 0.0479745f, 0.435512f},  {-0.898904f, -0.0479745f, -0.435512f}, {0.0479745f, 0.898904f, 0.435512f},
    {-0.0479745f, 0.898904f, -0.435512f}, {-0.435512f, 0.898904f, 0.0479745f},  {0.435512f, 0.898904f, -0.0479745f},
    {-0.0479745f, -0.898904f, 0.435512f}, {0.0479745f, -0.898904f, -0.435512f}, {0.435512f, -0.898904f, 0.0479745f},
    {-0.435512f, -0.898904f, -0.0479745f}, {0.435512f, 0.0479745f, 0.898904f},  {-0.435512f, -0.0479745f, 0.898904f},
    {0.0479745f, -0.435512f, 0.898904f},  {-0.0479745f, 0.435512f, 0.898904f},  {0.435512f, -0.0479745f, -0.898904f},
    {-0.435512f, 0.0479745f, -0.898904f}, {0.0479745f, 0.435512f, -0.898904f},  {-0.0479745f, -0.435512f, -0.898904f},
    {0.57735f, 0.57735f, 0.57735f},       {0.57735f, 0.57735f, -0.57735f},      {0.57735f, -0.57735f, 0.57735f},
    {0.57735f, -0.57735f, -0.57735f},     {-0.57735f, 0.57735f, 0.57735f},      {-0.57735f, 0.57735f, -0.57735f},
    {-0.57735f, -0.57735f, 0.57735f},     {-0.57735f, -0.57735f, -0.57735f}};
static const float kAperture32 = 0.628319f;
static const float kMinTraceStepFactor = 0.2f;
static const float kMaxTraceDistance = 30.0f;
static const float kMinSpecularAperture = 0.05f;
static const int kClipLevels = 6;
static const int kFaces = 6;

struct TraceDesc {
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
};

template <class T, class Fetch>
struct ClipmapTracer {
    const TraceDesc& d;
    const Fetch& fetch;
    Atlas A;
    uint64_t steps = 0;

    V4<T> sample_clipmap(V3<T> p, int level, V3<T> face_offset, V3<T> weight) const {
        T vs = T(d.voxel_size) * std::exp2(T(level));
        T extent = vs * T(d.volume_dimension);
        T dim = T(d.volume_dimension);
        V3<T> sp((fractv(p.x / extent) * dim + T(1)) / (dim + T(2)),
                 (fractv(p.y / extent) * dim + T(1)) / (dim + T(2)),
                 (fractv(p.z / extent) * dim + T(1)) / (dim + T(2)));
        sp.y = sp.y + T(level);
        sp.y = sp.y / T(kClipLevels);
        sp.x = sp.x / T(kFaces);
        V4<T> a = texture3d<T>(fetch, A, V3<T>(sp.x + face_offset.x, sp.y, sp.z));
        V4<T> b = texture3d<T>(fetch, A, V3<T>(sp.x + face_offset.y, sp.y, sp.z));
        V4<T> c = texture3d<T>(fetch, A, V3<T>(sp.x + face_offset.z, sp.y, sp.z));
        return a * weight.x + b * weight.y + c * weight.z;
    }

    V4<T> sample_clipmap_linear(V3<T> p, T cur_level, const int face_index[3], V3<T> weight) const {
        int lower = (int)std::floor(cur_level);
        int upper = (int)std::ceil(cur_level);
        V3<T> fo(T(face_index[0]) / T(kFaces), T(face_index[1]) / T(kFaces), T(face_index[2]) / T(kFaces));
        V4<T> lo = sample_clipmap(p, lower, fo, weight);
        V4<T> hi = sample_clipmap(p, upper, fo, weight);
        T f = fractv(cur_level);
        return V4<T>(mixv(lo.x, hi.x, f), mixv(lo.y, hi.y, f), mixv(lo.z, hi.z, f), mixv(lo.w, hi.w, f));
    }

    V4<T> trace_cone(V3<T> start, V3<T> dir, T aperture, T max_dist, T start_level, T step_factor) {
        V4<T> result(T(0));
        const T uvs = T(d.voxel_size);
        const T cone_coef = T(2) * std::tan(aperture * T(0.5));
        T cur_level = start_level;
        T vs = uvs * std::exp2(cur_level);
        start = start + dir * (vs * T(d.trace_start_offset) * T(0.5));
        T step = T(0);
        T diameter = std::max(step * cone_coef, uvs);
        T occlusion = T(0);
        const int face_index[3] = {dir.x > T(0) ? 0 : 1, dir.y > T(0) ? 2 : 3, dir.z > T(0) ? 4 : 5};
        const V3<T> weight = dir * dir;
        T seg = vs;
        const T min_radius = uvs * T(d.volume_dimension) * T(0.5);
        const V3<T> center(T(d.volume_center[0]), T(d.volume_center[1]), T(d.volume_center[2]));
        while (step < max_dist && occlusion < T(1)) {
            ++steps;
            V3<T> pos = start + dir * step;
            T dist = length(center - pos);
            T min_level = std::ceil(std::log2(dist / min_radius));
            cur_level = std::log2(diameter / uvs);
            cur_level = std::min(std::max(std::max(start_level, cur_level), min_level), T(kClipLevels - 1));
            V4<T> s = sample_clipmap_linear(pos, cur_level, face_index, weight);
            vs = uvs * std::exp2(cur_level);
            T correction = seg / vs;
            V3<T> radiance(s.x * correction, s.y * correction, s.z * correction);
            // a filtered alpha that rounds above 1 would give pow a negative base (undefined in GLSL); the
            // base is taken as 0 there (the sample is opaque), pinned the same way in every GPU form
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
        return V4<T>(result.x, result.y, result.z, T(1) - occlusion);
    }

    T calc_min_level(V3<T> wp) const {
        const V3<T> center(T(d.volume_center[0]), T(d.volume_center[1]), T(d.volume_center[2]));
        T dist = length(center - wp);
        T min_radius = T(d.voxel_size) * T(d.volume_dimension) * T(0.5);
        T min_level = std::max(std::log2(dist / min_radius), T(0));
        T radius = min_radius * std::exp2(std::ceil(min_level));
        T f = dist / radius;
        const T ts = T(0.5);
        T c = T(1) / (T(1) - ts);
        if (f > ts) return std::ceil(min_level) + (f - ts) * c;
        return std::ceil(min_level);
    }
};

// microfacetBRDF (brdf.glsl:28-78) on the PBRInfo built in
// voxelConeTracing.frag:225-252.
template <class T>
inline V3<T> microfacet_brdf(T NdotL, T NdotV, T NdotH, T VdotH, V3<T> r0, V3<T> r90, T alpha_r, V3<T> diffuse_color) {
    const T kPi = T(3.141592);
    T fres = std::pow(clampv(T(1) - VdotH, T(0), T(1)), T(5));
    V3<T> F(r0.x + (r90.x - r0.x) * fres, r0.y + (r90.y - r0.y) * fres, r0.z + (r90.z - r0.z) * fres);
    T r = alpha_r;
    T attL = T(2) * NdotL / (NdotL + std::sqrt(r * r + (T(1) - r * r) * (NdotL * NdotL)));
    T attV = T(2) * NdotV / (NdotV + std::sqrt(r * r + (T(1) - r * r) * (NdotV * NdotV)));
    T G = attL * attV;
    T rsq = alpha_r * alpha_r;
    T f = (NdotH * rsq - NdotH) * NdotH + T(1);
    T D = rsq / (kPi * f * f);
    V3<T> diff(diffuse_color.x / kPi, diffuse_color.y / kPi, diffuse_color.z / kPi);
    V3<T> out;
    for (int i = 0; i < 3; ++i) {
        T Fi = F[i];
        T dc = (T(1) - Fi) * diff[i];
        T sc = Fi * G * D / (T(4) * NdotL * NdotV);
        out[i] = NdotL * T(1) * (dc + sc);
    }
    return out;
}

struct LightDesc {
    float direction[3];
    float intensity;
    float color[3];
    int32_t padding;
};

struct SurfaceSample {
    float position[3];
    float depth;
    float normal_texel[3];
    float pad0;
    float diffuse_texel[4];
    float specular_texel[4];
    float emission_texel[3];
    float pad1;
};

// voxelConeTracing.frag main() (:143-294) for one G-buffer texel set.
// Writes diffuse/specular RGBA; returns false if the fragment is discarded.
template <class T, class Fetch>
inline bool trace_sample(ClipmapTracer<T, Fetch>& tr, const float eye[3], const float* shadow, int sw, int sh,
                         const ShadowDesc& sd, const LightDesc& light, const SurfaceSample& s, T out_d[4], T out_s[4],
                         float diffuse_aperture = 0.0f) {
    const TraceDesc& d = tr.d;
    if (T(s.depth) == T(1)) return false;
    V3<T> wp(T(s.position[0]), T(s.position[1]), T(s.position[2]));
    V3<T> view = normalize(V3<T>(T(eye[0]), T(eye[1]), T(eye[2])) - wp);
    V3<T> diffuse_color(T(s.diffuse_texel[0]), T(s.diffuse_texel[1]), T(s.diffuse_texel[2]));
    T perceptual_roughness = T(s.diffuse_texel[3]);
    V3<T> normal = normalize(V3<T>(T(s.normal_texel[0]) * T(2) - T(1), T(s.normal_texel[1]) * T(2) - T(1),
                                   T(s.normal_texel[2]) * T(2) - T(1)));
    V3<T> specular_color(T(s.specular_texel[0]), T(s.specular_texel[1]), T(s.specular_texel[2]));
    T metallic = T(s.specular_texel[3]);
    V3<T> emission(T(s.emission_texel[0]), T(s.emission_texel[1]), T(s.emission_texel[2]));
    bool has_emission = emission.x > T(0) || emission.y > T(0) || emission.z > T(0);

    T min_level = tr.calc_min_level(wp);
    T vs = T(d.voxel_size) * std::exp2(min_level);
    V3<T> start = wp + normal * (vs * T(d.trace_start_offset));

    V4<T> indirect(T(0), T(0), T(0), T(1));
    const bool c32 = d.enable_32_cones != 0;
    const int n = c32 ? 32 : 16;
    // the shader's constant, or a configured aperture (vct_trace_options)
    const T aperture = T(diffuse_aperture != 0.0f ? diffuse_aperture : (c32 ? kAperture32 : kAperture16));
    const T sf = std::max(T(kMinTraceStepFactor), T(d.min_trace_step_factor));
    for (int i = 0; i < n; ++i) {
        const float* dd = c32 ? kDirs32[i] : kDirs16[i];
        V3<T> dir{T(dd[0]), T(dd[1]), T(dd[2])};
        T cos_t = dot(normal, dir);
        if (cos_t < T(0)) continue;
        V4<T> c = tr.trace_cone(start, dir, aperture, T(kMaxTraceDistance), min_level, sf);
        indirect = indirect + c * cos_t;
    }
    indirect = V4<T>(indirect.x / T(n), indirect.y / T(n), indirect.z / T(n), indirect.w / T(n));
    indirect.w = indirect.w * T(d.ambient_occlusion_factor);
    const T idi = T(d.indirect_diffuse_intensity);
    indirect.x = indirect.x * (diffuse_color.x * idi);
    indirect.y = indirect.y * (diffuse_color.y * idi);
    indirect.z = indirect.z * (diffuse_color.z * idi);

    V3<T> ispec(T(0));
    if ((specular_color.x > T(1e-6f) || specular_color.y > T(1e-6f) || specular_color.z > T(1e-6f)) &&
        metallic > T(1e-6f)) {
        V3<T> sdir = reflect(-view, normal);
        V4<T> c = tr.trace_cone(start, sdir, std::max(perceptual_roughness, T(kMinSpecularAperture)),
                                T(kMaxTraceDistance), min_level, T(d.voxel_size));
        const T isi = T(d.indirect_specular_intensity);
        ispec = V3<T>(c.x * specular_color.x * isi, c.y * specular_color.y * isi, c.z * specular_color.z * isi);
    }

    V3<T> direct(T(0));
    if (has_emission) {
        direct = emission;
    } else {
        T alpha_r = perceptual_roughness * perceptual_roughness;
        T reflectance = std::max(std::max(specular_color.x, specular_color.y), specular_color.z);
        V3<T> r90(clampv(reflectance * T(50), T(0), T(1)));
        V3<T> l = normalize(-V3<T>(T(light.direction[0]), T(light.direction[1]), T(light.direction[2])));
        V3<T> h = normalize(l + view);
        T NdotL = clampv(dot(normal, l), T(0.001f), T(1));
        T NdotV = clampv(std::fabs(dot(normal, view)), T(0.001f), T(1));
        T NdotH = clampv(dot(normal, h), T(0), T(1));
        T VdotH = clampv(dot(view, h), T(0), T(1));
        T vis = calc_visibility<T>(shadow, sw, sh, sd, wp);
        V3<T> b = microfacet_brdf<T>(NdotL, NdotV, NdotH, VdotH, specular_color, r90, alpha_r, diffuse_color);
        direct = b * vis;
    }

    V4<T> dout(T(0), T(0), T(0), T(1)), sout(T(0), T(0), T(0), T(1));
    switch (d.rendering_mode) {
        case 0: dout = V4<T>(diffuse_color.x, diffuse_color.y, diffuse_color.z, T(1)); break;
        case 1: dout = V4<T>(specular_color.x, specular_color.y, specular_color.z, T(1)); break;
        case 2:
            dout = V4<T>(normal.x * T(0.5) + T(0.5), normal.y * T(0.5) + T(0.5), normal.z * T(0.5) + T(0.5), T(1));
            break;
        case 3: {
            static const float colors[7][4] = {{1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {1, 1, 0, 1},
                                               {0, 1, 1, 1}, {1, 0, 1, 1}, {1, 1, 1, 1}};
            int lo = (int)std::floor(min_level);
            lo = std::min(std::max(lo, 0), 5);
            T f = fractv(min_level);
            for (int c = 0; c < 4; ++c) {
                T v = mixv(T(colors[lo][c]), T(colors[lo + 1][c]), f) * T(0.5);
                if (c == 0) dout.x = v;
                else if (c == 1) dout.y = v;
                else if (c == 2) dout.z = v;
                else dout.w = v;
            }
            break;
        }
        case 4:
            direct = direct * indirect.w;
            dout = V4<T>(direct.x, direct.y, direct.z, T(1));
            break;
        case 5:
            direct = direct * indirect.w;
            dout.x = dout.x + direct.x + indirect.x;
            dout.y = dout.y + direct.y + indirect.y;
            dout.z = dout.z + direct.z + indirect.z;
            break;
        case 6:
            sout.x = sout.x + ispec.x;
            sout.y = sout.y + ispec.y;
            sout.z = sout.z + ispec.z;
            break;
        case 7: dout = V4<T>(indirect.w, indirect.w, indirect.w, T(1)); break;
        case 8:
        default:
            direct = direct * indirect.w;
            dout.x = dout.x + direct.x + indirect.x;
            dout.y = dout.y + direct.y + indirect.y;
            dout.z = dout.z + direct.z + indirect.z;
            sout.x = sout.x + ispec.x;
            sout.y = sout.y + ispec.y;
            sout.z = sout.z + ispec.z;
            break;
    }
    out_d[0] = dout.x; out_d[1] = dout.y; out_d[2] = dout.z; out_d[3] = dout.w;
    out_s[0] = sout.x; out_s[1] = sout.y; out_s[2] = sout.z; out_s[3] = sout.w;
    return true;
}

}  // namespace vcto
