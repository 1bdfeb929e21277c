// raster.cu -- the rasterisation-driven passes as CUDA kernels:
//   vct_voxelize_opacity  (VoxelizationPass + msaaVoxelizer.*),
//   vct_shadow_depth      (ReflectiveShadowMapPass depth, reflectiveShadowPass.vert),
//   vct_inject_radiance   (RadianceInjectionPass + msaaInjectRadiance.*),
//   vct_svo_fragments     (SparseVoxelizer + voxelizer.*).
//
// The fixed-function rasteriser is restated in software with a pinned rule
// (the reference's MSAA pattern and shading rate are implementation-defined):
// 8x MSAA at the Vulkan standard sample locations (one centre sample for the
// depth-only pass), vertices snapped to 1/256 pixel, exact 64-bit edge
// functions with a one-owner tie rule, depth clip [0,1], FP32 barycentrics
// float(e_i) * (1 / float(area)), the fragment shader at every covered sample.
//
// Work decomposition: one item per (triangle, clip level); each item's
// bounding box is cut into 8x8-pixel tiles (pixels row-major, samples in index
// order).  Items' tile counts are prefix-summed and a warp sets up 32 tiles
// (found by binary search, so no per-tile list is materialised) and then
// walks their pixels as one flattened list, a pixel per lane (k_cover).
// Order-dependent passes (RGBA8 running averages, the SVO
// fragment list) use a coverage count pass + prefix sum + an emit pass that
// writes one compact descriptor per covered sample in traversal order (item,
// tile, pixel, sample); a shading kernel then runs one thread per covered
// sample, so neighbouring lanes shade neighbouring samples of one triangle
// (their shadow-map taps share cache lines).  The injection's records are
// stably sorted by texel and folded sequentially per texel run, which
// reproduces the serial order of the reference's CAS loops bit for bit.
// Compiled with -fmad=false: the fragment arithmetic is the FP32 GLSL in its
// written order.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "trace_common.cuh"

namespace vct {

// ------------------------------------------------------------------ math
struct M4 {
    float m[16];
};

__host__ __device__ inline float4 mat_vec4(const float* M, float x, float y, float z, float w) {
    float r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float a = M[i] * x + M[4 + i] * y;
        float b = M[8 + i] * z + M[12 + i] * w;
        r[i] = a + b;
    }
    return make_float4(r[0], r[1], r[2], r[3]);
}

__host__ __device__ inline M4 mat_mul4(const float* A, const float* B) {
    M4 R;
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 4; ++r) {
            float s = A[r] * B[i * 4 + 0];
            s = s + A[4 + r] * B[i * 4 + 1];
            s = s + A[8 + r] * B[i * 4 + 2];
            s = s + A[12 + r] * B[i * 4 + 3];
            R.m[i * 4 + r] = s;
        }
    return R;
}

__host__ __device__ inline float3 cross3h(float3 a, float3 b) {
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__host__ __device__ inline float dot3h(float3 a, float3 b) {
    float t0 = a.x * b.x, t1 = a.y * b.y, t2 = a.z * b.z;
    return (t0 + t1) + t2;
}
__host__ __device__ inline float3 normalize3h(float3 v) {
    float inv = 1.0f / sqrtf(dot3h(v, v));
    return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

// glm::lookAtLH and glm::orthoLH_ZO (column-major).
__host__ inline M4 look_at_lh(float3 eye, float3 center, float3 up) {
    float3 f = normalize3h(make_float3(center.x - eye.x, center.y - eye.y, center.z - eye.z));
    float3 s = normalize3h(cross3h(up, f));
    float3 u = cross3h(f, s);
    M4 R = {};
    R.m[0] = s.x; R.m[4] = s.y; R.m[8] = s.z;
    R.m[1] = u.x; R.m[5] = u.y; R.m[9] = u.z;
    R.m[2] = f.x; R.m[6] = f.y; R.m[10] = f.z;
    R.m[12] = -dot3h(s, eye);
    R.m[13] = -dot3h(u, eye);
    R.m[14] = -dot3h(f, eye);
    R.m[15] = 1.0f;
    return R;
}
__host__ inline M4 ortho_lh_zo(float l, float r, float b, float t, float n, float f) {
    M4 R = {};
    R.m[0] = 2.0f / (r - l);
    R.m[5] = 2.0f / (t - b);
    R.m[10] = 1.0f / (f - n);
    R.m[12] = -(r + l) / (r - l);
    R.m[13] = -(t + b) / (t - b);
    R.m[14] = -n / (f - n);
    R.m[15] = 1.0f;
    return R;
}

// glm::perspectiveLH_ZO (column-major): fovy in radians.
__host__ inline M4 perspective_lh_zo(float fovy, float aspect, float n, float f) {
    const float th = tanf(fovy / 2.0f);
    M4 R = {};
    R.m[0] = 1.0f / (aspect * th);
    R.m[5] = 1.0f / th;
    R.m[10] = f / (f - n);
    R.m[11] = 1.0f;
    R.m[14] = -(f * n) / (f - n);
    return R;
}

// General 4x4 inverse by cofactors, in glm::inverse's evaluation order
// (glm 0.9.9 detail/func_matrix.inl, compute_inverse<4, 4>): the 2x2 minors
// of columns 2-3 (and 1-3, 1-2) taken over row pairs, each adjugate entry as
// (a * m0 - b * m1) + c * m2 with its checkerboard sign, then a scale by
// 1 / det where det = (c0 + c1) + (c2 + c3) over column 0's products with the
// adjugate's row 0.  M[c * 4 + r] is column c, row r.
__host__ inline M4 inverse4(const float* M) {
    auto e = [&](int c, int r) { return M[c * 4 + r]; };
    // F[f][j]: the 2x2 minor of rows fr[f] and columns cp[j] (glm's Fac0..Fac5)
    const int cp[4][2] = {{2, 3}, {2, 3}, {1, 3}, {1, 2}};
    const int fr[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
    float F[6][4];
    for (int f = 0; f < 6; ++f)
        for (int j = 0; j < 4; ++j) {
            const int a = cp[j][0], b = cp[j][1], r0 = fr[f][0], r1 = fr[f][1];
            F[f][j] = e(a, r0) * e(b, r1) - e(b, r0) * e(a, r1);
        }
    float V[4][4];  // V[r][j] = element (column 1 for j == 0 else column 0, row r)
    for (int r = 0; r < 4; ++r)
        for (int j = 0; j < 4; ++j) V[r][j] = e(j == 0 ? 1 : 0, r);
    // adjugate column k = (V_p * F_q - V_s * F_t) + V_u * F_v, {p, q, s, t, u, v} = tab[k]
    const int tab[4][6] = {{1, 0, 2, 1, 3, 2}, {0, 0, 2, 3, 3, 4}, {0, 1, 1, 3, 3, 5}, {0, 2, 1, 4, 2, 5}};
    M4 I;
    for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 4; ++j) {
            const float sgn = ((k + j) & 1) ? -1.0f : 1.0f;
            const float v = (V[tab[k][0]][j] * F[tab[k][1]][j] - V[tab[k][2]][j] * F[tab[k][3]][j]) +
                            V[tab[k][4]][j] * F[tab[k][5]][j];
            I.m[k * 4 + j] = v * sgn;
        }
    const float d0 = e(0, 0) * I.m[0], d1 = e(0, 1) * I.m[4], d2 = e(0, 2) * I.m[8], d3 = e(0, 3) * I.m[12];
    const float det = (d0 + d1) + (d2 + d3);
    const float inv = 1.0f / det;
    for (int i = 0; i < 16; ++i) I.m[i] = I.m[i] * inv;
    return I;
}

// Voxelizer::setViewProjection over the extended region (min - 1, extent + 2).
__host__ void voxel_view_proj(const vct_clipmap_region& r, float out[48]) {
    const float vs = r.voxel_size;
    float3 rg = make_float3((float)(r.extent[0] + 2u) * vs, (float)(r.extent[1] + 2u) * vs, (float)(r.extent[2] + 2u) * vs);
    float3 mcg = make_float3((float)(r.min_corner[0] - 1) * vs, (float)(r.min_corner[1] - 1) * vs,
                             (float)(r.min_corner[2] - 1) * vs);
    float3 eye = make_float3(mcg.x + 0.0f, mcg.y + 0.0f, mcg.z + rg.z);
    M4 v0 = look_at_lh(eye, make_float3(eye.x + 1.0f, eye.y + 0.0f, eye.z + 0.0f), make_float3(0.f, 1.f, 0.f));
    M4 v1 = look_at_lh(eye, make_float3(eye.x + 0.0f, eye.y + 1.0f, eye.z + 0.0f), make_float3(0.f, 0.f, -1.f));
    M4 v2 = look_at_lh(mcg, make_float3(mcg.x + 0.0f, mcg.y + 0.0f, mcg.z + 1.0f), make_float3(0.f, 1.f, 0.f));
    M4 p0 = ortho_lh_zo(-rg.z, rg.z, -rg.y, rg.y, 0.1f, rg.x);
    M4 p1 = ortho_lh_zo(-rg.x, rg.x, -rg.z, rg.z, 0.1f, rg.y);
    M4 p2 = ortho_lh_zo(-rg.x, rg.x, -rg.y, rg.y, 0.1f, rg.z);
    M4 m0 = mat_mul4(p0.m, v0.m), m1 = mat_mul4(p1.m, v1.m), m2 = mat_mul4(p2.m, v2.m);
    memcpy(out, m0.m, 64);
    memcpy(out + 16, m1.m, 64);
    memcpy(out + 32, m2.m, 64);
}

__host__ vct_voxelization_desc voxelization_desc(const vct_clipmap_region* regions, int level, int R) {
    vct_voxelization_desc d;
    memset(&d, 0, sizeof(d));
    const vct_clipmap_region& r = regions[level];
    for (int a = 0; a < 3; ++a) {
        d.region_min_corner[a] = (float)r.min_corner[a] * r.voxel_size - 1e-6f;
        d.region_max_corner[a] = (float)(r.min_corner[a] + (int32_t)r.extent[a]) * r.voxel_size + 1e-6f;
    }
    d.clip_level = (uint32_t)level;
    d.clip_max_extent = (float)r.extent[0] * r.voxel_size;
    d.voxel_size = r.voxel_size;
    if (level > 0) {
        const vct_clipmap_region& p = regions[level - 1];
        for (int a = 0; a < 3; ++a) {
            d.prev_region_min_corner[a] = (float)p.min_corner[a] * p.voxel_size;
            d.prev_region_max_corner[a] = (float)(p.min_corner[a] + (int32_t)p.extent[a]) * p.voxel_size;
        }
    }
    d.clipmap_resolution = R;
    return d;
}

// ------------------------------------------------------------------ scene
struct WTri {
    float3 p[3], n[3];
    uint32_t material;
};

__device__ inline WTri world_triangle(const vct_scene& s, int64_t t) {
    WTri w;
    // instance and vertex indices are clamped to the scene's arrays (a bad
    // index reads the last entry instead of out of bounds)
    const uint32_t inst = s.triangle_instance ? min(__ldg(s.triangle_instance + t), (uint32_t)max(s.instance_count - 1, 0)) : 0u;
    const float* model = s.node_matrices ? s.node_matrices + 32 * (int64_t)inst : nullptr;
    const uint32_t vmax = (uint32_t)max(s.vertex_count - 1, (int64_t)0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = min(__ldg(s.indices + 3 * t + k), vmax);
        const float* p = s.positions + 3 * (int64_t)vi;
        const float* n = s.normals + 3 * (int64_t)vi;
        float px = __ldg(p), py = __ldg(p + 1), pz = __ldg(p + 2);
        float nx = __ldg(n), ny = __ldg(n + 1), nz = __ldg(n + 2);
        if (model) {
            float4 wp = mat_vec4(model, px, py, pz, 1.0f);
            float4 wn = mat_vec4(model + 16, nx, ny, nz, 0.0f);
            w.p[k] = make_float3(wp.x, wp.y, wp.z);
            w.n[k] = make_float3(wn.x, wn.y, wn.z);
        } else {
            float4 wp = make_float4(px, py, pz, 1.0f);
            float4 wn = make_float4(nx, ny, nz, 0.0f);
            // identity model: mat_vec4 with the identity is exact, keep the values
            w.p[k] = make_float3(wp.x, wp.y, wp.z);
            w.n[k] = make_float3(wn.x, wn.y, wn.z);
        }
    }
    w.material = s.triangle_material ? __ldg(s.triangle_material + t) : 0u;
    return w;
}

__device__ inline int dominant_axis(const float3 p[3]) {
    float3 e1 = make_float3(p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z);
    float3 e2 = make_float3(p[2].x - p[0].x, p[2].y - p[0].y, p[2].z - p[0].z);
    float3 c = cross3h(e1, e2);
    float nx = fabsf(c.x), ny = fabsf(c.y), nz = fabsf(c.z);
    return (nx > ny && nx > nz) ? 0 : ((ny > nz) ? 1 : 2);
}

__device__ inline float4 texture_1x1(const vct_scene& s, int32_t id) {
    if (!s.textures || id < 0 || id >= s.texture_count) return make_float4(0.f, 0.f, 0.f, 0.f);
    return unpack_rgba8(__ldg(s.textures + id));
}

// ------------------------------------------------------------- rasteriser
__constant__ int c_sample_loc8[8][2] = {{144, 80}, {112, 176}, {208, 144}, {80, 48},
                                        {48, 208}, {16, 112}, {176, 240}, {240, 16}};

struct RSetup {
    long long X[3], Y[3];
    float z[3];
    bool swapped;  // vertices 1 and 2 exchanged to make the winding counter-clockwise
    long long area;
    float inv_area;
    int px0, py0, px1, py1;
    int owned;  // bit i: edge i owns its samples
    bool ok;
};

__device__ inline long long floor_div256(long long v) { return v >= 0 ? v / 256 : -((-v + 255) / 256); }

__device__ inline RSetup raster_setup(const float4 c[3], int W, int H) {
    RSetup r;
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    long long X[3], Y[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        X[k] = __float2ll_rn((hw * c[k].x + hw) * 256.0f);
        Y[k] = __float2ll_rn((hh * c[k].y + hh) * 256.0f);
    }
    long long area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
    r.ok = area != 0;
    if (!r.ok) return r;
    // counter-clockwise vertex order: swap vertices 1 and 2 of a clockwise triangle
    const bool sw = area < 0;
    if (sw) area = -area;
    r.X[0] = X[0];
    r.Y[0] = Y[0];
    r.z[0] = c[0].z;
    r.X[1] = sw ? X[2] : X[1];
    r.Y[1] = sw ? Y[2] : Y[1];
    r.z[1] = sw ? c[2].z : c[1].z;
    r.X[2] = sw ? X[1] : X[2];
    r.Y[2] = sw ? Y[1] : Y[2];
    r.z[2] = sw ? c[1].z : c[2].z;
    r.swapped = sw;
    r.area = area;
    r.inv_area = 1.0f / (float)area;
    r.owned = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
        const long long dy = r.Y[b] - r.Y[a], dx = r.X[b] - r.X[a];
        if (dy > 0 || (dy == 0 && dx > 0)) r.owned |= 1 << i;
    }
    long long mnx = min(r.X[0], min(r.X[1], r.X[2])), mxx = max(r.X[0], max(r.X[1], r.X[2]));
    long long mny = min(r.Y[0], min(r.Y[1], r.Y[2])), mxy = max(r.Y[0], max(r.Y[1], r.Y[2]));
    long long px0 = max(floor_div256(mnx), 0LL), px1 = min(floor_div256(mxx), (long long)W - 1);
    long long py0 = max(floor_div256(mny), 0LL), py1 = min(floor_div256(mxy), (long long)H - 1);
    if (px0 > px1 || py0 > py1) {
        r.ok = false;
        return r;
    }
    r.px0 = (int)px0;
    r.px1 = (int)px1;
    r.py0 = (int)py0;
    r.py1 = (int)py1;
    return r;
}

__device__ inline uint32_t tiles_of(const RSetup& r) {
    if (!r.ok) return 0u;
    return (uint32_t)(((r.px1 - r.px0) >> 3) + 1) * (uint32_t)(((r.py1 - r.py0) >> 3) + 1);
}

__device__ inline float3 interp3(const float b[3], const float3 v[3]) {
    return make_float3((b[0] * v[0].x + b[1] * v[1].x) + b[2] * v[2].x, (b[0] * v[0].y + b[1] * v[1].y) + b[2] * v[2].y,
                       (b[0] * v[0].z + b[1] * v[1].z) + b[2] * v[2].z);
}

// ------------------------------------------------------------ pass params
// K_OPA_COUNT: the opacity voxelisation and the injection's coverage count in
// one pass (the frame's items are the same for both).
// K_GBUFFER: the camera's visibility pass (closest fragment per pixel centre).
enum Kind { K_OPACITY = 0, K_INJECT = 1, K_SHADOW = 2, K_SVO = 3, K_OPA_COUNT = 4, K_GBUFFER = 5 };
enum Phase { P_DIRECT = 0, P_COUNT = 1, P_WRITE = 2 };

struct RasterArgs {
    vct_scene s;
    int kind;
    int R;                 // clipmap resolution (clipmap passes) or octree resolution (SVO)
    int W, H;              // viewport
    int nlevels;           // clip levels rasterised per triangle
    int levels[6];
    float vp[6][3][16];    // per level, per axis view-projection
    vct_voxelization_desc vd[6];
    float pv[16];          // shadow pass: proj * view
    // lighting (injection / SVO)
    TraceParams light;     // light, shadow map and its desc (trace-shared struct)
    float ldir[3];
    // SVO normalisation
    float center[3], ev;
    // outputs
    uint32_t* atlas;
    float* depth;
    uint32_t* frags;
    int64_t frag_capacity;
    int64_t items;
    uint32_t invalid_key;  // injection record key that sorts past every texel
    uint32_t count_levels; // injection: the clip levels (bit l) whose samples are counted and emitted
    unsigned long long* vis;  // G-buffer: per pixel (depth bits << 32 | triangle * 6 + sub-triangle), min wins
    // toroidal revoxelisation: levels whose bit is set keep only the opacity
    // fragments inside the union of their slabs (axis a: slab_lo[l][a] <=
    // p.a <= slab_hi[l][a]; an empty interval has lo > hi)
    uint32_t slab_levels;
    float slab_lo[6][3], slab_hi[6][3];
    int opa_r8;  // the opacity atlas holds one byte per texel (alpha only)
};

// A fragment at world position p of a slab-restricted level is kept when it
// lies inside one of the level's slabs.
__device__ inline bool in_slabs(const RasterArgs& A, int lvl, float3 p) {
    const float* lo = A.slab_lo[lvl];
    const float* hi = A.slab_hi[lvl];
    return (p.x >= lo[0] && p.x <= hi[0]) || (p.y >= lo[1] && p.y <= hi[1]) || (p.z >= lo[2] && p.z <= hi[2]);
}

// Conservative triangle cull for a slab-restricted level: false when no
// interpolated point of the triangle can fall inside a slab (the margin
// covers the rounding of the FP32 barycentric interpolation).
__device__ inline bool tri_meets_slabs(const RasterArgs& A, int lvl, const float3 p[3]) {
    const float mn[3] = {fminf(fminf(p[0].x, p[1].x), p[2].x), fminf(fminf(p[0].y, p[1].y), p[2].y),
                         fminf(fminf(p[0].z, p[1].z), p[2].z)};
    const float mx[3] = {fmaxf(fmaxf(p[0].x, p[1].x), p[2].x), fmaxf(fmaxf(p[0].y, p[1].y), p[2].y),
                         fmaxf(fmaxf(p[0].z, p[1].z), p[2].z)};
    bool hit = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float lo = A.slab_lo[lvl][a], hi = A.slab_hi[lvl][a];
        const float m = 1e-5f * (fabsf(mn[a]) + fabsf(mx[a])) + 1e-6f;
        hit = hit || (lo <= hi && mx[a] + m >= lo && mn[a] - m <= hi);
    }
    return hit;
}

// Items are numbered triangle-major (item = tri * nlevels + level index) and
// stay below 2^31, so 32-bit arithmetic suffices.
__device__ inline void item_of(const RasterArgs& A, int64_t item, int64_t& tri, int& lvl) {
    const uint32_t it = (uint32_t)item, nl = (uint32_t)A.nlevels;
    const uint32_t t = nl == 1u ? it : it / nl;
    tri = t;
    lvl = A.levels[it - t * nl];
}

// ---------------------------------------------------------- camera clipping
// The G-buffer pass draws with a perspective camera, so a triangle is clipped
// in homogeneous space before the divide: against the near plane z >= 0 (the
// zero-to-one depth range; it also keeps w >= zNear > 0) and a guard band
// |x|, |y| <= 16 w, which bounds the snapped screen coordinates so the 64-bit
// edge functions cannot overflow (pixels outside the viewport are never
// tested, so the band changes no coverage).  Sutherland-Hodgman over the five
// planes leaves at most 8 vertices; the polygon is fanned from its first
// vertex into at most 6 sub-triangles.  Every vertex carries its barycentric
// coordinates in the original triangle, so attributes interpolate
// perspective-correctly across sub-triangles.  FP32, no contraction; the
// oracle restates the same steps.
struct ClipVert {
    float x, y, z, w;  // clip coordinates
    float l[3];        // barycentric coordinates in the original triangle
};

constexpr float kGuardBand = 16.0f;

__host__ __device__ inline float clip_dist(const ClipVert& v, int plane) {
    switch (plane) {
        case 0: return v.z;
        case 1: return v.x + kGuardBand * v.w;
        case 2: return kGuardBand * v.w - v.x;
        case 3: return v.y + kGuardBand * v.w;
        default: return kGuardBand * v.w - v.y;
    }
}

// Clips triangle c[3] (clip coordinates) into poly[]; returns the vertex count (0 or 3..8).
__host__ __device__ inline int clip_triangle(const float4 c[3], ClipVert poly[8]) {
    ClipVert a[8], b[8];
    int n = 3;
    for (int k = 0; k < 3; ++k) {
        a[k].x = c[k].x;
        a[k].y = c[k].y;
        a[k].z = c[k].z;
        a[k].w = c[k].w;
        a[k].l[0] = k == 0 ? 1.0f : 0.0f;
        a[k].l[1] = k == 1 ? 1.0f : 0.0f;
        a[k].l[2] = k == 2 ? 1.0f : 0.0f;
    }
    ClipVert* src = a;
    ClipVert* dst = b;
    for (int plane = 0; plane < 5; ++plane) {
        bool all_in = true;
        for (int k = 0; k < n; ++k) all_in = all_in && clip_dist(src[k], plane) >= 0.0f;
        if (all_in) continue;
        int m = 0;
        for (int k = 0; k < n; ++k) {
            const ClipVert& p = src[k];
            const ClipVert& q = src[(k + 1) % n];
            const float dp = clip_dist(p, plane), dq = clip_dist(q, plane);
            if (dp >= 0.0f) dst[m++] = p;
            if ((dp >= 0.0f) != (dq >= 0.0f)) {
                const float t = dp / (dp - dq);
                ClipVert r;
                r.x = p.x + t * (q.x - p.x);
                r.y = p.y + t * (q.y - p.y);
                r.z = p.z + t * (q.z - p.z);
                r.w = p.w + t * (q.w - p.w);
                for (int i = 0; i < 3; ++i) r.l[i] = p.l[i] + t * (q.l[i] - p.l[i]);
                dst[m++] = r;
            }
        }
        n = m;
        ClipVert* t = src;
        src = dst;
        dst = t;
        if (n < 3) return 0;
    }
    for (int k = 0; k < n; ++k) poly[k] = src[k];
    return n;
}

// Sub-triangle `sub` of the clipped triangle (fan from vertex 0), or false.
__host__ __device__ inline bool clip_sub_triangle(const float4 c[3], int sub, ClipVert v[3]) {
    ClipVert poly[8];
    const int n = clip_triangle(c, poly);
    if (sub + 2 >= n) return false;
    v[0] = poly[0];
    v[1] = poly[sub + 1];
    v[2] = poly[sub + 2];
    return true;
}

// Clip-space vertices of item (tri, level) for the pass.
// KIND is the pass's kind (A.kind) as a template argument, so each kernel
// holds only its own projection (the G-buffer clipper's local arrays and the
// other kinds' branches cost the coverage kernels instruction-cache misses
// and a large stack frame).
template <int KIND>
__device__ inline bool item_setup(const RasterArgs& A, const WTri& w, int lvl, RSetup& rs, float3 pos[3]) {
    float4 c[3];
    if constexpr (KIND == K_SHADOW) {
#pragma unroll
        for (int k = 0; k < 3; ++k) c[k] = mat_vec4(A.pv, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
    } else if constexpr (KIND == K_GBUFFER) {  // `lvl` is the sub-triangle of the clipped triangle
        float4 h[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) h[k] = mat_vec4(A.pv, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
        ClipVert v[3];
        if (!clip_sub_triangle(h, lvl, v)) {
            rs.ok = false;
            return false;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) c[k] = make_float4(v[k].x / v[k].w, v[k].y / v[k].w, v[k].z / v[k].w, 1.0f);
    } else if constexpr (KIND == K_SVO) {
        float3 q[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            q[k] = make_float3((w.p[k].x - A.center[0]) / A.ev, (w.p[k].y - A.center[1]) / A.ev,
                               (w.p[k].z - A.center[2]) / A.ev);
            pos[k] = make_float3((q[k].x + 1.0f) * 0.5f, (q[k].y + 1.0f) * 0.5f, (q[k].z + 1.0f) * 0.5f);
        }
        const int axis = dominant_axis(q);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = axis == 0 ? q[k].y : q[k].x;
            const float b = axis == 2 ? q[k].y : q[k].z;
            c[k] = make_float4(a, b, 1.0f, 1.0f);
        }
    } else {
        // toroidal revoxelisation: a level restricted to its slabs skips the
        // triangles that cannot reach them, unless the fused pass also counts
        // the level's injection samples
        if ((A.slab_levels >> lvl) & 1u) {
            const bool counted = KIND == K_OPA_COUNT && ((A.count_levels >> lvl) & 1u);
            if ((KIND == K_OPACITY || KIND == K_OPA_COUNT) && !counted && !tri_meets_slabs(A, lvl, w.p)) {
                rs.ok = false;
                return false;
            }
        }
        const int axis = dominant_axis(w.p);
        const float* M = A.vp[lvl][axis];
#pragma unroll
        for (int k = 0; k < 3; ++k) c[k] = mat_vec4(M, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
    }
    rs = raster_setup(c, A.W, A.H);
    return rs.ok;
}

__device__ inline int3 clip_image_coords(const vct_voxelization_desc& d, float3 wp) {
    const float c = d.voxel_size * 0.25f;
    const float lo = d.region_min_corner[0] + c, hi = d.region_max_corner[0] - c;
    float p[3] = {fminf(fmaxf(wp.x, lo), hi), fminf(fmaxf(wp.y, lo), hi), fminf(fmaxf(wp.z, lo), hi)};
    const int R = d.clipmap_resolution;
    int ic[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float q = p[a] / d.clip_max_extent;
        float f = q - floorf(q);
        ic[a] = ((int)(f * (float)R)) & (R - 1);  // f >= 0 and R a power of two: the value % R
    }
    return make_int3(ic[0] + 1, ic[1] + 1 + (R + 2) * (int)d.clip_level, ic[2] + 1);
}

__device__ inline uint32_t conv_rgba8(float x, float y, float z, float w) {
    return (((uint32_t)w & 0xffu) << 24) | (((uint32_t)z & 0xffu) << 16) | (((uint32_t)y & 0xffu) << 8) |
           ((uint32_t)x & 0xffu);
}

// The CAS-loop body of imageAtomicRGBA8Avg / atomicRGBA8Avg for one observed value.
__device__ inline uint32_t rgba8_avg_fold(uint32_t cur, float vr, float vg, float vb, float va) {
    if (cur == 0u) return conv_rgba8(vr, vg, vb, va);
    float rx = (float)(cur & 0xffu), ry = (float)((cur >> 8) & 0xffu), rz = (float)((cur >> 16) & 0xffu),
          rw = (float)(cur >> 24);
    rx = rx * rw;
    ry = ry * rw;
    rz = rz * rw;
    float cx = rx + vr, cy = ry + vg, cz = rz + vb, cw = rw + va;
    cx = cx / cw;
    cy = cy / cw;
    cz = cz / cw;
    return conv_rgba8(cx, cy, cz, cw);
}

// The reference's CAS loop itself (faithful atomic mode), bounded: gives up
// after 1<<20 retries (never observed) and reports through `err`.
__device__ inline void rgba8_avg_atomic(uint32_t* cell, float vr, float vg, float vb, float va, int* err) {
    uint32_t prev = 0u, newv = conv_rgba8(vr, vg, vb, va), cur;
    int guard = 0;
    while ((cur = atomicCAS(cell, prev, newv)) != prev) {
        prev = cur;
        newv = rgba8_avg_fold(cur, vr, vg, vb, va);
        if (++guard > (1 << 20)) {
            atomicExch(err, 1);
            return;
        }
    }
}

struct InjRecord {  // one face update of the injection, in traversal order
    uint32_t key;
    float r, g, b;
};

// Injection fragment (msaaInjectRadiance.frag:68-155) -> up to 6 face updates.
// `wp` and `n` are the interpolated world position and (unnormalised) normal.
// Returns the number of updates; writes them to upd[] (key, r, g, b) with a = 1.
__device__ inline int inject_fragment(const RasterArgs& A, const vct_gltf_shade_material& mat, int lvl, float3 wp,
                                      float3 n, InjRecord upd[6]) {
    const vct_voxelization_desc& d = A.vd[lvl];
    const int3 ic = clip_image_coords(d, wp);
    if (mat.occlusion_texture > -1 && texture_1x1(A.s, mat.occlusion_texture).x < 0.1f) return 0;
    const AtlasDims AD(A.R);
    const int rb = A.R + 2;
    const bool emissive = mat.emissive_factor[0] > 0.0f || mat.emissive_factor[1] > 0.0f || mat.emissive_factor[2] > 0.0f;
    if (emissive) {
        float e[3] = {mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]};
        if (mat.emissive_texture > -1) {
            float4 tx = texture_1x1(A.s, mat.emissive_texture);
            e[0] = e[0] + tx.x;
            e[1] = e[1] + tx.y;
            e[2] = e[2] + tx.z;
        }
        for (int k = 0; k < 3; ++k) e[k] = fminf(fmaxf(e[k], 0.0f), 1.0f) * 255.0f;
        for (int f = 0; f < 6; ++f) upd[f] = InjRecord{(uint32_t)AD.index(ic.x + rb * f, ic.y, ic.z), e[0], e[1], e[2]};
        return 6;
    }
    float4 color = make_float4(mat.pbr_base_color_factor[0], mat.pbr_base_color_factor[1], mat.pbr_base_color_factor[2],
                               mat.pbr_base_color_factor[3]);
    if (mat.pbr_base_color_texture > -1) {
        float4 tx = texture_1x1(A.s, mat.pbr_base_color_texture);
        color = make_float4(color.x * tx.x, color.y * tx.y, color.z * tx.z, color.w * tx.w);
    }
    const float3 nrm = normalize3h(n);
    const float3 ld = make_float3(A.ldir[0], A.ldir[1], A.ldir[2]);
    const float NdotL = fminf(fmaxf(dot3h(nrm, ld), 0.001f), 1.0f);
    const float vis = calc_visibility(A.light, wp);
    float lc[3];
    for (int k = 0; k < 3; ++k) lc[k] = 0.0f + NdotL * vis * A.light.light.color[k] * A.light.light.intensity;
    if (lc[0] == 0.0f && lc[1] == 0.0f && lc[2] == 0.0f) return 0;
    float rad[3] = {lc[0] * color.x * color.w, lc[1] * color.y * color.w, lc[2] * color.z * color.w};
    for (int k = 0; k < 3; ++k) rad[k] = fminf(fmaxf(rad[k], 0.0f), 1.0f);
    const int face[3] = {-nrm.x > 0.0f ? 0 : 1, -nrm.y > 0.0f ? 2 : 3, -nrm.z > 0.0f ? 4 : 5};
    const float wgt[3] = {fabsf(nrm.x), fabsf(nrm.y), fabsf(nrm.z)};
    for (int k = 0; k < 3; ++k)
        upd[k] = InjRecord{(uint32_t)AD.index(ic.x + rb * face[k], ic.y, ic.z), rad[0] * wgt[k] * 255.0f,
                           rad[1] * wgt[k] * 255.0f, rad[2] * wgt[k] * 255.0f};
    return 3;
}

// SVO fragment (voxelizer.frag:48-103).  `fp` is the interpolated normalised
// position and `n` the interpolated (unnormalised) normal.  Returns 0 if the
// occlusion texture discards it (no slot), 1 with `*valid` false if the light
// test discards it after the counter increment (slot left untouched), else 1
// and the packed pair.
__device__ inline int svo_fragment(const RasterArgs& A, const vct_gltf_shade_material& mat, float3 fp, float3 n,
                                   bool* valid, uint2* out) {
    if (mat.occlusion_texture > -1 && texture_1x1(A.s, mat.occlusion_texture).x < 0.1f) return 0;
    *valid = false;
    float rad[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    const bool emissive = mat.emissive_factor[0] > 0.0f || mat.emissive_factor[1] > 0.0f || mat.emissive_factor[2] > 0.0f;
    if (emissive) {
        float e[3] = {mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]};
        if (mat.emissive_texture > -1) {
            float4 tx = texture_1x1(A.s, mat.emissive_texture);
            e[0] = e[0] + tx.x;
            e[1] = e[1] + tx.y;
            e[2] = e[2] + tx.z;
        }
        for (int k = 0; k < 3; ++k) rad[k] = fminf(fmaxf(e[k], 0.0f), 1.0f);
    } else {
        float4 color = make_float4(0.f, 0.f, 0.f, 1.f);
        if (mat.pbr_base_color_texture > -1) {
            float4 tx = texture_1x1(A.s, mat.pbr_base_color_texture);
            color = make_float4(tx.x * mat.pbr_base_color_factor[0], tx.y * mat.pbr_base_color_factor[1],
                                tx.z * mat.pbr_base_color_factor[2], tx.w * mat.pbr_base_color_factor[3]);
        }
        const float3 nrm = normalize3h(n);
        const float3 ld = make_float3(A.ldir[0], A.ldir[1], A.ldir[2]);
        const float NdotL = fminf(fmaxf(dot3h(nrm, ld), 0.001f), 1.0f);
        const float vis = calc_visibility(A.light, fp);
        float lc[3];
        for (int k = 0; k < 3; ++k) lc[k] = 0.0f + NdotL * vis * A.light.light.color[k] * A.light.light.intensity;
        if (lc[0] == 0.0f && lc[1] == 0.0f && lc[2] == 0.0f) return 1;
        const float cc[3] = {color.x, color.y, color.z};
        for (int k = 0; k < 3; ++k) rad[k] = fminf(fmaxf(lc[k] * cc[k] * color.w, 0.0f), 1.0f);
        rad[3] = 1.0f;
    }
    const float res = (float)A.R;
    const uint32_t vx = (uint32_t)fminf(fmaxf(fp.x * res, 0.0f), res);
    const uint32_t vy = (uint32_t)fminf(fmaxf(fp.y * res, 0.0f), res);
    const uint32_t vz = (uint32_t)fminf(fmaxf(fp.z * res, 0.0f), res);
    const uint32_t rgba = conv_rgba8(rad[0] * 255.0f, rad[1] * 255.0f, rad[2] * 255.0f, rad[3] * 255.0f);
    out->x = vx | (vy << 12) | ((vz & 0xffu) << 24);
    out->y = ((vz >> 8) << 28) | (rgba & 0xfffffffu);
    *valid = true;
    return 1;
}

// ---------------------------------------------------------------- kernels
struct TilePlan {
    const uint32_t* tile_end;   // inclusive prefix of the items' tile counts
    const uint32_t* tile_item;  // item of every tile
    uint32_t total;             // tiles
    unsigned int* ticket;       // the next chunk of 32 tiles a coverage warp takes (zeroed per launch)
};

// Item of every tile: item i owns tiles [tile_end[i-1], tile_end[i]).  A warp
// takes 32 items; a lane writes its own item's tiles when there are at most
// eight, and the warp writes the larger items' together, so an item with
// thousands of tiles (a floor quad in a 2048^2 shadow map) is spread over the
// lanes.
__global__ void k_tile_items(const uint32_t* __restrict__ tile_end, int64_t items, uint32_t* __restrict__ tile_item) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < items; base += nwarps * 32) {
        const int64_t i = base + lane;
        const uint32_t e_i = i < items ? tile_end[i] : 0u;
        const uint32_t b_i = i < items ? (i > 0 ? tile_end[i - 1] : 0u) : 0u;
        if (e_i - b_i <= 8u)
            for (uint32_t g = b_i; g < e_i; ++g) tile_item[g] = (uint32_t)i;
        for (unsigned big = __ballot_sync(0xffffffffu, e_i - b_i > 8u); big; big &= big - 1u) {
            const int j = __ffs(big) - 1;
            const uint32_t b = __shfl_sync(0xffffffffu, b_i, j), e = __shfl_sync(0xffffffffu, e_i, j);
            for (uint32_t g = b + (uint32_t)lane; g < e; g += 32u) tile_item[g] = (uint32_t)(base + j);
        }
    }
}

template <int KIND>
__global__ void k_item_tiles(const __grid_constant__ RasterArgs A, uint32_t* __restrict__ tiles) {
    for (int64_t item = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; item < A.items;
         item += (int64_t)gridDim.x * blockDim.x) {
        int64_t tri;
        int lvl;
        item_of(A, item, tri, lvl);
        WTri w = world_triangle(A.s, tri);
        RSetup rs;
        float3 pos[3];
        tiles[item] = item_setup<KIND>(A, w, lvl, rs, pos) ? tiles_of(rs) : 0u;
    }
}

// One covered sample of the injection or SVO pass, compacted in traversal
// order for the shading kernels: the interpolated position (world space for
// the injection, the normalised [0,1] cube for the SVO), the output slot (the
// first face record of the injection, the fragment-list slot of the SVO),
// the interpolated unnormalised normal, and level | material << 3.
struct FragDesc {
    float4 p;  // x, y, z, slot (bits)
    float4 n;  // x, y, z, meta (bits)
};

__device__ inline vct_gltf_shade_material material_of(const vct_scene& s, uint32_t mi) {
    return s.materials ? s.materials[min((int)mi, s.material_count - 1)] : vct_gltf_shade_material{};
}

__device__ inline bool item_discarded(const RasterArgs& A, const vct_gltf_shade_material& mat) {
    // occlusion textures are 1x1, so their discard test is per material
    return mat.occlusion_texture > -1 && texture_1x1(A.s, mat.occlusion_texture).x < 0.1f;
}

// gBufferPass.frag:103-106: alpha-tested materials discard below the cutoff
// (1x1 textures make the base colour's alpha per material).
__device__ inline float4 gbuffer_base_color(const RasterArgs& A, const vct_gltf_shade_material& mat) {
    float4 c = make_float4(mat.pbr_base_color_factor[0], mat.pbr_base_color_factor[1], mat.pbr_base_color_factor[2],
                           mat.pbr_base_color_factor[3]);
    if (mat.pbr_base_color_texture > -1) {
        const float4 t = texture_1x1(A.s, mat.pbr_base_color_texture);
        c = make_float4(c.x * t.x, c.y * t.y, c.z * t.z, c.w * t.w);
    }
    return c;
}

__device__ inline bool gbuffer_discarded(const RasterArgs& A, const vct_gltf_shade_material& mat) {
    return mat.alpha_mode > 0 && gbuffer_base_color(A, mat).w < mat.alpha_cutoff;
}

__device__ inline uint32_t inject_per_fragment(const vct_gltf_shade_material& mat) {
    const bool emissive = mat.emissive_factor[0] > 0.0f || mat.emissive_factor[1] > 0.0f || mat.emissive_factor[2] > 0.0f;
    return emissive ? 6u : 3u;
}

// 8x MSAA standard sample positions in 1/256 pixel (the c_sample_loc8 table
// as constant expressions, so unrolled sample loops fold them).
__host__ __device__ constexpr int sample_x(int s) {
    return s == 0 ? 144 : s == 1 ? 112 : s == 2 ? 208 : s == 3 ? 80 : s == 4 ? 48 : s == 5 ? 16 : s == 6 ? 176 : 240;
}
__host__ __device__ constexpr int sample_y(int s) {
    return s == 0 ? 80 : s == 1 ? 176 : s == 2 ? 144 : s == 3 ? 48 : s == 4 ? 208 : s == 5 ? 112 : s == 6 ? 240 : 16;
}

// The set-up triangle of one tile in the form the per-pixel tests use.  Edge
// i runs from vertex a = (i+1)%3 to c = (i+2)%3 and
//   e_i(x, y) = dX_i * (y - Y_a) - dY_i * (x - X_a)        (1/256-pixel units),
// the pinned edge function: a sample is covered when every e_i > 0, or
// e_i == 0 on an edge that owns its ties, and its interpolated depth
// (b0 z0 + b1 z1) + b2 z2 with b_i = float(e_i) * inv_area lies in [0, 1].
// The tile keeps E_i = e_i at its corner
// (tx * 256, ty * 256); a sample at offset (ox, oy) from that corner has
// e_i = E_i + dX_i * oy - dY_i * ox, the same int64 value (equal modulo 2^64
// even where a product wrapped).
//   small: every |dX_i|, |dY_i| < 2^17.  A sample of the tile is then within
//          Mt_i = (|dX_i| + |dY_i|) * 2032 < 2^29 of E_i (offsets < 7 * 256 +
//          240), so an edge with E_i > Mt_i passes every sample of the tile,
//          E_i < -Mt_i empties the tile, and the others run in 32 bits;
//   zsafe: every vertex depth lies in [0, 1 - 2^-20].  The interpolated depth
//          of a covered sample is then inside the [0, 1] clip: its weights
//          are >= 0 and sum to at most (1 + 2^-24)^3 (area = sum of e_i, three
//          roundings each) and the five roundings of the dot product add at
//          most a factor (1 + 2^-24)^3, so z <= (1 + 2^-24)^6 (1 - 2^-20) < 1.
struct TileRegs {
    long long E[3];     // e_i at the tile corner
    int dX[3], dY[3];   // small tiles: the edge deltas
    float z[3], inv_area;
    uint32_t flags;     // bits 0-2: edge i owns its ties; 3: vertices 1 and 2 swapped;
                        // 4: small; 5: zsafe; 6-8: edge i passes every sample of the tile
};

// Per-tile state that the lanes of one warp share: one slot per lane's tile.
struct TileSlot {
    TileRegs t;                // the set-up triangle, ready for the per-pixel tests
    long long dXl[3], dYl[3];  // the edge deltas in 64 bits (tiles that are not small)
    int tx, ty, tw;            // tile origin and clipped width in pixels
    uint32_t tw_magic;         // ceil(2^32 / tw) (tw > 1): n / tw = umulhi(n, tw_magic) for n < 64
    uint32_t px_end;           // inclusive prefix of the warp's tile pixel counts
    uint32_t done;             // covered samples of this tile met in earlier rounds
    uint32_t base_f, base_r, per, meta;
    uint32_t item;             // the tile's (triangle, level or sub-triangle) item
    float3 p[3], n[3];         // interpolation sources (position, normal)
};

// Fills the slot's test state for tile (tx, ty); returns false if an edge
// rejects every sample of the tile.
__device__ inline bool tile_regs(const RSetup& rs, int tx, int ty, TileSlot& T) {
    TileRegs& t = T.t;
    bool small = true;
    long long Mt[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, c = (i + 2) % 3;
        const long long dX = rs.X[c] - rs.X[a], dY = rs.Y[c] - rs.Y[a];
        T.dXl[i] = dX;
        T.dYl[i] = dY;
        t.E[i] = dX * ((long long)ty * 256 - rs.Y[a]) - dY * ((long long)tx * 256 - rs.X[a]);
        const bool si = dX > -(1LL << 17) && dX < (1LL << 17) && dY > -(1LL << 17) && dY < (1LL << 17);
        small = small && si;
        t.dX[i] = (int)dX;  // meaningful only when small
        t.dY[i] = (int)dY;
        Mt[i] = si ? (llabs(dX) + llabs(dY)) * 2032 : 0;
        t.z[i] = rs.z[i];
    }
    uint32_t flags = (uint32_t)rs.owned | (rs.swapped ? 8u : 0u);
    if (small) {
        flags |= 16u;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (t.E[i] < -Mt[i]) return false;
            if (t.E[i] > Mt[i]) flags |= 64u << i;
        }
    }
    const float zhi = 0.99999904632568359375f;  // 1 - 2^-20
    if (rs.z[0] >= 0.0f && rs.z[1] >= 0.0f && rs.z[2] >= 0.0f && rs.z[0] <= zhi && rs.z[1] <= zhi && rs.z[2] <= zhi)
        flags |= 32u;
    t.flags = flags;
    t.inv_area = rs.inv_area;
    return true;
}

// Barycentrics and depth of the sample at offset (ox, oy) from the tile
// corner: the pinned FP32 barycentrics and depth.
__device__ inline void sample_bz(const TileRegs& t, const TileSlot& T, int ox, int oy, float b[3], float& z) {
    float bo[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const long long e = (t.flags & 16u) ? t.E[i] + (long long)(t.dX[i] * oy - t.dY[i] * ox)
                                            : t.E[i] + (T.dXl[i] * oy - T.dYl[i] * ox);
        bo[i] = (float)e * t.inv_area;
    }
    z = (bo[0] * t.z[0] + bo[1] * t.z[1]) + bo[2] * t.z[2];
    b[0] = bo[0];
    b[1] = (t.flags & 8u) ? bo[2] : bo[1];
    b[2] = (t.flags & 8u) ? bo[1] : bo[2];
}

// Coverage mask of the NS samples of the pixel at offset (ox0, oy0) from the
// tile corner (bit s: sample s covered and inside the depth clip).
template <int NS>
__device__ inline uint32_t cover_pixel(const TileRegs& t, const TileSlot& T, int ox0, int oy0) {
    uint32_t mask = 0;
    if (t.flags & 16u) {
        int base[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) base[i] = (int)t.E[i] + (t.dX[i] * oy0 - t.dY[i] * ox0);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const int ox = NS == 1 ? 128 : sample_x(s), oy = NS == 1 ? 128 : sample_y(s);
            bool cov = true;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (!((t.flags >> (6 + i)) & 1u)) {
                    const int e = base[i] + (t.dX[i] * oy - t.dY[i] * ox);
                    cov = cov && (e > 0 || (e == 0 && ((t.flags >> i) & 1u)));
                }
            }
            if (cov && !(t.flags & 32u)) {
                float b[3], z;
                sample_bz(t, T, ox0 + ox, oy0 + oy, b, z);
                cov = z >= 0.0f && z <= 1.0f;
            }
            mask |= (uint32_t)cov << s;
        }
    } else {
#pragma unroll 1
        for (int s = 0; s < NS; ++s) {
            const int ox = ox0 + (NS == 1 ? 128 : c_sample_loc8[s][0]), oy = oy0 + (NS == 1 ? 128 : c_sample_loc8[s][1]);
            bool cov = true;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const long long e = t.E[i] + (T.dXl[i] * oy - T.dYl[i] * ox);
                cov = cov && (e > 0 || (e == 0 && ((t.flags >> i) & 1u)));
            }
            if (cov) {
                float b[3], z;
                sample_bz(t, T, ox, oy, b, z);
                cov = z >= 0.0f && z <= 1.0f;
            }
            mask |= (uint32_t)cov << s;
        }
    }
    return mask;
}

// Per-sample work of the coverage kernels (opacity stores, fragment
// emission) over the round's covered samples dealt one per lane (true), or
// over each lane's own pixel mask (false).
constexpr bool kDealCoveredSamples = true;

// The covered samples of a warp's 32 pixels (lane i's pixel has coverage
// mask `mask`), dealt one per lane in (pixel, sample) order, 32 per round:
// fn(valid, o, s, r) runs on every lane (valid false on the lanes past the
// last sample) for the r-th covered sample s of lane o's pixel.  Every lane
// does the same per-sample work whatever its own pixel's coverage; fn may
// shuffle (all lanes call it together).
template <class Fn>
__device__ __forceinline__ void for_each_covered(uint32_t mask, int lane, Fn&& fn) {
    constexpr unsigned FULL = 0xffffffffu;
    const uint32_t c = __popc(mask);
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31), excl = incl - c;
    for (uint32_t k0 = 0; k0 < total; k0 += 32u) {
        const uint32_t k = k0 + (uint32_t)lane;
        int o = 0;  // the first lane whose inclusive count exceeds k
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1)
            if (__shfl_sync(FULL, incl, o + step - 1) <= k) o += step;
        o = min(o, 31);
        const uint32_t mo = __shfl_sync(FULL, mask, o), r = k - __shfl_sync(FULL, excl, o);
        const bool valid = k < total;
        fn(valid, o, valid ? (int)__fns(mo, 0u, (int)r + 1) : 0, r);
    }
}

// The next chunk of 32 tiles for the calling warp.
__device__ __forceinline__ uint32_t next_chunk(unsigned int* ticket, int lane) {
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(ticket, 1u);
    return __shfl_sync(0xffffffffu, c, 0);
}

// Coverage kernels.  A warp takes 32 consecutive 8x8 tiles of (triangle,
// level) items -- one per lane -- sets each up once into shared memory, then
// flattens the (tile, pixel) pairs of all 32 tiles and walks them 32 at a
// time, one pixel (all of its samples) per lane, so every lane does the same
// work however unequal the tiles are.  Pixel q of the flattened list belongs
// to the first tile whose inclusive pixel sum exceeds q; within a tile pixels
// are row-major, so the list is in traversal order (item, tile, pixel, sample).
//   P_DIRECT writes the pass's output (opacity, shadow depth, atomic injection);
//   P_COUNT counts covered samples and their records per tile;
//   P_WRITE emits one FragDesc per covered sample at its rank within the tile
//   (earlier rounds' count + a warp scan over the lanes of the same tile),
//   skipping the tiles whose count (`counts`, from P_COUNT) is zero.
// A tile's item comes from the tile plan's tile -> item array.
template <int KIND, int PHASE>
__global__ void __launch_bounds__(128, 6) k_cover(const __grid_constant__ RasterArgs A, const TilePlan plan,
                                               uint2* __restrict__ counts, const uint2* __restrict__ offs,
                                               FragDesc* __restrict__ frags, int* __restrict__ err) {
    constexpr int NS = (KIND == K_SHADOW || KIND == K_GBUFFER) ? 1 : 8;
    constexpr bool RANKED = PHASE != P_DIRECT;
    // the opacity writes run over the round's covered samples dealt to the lanes
    constexpr bool FLAT_OPACITY = kDealCoveredSamples && (KIND == K_OPACITY || KIND == K_OPA_COUNT) && PHASE != P_WRITE;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ TileSlot slots[4][32];
    const int lane = threadIdx.x & 31;
    TileSlot* S = slots[threadIdx.x >> 5];
    const uint32_t* __restrict__ tile_end = plan.tile_end;
    const uint32_t total = plan.total;
    const uint32_t nchunks = (total + 31u) >> 5;
    // chunks are dealt to the warps as they free up (a ticket), so unequal chunks do not leave SMs idle at the
    // end; every chunk's results depend only on its index
    for (uint32_t ch = next_chunk(plan.ticket, lane); ch < nchunks; ch = next_chunk(plan.ticket, lane)) {
        const uint32_t g = ch * 32u + lane;
        uint32_t npx = 0;
        // the emit phase skips tiles whose count pass found no covered sample
        if (g < total && !(PHASE == P_WRITE && counts[g].x == 0u)) {
            const int64_t item = plan.tile_item[g];
            const uint32_t local = g - (item > 0 ? tile_end[item - 1] : 0u);
            int64_t tri;
            int lvl;
            item_of(A, item, tri, lvl);
            const WTri w = world_triangle(A.s, tri);
            RSetup rs;
            float3 pos[3];
            bool live = item_setup<KIND>(A, w, lvl, rs, pos);
            const uint32_t mi = min(w.material, (uint32_t)max(A.s.material_count - 1, 0));
            uint32_t per = 1u;
            if (KIND == K_GBUFFER) live = live && !gbuffer_discarded(A, material_of(A.s, mi));
            if (KIND != K_SHADOW && KIND != K_GBUFFER) {
                const vct_gltf_shade_material mat = material_of(A.s, mi);
                live = live && !item_discarded(A, mat);
                if (KIND == K_INJECT || KIND == K_OPA_COUNT) per = inject_per_fragment(mat);
                if (KIND == K_INJECT) live = live && ((A.count_levels >> lvl) & 1u);
            }
            TileSlot& T = S[lane];
            T.per = per;
            if (live) {
                const int tcols = ((rs.px1 - rs.px0) >> 3) + 1;
                const int tx = rs.px0 + 8 * (int)(local % (uint32_t)tcols), ty = rs.py0 + 8 * (int)(local / (uint32_t)tcols);
                const int tw = min(tx + 7, rs.px1) - tx + 1, th = min(ty + 7, rs.py1) - ty + 1;
                npx = tile_regs(rs, tx, ty, T) ? (uint32_t)(tw * th) : 0u;
                T.tx = tx;
                T.ty = ty;
                T.tw = tw;
                T.tw_magic = tw > 1 ? (uint32_t)(0xffffffffu / (uint32_t)tw) + 1u : 0u;
                T.meta = (uint32_t)lvl | (mi << 3);
                T.item = (uint32_t)item;
                if (KIND != K_SHADOW && KIND != K_GBUFFER) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        T.p[k] = KIND == K_SVO ? pos[k] : w.p[k];
                        T.n[k] = w.n[k];
                    }
                }
                if (PHASE == P_WRITE) {
                    const uint2 b = offs[g];
                    T.base_f = b.x;
                    T.base_r = b.y;
                }
            }
        }
        // ---- flattened pixel list of the warp's tiles
        uint32_t incl = npx;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL, incl, d);
            if (lane >= d) incl += v;
        }
        S[lane].px_end = incl;
        S[lane].done = 0u;
        const uint32_t P = __shfl_sync(FULL, incl, 31);
        __syncwarp();
        TileRegs t;
        int cj = -1;
        if (KIND == K_SHADOW || KIND == K_GBUFFER) {
            // one centre sample per pixel: each lane takes four consecutive
            // pixels of the list per round, so the tile search and slot reload
            // are shared by four depth tests
            for (uint32_t q0 = (uint32_t)lane * 4u; q0 < P; q0 += 128u) {
                int lo = 0, hi = 31;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (S[mid].px_end > q0) hi = mid;
                    else lo = mid + 1;
                }
                int j = lo;
                for (uint32_t q = q0; q < q0 + 4u && q < P; ++q) {
                    while (S[j].px_end <= q) ++j;  // the next pixel's tile (at most 3 steps)
                    if (j != cj) {
                        t = S[j].t;
                        cj = j;
                    }
                    const uint32_t start = j > 0 ? S[j - 1].px_end : 0u;
                    const uint32_t lp = q - start, tw = (uint32_t)S[j].tw;
                    const uint32_t row = tw > 1u ? __umulhi(lp, S[j].tw_magic) : lp;
                    const int ox0 = (int)(lp - row * tw) * 256, oy0 = (int)row * 256;
                    if (cover_pixel<1>(t, S[j], ox0, oy0)) {
                        float b[3], z;
                        sample_bz(t, S[j], ox0 + 128, oy0 + 128, b, z);
                        const int px = S[j].tx + (ox0 >> 8), py = S[j].ty + (oy0 >> 8);
                        if (KIND == K_SHADOW) {
                            atomicMin(reinterpret_cast<unsigned int*>(A.depth) + (int64_t)py * A.W + px,
                                      __float_as_uint(z));
                        } else if (z < 1.0f) {  // depth test LESS against the cleared 1.0
                            // z >= 0 here; -0 is keyed as +0 so the bit order is the numeric order
                            atomicMin(A.vis + (int64_t)py * A.W + px,
                                      ((unsigned long long)(__float_as_uint(z) & 0x7fffffffu) << 32) | S[j].item);
                        }
                    }
                }
            }
            __syncwarp();
            continue;
        }
        for (uint32_t q0 = 0; q0 < P; q0 += 32u) {
            const uint32_t q = q0 + lane;
            const bool act = q < P;
            int j = 0;
            uint32_t start = 0, mask = 0;
            int px = 0, py = 0, ox0 = 0, oy0 = 0;
            if (act) {
                int lo = 0, hi = 31;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (S[mid].px_end > q) hi = mid;
                    else lo = mid + 1;
                }
                j = lo;
                start = j > 0 ? S[j - 1].px_end : 0u;
                if (j != cj) {
                    t = S[j].t;
                    cj = j;
                }
                const uint32_t lp = q - start, tw = (uint32_t)S[j].tw;
                const uint32_t row = tw > 1u ? __umulhi(lp, S[j].tw_magic) : lp;
                ox0 = (int)(lp - row * tw) * 256;
                oy0 = (int)row * 256;
                px = S[j].tx + (ox0 >> 8);
                py = S[j].ty + (oy0 >> 8);
                mask = cover_pixel<NS>(t, S[j], ox0, oy0);
                if (!FLAT_OPACITY && (PHASE == P_DIRECT || KIND == K_OPA_COUNT) && mask) {
                    const TileSlot& T = S[j];
                    const int lvl = (int)(T.meta & 7u);
                    int3 last_ic = make_int3(-1, -1, -1);  // opacity: the previous sample's voxel (stores are idempotent)
                    for (uint32_t m = mask; m; m &= m - 1u) {
                        const int s = __ffs(m) - 1;
                        float b[3], z;
                        sample_bz(t, T, ox0 + (NS == 1 ? 128 : c_sample_loc8[s][0]),
                                  oy0 + (NS == 1 ? 128 : c_sample_loc8[s][1]), b, z);
                        if (KIND == K_SHADOW) {
                            atomicMin(reinterpret_cast<unsigned int*>(A.depth) + (int64_t)py * A.W + px, __float_as_uint(z));
                        } else if (KIND == K_OPACITY || KIND == K_OPA_COUNT) {
                            const vct_voxelization_desc& d = A.vd[lvl];
                            const float3 wp = interp3(b, T.p);
                            if (wp.x < d.region_min_corner[0] || wp.y < d.region_min_corner[1] ||
                                wp.z < d.region_min_corner[2] || wp.x > d.region_max_corner[0] ||
                                wp.y > d.region_max_corner[1] || wp.z > d.region_max_corner[2])
                                continue;
                            if (((A.slab_levels >> lvl) & 1u) && !in_slabs(A, lvl, wp)) continue;
                            const AtlasDims AD(A.R);
                            const int3 ic = clip_image_coords(d, wp);
                            if (ic.x == last_ic.x && ic.y == last_ic.y && ic.z == last_ic.z) continue;
                            last_ic = ic;
                            if (A.opa_r8) {
                                uint8_t* a8 = reinterpret_cast<uint8_t*>(A.atlas);
                                for (int f = 0; f < 6; ++f) a8[AD.index(ic.x + (A.R + 2) * f, ic.y, ic.z)] = 0xFFu;
                            } else {
                                for (int f = 0; f < 6; ++f) A.atlas[AD.index(ic.x + (A.R + 2) * f, ic.y, ic.z)] = 0xFFFFFFFFu;
                            }
                        } else if (KIND == K_INJECT) {
                            const vct_gltf_shade_material mat = material_of(A.s, T.meta >> 3);
                            InjRecord upd[6];
                            const int k = inject_fragment(A, mat, lvl, interp3(b, T.p), interp3(b, T.n), upd);
                            for (int i = 0; i < k; ++i)
                                rgba8_avg_atomic(A.atlas + upd[i].key, upd[i].r, upd[i].g, upd[i].b, 1.0f, err);
                        }
                    }
                }
            }
            if constexpr (FLAT_OPACITY) {
                // opacity: every covered sample inside its level's region (and
                // slabs) marks its voxel on all six faces; a sample in the same
                // voxel as the previous one of its pixel skips the (idempotent) stores
                for_each_covered(mask, lane, [&](bool valid, int o, int s, uint32_t) {
                    const int jo = __shfl_sync(FULL, j, o), oxo = __shfl_sync(FULL, ox0, o),
                              oyo = __shfl_sync(FULL, oy0, o);
                    int3 ic = make_int3(-1, -1, -1);
                    bool keep = false;
                    if (valid) {
                        const TileSlot& T = S[jo];
                        const int lvl = (int)(T.meta & 7u);
                        float b[3], z;
                        sample_bz(T.t, T, oxo + c_sample_loc8[s][0], oyo + c_sample_loc8[s][1], b, z);
                        const vct_voxelization_desc& d = A.vd[lvl];
                        const float3 wp = interp3(b, T.p);
                        const bool inside = !(wp.x < d.region_min_corner[0] || wp.y < d.region_min_corner[1] ||
                                              wp.z < d.region_min_corner[2] || wp.x > d.region_max_corner[0] ||
                                              wp.y > d.region_max_corner[1] || wp.z > d.region_max_corner[2]) &&
                                            !(((A.slab_levels >> lvl) & 1u) && !in_slabs(A, lvl, wp));
                        if (inside) {
                            ic = clip_image_coords(d, wp);
                            keep = true;
                        }
                    }
                    const int po = __shfl_up_sync(FULL, keep ? o : -1, 1), qx = __shfl_up_sync(FULL, ic.x, 1),
                              qy = __shfl_up_sync(FULL, ic.y, 1), qz = __shfl_up_sync(FULL, ic.z, 1);
                    const bool dup = lane > 0 && po == o && qx == ic.x && qy == ic.y && qz == ic.z;
                    if (keep && !dup) {
                        const AtlasDims AD(A.R);
                        if (A.opa_r8) {
                            uint8_t* a8 = reinterpret_cast<uint8_t*>(A.atlas);
                            for (int f = 0; f < 6; ++f) a8[AD.index(ic.x + (A.R + 2) * f, ic.y, ic.z)] = 0xFFu;
                        } else {
                            for (int f = 0; f < 6; ++f) A.atlas[AD.index(ic.x + (A.R + 2) * f, ic.y, ic.z)] = 0xFFFFFFFFu;
                        }
                    }
                });
            }
            if (RANKED) {
                if (KIND == K_OPA_COUNT && act && !((A.count_levels >> (S[j].meta & 7u)) & 1u)) mask = 0u;
                const uint32_t c = __popc(mask);
                uint32_t ci = c;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t v = __shfl_up_sync(FULL, ci, d);
                    if (lane >= d) ci += v;
                }
                const uint32_t cx = ci - c;
                const int first = (act && start > q0) ? (int)(start - q0) : 0;  // first lane of my tile this round
                const uint32_t cx_first = __shfl_sync(FULL, cx, first);
                const uint32_t rank = act ? S[j].done + (cx - cx_first) : 0u;
                const bool last = act && (lane == 31 || q + 1u == P || q + 1u == S[j].px_end);
                __syncwarp();
                if (last) S[j].done += ci - cx_first;
                __syncwarp();
                if constexpr (PHASE == P_WRITE && !kDealCoveredSamples) {
                    if (mask) {
                        const TileSlot& T = S[j];
                        uint32_t k = rank;
                        for (uint32_t m = mask; m; m &= m - 1u) {
                            const int s = __ffs(m) - 1;
                            float b[3], z;
                            sample_bz(t, T, ox0 + c_sample_loc8[s][0], oy0 + c_sample_loc8[s][1], b, z);
                            const float3 p = interp3(b, T.p);
                            const float3 nn = interp3(b, T.n);
                            FragDesc d;
                            d.p = make_float4(p.x, p.y, p.z, __uint_as_float(T.base_r + k * T.per));
                            d.n = make_float4(nn.x, nn.y, nn.z, __uint_as_float(T.meta));
                            frags[T.base_f + k] = d;
                            ++k;
                        }
                    }
                }
                if constexpr (PHASE == P_WRITE && kDealCoveredSamples) {
                    // the r-th covered sample of a pixel goes to its tile's slot rank + r
                    for_each_covered(mask, lane, [&](bool valid, int o, int s, uint32_t r) {
                        const int jo = __shfl_sync(FULL, j, o), oxo = __shfl_sync(FULL, ox0, o),
                                  oyo = __shfl_sync(FULL, oy0, o);
                        const uint32_t k = __shfl_sync(FULL, rank, o) + r;
                        if (valid) {
                            const TileSlot& T = S[jo];
                            float b[3], z;
                            sample_bz(T.t, T, oxo + c_sample_loc8[s][0], oyo + c_sample_loc8[s][1], b, z);
                            const float3 p = interp3(b, T.p);
                            const float3 nn = interp3(b, T.n);
                            FragDesc d;
                            d.p = make_float4(p.x, p.y, p.z, __uint_as_float(T.base_r + k * T.per));
                            d.n = make_float4(nn.x, nn.y, nn.z, __uint_as_float(T.meta));
                            frags[T.base_f + k] = d;
                        }
                    });
                }
            }
        }
        __syncwarp();
        if (PHASE == P_COUNT && g < total) counts[g] = make_uint2(S[lane].done, S[lane].done * S[lane].per);
        __syncwarp();
    }
}

template <int KIND, int PHASE>
static void launch_cover(const RasterArgs& A, const TilePlan& plan, uint2* counts, const uint2* offs, FragDesc* frags,
                         int* err, cudaStream_t st) {
    const uint32_t nchunks = (plan.total + 31u) >> 5;
    int blocks = (int)((nchunks + 3u) >> 2);
    blocks = blocks < 1 ? 1 : (blocks > 152 * 16 ? 152 * 16 : blocks);
    // (an error of the zeroing is the thread's last error, which the callers' launch check reads)
    cudaMemsetAsync(plan.ticket, 0, sizeof(unsigned int), st);
    k_cover<KIND, PHASE><<<blocks, 128, 0, st>>>(A, plan, counts, offs, frags, err);
}

// Injection shading, one thread per covered sample: writes its face records
// (texel key, colour) at the scanned record offset; the records that the
// fragment shader does not produce (a fragment in shadow produces none) get
// the invalid key and are dropped before the sort.
__global__ void __launch_bounds__(256) k_inject_shade(const __grid_constant__ RasterArgs A, const FragDesc* __restrict__ frags,
                                                      uint32_t nfrag, uint32_t* __restrict__ keys,
                                                      float4* __restrict__ rgb) {
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nfrag; f += gridDim.x * blockDim.x) {
        const FragDesc d = frags[f];
        const uint32_t rec = __float_as_uint(d.p.w), meta = __float_as_uint(d.n.w);
        const vct_gltf_shade_material mat = material_of(A.s, meta >> 3);
        InjRecord upd[6];
        const int k = inject_fragment(A, mat, (int)(meta & 7u), make_float3(d.p.x, d.p.y, d.p.z),
                                      make_float3(d.n.x, d.n.y, d.n.z), upd);
        const uint32_t per = inject_per_fragment(mat);
        for (uint32_t i = 0; i < per; ++i) {
            const bool v = (int)i < k;
            keys[rec + i] = v ? upd[i].key : A.invalid_key;
            if (v) rgb[rec + i] = make_float4(upd[i].r, upd[i].g, upd[i].b, 0.0f);
        }
    }
}

// SVO fragment shading, one thread per covered sample: writes the packed
// (position, colour) pair into its slot; light-discarded slots stay zero.
__global__ void __launch_bounds__(256) k_svo_shade(const __grid_constant__ RasterArgs A, const FragDesc* __restrict__ frags,
                                                   uint32_t nfrag) {
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nfrag; f += gridDim.x * blockDim.x) {
        const FragDesc d = frags[f];
        const uint32_t slot = __float_as_uint(d.p.w), meta = __float_as_uint(d.n.w);
        const vct_gltf_shade_material mat = material_of(A.s, meta >> 3);
        bool valid = false;
        uint2 v;
        svo_fragment(A, mat, make_float3(d.p.x, d.p.y, d.p.z), make_float3(d.n.x, d.n.y, d.n.z), &valid, &v);
        if (valid && (int64_t)slot < A.frag_capacity) reinterpret_cast<uint2*>(A.frags)[slot] = v;
    }
}

// Boundaries of the texel runs in the sorted record keys over positions
// [0, n]: every position whose key differs from its predecessor, plus 0 and
// n, so run h is [heads[h], heads[h + 1]).  (The fold would skip a run of
// invalid keys; the compaction before the sort leaves none.)
struct RunHead {
    const uint32_t* keys;
    uint32_t n;
    __device__ bool operator()(uint32_t i) const { return i == 0 || i == n || keys[i - 1] != keys[i]; }
};

// The records the fragment shader produced (stable compaction before the sort).
struct ValidKey {
    uint32_t invalid;
    __device__ bool operator()(uint32_t k) const { return k != invalid; }
};
struct ValidRecord {
    const uint32_t* keys;
    uint32_t invalid;
    __device__ bool operator()(uint32_t i) const { return keys[i] != invalid; }
};

struct SumU2 {
    __host__ __device__ uint2 operator()(uint2 a, uint2 b) const { return make_uint2(a.x + b.x, a.y + b.y); }
};

// gBufferPass.frag at each pixel's closest fragment, written as the
// vct_surface_sample the trace reads: the sub-triangle the visibility pass
// kept is set up again, its FP32 barycentrics at the pixel centre are made
// perspective-correct (b_k / w_k, normalised) and mapped to the original
// triangle's, the world normal and the material give the attachments' values,
// which are stored through their formats (diffuse / specular RGBA8 UNORM,
// normal / emission RGBA16F), and the world position is rebuilt from the depth
// as worldPosFromDepth does (voxelConeTracing.frag:305-311).  Pixels with no
// fragment keep depth 1 (the trace leaves them untouched).
__device__ inline float u8_texel(float x) { return unorm8_decode(unorm8_store(x)); }
__device__ inline float f16_texel(float x) { return __half2float(__float2half_rn(x)); }

__global__ void __launch_bounds__(256) k_gbuffer_resolve(const __grid_constant__ RasterArgs A, const M4 vp_inv,
                                                         vct_surface_sample* __restrict__ out) {
    const int64_t npx = (int64_t)A.W * A.H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npx; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = A.vis[i];
        const int px = (int)(i % A.W), py = (int)(i / A.W);
        // the attachments' clear values: colour (0, 0, 0, 1), depth 1
        float depth = 1.0f;
        float4 r1 = make_float4(0.f, 0.f, 0.f, 1.0f), r2 = r1, r3 = r1, r4 = r1;
        if (key != ~0ull) {
            depth = __uint_as_float((uint32_t)(key >> 32));
            const uint32_t item = (uint32_t)key;
            const int64_t tri = item / 6u;
            const int sub = (int)(item % 6u);
            const WTri w = world_triangle(A.s, tri);
            float4 h[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) h[k] = mat_vec4(A.pv, w.p[k].x, w.p[k].y, w.p[k].z, 1.0f);
            ClipVert v[3];
            clip_sub_triangle(h, sub, v);  // the visibility pass drew this sub-triangle
            float4 c[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) c[k] = make_float4(v[k].x / v[k].w, v[k].y / v[k].w, v[k].z / v[k].w, 1.0f);
            const RSetup rs = raster_setup(c, A.W, A.H);
            const long long sx = (long long)px * 256 + 128, sy = (long long)py * 256 + 128;
            float bo[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const int a = (e + 1) % 3, cc = (e + 2) % 3;
                const long long ev = (rs.X[cc] - rs.X[a]) * (sy - rs.Y[a]) - (rs.Y[cc] - rs.Y[a]) * (sx - rs.X[a]);
                bo[e] = (float)ev * rs.inv_area;
            }
            const float b[3] = {bo[0], rs.swapped ? bo[2] : bo[1], rs.swapped ? bo[1] : bo[2]};
            // perspective-correct weights of the sub-triangle's vertices, then
            // of the original triangle's
            float q[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) q[k] = b[k] / v[k].w;
            const float qs = (q[0] + q[1]) + q[2];
#pragma unroll
            for (int k = 0; k < 3; ++k) q[k] = q[k] / qs;
            float lam[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) lam[j] = (q[0] * v[0].l[j] + q[1] * v[1].l[j]) + q[2] * v[2].l[j];
            const float3 nrm = normalize3h(interp3(lam, w.n));
            // gBufferPass.frag:64-121 with 1x1 textures (no tangents: the
            // normal texture is not applied)
            const vct_gltf_shade_material mat = material_of(A.s, w.material);
            float rough = mat.pbr_roughness_factor, metal = mat.pbr_metallic_factor;
            if (mat.pbr_metallic_roughness_texture > -1) {
                const float4 mr = texture_1x1(A.s, mat.pbr_metallic_roughness_texture);
                rough = rough * mr.y;
                metal = metal * mr.z;
            } else {
                rough = fminf(fmaxf(rough, 0.04f), 1.0f);
                metal = fminf(fmaxf(metal, 0.0f), 1.0f);
            }
            const float4 base = gbuffer_base_color(A, mat);
            const float dk = 1.0f - metal;
            const float3 diff = make_float3(base.x * 0.96f * dk, base.y * 0.96f * dk, base.z * 0.96f * dk);
            const float3 spec = make_float3(mix_rn(0.04f, base.x, metal), mix_rn(0.04f, base.y, metal),
                                            mix_rn(0.04f, base.z, metal));
            float3 em = make_float3(mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]);
            if (mat.emissive_texture > -1) {
                const float4 t = texture_1x1(A.s, mat.emissive_texture);
                em = make_float3(em.x * powf(t.x, 2.2f), em.y * powf(t.y, 2.2f), em.z * powf(t.z, 2.2f));
            }
            r1 = make_float4(f16_texel(nrm.x * 0.5f + 0.5f), f16_texel(nrm.y * 0.5f + 0.5f), f16_texel(nrm.z * 0.5f + 0.5f),
                             1.0f);
            r2 = make_float4(u8_texel(diff.x), u8_texel(diff.y), u8_texel(diff.z), u8_texel(rough));
            r3 = make_float4(u8_texel(spec.x), u8_texel(spec.y), u8_texel(spec.z), u8_texel(metal));
            r4 = make_float4(f16_texel(em.x), f16_texel(em.y), f16_texel(em.z), 1.0f);
        }
        // worldPosFromDepth (voxelConeTracing.frag:305-311) at the pixel centre
        const float u = ((float)px + 0.5f) / (float)A.W, vv = ((float)py + 0.5f) / (float)A.H;
        const float4 wp = mat_vec4(vp_inv.m, u * 2.0f - 1.0f, vv * 2.0f - 1.0f, depth, 1.0f);
        float4* o = reinterpret_cast<float4*>(out + i);
        o[0] = make_float4(wp.x / wp.w, wp.y / wp.w, wp.z / wp.w, depth);
        o[1] = r1;
        o[2] = r2;
        o[3] = r3;
        o[4] = r4;
    }
}

// Sequential per-texel fold of the stably sorted injection records, one
// thread per texel run.
//
// Only the tail of a long run matters.  Every injection record has alpha 1,
// so a step maps the stored alpha byte a to (a + 1) & 0xff whatever the colour
// (the store truncates the float sum a + 1 and keeps its low byte): alpha is
// a step counter mod 256.  A step whose input has alpha 0 computes
// rgb * 0 + v over 0 + 1, i.e. exactly the record's own value with alpha 1,
// which is also what it computes from an empty (zero) texel.  So if k* is
// the last step of the run whose input alpha is 0, the result equals the fold
// of records k*.. from zero, and a run costs at most 256 serial steps however
// many records land on its texel (fragments clamped onto region borders pile
// hundreds of thousands onto single texels).
// `touched` (the frame's path, may be null): the texels start from zero (their
// level is being refreshed) and each one written is marked in the bitmap.
__global__ void __launch_bounds__(256) k_inject_fold(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ order,
                                                     const float4* __restrict__ rgb, const uint32_t* __restrict__ heads,
                                                     const uint32_t* __restrict__ nheads, uint32_t invalid_key,
                                                     uint32_t* __restrict__ atlas, uint32_t* __restrict__ touched) {
    const uint32_t nruns = *nheads - 1u;
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nruns; h += gridDim.x * blockDim.x) {
        const uint32_t s = heads[h], e = heads[h + 1];
        const uint32_t key = keys[s];
        if (key == invalid_key) continue;
        uint32_t cell = 0u;
        if (touched) atomicOr(touched + (key >> 5), 1u << (key & 31u));
        else cell = atlas[key];
        const uint32_t len = e - s;
        const uint32_t k0 = (256u - (cell >> 24)) & 255u;  // first step whose input alpha is 0
        uint32_t j = s;
        if (k0 < len) {
            j = s + k0 + ((len - 1u - k0) & ~255u);  // the last such step
            cell = 0u;
        }
        // the fold is a serial chain; fetch four records ahead of it
        for (; j < e; j += 4) {
            float4 r4[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + u < e) r4[u] = rgb[order[j + u]];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + u < e) cell = rgba8_avg_fold(cell, r4[u].x, r4[u].y, r4[u].z, 1.0f);
        }
        atlas[key] = cell;
    }
}

__global__ void k_fill_f32(float* p, int64_t n, float v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// ---------------------------------------------------------------- host side
static int grid_of(int64_t n, int block, int cap = 152 * 32) {
    int64_t g = (n + block - 1) / block;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

int workspace_reserve(vct_workspace_s* ws, size_t bytes) {
    if (ws->bytes >= bytes) return VCT_OK;
    if (ws->ptr) {
        VCT_CUDA_TRY(cudaDeviceSynchronize());
        VCT_CUDA_TRY(cudaFree(ws->ptr));
        ws->ptr = nullptr;
        ws->bytes = 0;
    }
    size_t want = bytes + bytes / 4;
    VCT_CUDA_TRY(cudaMalloc(&ws->ptr, want));
    ws->bytes = want;
    return VCT_OK;
}

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

static int check_scene(const vct_scene* s) {
    VCT_CHECK_ARG(s, "null scene");
    VCT_CHECK_ARG(s->triangle_count >= 0 && s->triangle_count < (1LL << 31), "scene triangle count out of range");
    if (s->triangle_count == 0) return VCT_OK;
    VCT_CHECK_ARG(s->positions && s->normals && s->indices, "scene positions / normals / indices are required");
    VCT_CHECK_ARG(s->materials && s->material_count > 0, "scene needs at least one material");
    VCT_CHECK_ARG(!s->node_matrices || s->instance_count > 0, "node matrices given without an instance count");
    VCT_CHECK_ARG(s->vertex_count > 0 && s->vertex_count <= (1LL << 32), "scene vertex count out of range");
    return VCT_OK;
}

// Tile plan shared by every pass: inclusive tile sums per item and the item
// of every tile, in the workspace from offset 0; `off` is advanced past them.
static int plan_tiles(RasterArgs& A, vct_workspace_s* ws, size_t& off, TilePlan* plan, cudaStream_t st) {
    VCT_CHECK_ARG(A.items < (1LL << 31), "rasteriser: more than 2^31 (triangle, level) items");
    const size_t n = (size_t)A.items;
    size_t scan_bytes = 0;
    VCT_CUDA_TRY(cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)n));
    const size_t need = a256(4 * n) * 2 + a256(scan_bytes) + 256;
    int rc = workspace_reserve(ws, need);
    if (rc != VCT_OK) return rc;
    char* base = (char*)ws->ptr;
    uint32_t* counts = (uint32_t*)base;
    uint32_t* tile_end = (uint32_t*)(base + a256(4 * n));
    void* tmp = base + 2 * a256(4 * n);
    off = 2 * a256(4 * n) + a256(scan_bytes);
    switch (A.kind) {
        case K_OPACITY: k_item_tiles<K_OPACITY><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        case K_INJECT: k_item_tiles<K_INJECT><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        case K_SHADOW: k_item_tiles<K_SHADOW><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        case K_SVO: k_item_tiles<K_SVO><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        case K_OPA_COUNT: k_item_tiles<K_OPA_COUNT><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        case K_GBUFFER: k_item_tiles<K_GBUFFER><<<grid_of(n, 128), 128, 0, st>>>(A, counts); break;
        default: return fail(VCT_E_BAD_ARG, "rasteriser: unknown pass kind");
    }
    VCT_LAUNCH_CHECK();
    VCT_CUDA_TRY(cub::DeviceScan::InclusiveSum(tmp, scan_bytes, counts, tile_end, (int)n, st));
    uint32_t total = 0;
    VCT_CUDA_TRY(cudaMemcpyAsync(&total, tile_end + (n - 1), 4, cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaStreamSynchronize(st));
    if (ws->bytes < off + a256(4 * (size_t)total) + 256) {
        rc = workspace_reserve(ws, off + a256(4 * (size_t)total) + 256);
        if (rc != VCT_OK) return rc;
        return plan_tiles(A, ws, off, plan, st);  // the arena moved: plan again
    }
    uint32_t* tile_item = (uint32_t*)(base + off);
    off += a256(4 * (size_t)total);
    unsigned int* ticket = (unsigned int*)(base + off);
    off += 256;
    if (total) {
        k_tile_items<<<grid_of(n, 256), 256, 0, st>>>(tile_end, A.items, tile_item);
        VCT_LAUNCH_CHECK();
    }
    plan->tile_end = tile_end;
    plan->tile_item = tile_item;
    plan->total = total;
    plan->ticket = ticket;
    return VCT_OK;
}

// Returned (positive) when the workspace had to grow: buffers carved before
// the growth moved, so the caller restarts its pass from the top.
constexpr int kWorkspaceGrew = 1;

// Coverage count + exclusive scan of (covered samples, records) per tile for
// the injection and the SVO pass.  On VCT_OK *counts_out and *offs (in the
// workspace, `off` advanced past them) hold each tile's counts and its first
// descriptor / record, and *nfrag / *nrec the totals (host).
template <int KIND>
static int count_tiles(RasterArgs& A, vct_workspace_s* ws, size_t& off, const TilePlan& plan, uint2** counts_out,
                       uint2** offs, uint32_t* nfrag, uint32_t* nrec, cudaStream_t st) {
    const uint32_t total = plan.total;
    size_t scan_bytes = 0;
    VCT_CUDA_TRY(cub::DeviceScan::ExclusiveScan(nullptr, scan_bytes, (uint2*)nullptr, (uint2*)nullptr, SumU2{},
                                                make_uint2(0u, 0u), (int)total));
    const size_t need = off + a256(8 * (size_t)total) * 2 + a256(scan_bytes) + 256;
    if (ws->bytes < need) {
        int rc = workspace_reserve(ws, need);
        return rc != VCT_OK ? rc : kWorkspaceGrew;
    }
    char* base = (char*)ws->ptr + off;
    uint2* counts = (uint2*)base;
    *counts_out = counts;
    *offs = (uint2*)(base + a256(8 * (size_t)total));
    void* tmp = base + 2 * a256(8 * (size_t)total);
    off += 2 * a256(8 * (size_t)total) + a256(scan_bytes);
    launch_cover<KIND, P_COUNT>(A, plan, counts, nullptr, nullptr, nullptr, st);
    VCT_LAUNCH_CHECK();
    VCT_CUDA_TRY(cub::DeviceScan::ExclusiveScan(tmp, scan_bytes, counts, *offs, SumU2{}, make_uint2(0u, 0u), (int)total, st));
    uint2 last[2];
    VCT_CUDA_TRY(cudaMemcpyAsync(&last[0], *offs + (total - 1), 8, cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaMemcpyAsync(&last[1], counts + (total - 1), 8, cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaStreamSynchronize(st));
    const uint64_t f = (uint64_t)last[0].x + last[1].x, r = (uint64_t)last[0].y + last[1].y;
    // the per-tile sums are 32-bit: a wrapped total shows as fewer records than fragments
    if (f >= (1ull << 31) || r >= (1ull << 31) || r < f)
        return fail(VCT_E_OVERFLOW, "rasteriser: more than 2^31 covered samples or records in one pass");
    *nfrag = (uint32_t)f;
    *nrec = (uint32_t)r;
    return VCT_OK;
}

// The deterministic injection after its coverage count: the emitted sample
// descriptors and the record arrays, carved from the workspace.
struct InjectState {
    TilePlan plan;
    uint32_t nfrag = 0, nrec = 0;
    FragDesc* fr = nullptr;
    float4* rgb = nullptr;
    uint32_t *kin = nullptr, *kout = nullptr, *vin = nullptr, *vout = nullptr, *heads = nullptr, *nheads = nullptr;
    uint32_t* nvalid = nullptr;
    void* stmp = nullptr;
    size_t sort_bytes = 0, select_bytes = 0;
    int key_bits = 0;
};

// Plan the tiles of `C`'s items, count covered samples and records per tile
// with the KIND kernel (K_INJECT; or K_OPA_COUNT, which also writes `C`'s
// opacity atlas), scan, read the totals back, reserve and carve everything
// the rest of the injection needs, and emit the descriptors with `I` (the
// injection's args over the same items).  Returns kWorkspaceGrew when the
// workspace moved: the caller restarts (every step here is idempotent).
template <int KIND>
static int inject_prepare(RasterArgs& C, RasterArgs& I, vct_workspace_s* ws, cudaStream_t st, InjectState* S) {
    size_t off;
    int rc = plan_tiles(C, ws, off, &S->plan, st);
    if (rc != VCT_OK) return rc;
    S->nfrag = S->nrec = 0;
    if (S->plan.total == 0) return VCT_OK;
    uint2 *counts, *offs;
    rc = count_tiles<KIND>(C, ws, off, S->plan, &counts, &offs, &S->nfrag, &S->nrec, st);
    if (rc != VCT_OK) return rc;  // including kWorkspaceGrew
    if (S->nfrag == 0) return VCT_OK;
    const uint32_t nfrag = S->nfrag, nrec = S->nrec;
    S->key_bits = 32 - __builtin_clz((unsigned)I.invalid_key);
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, S->sort_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                 (uint32_t*)nullptr, (uint32_t*)nullptr, (int)nrec, 0, S->key_bits));
    VCT_CUDA_TRY(cub::DeviceSelect::If(nullptr, S->select_bytes, thrust::counting_iterator<uint32_t>(0u),
                                       (uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)nrec + 1,
                                       RunHead{nullptr, nrec}));
    size_t sel_keys = 0, sel_recs = 0;
    VCT_CUDA_TRY(cub::DeviceSelect::If(nullptr, sel_keys, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                       (int64_t)nrec, ValidKey{0u}));
    VCT_CUDA_TRY(cub::DeviceSelect::If(nullptr, sel_recs, thrust::counting_iterator<uint32_t>(0u), (uint32_t*)nullptr,
                                       (uint32_t*)nullptr, (int64_t)nrec, ValidRecord{nullptr, 0u}));
    if (sel_keys > S->select_bytes) S->select_bytes = sel_keys;
    if (sel_recs > S->select_bytes) S->select_bytes = sel_recs;
    const size_t r4 = a256(4 * (size_t)nrec + 4);
    const size_t need = off + a256(sizeof(FragDesc) * (size_t)nfrag) + a256(16 * (size_t)nrec) + 5 * r4 + 256 +
                        a256(S->sort_bytes > S->select_bytes ? S->sort_bytes : S->select_bytes);
    if (ws->bytes < need) {
        rc = workspace_reserve(ws, need);
        return rc != VCT_OK ? rc : kWorkspaceGrew;
    }
    char* p = (char*)ws->ptr + off;
    S->fr = (FragDesc*)p;
    p += a256(sizeof(FragDesc) * (size_t)nfrag);
    S->rgb = (float4*)p;
    p += a256(16 * (size_t)nrec);
    S->kin = (uint32_t*)p;
    S->kout = (uint32_t*)(p + r4);
    S->vin = (uint32_t*)(p + 2 * r4);
    S->vout = (uint32_t*)(p + 3 * r4);
    S->heads = (uint32_t*)(p + 4 * r4);
    S->nheads = (uint32_t*)(p + 5 * r4);
    S->nvalid = (uint32_t*)(p + 5 * r4 + 128);
    S->stmp = p + 5 * r4 + 256;
    launch_cover<K_INJECT, P_WRITE>(I, S->plan, counts, offs, S->fr, nullptr, st);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

// Shade the emitted samples into face records (needs the light and shadow
// map in `I`), keep the records the shader produced (stable compaction: the
// keys, and their record indices as the sort's values), sort them stably by
// texel and fold every texel's run.  The count of kept records is read back
// for the sort (a frame keeps the GPU busy meanwhile with its opacity mips on
// the side stream).
static int inject_finish(const RasterArgs& I, const InjectState& S, uint32_t* touched, cudaStream_t st) {
    if (S.nfrag == 0) return VCT_OK;
    const uint32_t nfrag = S.nfrag, nrec = S.nrec;
    k_inject_shade<<<grid_of(nfrag, 256), 256, 0, st>>>(I, S.fr, nfrag, S.kin, S.rgb);
    VCT_LAUNCH_CHECK();
    size_t tb = S.select_bytes;
    VCT_CUDA_TRY(cub::DeviceSelect::If(S.stmp, tb, S.kin, S.kout, S.nvalid, (int64_t)nrec, ValidKey{I.invalid_key}, st));
    tb = S.select_bytes;
    VCT_CUDA_TRY(cub::DeviceSelect::If(S.stmp, tb, thrust::counting_iterator<uint32_t>(0u), S.vout, S.nvalid,
                                       (int64_t)nrec, ValidRecord{S.kin, I.invalid_key}, st));
    uint32_t nv = 0;
    VCT_CUDA_TRY(cudaMemcpyAsync(&nv, S.nvalid, sizeof(nv), cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaStreamSynchronize(st));
    if (nv == 0) return VCT_OK;
    tb = S.sort_bytes;
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(S.stmp, tb, S.kout, S.kin, S.vout, S.vin, (int)nv, 0, S.key_bits, st));
    tb = S.select_bytes;
    VCT_CUDA_TRY(cub::DeviceSelect::If(S.stmp, tb, thrust::counting_iterator<uint32_t>(0u), S.heads, S.nheads,
                                       (int64_t)nv + 1, RunHead{S.kin, nv}, st));
    k_inject_fold<<<grid_of(nv, 256), 256, 0, st>>>(S.kin, S.vin, S.rgb, S.heads, S.nheads, I.invalid_key, I.atlas,
                                                    touched);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

static void fill_clipmap_levels(RasterArgs& A, const vct_clipmap_region* regions, int R, uint32_t level_mask) {
    A.nlevels = 0;
    for (int l = 0; l < 6; ++l) {
        voxel_view_proj(regions[l], &A.vp[l][0][0]);
        A.vd[l] = voxelization_desc(regions, l, R);
        if ((level_mask >> l) & 1u) A.levels[A.nlevels++] = l;
    }
}

static int fill_light(RasterArgs& A, const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                      const vct_directional_light_shadow_desc* light_shadow) {
    VCT_CHECK_ARG(light, "null light");
    memset(&A.light, 0, sizeof(A.light));
    A.light.light = *light;
    if (shadow && shadow->depth) {
        VCT_CHECK_ARG(light_shadow, "shadow map given without its light shadow desc");
        VCT_CHECK_ARG(shadow->width > 0 && shadow->height > 0, "bad shadow map size");
        A.light.shadow = shadow->depth;
        A.light.shadow_w = shadow->width;
        A.light.shadow_h = shadow->height;
        A.light.shadow_desc = *light_shadow;
    }
    float3 l = normalize3h(make_float3(-light->direction[0], -light->direction[1], -light->direction[2]));
    A.ldir[0] = l.x;
    A.ldir[1] = l.y;
    A.ldir[2] = l.z;
    return VCT_OK;
}

}  // namespace vct

using namespace vct;

extern "C" int vct_workspace_create(size_t initial_bytes, vct_workspace_s** out) {
    VCT_CHECK_ARG(out, "vct_workspace_create: null output");
    auto* w = new vct_workspace_s();
    if (initial_bytes) {
        cudaError_t e = cudaMalloc(&w->ptr, initial_bytes);
        if (e != cudaSuccess) {
            delete w;
            return cuda_fail(e, "cudaMalloc (workspace)");
        }
        w->bytes = initial_bytes;
    }
    *out = w;
    return VCT_OK;
}

extern "C" int vct_workspace_destroy(vct_workspace_s* w) {
    if (!w) return VCT_OK;
    cudaError_t e = w->ptr ? cudaFree(w->ptr) : cudaSuccess;
    if (w->aux) {
        cudaError_t e2 = cudaFree(w->aux);
        if (e == cudaSuccess) e = e2;
    }
    if (w->side) {
        cudaError_t e2 = cudaStreamSynchronize(w->side);
        if (e == cudaSuccess) e = e2;
        e2 = cudaStreamDestroy(w->side);
        if (e == cudaSuccess) e = e2;
    }
    if (w->fork) cudaEventDestroy(w->fork);
    if (w->join) cudaEventDestroy(w->join);
    if (w->side_ws) {
        const int rc = vct_workspace_destroy(w->side_ws);
        if (rc != VCT_OK && e == cudaSuccess) e = cudaErrorUnknown;
    }
    delete w;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree (workspace)");
    return VCT_OK;
}

extern "C" int64_t vct_workspace_bytes(vct_workspace_s* w) { return w ? (int64_t)w->bytes : -1; }

extern "C" int vct_voxelization_view_proj(const vct_clipmap_region* region, float out[48]) {
    VCT_CHECK_ARG(region && out, "vct_voxelization_view_proj: null argument");
    voxel_view_proj(*region, out);
    return VCT_OK;
}

extern "C" int vct_voxelization_desc_for(const vct_clipmap_region regions[6], int32_t level, int32_t R,
                                         vct_voxelization_desc* out) {
    VCT_CHECK_ARG(regions && out && level >= 0 && level < 6, "vct_voxelization_desc_for: bad argument");
    *out = voxelization_desc(regions, level, R);
    return VCT_OK;
}

extern "C" int vct_camera_matrix(const float position[3], const float direction[3], const float up[3],
                                 float fovy_degrees, float aspect, vct_cam_matrix* out) {
    VCT_CHECK_ARG(position && direction && up && out, "vct_camera_matrix: null argument");
    VCT_CHECK_ARG(aspect > 0.0f && fovy_degrees > 0.0f && fovy_degrees < 180.0f, "vct_camera_matrix: bad fovy or aspect");
    const float dd = direction[0] * direction[0] + direction[1] * direction[1] + direction[2] * direction[2];
    const float3 side = cross3h(make_float3(up[0], up[1], up[2]), make_float3(direction[0], direction[1], direction[2]));
    VCT_CHECK_ARG(dd > 0.0f && dot3h(side, side) > 0.0f, "vct_camera_matrix: zero direction or direction parallel to up");
    const float3 eye = make_float3(position[0], position[1], position[2]);
    const M4 view = look_at_lh(eye, make_float3(eye.x + direction[0], eye.y + direction[1], eye.z + direction[2]),
                               make_float3(up[0], up[1], up[2]));
    const float fovy = fovy_degrees * (float)0.01745329251994329576923690768489;  // glm::radians
    const M4 proj = perspective_lh_zo(fovy, aspect, 0.01f, 5000.0f);
    const M4 vp = mat_mul4(proj.m, view.m);
    const M4 vinv = inverse4(view.m), pinv = inverse4(proj.m);
    const M4 vpi = mat_mul4(vinv.m, pinv.m);
    memcpy(out->view_proj, vp.m, 64);
    memcpy(out->view_proj_inv, vpi.m, 64);
    out->eye_pos[0] = position[0];
    out->eye_pos[1] = position[1];
    out->eye_pos[2] = position[2];
    out->padding = 0;
    return VCT_OK;
}

extern "C" int vct_directional_light_shadow(const float origin[3], const float direction[3], float z_near, float z_far,
                                            vct_directional_light_shadow_desc* out) {
    VCT_CHECK_ARG(origin && direction && out, "vct_directional_light_shadow: null argument");
    VCT_CHECK_ARG(z_far > z_near, "vct_directional_light_shadow: far must exceed near");
    float3 o = make_float3(origin[0], origin[1], origin[2]);
    float3 d = normalize3h(make_float3(direction[0], direction[1], direction[2]));
    M4 view = look_at_lh(o, make_float3(o.x + d.x, o.y + d.y, o.z + d.z), make_float3(0.f, 1.f, 0.f));
    M4 proj = ortho_lh_zo(-16.0f, 16.0f, -16.0f, 16.0f, z_near, z_far);
    memcpy(out->view, view.m, 64);
    memcpy(out->proj, proj.m, 64);
    out->z_near = z_near;
    out->z_far = z_far;
    return VCT_OK;
}

extern "C" int vct_clear_atlas(uint32_t* atlas, int32_t R, void* stream) {
    VCT_CHECK_ARG(atlas && valid_resolution(R), "vct_clear_atlas: bad argument");
    VCT_CUDA_TRY(cudaMemsetAsync(atlas, 0, sizeof(uint32_t) * AtlasDims(R).texels(), as_stream(stream)));
    return VCT_OK;
}

namespace vct {

// The opacity pass's restriction for a toroidal update from its slab list
// (vct_update_clip_regions' output): a level with a whole-region slab is
// voxelised in full; every other level keeps only the fragments inside its
// slabs, each slab bounded like the region Voxelizer::cmdVoxelize would be
// given for it (min * voxel size - 1e-6, max * voxel size + 1e-6; the other
// two axes span the level's region, whose bounds the pass already applies).
struct SlabPlan {
    uint32_t restricted = 0;  // levels limited to their slabs
    uint32_t changed = 0;     // levels with at least one slab (cleared, voxelised, mipped)
    float lo[6][3], hi[6][3];
};

int slab_plan(const vct_clipmap_region regions[6], int R, const vct_clipmap_region* slabs, const int32_t* levels,
              int n, SlabPlan* P) {
    VCT_CHECK_ARG(n >= 0 && n <= 18 && (n == 0 || (slabs && levels)), "toroidal update: bad slab list");
    uint32_t full = 0;
    for (int l = 0; l < 6; ++l)
        for (int a = 0; a < 3; ++a) {
            P->lo[l][a] = 3.0e38f;
            P->hi[l][a] = -3.0e38f;
        }
    for (int i = 0; i < n; ++i) {
        const int l = levels[i];
        VCT_CHECK_ARG(l >= 0 && l < 6, "toroidal update: slab level out of range");
        const vct_clipmap_region& sr = slabs[i];
        const vct_clipmap_region& r = regions[l];
        VCT_CHECK_ARG(sr.voxel_size == r.voxel_size, "toroidal update: slab voxel size differs from its level's");
        int thin = -1, nthin = 0;
        for (int a = 0; a < 3; ++a) {
            VCT_CHECK_ARG(sr.extent[a] >= 1 && sr.extent[a] <= (uint32_t)R, "toroidal update: bad slab extent");
            if (sr.extent[a] != (uint32_t)R) {
                thin = a;
                ++nthin;
            }
        }
        VCT_CHECK_ARG(nthin <= 1, "toroidal update: a slab is thin along one axis at most");
        P->changed |= 1u << l;
        if (nthin == 0) {
            full |= 1u << l;
            continue;
        }
        const float vs = sr.voxel_size;
        P->lo[l][thin] = fminf(P->lo[l][thin], (float)sr.min_corner[thin] * vs - 1e-6f);
        P->hi[l][thin] = fmaxf(P->hi[l][thin], (float)(sr.min_corner[thin] + (int32_t)sr.extent[thin]) * vs + 1e-6f);
    }
    P->restricted = 0x3Fu & ~full;
    return VCT_OK;
}

// ClipmapCleaner::cmdClearOpacityClipRegion of every slab, at its corner
// wrapped into the level ((min % extent + extent) % extent,
// VoxelizationPass.cpp:127-141).
int clear_slabs(uint32_t* atlas, int R, const vct_clipmap_region* slabs, const int32_t* levels, int n, void* stream) {
    for (int i = 0; i < n; ++i) {
        vct_image_cleaning_desc c;
        for (int a = 0; a < 3; ++a) {
            c.region_min_corner[a] = ((slabs[i].min_corner[a] % R) + R) % R;
            c.clip_max_extent[a] = slabs[i].extent[a];
        }
        c.clip_level = levels[i];
        c.clipmap_resolution = R;
        c.face_count = VCT_FACE_COUNT;
        int rc = vct_clear_region(atlas, &c, stream);
        if (rc != VCT_OK) return rc;
    }
    return VCT_OK;
}

void apply_slabs(RasterArgs& A, const SlabPlan& P) {
    A.slab_levels = P.restricted;
    memcpy(A.slab_lo, P.lo, sizeof(P.lo));
    memcpy(A.slab_hi, P.hi, sizeof(P.hi));
}

}  // namespace vct

extern "C" int vct_voxelize_opacity_slabs(const vct_scene* scene, const vct_clipmap_region regions[6], int32_t R,
                                          uint32_t* atlas, const vct_clipmap_region* slabs, const int32_t* slab_levels,
                                          int32_t slab_count, vct_workspace_s* ws, void* stream) {
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(regions && atlas && ws && valid_resolution(R), "vct_voxelize_opacity_slabs: bad argument");
    SlabPlan P;
    if ((rc = slab_plan(regions, R, slabs, slab_levels, slab_count, &P)) != VCT_OK) return rc;
    if ((rc = clear_slabs(atlas, R, slabs, slab_levels, slab_count, stream)) != VCT_OK) return rc;
    if (scene->triangle_count == 0 || P.changed == 0) return VCT_OK;
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_OPACITY;
    A.R = R;
    A.W = A.H = R + 2;
    fill_clipmap_levels(A, regions, R, P.changed);
    apply_slabs(A, P);
    A.items = scene->triangle_count * A.nlevels;
    A.atlas = atlas;
    cudaStream_t st = as_stream(stream);
    size_t off;
    TilePlan plan;
    rc = plan_tiles(A, ws, off, &plan, st);
    if (rc != VCT_OK) return rc;
    if (plan.total) launch_cover<K_OPACITY, P_DIRECT>(A, plan, nullptr, nullptr, nullptr, nullptr, st);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_voxelize_opacity(const vct_scene* scene, const vct_clipmap_region regions[6], int32_t R,
                                    uint32_t* atlas, uint32_t level_mask, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_voxelize_opacity");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(regions && atlas && ws && valid_resolution(R), "vct_voxelize_opacity: bad argument");
    VCT_CHECK_ARG((level_mask & ~0x3Fu) == 0, "vct_voxelize_opacity: level mask has bits above level 5");
    if (scene->triangle_count == 0 || level_mask == 0) return VCT_OK;
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_OPACITY;
    A.R = R;
    A.W = A.H = R + 2;
    fill_clipmap_levels(A, regions, R, level_mask);
    A.items = scene->triangle_count * A.nlevels;
    A.atlas = atlas;
    cudaStream_t st = as_stream(stream);
    size_t off;
    TilePlan plan;
    rc = plan_tiles(A, ws, off, &plan, st);
    if (rc != VCT_OK) return rc;
    if (plan.total) launch_cover<K_OPACITY, P_DIRECT>(A, plan, nullptr, nullptr, nullptr, nullptr, st);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

// ------------------------------------------------ conservative voxels
// The conservative voxelisation mode: every voxel of a level's region that
// the triangle touches, by the triangle / box overlap test of M. Schwarz and
// H.-P. Seidel ("Fast parallel surface and solid voxelization on GPUs",
// SIGGRAPH Asia 2010, section 3.1): the box overlaps the triangle's plane
// (the plane's values at the box's two critical corners differ in sign or
// vanish) and, in each axis projection, lies on the inner side of every edge
// line shifted outward by the box's extent.  FP32 without contraction in the
// level's voxel units u = p * (1 / voxel_size) - min_corner, the voxel
// (i, j, k) being the box [i, i+1] x [j, j+1] x [k, k+1] -- the oracle's
// arithmetic, so the voxel sets are equal bit for bit.
namespace vct {
namespace {

struct ConsTri {
    float u[3][3];
    float n[3];
    float d1, d2;
    float ne[3][3][2];
    float de[3][3];
    int lo[3], hi[3];
    bool ok;
};

__device__ __forceinline__ float fmax0(float x) { return x > 0.0f ? x : 0.0f; }

__device__ inline ConsTri cons_setup(const float3 p[3], const vct_clipmap_region& rg, int R) {
    ConsTri t;
    const float inv = 1.0f / rg.voxel_size;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t.u[k][0] = p[k].x * inv - (float)rg.min_corner[0];
        t.u[k][1] = p[k].y * inv - (float)rg.min_corner[1];
        t.u[k][2] = p[k].z * inv - (float)rg.min_corner[2];
    }
    t.ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float mn = fminf(fminf(t.u[0][a], t.u[1][a]), t.u[2][a]);
        const float mx = fmaxf(fmaxf(t.u[0][a], t.u[1][a]), t.u[2][a]);
        const float fl = floorf(mn), fh = floorf(mx);
        t.lo[a] = fl < 0.0f ? 0 : (fl > (float)(R - 1) ? R : (int)fl);
        t.hi[a] = fh > (float)(R - 1) ? R - 1 : (fh < 0.0f ? -1 : (int)fh);
        if (t.lo[a] > t.hi[a]) t.ok = false;
    }
    float e0[3], e1[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        e0[a] = t.u[1][a] - t.u[0][a];
        e1[a] = t.u[2][a] - t.u[0][a];
    }
    t.n[0] = e0[1] * e1[2] - e0[2] * e1[1];
    t.n[1] = e0[2] * e1[0] - e0[0] * e1[2];
    t.n[2] = e0[0] * e1[1] - e0[1] * e1[0];
    float c[3], c2[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = t.n[a] > 0.0f ? 1.0f : 0.0f;
        c2[a] = 1.0f - c[a];
    }
    t.d1 = t.n[0] * (c[0] - t.u[0][0]) + t.n[1] * (c[1] - t.u[0][1]) + t.n[2] * (c[2] - t.u[0][2]);
    t.d2 = t.n[0] * (c2[0] - t.u[0][0]) + t.n[1] * (c2[1] - t.u[0][1]) + t.n[2] * (c2[2] - t.u[0][2]);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int a0 = q, a1 = (q + 1) % 3, a2 = (q + 2) % 3;  // projections xy, yz, zx
        const float sg = t.n[a2] >= 0.0f ? 1.0f : -1.0f;
#pragma unroll
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

__device__ inline bool cons_overlap(const ConsTri& t, int i, int j, int k) {
    if (i < t.lo[0] || i > t.hi[0] || j < t.lo[1] || j > t.hi[1] || k < t.lo[2] || k > t.hi[2]) return false;
    const float p[3] = {(float)i, (float)j, (float)k};
    const float np = t.n[0] * p[0] + t.n[1] * p[1] + t.n[2] * p[2];
    if ((np + t.d1) * (np + t.d2) > 0.0f) return false;
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int e = 0; e < 3; ++e)
            if (t.ne[q][e][0] * p[q] + t.ne[q][e][1] * p[(q + 1) % 3] + t.de[q][e] < 0.0f) return false;
    return true;
}

struct ConsArgs {
    vct_scene s;
    vct_clipmap_region rg[6];
    int levels[6];
    int nlevels;
    int R;
    uint32_t* atlas;
};

// One warp per (triangle, level) item, the item's bounding-box voxels dealt
// over the lanes (a large triangle's box has thousands of voxels, a small
// one's a few).
__global__ void __launch_bounds__(256) k_voxelize_conservative(const __grid_constant__ ConsArgs A, int64_t items) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int rb = A.R + 2;
    const int64_t W = (int64_t)rb * 6, H = (int64_t)rb * 6;
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < items; it += nwarps) {
        const int64_t tri = it / A.nlevels;
        const int level = A.levels[it - tri * A.nlevels];
        const WTri w = world_triangle(A.s, tri);
        const vct_gltf_shade_material mat = material_of(A.s, w.material);
        if (mat.occlusion_texture > -1 && texture_1x1(A.s, mat.occlusion_texture).x < 0.1f) continue;
        const vct_clipmap_region& rg = A.rg[level];
        const ConsTri t = cons_setup(w.p, rg, A.R);
        if (!t.ok) continue;
        const int nx = t.hi[0] - t.lo[0] + 1, ny = t.hi[1] - t.lo[1] + 1, nz = t.hi[2] - t.lo[2] + 1;
        const int64_t nv = (int64_t)nx * ny * nz;
        for (int64_t v = lane; v < nv; v += 32) {
            const int64_t r = v / nx;
            const int i = t.lo[0] + (int)(v - r * nx), j = t.lo[1] + (int)(r % ny), k = t.lo[2] + (int)(r / ny);
            if (!cons_overlap(t, i, j, k)) continue;
            const int x = (((rg.min_corner[0] + i) % A.R) + A.R) % A.R + 1;
            const int y = (((rg.min_corner[1] + j) % A.R) + A.R) % A.R + 1 + rb * level;
            const int z = (((rg.min_corner[2] + k) % A.R) + A.R) % A.R + 1;
            const int64_t base = ((int64_t)z * H + y) * W + x;
#pragma unroll
            for (int f = 0; f < 6; ++f) A.atlas[base + (int64_t)rb * f] = 0xFFFFFFFFu;
        }
    }
}

}  // namespace
}  // namespace vct

extern "C" int vct_voxelize_opacity_conservative(const vct_scene* scene, const vct_clipmap_region regions[6],
                                                 int32_t R, uint32_t* atlas, uint32_t level_mask, void* stream) {
    vct::NvtxRange nvtx_range("vct_voxelize_opacity_conservative");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(regions && atlas && valid_resolution(R), "vct_voxelize_opacity_conservative: bad argument");
    VCT_CHECK_ARG((level_mask & ~0x3Fu) == 0, "vct_voxelize_opacity_conservative: level mask has bits above level 5");
    if (scene->triangle_count == 0 || level_mask == 0) return VCT_OK;
    vct::ConsArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.R = R;
    A.atlas = atlas;
    for (int l = 0; l < 6; ++l) {
        A.rg[l] = regions[l];
        VCT_CHECK_ARG(regions[l].voxel_size > 0.0f, "vct_voxelize_opacity_conservative: non-positive voxel size");
        if ((level_mask >> l) & 1u) A.levels[A.nlevels++] = l;
    }
    const int64_t items = scene->triangle_count * (int64_t)A.nlevels;
    int64_t blocks = (items * 32 + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    vct::k_voxelize_conservative<<<(int)blocks, 256, 0, as_stream(stream)>>>(A, items);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_shadow_depth(const vct_scene* scene, const vct_directional_light_shadow_desc* sd, float* depth,
                                int32_t W, int32_t H, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_shadow_depth");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(sd && depth && ws && W > 0 && H > 0 && W <= 32768 && H <= 32768, "vct_shadow_depth: bad argument");
    cudaStream_t st = as_stream(stream);
    const int64_t npx = (int64_t)W * H;
    k_fill_f32<<<grid_of(npx, 256), 256, 0, st>>>(depth, npx, 1.0f);
    VCT_LAUNCH_CHECK();
    if (scene->triangle_count == 0) return VCT_OK;
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_SHADOW;
    A.W = W;
    A.H = H;
    A.nlevels = 1;
    A.levels[0] = 0;
    M4 pv = mat_mul4(sd->proj, sd->view);
    memcpy(A.pv, pv.m, 64);
    A.items = scene->triangle_count;
    A.depth = depth;
    size_t off;
    TilePlan plan;
    rc = plan_tiles(A, ws, off, &plan, st);
    if (rc != VCT_OK) return rc;
    if (plan.total) launch_cover<K_SHADOW, P_DIRECT>(A, plan, nullptr, nullptr, nullptr, nullptr, st);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

extern "C" int vct_inject_radiance(const vct_scene* scene, const vct_clipmap_region regions[6], int32_t R,
                                   const vct_shadow_map* shadow, const vct_directional_light_desc* light,
                                   const vct_directional_light_shadow_desc* light_shadow, uint32_t* atlas,
                                   uint32_t level_mask, int32_t mode, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_inject_radiance");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(regions && atlas && ws && valid_resolution(R), "vct_inject_radiance: bad argument");
    VCT_CHECK_ARG(mode == VCT_INJECT_DETERMINISTIC || mode == VCT_INJECT_ATOMIC, "vct_inject_radiance: bad mode");
    VCT_CHECK_ARG((level_mask & ~0x3Fu) == 0, "vct_inject_radiance: level mask has bits above level 5");
    if (scene->triangle_count == 0 || level_mask == 0) return VCT_OK;
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_INJECT;
    A.R = R;
    {  // all-ones key of the smallest width that covers every texel index
        const uint32_t texels = (uint32_t)AtlasDims(R).texels();
        A.invalid_key = 0xffffffffu >> __builtin_clz(texels);
    }
    A.W = A.H = R + 2;
    fill_clipmap_levels(A, regions, R, level_mask);
    rc = fill_light(A, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    A.items = scene->triangle_count * A.nlevels;
    A.atlas = atlas;
    A.count_levels = 0x3Fu;  // every level of the item list
    cudaStream_t st = as_stream(stream);
    if (mode == VCT_INJECT_ATOMIC) {
        size_t off;
        TilePlan plan;
        rc = plan_tiles(A, ws, off, &plan, st);
        if (rc != VCT_OK) return rc;
        if (plan.total == 0) return VCT_OK;
        int* err = (int*)((char*)ws->ptr + off);
        VCT_CUDA_TRY(cudaMemsetAsync(err, 0, 4, st));
        launch_cover<K_INJECT, P_DIRECT>(A, plan, nullptr, nullptr, nullptr, err, st);
        VCT_LAUNCH_CHECK();
        int herr = 0;
        VCT_CUDA_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
        VCT_CUDA_TRY(cudaStreamSynchronize(st));
        if (herr) return fail(VCT_E_TIMEOUT, "vct_inject_radiance: a CAS loop gave up after 2^20 retries");
        return VCT_OK;
    }
    // deterministic: count -> scan -> emit covered samples -> shade into records
    // -> stable sort by texel -> fold each texel's run in traversal order
    InjectState S;
    rc = inject_prepare<K_INJECT>(A, A, ws, st, &S);
    if (rc == kWorkspaceGrew)
        return vct_inject_radiance(scene, regions, R, shadow, light, light_shadow, atlas, level_mask, mode, ws, stream);
    if (rc != VCT_OK) return rc;
    return inject_finish(A, S, nullptr, st);
}

extern "C" int vct_gbuffer(const vct_scene* scene, const vct_cam_matrix* cam, int32_t width, int32_t height,
                           vct_surface_sample* out, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_gbuffer");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(cam && out && ws, "vct_gbuffer: null argument");
    VCT_CHECK_ARG(width > 0 && height > 0 && width <= 16384 && height <= 16384, "vct_gbuffer: bad image size");
    VCT_CHECK_ARG(((uintptr_t)out & 15) == 0, "vct_gbuffer: the output must be 16-byte aligned");
    VCT_CHECK_ARG(scene->triangle_count < (1LL << 28), "vct_gbuffer: more than 2^28 triangles");
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_GBUFFER;
    A.W = width;
    A.H = height;
    A.nlevels = 6;  // up to six sub-triangles per clipped triangle
    for (int l = 0; l < 6; ++l) A.levels[l] = l;
    memcpy(A.pv, cam->view_proj, 64);
    A.items = scene->triangle_count * 6;
    cudaStream_t st = as_stream(stream);
    const int64_t npx = (int64_t)width * height;
    size_t off = 0;
    TilePlan plan;
    plan.total = 0;
    if (scene->triangle_count > 0) {
        rc = plan_tiles(A, ws, off, &plan, st);
        if (rc != VCT_OK) return rc;
    }
    const size_t need = off + a256(8 * (size_t)npx);
    if (ws->bytes < need) {
        rc = workspace_reserve(ws, need);
        if (rc != VCT_OK) return rc;
        return vct_gbuffer(scene, cam, width, height, out, ws, stream);  // the plan moved with the arena
    }
    A.vis = (unsigned long long*)((char*)ws->ptr + off);
    M4 vp_inv;
    memcpy(vp_inv.m, cam->view_proj_inv, 64);
    VCT_CUDA_TRY(cudaMemsetAsync(A.vis, 0xff, 8 * (size_t)npx, st));
    if (plan.total) launch_cover<K_GBUFFER, P_DIRECT>(A, plan, nullptr, nullptr, nullptr, nullptr, st);
    VCT_LAUNCH_CHECK();
    k_gbuffer_resolve<<<grid_of(npx, 256), 256, 0, st>>>(A, vp_inv, out);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}

namespace vct {

// The rasterised part of a frame with the deterministic injection
// (Application::run's VoxelizationPass, RSMPass and RadianceInjectionPass up to
// the fold).  The opacity voxelisation and the injection's coverage count
// share one tile plan and one coverage pass -- their items (every triangle at
// every level, the same projections and viewport) are the same -- so the
// order is: clear opacity, shadow depth (it does not depend on the atlases),
// opacity + count + emit, opacity mips, border, clear of the due radiance
// levels, then shading, sort and fold.  The results equal the passes run one
// by one in the reference's order.
// The workspace's side stream, created on first use on the current device
// (non-blocking, with its fork and join events); null when the current
// device is not the one it was created on (the frame then runs serially).
static cudaStream_t side_stream(vct_workspace_s* ws) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if (ws->side) return ws->side_device == dev ? ws->side : nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    if (cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        cudaStreamDestroy(s);
        return nullptr;
    }
    ws->side = s;
    ws->fork = a;
    ws->join = b;
    ws->side_device = dev;
    ws->side_ws = new vct_workspace_s();
    return s;
}

// `side` continues after everything enqueued on `st` so far.
static int fork_side(vct_workspace_s* ws, cudaStream_t side, cudaStream_t st) {
    VCT_CUDA_TRY(cudaEventRecord(ws->fork, st));
    VCT_CUDA_TRY(cudaStreamWaitEvent(side, ws->fork, 0));
    return VCT_OK;
}

// `st` continues after everything enqueued on `side` so far.
static int join_side(vct_workspace_s* ws, cudaStream_t side, cudaStream_t st) {
    VCT_CUDA_TRY(cudaEventRecord(ws->join, side));
    VCT_CUDA_TRY(cudaStreamWaitEvent(st, ws->join, 0));
    return VCT_OK;
}

int frame_raster_passes(const vct_scene* scene, const vct_frame_desc* f, const vct_clipmap_region regions[6],
                        uint32_t due, const vct_clipmap_region* slabs, const int32_t* slab_levels, int nslabs,
                        uint32_t* opacity, uint32_t* radiance, float* shadow_depth, vct_workspace_s* ws,
                        const uint32_t** touched_out, cudaStream_t st) {
    const int R = f->clipmap_resolution;
    void* stream = st;
    int rc;
    const bool toroidal = nslabs >= 0;
    SlabPlan P;
    if (toroidal && (rc = slab_plan(regions, R, slabs, slab_levels, nslabs, &P)) != VCT_OK) return rc;
    // the touched-texel bitmap, one bit per atlas texel, cleared every frame
    const size_t bm_bytes = a256(((size_t)AtlasDims(R).texels() + 31) / 32 * 4);
    if (ws->aux_bytes < bm_bytes) {
        if (ws->aux) {
            VCT_CUDA_TRY(cudaDeviceSynchronize());
            VCT_CUDA_TRY(cudaFree(ws->aux));
            ws->aux = nullptr;
            ws->aux_bytes = 0;
        }
        VCT_CUDA_TRY(cudaMalloc(&ws->aux, bm_bytes));
        ws->aux_bytes = bm_bytes;
    }
    uint32_t* touched = (uint32_t*)ws->aux;
    VCT_CUDA_TRY(cudaMemsetAsync(touched, 0, bm_bytes, st));
    *touched_out = touched;
    // Two stretches run on the side stream (with its own workspace), beside
    // main-stream work they share no buffer with: the shadow pass beside the
    // opacity clear, voxelisation and injection count / emission (the shadow
    // map is read only by the injection's shading, after the join), and the
    // opacity mips + border wrap beside the shading, sort and fold.  The
    // results are those of the serial order.
    cudaStream_t side = side_stream(ws);
    cudaStream_t sst = side ? side : st;  // the shadow pass's stream
    vct_workspace_s* sws = side ? ws->side_ws : ws;
    if (side && (rc = fork_side(ws, side, st)) != VCT_OK) return rc;
    const bool r8 = f->opacity_format == VCT_OPACITY_R8;  // (full revoxelisation only: checked by the caller)
    if (toroidal) rc = clear_slabs(opacity, R, slabs, slab_levels, nslabs, stream);
    else if (r8) rc = cudaMemsetAsync(opacity, 0, (size_t)AtlasDims(R).texels(), st) == cudaSuccess
                          ? VCT_OK : fail(VCT_E_CUDA, "cudaMemsetAsync (opacity clear)");
    else rc = vct_clear_atlas(opacity, R, stream);
    if (rc != VCT_OK) return rc;
    vct_shadow_map sm = {nullptr, 0, 0};
    if (f->shadow_width > 0) {
        if ((rc = vct_shadow_depth(scene, &f->light_shadow, shadow_depth, f->shadow_width, f->shadow_height, sws,
                                   sst)) != VCT_OK)
            return rc;
        sm.depth = shadow_depth;
        sm.width = f->shadow_width;
        sm.height = f->shadow_height;
    }
    if ((rc = check_scene(scene)) != VCT_OK) return rc;
    cudaStream_t ost = side ? side : st;  // the opacity mips' stream
    InjectState S;
    RasterArgs I;
    memset(&I, 0, sizeof(I));
    if (scene->triangle_count > 0) {
        RasterArgs C;  // the opacity pass over all six levels, counting the due levels' samples
        memset(&C, 0, sizeof(C));
        C.s = *scene;
        C.kind = K_OPA_COUNT;
        C.R = R;
        C.W = C.H = R + 2;
        fill_clipmap_levels(C, regions, R, 0x3Fu);
        if (toroidal) apply_slabs(C, P);
        C.items = scene->triangle_count * C.nlevels;
        C.atlas = opacity;
        C.opa_r8 = r8 ? 1 : 0;
        C.count_levels = due;
        I = C;  // the injection's args over the same items
        I.kind = K_INJECT;
        I.atlas = radiance;
        I.opa_r8 = 0;
        I.invalid_key = 0xffffffffu >> __builtin_clz((uint32_t)AtlasDims(R).texels());
        if ((rc = fill_light(I, &sm, &f->light, &f->light_shadow)) != VCT_OK) return rc;
        for (;;) {
            rc = inject_prepare<K_OPA_COUNT>(C, I, ws, st, &S);
            if (rc != kWorkspaceGrew) break;
        }
        if (rc != VCT_OK) return rc;
    }
    // the shading below reads the shadow map; the mips read the voxelised opacity
    if (side && (rc = join_side(ws, side, st)) != VCT_OK) return rc;
    if (side && (rc = fork_side(ws, side, st)) != VCT_OK) return rc;
    if (r8) {
        if ((rc = opacity_r8_mips(reinterpret_cast<uint8_t*>(opacity), regions, R, ost)) != VCT_OK) return rc;
    } else if (!toroidal) {
        if ((rc = vct_downsample_all(opacity, regions, R, VCT_DOWNSAMPLE_OPACITY, ost)) != VCT_OK) return rc;
    } else {
        // VoxelizationPass::onEndRenderPass: the mips of the levels that were revoxelised
        for (int l = 1; l < 6; ++l) {
            if (!((P.changed >> l) & 1u)) continue;
            vct_downsample_desc d;
            for (int a = 0; a < 3; ++a) d.prev_region_min_corner[a] = regions[l - 1].min_corner[a];
            d.clip_level = l;
            d.clipmap_resolution = R;
            d.downsample_region_size = VCT_DOWNSAMPLE_REGION_SIZE;
            if ((rc = vct_downsample(opacity, &d, VCT_DOWNSAMPLE_OPACITY, ost)) != VCT_OK) return rc;
        }
    }
    vct_border_wrapping_desc bw = {(uint32_t)R, VCT_VOXEL_BORDER, VCT_FACE_COUNT, VCT_CLIP_LEVEL_COUNT};
    if (r8) rc = wrap_border_r8(reinterpret_cast<uint8_t*>(opacity), R, ost);
    else rc = vct_wrap_border(opacity, &bw, ost);
    if (rc != VCT_OK) return rc;
    // the due radiance levels' clear is folded into the fold (texels start from
    // zero) and the copy-alpha / mip passes (unmarked texels read as zero rgb)
    if (scene->triangle_count > 0 && (rc = inject_finish(I, S, touched, st)) != VCT_OK) return rc;
    // the copy-alpha and radiance mip passes that follow read the final opacity
    if (side && (rc = join_side(ws, side, st)) != VCT_OK) return rc;
    return VCT_OK;
}

}  // namespace vct

extern "C" int vct_svo_fragments(const vct_scene* scene, int32_t octree_level, const float bb_min[3],
                                 const float bb_max[3], const vct_shadow_map* shadow,
                                 const vct_directional_light_desc* light,
                                 const vct_directional_light_shadow_desc* light_shadow, uint32_t* frags,
                                 int64_t capacity, int64_t* count, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_svo_fragments");
    int rc = check_scene(scene);
    if (rc != VCT_OK) return rc;
    VCT_CHECK_ARG(count && bb_min && bb_max && ws, "vct_svo_fragments: null argument");
    VCT_CHECK_ARG(octree_level >= 1 && octree_level <= 11, "vct_svo_fragments: octree level must be 1..11");
    VCT_CHECK_ARG(capacity >= 0 && (capacity == 0 || frags), "vct_svo_fragments: bad fragment buffer");
    *count = 0;
    if (scene->triangle_count == 0) return VCT_OK;
    RasterArgs A;
    memset(&A, 0, sizeof(A));
    A.s = *scene;
    A.kind = K_SVO;
    A.R = 1 << octree_level;
    A.W = A.H = A.R;
    A.nlevels = 1;
    A.levels[0] = 0;
    rc = fill_light(A, shadow, light, light_shadow);
    if (rc != VCT_OK) return rc;
    float ext[3];
    for (int a = 0; a < 3; ++a) {
        ext[a] = bb_max[a] - bb_min[a];
        A.center[a] = (bb_min[a] + bb_max[a]) * 0.5f;
    }
    A.ev = fmaxf(ext[0], fmaxf(ext[1], ext[2])) * 0.5f;
    VCT_CHECK_ARG(A.ev > 0.0f, "vct_svo_fragments: empty scene bounding box");
    A.items = scene->triangle_count;
    A.frags = frags;
    A.frag_capacity = capacity;
    cudaStream_t st = as_stream(stream);
    size_t off;
    TilePlan plan;
    rc = plan_tiles(A, ws, off, &plan, st);
    if (rc != VCT_OK) return rc;
    if (plan.total == 0) return VCT_OK;
    // count pass (SparseVoxelizer::preVoxelize), host readback of the count
    uint2 *counts, *offs;
    uint32_t nfrag, nslot;
    rc = count_tiles<K_SVO>(A, ws, off, plan, &counts, &offs, &nfrag, &nslot, st);
    if (rc == kWorkspaceGrew)
        return vct_svo_fragments(scene, octree_level, bb_min, bb_max, shadow, light, light_shadow, frags, capacity,
                                 count, ws, stream);
    if (rc != VCT_OK) return rc;
    *count = (int64_t)nslot;
    if (capacity == 0 || nfrag == 0) return VCT_OK;  // count-only call
    if (*count > capacity) return fail(VCT_E_OVERFLOW, "vct_svo_fragments: fragment list capacity too small");
    const size_t need = off + a256(sizeof(FragDesc) * (size_t)nfrag) + 256;
    if (ws->bytes < need) {
        rc = workspace_reserve(ws, need);
        if (rc != VCT_OK) return rc;
        return vct_svo_fragments(scene, octree_level, bb_min, bb_max, shadow, light, light_shadow, frags, capacity,
                                 count, ws, stream);
    }
    FragDesc* fr = (FragDesc*)((char*)ws->ptr + off);
    // write pass (SparseVoxelizer::cmdVoxelize); discarded slots stay zero
    VCT_CUDA_TRY(cudaMemsetAsync(frags, 0, sizeof(uint32_t) * 2 * (size_t)*count, st));
    launch_cover<K_SVO, P_WRITE>(A, plan, counts, offs, fr, nullptr, st);
    VCT_LAUNCH_CHECK();
    k_svo_shade<<<grid_of(nfrag, 256), 256, 0, st>>>(A, fr, nfrag);
    VCT_LAUNCH_CHECK();
    return VCT_OK;
}
