"""Seeded synthetic inputs in the reference's input layout.

The reference loads Sponza from glTF (its mesh .bin is not shipped), so the
benchmark configurations use procedural scenes instead:

* ``room_scene`` -- configuration 1: a 20x10x10 box (12 quads), 16 cylinders
  (32 segments) and 20k random triangles with edges U(0.05, 0.5), one
  uniform-random RGBA8 albedo per triangle (about 34k triangles).
* ``hall_scene`` -- configuration 2: instanced columns, arches and random
  clutter, about 1M triangles.
* ``terrain_scene`` -- configuration 3 (the large octree): a gradient-noise
  heightfield plus 10k boxes, about 4M triangles (58M SVO fragments at 512^3).

Geometry comes out as separate fp32 position / normal streams and uint32
indices (the reference binds one vertex stream per attribute,
VFS/SceneManager.cpp:124-204) plus one material index per triangle.  Each
material is a GltfShadeMaterial whose base colour is a 1x1 RGBA8 texture with
factor 1, so that both the SVO voxeliser (which ignores the factor when there
is no texture) and the injection pass see the albedo.

``surface_samples`` produces G-buffer texel sets (vct_surface_sample) at
area-uniform points with face normals, filled the way gBufferPass.frag would
(diffuse = base * 0.96 * (1 - metallic), specular = mix(0.04, base, metallic),
RGBA8 / RGBA16F quantisation of the attachments).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SAMPLE_DTYPE = np.dtype([
    ("position", np.float32, 3), ("depth", np.float32),
    ("normal_texel", np.float32, 3), ("pad0", np.float32),
    ("diffuse_texel", np.float32, 4), ("specular_texel", np.float32, 4),
    ("emission_texel", np.float32, 3), ("pad1", np.float32),
])
assert SAMPLE_DTYPE.itemsize == 80

MATERIAL_DTYPE = np.dtype([
    ("pbr_base_color_factor", np.float32, 4), ("pbr_base_color_texture", np.int32),
    ("pbr_metallic_factor", np.float32), ("pbr_roughness_factor", np.float32),
    ("pbr_metallic_roughness_texture", np.int32), ("emissive_texture", np.int32), ("alpha_mode", np.int32),
    ("alpha_cutoff", np.float32), ("double_sided", np.int32), ("emissive_factor", np.float32, 3),
    ("normal_texture", np.int32), ("normal_texture_scale", np.float32), ("occlusion_texture", np.int32),
    ("occlusion_texture_strength", np.float32), ("padding", np.int32),
])
assert MATERIAL_DTYPE.itemsize == 80


@dataclass
class Scene:
    positions: np.ndarray   # (V, 3) f32, object space (world space without node matrices)
    normals: np.ndarray     # (V, 3) f32
    indices: np.ndarray     # (T, 3) u32, into the whole vertex arrays
    tri_material: np.ndarray  # (T,) u32
    materials: np.ndarray   # (M,) MATERIAL_DTYPE
    textures: np.ndarray    # (X,) u32 RGBA8 1x1 texels, indexed by the materials' texture ids
    node_matrices: np.ndarray | None = None  # (N, 32) f32: NodeMatrix {model, itModel}, column-major
    tri_instance: np.ndarray | None = None   # (T,) u32: the NodeMatrix of each triangle

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])

    def triangles(self) -> np.ndarray:
        return self.positions[self.indices]  # (T, 3, 3)


def world_positions(scene: Scene) -> np.ndarray:
    """World-space corners of every triangle, (3T, 3) f32: NodeMatrix.model * (p, 1) in glm's
    mat4 * vec4 order ((c0 x + c1 y) + (c2 z + c3 w)); the object positions without node matrices."""
    if scene.node_matrices is None:
        return np.asarray(scene.positions, np.float32)
    # indices past the arrays read the last entry, as on the device
    idx = np.minimum(np.asarray(scene.indices, np.int64).reshape(-1), scene.positions.shape[0] - 1)
    inst = np.minimum(np.repeat(np.asarray(scene.tri_instance, np.int64), 3), scene.node_matrices.shape[0] - 1)
    m = np.asarray(scene.node_matrices, np.float32)[inst, :16]
    p = np.asarray(scene.positions, np.float32)[idx]
    x, y, z = p[:, 0:1], p[:, 1:2], p[:, 2:3]
    r = (m[:, 0:4] * x + m[:, 4:8] * y) + (m[:, 8:12] * z + m[:, 12:16])
    return r[:, :3].astype(np.float32)


def _rgba8(rng, n):
    c = rng.integers(0, 256, size=(n, 4), dtype=np.uint32)
    c[:, 3] = 255
    return (c[:, 0] | (c[:, 1] << 8) | (c[:, 2] << 16) | (c[:, 3] << 24)).astype(np.uint32)


def _materials_for(textures: np.ndarray) -> np.ndarray:
    m = np.zeros(textures.shape[0], MATERIAL_DTYPE)
    m["pbr_base_color_factor"] = 1.0
    m["pbr_base_color_texture"] = np.arange(textures.shape[0], dtype=np.int32)
    m["pbr_metallic_factor"] = 0.0
    m["pbr_roughness_factor"] = 1.0
    m["pbr_metallic_roughness_texture"] = -1
    m["emissive_texture"] = -1
    m["normal_texture"] = -1
    m["occlusion_texture"] = -1
    m["normal_texture_scale"] = 1.0
    m["occlusion_texture_strength"] = 1.0
    return m


def _quad(p0, p1, p2, p3):
    return [(p0, p1, p2), (p0, p2, p3)]


def _box_quads(lo, hi, splits=(2, 1, 1)):
    """Inward-facing axis-aligned box as quads; each face split in two (12 quads)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    tris = []
    for axis in range(3):
        u, v = [a for a in range(3) if a != axis]
        for side in (0, 1):
            c = hi[axis] if side else lo[axis]
            # split along the longest in-plane axis
            su = 2 if (hi[u] - lo[u]) >= (hi[v] - lo[v]) else 1
            sv = 3 - su
            for i in range(su):
                for j in range(sv):
                    u0 = lo[u] + (hi[u] - lo[u]) * i / su
                    u1 = lo[u] + (hi[u] - lo[u]) * (i + 1) / su
                    v0 = lo[v] + (hi[v] - lo[v]) * j / sv
                    v1 = lo[v] + (hi[v] - lo[v]) * (j + 1) / sv
                    pts = []
                    for (a, b) in ((u0, v0), (u1, v0), (u1, v1), (u0, v1)):
                        p = np.zeros(3)
                        p[axis] = c
                        p[u] = a
                        p[v] = b
                        pts.append(p)
                    tris += _quad(*pts)
    return tris


def _cylinder(center, radius, height, segments, rings):
    cx, cy, cz = center
    th = np.linspace(0, 2 * np.pi, segments + 1)
    hs = np.linspace(0, height, rings + 1)
    tris = []
    for r in range(rings):
        for s in range(segments):
            a = [cx + radius * np.cos(th[s]), cy + hs[r], cz + radius * np.sin(th[s])]
            b = [cx + radius * np.cos(th[s + 1]), cy + hs[r], cz + radius * np.sin(th[s + 1])]
            c = [cx + radius * np.cos(th[s + 1]), cy + hs[r + 1], cz + radius * np.sin(th[s + 1])]
            d = [cx + radius * np.cos(th[s]), cy + hs[r + 1], cz + radius * np.sin(th[s])]
            tris += _quad(np.array(a), np.array(b), np.array(c), np.array(d))
    return tris


def _cylinder_np(centers, radius, height, segments, rings):
    """Vectorised cylinders: (N, rings*segments*2, 3, 3)."""
    th = np.linspace(0, 2 * np.pi, segments + 1)
    hs = np.linspace(0, height, rings + 1)
    s, r = np.meshgrid(np.arange(segments), np.arange(rings), indexing="xy")
    s = s.ravel()
    r = r.ravel()
    def pt(ti, hi):
        return np.stack([radius * np.cos(th[ti]), hs[hi], radius * np.sin(th[ti])], -1)
    a, b, c, d = pt(s, r), pt(s + 1, r), pt(s + 1, r + 1), pt(s, r + 1)
    quad = np.stack([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], 1).reshape(-1, 3, 3)
    return centers[:, None, None, :] + quad[None]


def _random_triangles(rng, n, lo, hi, edge_lo=0.05, edge_hi=0.5):
    c = rng.uniform(lo, hi, size=(n, 3))
    # two random edge vectors of length U(edge_lo, edge_hi)
    def rand_dir(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    e1 = rand_dir(n) * rng.uniform(edge_lo, edge_hi, size=(n, 1))
    e2 = rand_dir(n) * rng.uniform(edge_lo, edge_hi, size=(n, 1))
    return np.stack([c, c + e1, c + e2], 1)


def _pack(tris: np.ndarray, rng, per_triangle_albedo=True) -> Scene:
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    T = tris.shape[0]
    pos = tris.reshape(-1, 3).copy()
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0, 1, 0], np.float32))
    nrm = np.repeat(n, 3, axis=0).astype(np.float32)
    idx = np.arange(3 * T, dtype=np.uint32).reshape(T, 3)
    textures = _rgba8(rng, T)
    return Scene(pos, nrm, idx, np.arange(T, dtype=np.uint32), _materials_for(textures), textures)


def room_scene(seed: int = 1, n_random: int = 20000) -> Scene:
    """Configuration 1: 20x10x10 room, 16 cylinders, 20k random triangles (~34k)."""
    rng = np.random.default_rng(seed)
    tris = [np.array(t) for t in _box_quads([-10, -1, -5], [10, 9, 5])]
    centers = np.array([[x, -1.0, z] for x in np.linspace(-8, 8, 8) for z in (-3.0, 3.0)])
    cyl = _cylinder_np(centers, 0.4, 10.0, 32, 14).reshape(-1, 3, 3)
    rnd = _random_triangles(rng, n_random, [-9.5, -0.5, -4.5], [9.5, 8.5, 4.5])
    allt = np.concatenate([np.stack(tris), cyl, rnd], 0)
    return _pack(allt, rng)


def hall_scene(seed: int = 2, target: int = 1_000_000) -> Scene:
    """Configuration 2: columns, arches and clutter, about `target` triangles."""
    rng = np.random.default_rng(seed)
    parts = [np.stack([np.array(t) for t in _box_quads([-30, -1, -30], [30, 20, 30])])]
    # columns: 16 segments x 12 rings x 2 = 384 tris each
    ncol = max(1, int(target * 0.55) // 384)
    cc = np.stack([rng.uniform(-28, 28, ncol), np.full(ncol, -1.0), rng.uniform(-28, 28, ncol)], 1)
    parts.append(_cylinder_np(cc, 0.5, 12.0, 16, 12).reshape(-1, 3, 3))
    # arches: half-ring tubes between column pairs
    narch = max(1, int(target * 0.15) // 512)
    u = np.linspace(0, np.pi, 33)
    v = np.linspace(0, 2 * np.pi, 9)
    uu, vv = np.meshgrid(np.arange(32), np.arange(8), indexing="xy")
    uu = uu.ravel()
    vv = vv.ravel()
    R0, r0 = 3.0, 0.35
    def tor(ui, vi):
        return np.stack([(R0 + r0 * np.cos(v[vi])) * np.cos(u[ui]), (R0 + r0 * np.cos(v[vi])) * np.sin(u[ui]),
                         r0 * np.sin(v[vi])], -1)
    a, b, c, d = tor(uu, vv), tor(uu + 1, vv), tor(uu + 1, vv + 1), tor(uu, vv + 1)
    arch = np.stack([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], 1).reshape(-1, 3, 3)
    ac = np.stack([rng.uniform(-25, 25, narch), rng.uniform(8, 12, narch), rng.uniform(-25, 25, narch)], 1)
    ang = rng.uniform(0, np.pi, narch)
    rot = np.zeros((narch, 3, 3))
    rot[:, 0, 0] = np.cos(ang)
    rot[:, 0, 2] = -np.sin(ang)
    rot[:, 1, 1] = 1
    rot[:, 2, 0] = np.sin(ang)
    rot[:, 2, 2] = np.cos(ang)
    parts.append((np.einsum("nij,tkj->ntki", rot, arch) + ac[:, None, None, :]).reshape(-1, 3, 3))
    used = sum(p.shape[0] for p in parts)
    parts.append(_random_triangles(rng, max(0, target - used), [-28, -0.5, -28], [28, 18, 28]))
    return _pack(np.concatenate(parts, 0), rng)


# Eight unit gradients for the 2D gradient noise below.
_GRAD2 = np.array([[1, 0], [-1, 0], [0, 1], [0, -1], [1, 1], [-1, 1], [1, -1], [-1, -1]], np.float64)
_GRAD2[4:] *= np.sqrt(0.5)


def gradient_noise2(x, y, perm: np.ndarray) -> np.ndarray:
    """Perlin's gradient noise in 2D (K. Perlin, "Improving Noise", SIGGRAPH 2002): each lattice point takes
    one of eight unit gradients through the hash perm[perm[i] + j] of a doubled 256-entry permutation, the
    four corner ramps are blended with the quintic fade 6t^5 - 15t^4 + 10t^3.  Values lie in [-1, 1]."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    x0, y0 = np.floor(x), np.floor(y)
    fx, fy = x - x0, y - y0
    i, j = x0.astype(np.int64) & 255, y0.astype(np.int64) & 255

    def ramp(di, dj):
        g = _GRAD2[perm[perm[i + di] + j + dj] & 7]
        return g[..., 0] * (fx - di) + g[..., 1] * (fy - dj)

    def fade(t):
        return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)

    u, v = fade(fx), fade(fy)
    a = ramp(0, 0) + u * (ramp(1, 0) - ramp(0, 0))
    b = ramp(0, 1) + u * (ramp(1, 1) - ramp(0, 1))
    return a + v * (b - a)


def _box_triangles(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    """Closed axis-aligned boxes, 12 outward-wound triangles each: (N, 12, 3, 3).  Corner c has the
    coordinates (hi if bit k of c else lo) on axis k."""
    quads = [(1, 3, 7, 5), (0, 4, 6, 2), (2, 6, 7, 3), (0, 1, 5, 4), (4, 5, 7, 6), (0, 2, 3, 1)]  # +x -x +y -y +z -z
    corners = np.stack([np.where(np.array([(c >> k) & 1 for k in range(3)], bool)[None], hi, lo)
                        for c in range(8)], 1)  # (N, 8, 3)
    tri = np.array([t for a, b, c, d in quads for t in ((a, b, c), (a, c, d))])  # (12, 3)
    return corners[:, tri]


def terrain_height(x, z, perm: np.ndarray, amplitude: float = 2.5, frequency: float = 0.11,
                   octaves: int = 5) -> np.ndarray:
    """Fractal sum of gradient noise: amplitude * sum_o 0.5^o noise(frequency 2^o (x, z))."""
    h = np.zeros(np.broadcast(np.asarray(x), np.asarray(z)).shape)
    for o in range(octaves):
        f = frequency * (2.0 ** o)
        h += (0.5 ** o) * gradient_noise2(np.asarray(x) * f, np.asarray(z) * f, perm)
    return amplitude * h


def terrain_scene(seed: int = 3, target: int = 4_000_000, boxes: int = 10_000, half: float = 15.0,
                  palette: int = 4096) -> Scene:
    """Configuration 3: a gradient-noise terrain over [-half, half]^2 (a regular grid, two up-facing triangles
    per cell) plus `boxes` closed boxes standing on it (footprint U(0.2, 0.9)^2, height U(0.2, 1.5)), about
    `target` triangles in all.  Albedo from a palette of `palette` RGBA8 texels, one entry per triangle."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm])
    cells = max(1, int(np.sqrt(max(target - 12 * boxes, 2) / 2.0)))
    g = np.linspace(-half, half, cells + 1)
    gx, gz = np.meshgrid(g, g, indexing="xy")
    gy = terrain_height(gx, gz, perm)
    v = np.stack([gx, gy, gz], -1)  # (cells+1, cells+1, 3), v[j, i] at (g[i], g[j])
    v00, v10, v01, v11 = v[:-1, :-1], v[:-1, 1:], v[1:, :-1], v[1:, 1:]
    # (v00, v01, v10) turns +y up: cross(v01 - v00, v10 - v00) = (0, dx dz, 0) on a flat cell
    terrain = np.stack([np.stack([v00, v01, v10], -2), np.stack([v10, v01, v11], -2)], -3).reshape(-1, 3, 3)
    parts = [terrain]
    if boxes:
        foot = rng.uniform(0.2, 0.9, size=(boxes, 2))
        tall = rng.uniform(0.2, 1.5, size=boxes)
        cx = rng.uniform(-half + 1.5, half - 1.5, boxes)
        cz = rng.uniform(-half + 1.5, half - 1.5, boxes)
        base = terrain_height(cx, cz, perm) - 0.2
        lo = np.stack([cx - 0.5 * foot[:, 0], base, cz - 0.5 * foot[:, 1]], 1)
        hi = np.stack([cx + 0.5 * foot[:, 0], base + tall, cz + 0.5 * foot[:, 1]], 1)
        parts.append(_box_triangles(lo, hi).reshape(-1, 3, 3))
    tris = np.concatenate(parts, 0).astype(np.float32)
    T = tris.shape[0]
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0, 1, 0], np.float32)).astype(np.float32)
    textures = _rgba8(rng, palette)
    tri_mat = rng.integers(0, palette, size=T, dtype=np.uint32)
    return Scene(tris.reshape(-1, 3).copy(), np.repeat(n, 3, axis=0), np.arange(3 * T, dtype=np.uint32).reshape(T, 3),
                 tri_mat, _materials_for(textures), textures)


def _f16(x):
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


def _u8(x):
    return (np.floor(np.clip(x, 0, 1) * 255.0 + 0.5) / 255.0).astype(np.float32)


def surface_samples(scene: Scene, n: int, seed: int = 11, roughness=(0.1, 0.9), metallic=(0.0, 1.0),
                    specular_fraction: float = 1.0) -> np.ndarray:
    """Area-uniform G-buffer samples with face normals (vct_surface_sample records)."""
    rng = np.random.default_rng(seed)
    t = scene.triangles().astype(np.float64)
    e1 = t[:, 1] - t[:, 0]
    e2 = t[:, 2] - t[:, 0]
    cr = np.cross(e1, e2)
    area = 0.5 * np.linalg.norm(cr, axis=1)
    cdf = np.cumsum(area)
    cdf /= cdf[-1]
    tri = np.searchsorted(cdf, rng.random(n), side="right").clip(0, len(area) - 1)
    r1 = np.sqrt(rng.random(n))
    r2 = rng.random(n)
    p = (1 - r1)[:, None] * t[tri, 0] + (r1 * (1 - r2))[:, None] * t[tri, 1] + (r1 * r2)[:, None] * t[tri, 2]
    nrm = cr[tri] / np.maximum(np.linalg.norm(cr[tri], axis=1, keepdims=True), 1e-30)
    tex = scene.textures[scene.tri_material[tri]]
    base = np.stack([(tex >> (8 * k)) & 0xFF for k in range(3)], 1).astype(np.float64) / 255.0
    met = rng.uniform(*metallic, size=n)
    if specular_fraction < 1.0:
        met = np.where(rng.random(n) < specular_fraction, met, 0.0)
    rough = rng.uniform(*roughness, size=n)
    f0 = 0.04
    diffuse = base * (1 - f0) * (1 - met)[:, None]
    specular = f0 * (1 - met)[:, None] + base * met[:, None]
    s = np.zeros(n, SAMPLE_DTYPE)
    s["position"] = p.astype(np.float32)
    s["depth"] = 0.0
    s["normal_texel"] = _f16(nrm * 0.5 + 0.5)
    s["diffuse_texel"][:, :3] = _u8(diffuse)
    s["diffuse_texel"][:, 3] = _u8(rough)
    s["specular_texel"][:, :3] = _u8(specular)
    s["specular_texel"][:, 3] = _u8(met)
    return s


def random_samples(n: int, center, half_extent: float, seed: int = 7, specular_fraction: float = 0.5) -> np.ndarray:
    """Samples at random points of a box with random normals and materials (test input)."""
    rng = np.random.default_rng(seed)
    s = np.zeros(n, SAMPLE_DTYPE)
    s["position"] = (np.asarray(center) + rng.uniform(-half_extent, half_extent, size=(n, 3))).astype(np.float32)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    s["normal_texel"] = _f16(v * 0.5 + 0.5)
    s["diffuse_texel"] = _u8(rng.random((n, 4)))
    s["diffuse_texel"][:, 3] = _u8(rng.uniform(0.1, 0.9, n))
    spec = rng.random(n) < specular_fraction
    s["specular_texel"][:, :3] = _u8(rng.random((n, 3)))
    s["specular_texel"][:, 3] = np.where(spec, _u8(rng.uniform(0.05, 1, n)), 0.0)
    emis = rng.random(n) < 0.05
    s["emission_texel"] = np.where(emis[:, None], _f16(rng.random((n, 3))), 0.0)
    return s


def atlas_shape(R: int) -> tuple[int, int, int]:
    """(depth, height, width) of the reference's atlas for resolution R."""
    return (R + 2, (R + 2) * 6, (R + 2) * 6)


def smooth_volume(R: int, seed: int = 5, max_alpha: float = 0.3, waves: int = 6, xp=np, device=None):
    """A float RGBA atlas (reference layout, (D, H, W, 4) float32) of smooth noise: each channel the mean
    of `waves` separable products sin(kx x + a) sin(ky y + b) sin(kz z + c) over the texel grid mapped to
    rgb in [0, 1] and alpha in [0, max_alpha] (the differentiable form's volume; alpha below 1 never
    saturates the march).  `xp` = numpy, or torch with `device` to build it on the GPU."""
    rng = np.random.default_rng(seed)
    D, H, W = atlas_shape(R)

    def axis(n):
        return xp.arange(n, dtype=xp.float32) if device is None else xp.arange(n, dtype=xp.float32, device=device)

    x, y, z = axis(W), axis(H), axis(D)
    if device is None:
        out = np.empty((D, H, W, 4), np.float32)
    else:
        out = xp.empty((D, H, W, 4), dtype=xp.float32, device=device)
    for c in range(4):
        acc = None
        for _ in range(waves):
            k = rng.uniform(0.02, 0.12, 3) * 2 * np.pi
            ph = rng.uniform(0, 2 * np.pi, 3)
            term = (xp.sin(z * float(k[2]) + float(ph[2]))[:, None, None] *
                    xp.sin(y * float(k[1]) + float(ph[1]))[None, :, None] *
                    xp.sin(x * float(k[0]) + float(ph[0]))[None, None, :])
            acc = term if acc is None else acc + term
        out[..., c] = (acc / waves * 0.5 + 0.5) * (max_alpha if c == 3 else 1.0)
    return out


def random_atlas(R: int, seed: int = 3, fill: float = 0.15) -> np.ndarray:
    """Sparse random RGBA8 atlas (uint32 words, reference layout): `fill` of the texels are occupied."""
    rng = np.random.default_rng(seed)
    shape = atlas_shape(R)
    occ = rng.random(shape) < fill
    rgb = rng.integers(0, 256, size=shape + (3,), dtype=np.uint32)
    a = rng.integers(64, 256, size=shape, dtype=np.uint32)
    word = rgb[..., 0] | (rgb[..., 1] << 8) | (rgb[..., 2] << 16) | (a << 24)
    return np.where(occ, word, 0).astype(np.uint32)


def default_trace_desc(regions: np.ndarray, R: int) -> dict:
    """VoxelConeTracingDesc as VoxelConeTracingPass::onUpdate fills it (VoxelConeTracingPass.cpp:90-102,
    defaults VoxelConeTracingPass.h:75-82)."""
    mc = regions[0, 0:3].astype(np.float32)
    ext = regions[0, 3:6].astype(np.float32)
    vs = np.float32(regions[0, 6:7].view(np.float32)[0])
    center = mc * vs + (ext * vs) * np.float32(0.5)
    return dict(volume_center=center.tolist(), rendering_mode=8, voxel_size=float(vs), volume_dimension=float(R),
                trace_start_offset=1.0, indirect_diffuse_intensity=8.0, ambient_occlusion_factor=0.5,
                min_trace_step_factor=1.0, indirect_specular_intensity=3.0, occlusion_decay=2.0, enable_32_cones=0)


def _mix32(h, xp):
    """32-bit integer finaliser (murmur3 fmix32) on int64 arrays holding uint32 values."""
    m = 0xFFFFFFFF
    h = h ^ (h >> 16)
    h = (h * 0x85EBCA6B) & m
    h = h ^ (h >> 13)
    h = (h * 0xC2B2AE35) & m
    h = h ^ (h >> 16)
    return h


def procedural_atlas_words(index, seed: int, fill: float, xp):
    """RGBA8 words of a sparse hash-random atlas at linear texel `index` (int64 array, numpy or torch).

    Identical on the CPU (numpy) and the GPU (torch): the benchmark's CPU and GPU
    arms trace the same clipmap."""
    m = 0xFFFFFFFF
    h = _mix32(((index * 0x9E3779B1) & m) ^ (seed & m), xp)
    h2 = _mix32((h * 0x27D4EB2F + 0x165667B1) & m, xp)
    occ = (h & 0xFFFF) < int(fill * 65536)
    alpha = 64 + ((h >> 16) % 192)
    word = (h2 & 0xFFFFFF) | (alpha << 24)
    return xp.where(occ, word, xp.zeros_like(word))


def procedural_atlas_numpy(R: int, seed: int = 3, fill: float = 0.05, chunk: int = 1 << 26) -> np.ndarray:
    shape = atlas_shape(R)
    n = int(np.prod(shape))
    out = np.empty(n, np.uint32)
    for s in range(0, n, chunk):
        idx = np.arange(s, min(n, s + chunk), dtype=np.int64)
        out[s:s + idx.shape[0]] = procedural_atlas_words(idx, seed, fill, np).astype(np.uint32)
    return out.reshape(shape)


def procedural_atlas_torch(R: int, seed: int = 3, fill: float = 0.05, device="cuda", chunk: int = 1 << 27):
    import torch
    shape = atlas_shape(R)
    n = int(np.prod(shape))
    out = torch.empty(n, dtype=torch.int32, device=device)
    for s in range(0, n, chunk):
        idx = torch.arange(s, min(n, s + chunk), dtype=torch.int64, device=device)
        w = procedural_atlas_words(idx, seed, fill, torch)
        out[s:s + idx.shape[0]] = (w - ((w >> 31) << 32)).to(torch.int32)  # reinterpret uint32 as int32
    return out.reshape(shape)
