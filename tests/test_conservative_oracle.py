"""The oracle's conservative voxelisation mode on the CPU: its triangle / box overlap decision (Schwarz &
Seidel 2010, FP32) against an independent separating-axis test (Akenine-Moller 2001, FP64) on random
triangles, and whole-scene properties (every vertex's voxel is marked; a flat quad marks exactly its
layer of voxels; triangles outside a level leave it empty)."""
import numpy as np
import pytest

R = 32


def _region(min_corner=(-16, -16, -16), vs=0.5):
    row = np.zeros(7, np.int32)
    row[0:3] = min_corner
    row[3:6] = R
    row[6] = np.float32(vs).view(np.int32)
    return row


def _sat_overlap(tri, lo, hi):
    """Separating-axis triangle / box test in FP64: the 13 axes (box normals, triangle normal, 9 edge
    cross products)."""
    c = 0.5 * (lo + hi)
    h = 0.5 * (hi - lo)
    v = tri - c
    e = [v[1] - v[0], v[2] - v[1], v[0] - v[2]]
    axes = [np.eye(3)[i] for i in range(3)] + [np.cross(e[0], e[1])]
    axes += [np.cross(np.eye(3)[i], ej) for i in range(3) for ej in e]
    for a in axes:
        if not np.any(a):
            continue
        p = v @ a
        r = np.abs(a) @ h
        if p.min() > r or p.max() < -r:
            return False
    return True


def test_overlap_matches_separating_axes(oracle):
    rng = np.random.default_rng(0)
    row = _region()
    vs = 0.5
    agree = disagree = 0
    for _ in range(1500):
        centre = rng.uniform(-6, 6, 3)
        tri = (centre + rng.normal(0, rng.choice([0.3, 1.0, 3.0]), (3, 3))).astype(np.float32)
        u = tri.astype(np.float64) / vs - row[0:3]
        lo = np.clip(np.floor(u.min(0)).astype(int) - 1, 0, R - 1)
        hi = np.clip(np.floor(u.max(0)).astype(int) + 1, 0, R - 1)
        for _ in range(6):
            ijk = [int(rng.integers(lo[a], hi[a] + 1)) for a in range(3)]
            got = oracle.cons_overlap(tri, row, R, *ijk)
            want = _sat_overlap(u, np.array(ijk, float), np.array(ijk, float) + 1.0)
            # boxes outside the triangle's bounding box are not candidates of the method (the voxel loop
            # visits the bounding box): compare only the boxes inside it
            if any(ijk[a] < np.floor(u[:, a].min()) or ijk[a] > np.floor(u[:, a].max()) for a in range(3)):
                assert not got
                continue
            if got == want:
                agree += 1
            else:  # FP32 ties on a face or edge of the box: the box must be within rounding of the triangle
                grown = _sat_overlap(u, np.array(ijk, float) - 1e-4, np.array(ijk, float) + 1.0 + 1e-4)
                shrunk = _sat_overlap(u, np.array(ijk, float) + 1e-4, np.array(ijk, float) + 1.0 - 1e-4)
                assert grown and not shrunk, (tri, ijk, got, want)
                disagree += 1
    assert agree > 2000 and disagree <= 0.002 * agree


def _scene_of(tris):
    from vk_voxel_cone_tracing_gb300.scene import _pack
    return _pack(np.asarray(tris, np.float32).reshape(-1, 3, 3), np.random.default_rng(0))


def _marked(atlas, level):
    """Voxels (x, y, z in atlas texel units of face 0) marked at `level`."""
    rb = R + 2
    sub = atlas[1:R + 1, rb * level + 1: rb * level + R + 1, 1:R + 1]
    z, y, x = np.nonzero(sub)
    return set(zip(x.tolist(), y.tolist(), z.tolist()))


def test_vertices_are_marked_and_a_flat_quad_marks_one_layer(oracle):
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    vs0 = float(regions[0, 6:7].view(np.float32)[0])
    mc = regions[0, 0:3].astype(np.int64)
    # a horizontal quad inside voxel layer j = 5 of level 0 (y in the middle of the layer), x, z spanning 8
    y = (mc[1] + 5.5) * vs0
    x0, x1 = (mc[0] + 3.0) * vs0, (mc[0] + 11.0) * vs0
    z0, z1 = (mc[2] + 4.0) * vs0, (mc[2] + 12.0) * vs0
    quad = [[[x0, y, z0], [x1, y, z0], [x1, y, z1]], [[x0, y, z0], [x1, y, z1], [x0, y, z1]]]
    atlas = oracle.voxelize_conservative(_scene_of(quad), R, regions, level_mask=1)
    got = _marked(atlas, 0)
    # voxels of the quad's bounding box [3, 11] x [4, 12] (in voxel units): the box starting on the far edge
    # (i = 11, k = 12) touches it, the box ending on the near edge (i = 2) lies outside the bounding box
    want = {(int((mc[0] + i) % R), int((mc[1] + 5) % R), int((mc[2] + k) % R)) for i in range(3, 12)
            for k in range(4, 13)}
    assert got == want
    assert np.count_nonzero(atlas[:, (R + 2):, :]) == 0  # other levels untouched


def test_random_scene_marks_every_vertex_voxel(oracle):
    rng = np.random.default_rng(5)
    regions = oracle.clip_regions((0.3, 0.2, -0.1), R)
    tris = rng.uniform(-9, 9, (1, 3)) + rng.normal(0, 0.6, (200, 3, 3))
    atlas = oracle.voxelize_conservative(_scene_of(tris), R, regions)
    for level in range(6):
        vs = float(regions[level, 6:7].view(np.float32)[0])
        mc = regions[level, 0:3].astype(np.int64)
        marked = _marked(atlas, level)
        for v in np.asarray(tris, np.float32).reshape(-1, 3):
            u = np.floor(v.astype(np.float64) / vs - mc).astype(int)
            if np.all((u >= 0) & (u < R)):
                assert tuple(((mc + u) % R).tolist()) in marked
    # a triangle far outside every level leaves the atlas empty
    far = oracle.voxelize_conservative(_scene_of([[[900, 900, 900], [901, 900, 900], [900, 901, 900]]]), R, regions)
    assert not far.any()
