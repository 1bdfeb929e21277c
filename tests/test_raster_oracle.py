"""CPU checks of the raster oracle and of the library's host-side math.

Analytic cases of the pinned rasteriser (a floor quad voxelises into a full
layer; shared edges are covered once; depth of a plane), and the library's
host helpers (view-projection, light matrices) against the reference's glm
golden vectors."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import capi
from vk_voxel_cone_tracing_gb300.scene import Scene, _materials_for

GOLDEN = Path(__file__).resolve().parent / "golden"


def _quad_scene(y=0.3, half=40.0, color=0xFF4080C0):
    p = np.array([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]], np.float32)
    tris = np.stack([p[[0, 1, 2]], p[[0, 2, 3]]])
    pos = tris.reshape(-1, 3).copy()
    nrm = np.tile(np.array([0, 1, 0], np.float32), (6, 1))
    idx = np.arange(6, dtype=np.uint32).reshape(2, 3)
    tex = np.array([color, color], np.uint32)
    return Scene(pos, nrm, idx, np.array([0, 1], np.uint32), _materials_for(tex), tex)


def test_floor_quad_fills_a_voxel_layer(oracle):
    R = 32
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    atlas = oracle.voxelize_opacity(_quad_scene(0.3), R, regions, level_mask=1)
    vs = oracle.region_voxel_size(regions, 0)
    iy = int(np.floor((0.3 / (R * vs) % 1.0) * R)) + 1
    face0 = atlas[1:R + 1, 1:R + 1, 1:R + 1]  # level 0, face 0 block: [z, y, x]
    layer = face0[:, iy - 1, :]
    assert (layer == 0xFFFFFFFF).all(), np.count_nonzero(layer != 0xFFFFFFFF)
    # nothing outside the layer, and the 6 face copies agree
    assert np.count_nonzero(face0) == R * R
    for f in range(1, 6):
        blk = atlas[1:R + 1, 1:R + 1, 1 + f * (R + 2):R + 1 + f * (R + 2)]
        assert np.array_equal(blk, face0)


def test_shared_edge_covered_once(oracle):
    """Shadow depth of two triangles sharing a diagonal: a plane at constant
    depth covers every pixel whose centre is inside it (no gaps on the edge)."""
    from oracle.oracle import light_shadow_desc
    # a light looking straight down (up = +y would be parallel: tilt it by 1e-3)
    sd = light_shadow_desc((0.0, 20.0, 0.0), (1e-3, -1.0, 0.0))
    depth = oracle.shadow_depth(_quad_scene(0.0, half=8.0), sd, 64, 64)
    inside = depth < 1.0
    # the quad spans +-8 of the +-16 ortho: the central half of the map, no holes
    assert inside[17:47, 17:47].all() and not inside[:15].any() and not inside[49:].any()
    assert inside.sum() in range(31 * 31, 34 * 34)
    z = depth[inside]
    assert np.ptp(z) < 1e-3 and 0.0 < z.min() < 1.0


def test_library_host_matrices_match_glm_golden(vct_lib):
    g = json.loads((GOLDEN / "glm_host_math.json").read_text())
    from vk_voxel_cone_tracing_gb300.clipmap import clip_regions
    for rec in g["regions"]:
        cam = np.array(rec["cam"], np.uint32).view(np.float32).tolist()
        regs = clip_regions(cam, rec["R"])
        out = (C.c_float * 48)()
        capi.call("vct_voxelization_view_proj", C.byref(regs[rec["level"]]), C.cast(out, C.c_void_p))
        got = np.frombuffer(bytes(out), np.uint32).reshape(3, 16)
        assert np.array_equal(got, np.array(rec["view_proj"], np.uint32).reshape(3, 16))
    from vk_voxel_cone_tracing_gb300.passes import light_shadow_desc
    for rec in g["lights"]:
        o = np.array(rec["origin"], np.uint32).view(np.float32).tolist()
        d = np.array(rec["direction"], np.uint32).view(np.float32).tolist()
        sd = light_shadow_desc(o, d)
        assert np.array_equal(np.frombuffer(bytes(sd.view), np.uint32), np.array(rec["view"], np.uint32))
        assert np.array_equal(np.frombuffer(bytes(sd.proj), np.uint32), np.array(rec["proj"], np.uint32))


def test_library_camera_matrix_matches_glm_golden(vct_lib):
    g = json.loads((GOLDEN / "glm_host_math.json").read_text())
    from vk_voxel_cone_tracing_gb300.passes import camera_matrix
    for rec in g["cameras"]:
        v = np.array(rec["in"], np.uint32).view(np.float32)
        cam = camera_matrix(v[0:3].tolist(), v[3:6].tolist(), v[6:9].tolist(), float(v[9]), float(v[10]))
        assert np.array_equal(np.frombuffer(bytes(cam.view_proj), np.uint32), np.array(rec["view_proj"], np.uint32))
        assert np.array_equal(np.frombuffer(bytes(cam.view_proj_inv), np.uint32),
                              np.array(rec["view_proj_inv"], np.uint32))
    with pytest.raises(capi.VctError):
        camera_matrix((0, 0, 0), (0, 0, 1), aspect=0.0)


def test_library_voxelization_desc_matches_oracle(vct_lib, oracle):
    from vk_voxel_cone_tracing_gb300.clipmap import clip_regions
    for cam, R in (((0.0, 0.0, 0.0), 128), ((1.3, 2.7, -5.1), 256)):
        regs = clip_regions(cam, R)
        oregs = oracle.clip_regions(cam, R)
        for lvl in range(6):
            d = capi.VoxelizationDesc()
            capi.call("vct_voxelization_desc_for", C.cast(regs, C.c_void_p), lvl, R, capi.ref(d))
            assert bytes(d) == oracle.voxelization_desc(oregs, lvl, R)


def test_svo_build_small_tree(oracle):
    """Two fragments in opposite corners at level 3: the flagged paths and leaf colours."""
    frags = np.zeros((2, 2), np.uint32)
    # positions (x, y, z) = (2, 2, 2) and (13, 13, 13) in a 2^4 grid; colours 28-bit
    for i, (p, c) in enumerate((((2, 2, 2), 0x0F102030), ((13, 13, 13), 0x0F405060))):
        x, y, z = p
        frags[i, 0] = x | (y << 12) | ((z & 0xFF) << 24)
        frags[i, 1] = ((z >> 8) << 28) | c
    pool, n = oracle.svo_build(frags, 4, capacity=4096)
    # level 1: both land in root child 0 (the ">> 1" quirk halves positions)
    assert pool[0, 0] & 0x80000000 and all(pool[k, 0] == 0 for k in range(1, 8))
    leaves = [k for k in range(n) if pool[k, 1] != 0 and (pool[k, 0] & 0x7FFFFFFF) == 0]
    assert len(leaves) >= 2
    cols = sorted(int(pool[k, 1]) for k in leaves)
    assert 0x0F102030 in cols and 0x0F405060 in cols
