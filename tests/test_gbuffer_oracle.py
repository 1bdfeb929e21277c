"""The G-buffer producer's oracle on small scenes (CPU): what GBufferPass draws
for a camera -- closest surface per pixel, world position rebuilt from depth,
attachment texels after their formats -- including triangles that cross the
near plane, alpha-tested discards and equal-depth ties."""
import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300.scene import Scene, _materials_for

W, H = 96, 64
ASPECT = W / H


def _quads_scene(quads, colors, materials=None):
    """Each quad (4 corners, normal) as two triangles with its own material."""
    pos, nrm, mat = [], [], []
    for qi, (p, n) in enumerate(quads):
        p = np.asarray(p, np.float32)
        for tri in ((0, 1, 2), (0, 2, 3)):
            pos.extend(p[list(tri)])
            nrm.extend([n] * 3)
            mat.append(qi)
    pos = np.asarray(pos, np.float32)
    idx = np.arange(len(pos), dtype=np.uint32).reshape(-1, 3)
    tex = np.asarray(colors, np.uint32)
    m = _materials_for(tex) if materials is None else materials
    return Scene(pos, np.asarray(nrm, np.float32), idx, np.asarray(mat, np.uint32), m, tex)


def _floor(y=0.0, half=20.0):
    return ([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]], (0.0, 1.0, 0.0))


def _wall(z, half=3.0):
    return ([[-half, -half, z], [half, -half, z], [half, half, z], [-half, half, z]], (0.0, 0.0, -1.0))


def _fields(g):
    return dict(pos=g[:, 0:3], depth=g[:, 3], normal=g[:, 4:7], diffuse=g[:, 8:12], specular=g[:, 12:16],
                emission=g[:, 16:19])


def test_floor_seen_from_above(oracle):
    cam = oracle.camera_matrix((0.0, 2.0, -5.0), (0.0, -0.3, 1.0), aspect=ASPECT)
    g = _fields(oracle.gbuffer(_quads_scene([_floor()], [0xFF4080C0]), cam, W, H))
    hit = g["depth"] < 1.0
    assert 0.3 * W * H < hit.sum() < 0.9 * W * H
    # world +y maps to NDC +y and NDC y -1 is row 0 (no flip, as the reference draws), so the
    # floor below the horizon fills the rows with the smaller index
    rows = hit.reshape(H, W).all(1)
    assert rows[0] and not rows[-1]
    assert np.abs(g["pos"][hit, 1]).max() < 2e-3
    assert np.all(g["depth"][hit] > 0.0)
    n = g["normal"][hit]
    assert np.array_equal(n, np.broadcast_to(np.float32([0.5, 1.0, 0.5]), n.shape))
    # diffuse = base * 0.96 stored as UNORM8, roughness 1; specular F0 0.04, metallic 0
    base = np.float32([0xC0, 0x80, 0x40]) / np.float32(255.0)
    want = np.floor(np.clip(base * np.float32(0.96), 0, 1) * np.float32(255.0) + np.float32(0.5)) / np.float32(255.0)
    assert np.array_equal(g["diffuse"][hit][:, :3], np.broadcast_to(want.astype(np.float32), (hit.sum(), 3)))
    assert (g["diffuse"][hit][:, 3] == 1.0).all() and (g["specular"][hit][:, 3] == 0.0).all()
    assert np.allclose(g["specular"][hit][:, :3], 10 / 255.0)
    # sky pixels: depth 1, the colour clear (0, 0, 0, 1)
    sky = ~hit
    assert (g["diffuse"][sky] == np.float32([0, 0, 0, 1])).all()


def test_near_plane_clipping_leaves_no_holes(oracle):
    """A floor that extends behind the camera crosses the near plane: clipped, drawn without gaps."""
    cam = oracle.camera_matrix((0.0, 1.0, 0.0), (0.0, -1.0, 0.6), aspect=ASPECT)
    g = _fields(oracle.gbuffer(_quads_scene([_floor(half=50.0)], [0xFFFFFFFF]), cam, W, H))
    hit = (g["depth"] < 1.0).reshape(H, W)
    # looking steeply down: the 60% of the image below the horizon is floor, with no hole
    assert hit[:int(0.6 * H)].all()
    pos = g["pos"][g["depth"] < 1.0]
    assert np.abs(pos[:, 1]).max() < 1e-3


def test_closest_surface_wins(oracle):
    cam = oracle.camera_matrix((0.0, 0.0, -5.0), (0.0, 0.0, 1.0), aspect=ASPECT)
    near, far = _wall(0.0, half=1.0), _wall(2.0, half=3.0)
    for order in ((far, near), (near, far)):
        colors = [0xFF0000FF, 0xFF00FF00] if order[0] is far else [0xFF00FF00, 0xFF0000FF]
        g = _fields(oracle.gbuffer(_quads_scene(list(order), colors), cam, W, H))
        c = (H // 2) * W + W // 2
        # the near wall at z = 0 (depth -> position in FP32 with near 0.01 loses ~1e-4 at 5 units)
        assert abs(g["pos"][c, 2] - 0.0) < 1e-3
        assert g["diffuse"][c, 1] > 0.9 and g["diffuse"][c, 0] == 0.0  # green (0xFF00FF00 is RGBA 0,255,0,255)


def test_equal_depth_tie_keeps_the_first_triangle(oracle):
    cam = oracle.camera_matrix((0.0, 0.0, -5.0), (0.0, 0.0, 1.0), aspect=ASPECT)
    g = _fields(oracle.gbuffer(_quads_scene([_wall(0.0), _wall(0.0)], [0xFF0000FF, 0xFFFF0000]), cam, W, H))
    hit = g["depth"] < 1.0
    assert hit.sum() > 100
    assert (g["diffuse"][hit][:, 0] > 0.9).all() and (g["diffuse"][hit][:, 2] == 0.0).all()  # red: the first quad


def test_alpha_tested_material_is_discarded(oracle):
    tex = np.asarray([0x20FFFFFF, 0xFFFFFFFF], np.uint32)  # alpha 0x20 / 0xFF
    m = _materials_for(tex)
    m["alpha_mode"] = 1
    m["alpha_cutoff"] = 0.5
    cam = oracle.camera_matrix((0.0, 0.0, -5.0), (0.0, 0.0, 1.0), aspect=ASPECT)
    g = _fields(oracle.gbuffer(_quads_scene([_wall(0.0, 1.0), _wall(1.0, 3.0)], tex, m), cam, W, H))
    c = (H // 2) * W + W // 2
    assert abs(g["pos"][c, 2] - 1.0) < 1e-3  # the cut-out near quad is not drawn


def test_materials_and_emission(oracle):
    tex = np.asarray([0xFF808080, 0xFF00FF00, 0xFFFFFFFF], np.uint32)
    m = _materials_for(tex[:1])
    m["pbr_metallic_factor"] = 0.75
    m["pbr_roughness_factor"] = 0.01  # clamped to 0.04
    m["emissive_factor"] = (0.5, 2.0, 0.0)
    m["emissive_texture"] = 2
    cam = oracle.camera_matrix((0.0, 0.0, -5.0), (0.0, 0.0, 1.0), aspect=ASPECT)
    sc = _quads_scene([_wall(0.0)], tex[:1], m)
    sc.textures = tex
    g = _fields(oracle.gbuffer(sc, cam, W, H))
    c = (H // 2) * W + W // 2
    b = np.float32(0x80) / np.float32(255.0)
    rough = np.floor(np.float32(0.04) * np.float32(255.0) + np.float32(0.5)) / np.float32(255.0)
    assert g["diffuse"][c, 3] == np.float32(rough)
    assert g["specular"][c, 3] == np.float32(np.floor(np.float32(0.75) * 255 + 0.5) / np.float32(255.0))
    spec = np.float32(0.04) * np.float32(0.25) + b * np.float32(0.75)
    assert abs(g["specular"][c, 0] - spec) <= 0.5 / 255.0 + 1e-7
    assert np.array_equal(g["emission"][c], np.float32([0.5, 2.0, 0.0]))  # texel 1.0 ^ 2.2 = 1


@pytest.mark.parametrize("seed", [0, 1])
def test_room_scene_depth_matches_positions(oracle, seed):
    """Every drawn pixel's rebuilt position projects back to its pixel centre at its depth."""
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    sc = room_scene(seed=seed, n_random=500)
    cam = oracle.camera_matrix((0.3, 2.0, -4.0), (0.2, -0.1, 1.0), aspect=ASPECT)
    g = _fields(oracle.gbuffer(sc, cam, W, H))
    hit = g["depth"] < 1.0
    assert hit.mean() > 0.95  # inside the room: every pixel sees a wall
    vp = cam[0:16].reshape(4, 4).T.astype(np.float64)
    p = np.concatenate([g["pos"][hit].astype(np.float64), np.ones((hit.sum(), 1))], 1) @ vp.T
    ndc = p[:, :3] / p[:, 3:4]
    iy, ix = np.divmod(np.nonzero(hit)[0], W)
    assert np.abs((ndc[:, 0] + 1) * 0.5 * W - (ix + 0.5)).max() < 1e-2
    assert np.abs((ndc[:, 1] + 1) * 0.5 * H - (iy + 0.5)).max() < 1e-2
    assert np.abs(ndc[:, 2] - g["depth"][hit]).max() < 1e-5
