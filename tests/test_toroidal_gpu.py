"""GPU parity of the toroidal revoxelisation: the slab pass on its own and whole
frames in VCT_REVOX_TOROIDAL mode, against the oracle running the same steps
(region update, slab clear + voxelisation, mips of the moved levels, border,
then the radiance passes of the due levels), bit for bit."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)
PATH = [(0.35, 2.1, -0.7), (0.9, 2.3, -1.2), (1.7, 2.0, -1.4), (1.75, 2.05, -1.4), (-3.0, 2.6, 0.4),
        (30.0, 4.0, -9.0)]


def _origin(center=(0.0, 4.0, 0.0), dist=15.0):
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - dist * d).astype(np.float32).tolist())


def _np_regions(regs):
    return np.frombuffer(bytes(regs), np.int32).reshape(6, 7).copy()


@pytest.mark.parametrize("R", [32, 64])
def test_slab_voxelisation_sequence_bit_exact(cuda, oracle, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    sc = room_scene(seed=4, n_random=3000)
    ds, ws = passes.DeviceScene(sc), passes.Workspace()
    regs = clipmap.clip_regions(PATH[0], R)
    o_regs = oracle.clip_regions(PATH[0], R).astype(np.int32).copy()
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity(ds, regs, R, atlas, ws)
    want = oracle.voxelize_opacity(sc, R, o_regs)
    moved = 0
    for cam in PATH[1:]:
        slabs, levels = passes.update_clip_regions(regs, cam, R)
        o_slabs, o_levels = oracle.update_clip_regions(o_regs, np.float32(cam), R)
        assert levels == o_levels.tolist()
        moved += len(levels)
        passes.voxelize_opacity_slabs(ds, regs, R, atlas, slabs, levels, ws)
        oracle.voxelize_opacity_slabs(sc, R, o_regs, want, o_slabs, o_levels)
        torch.cuda.synchronize()
        got = atlas.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want), f"camera {cam}: {np.count_nonzero(got != want)} texels differ"
    assert moved >= 6 and np.count_nonzero(want) > 1000


def test_toroidal_frames_bit_exact(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    R, S = 32, 256
    sc = room_scene(seed=5, n_random=3000)
    ds, ws = passes.DeviceScene(sc), passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((S, S), dtype=torch.float32, device="cuda")
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(_origin(), LIGHT_DIR)
    state = (capi.ClipmapRegion * 6)()
    sd_o = oracle.light_shadow_desc(_origin(), LIGHT_DIR)
    w_sh = oracle.shadow_depth(sc, sd_o, S, S)
    w_op = w_rad = o_regs = None
    for k, cam in enumerate(PATH[:5]):
        mode = capi.REVOX_FULL if k == 0 else capi.REVOX_TOROIDAL
        passes.clipmap_frame(ds, cam, R, op, rad, sh, light, lsd, ws, frame_index=k, revoxelization=mode,
                             regions_state=state)
        # the oracle's frame k
        due = [l for l in range(6) if k % (1 << l) == 0]
        if k == 0:
            o_regs = oracle.clip_regions(cam, R).astype(np.int32).copy()
            w_op = oracle.voxelize_opacity(sc, R, o_regs)
            mip_levels = range(1, 6)
            w_rad = np.zeros_like(w_op)
        else:
            o_slabs, o_levels = oracle.update_clip_regions(o_regs, np.float32(cam), R)
            oracle.voxelize_opacity_slabs(sc, R, o_regs, w_op, o_slabs, o_levels)
            mip_levels = sorted({int(l) for l in o_levels if l >= 1})
        for level in mip_levels:
            oracle.downsample(w_op, R, o_regs[level - 1, 0:3], level, 0)
        oracle.wrap_border(w_op, R)
        for level in due:
            oracle.clear_region(w_rad, R, (0, 0, 0), (R, R, R), level)
        mask = sum(1 << l for l in due)
        w_rad = oracle.inject_radiance(sc, R, o_regs, w_sh, sd_o, level_mask=mask, atlas=w_rad)
        for level in due:
            oracle.copy_alpha(w_rad, w_op, R, level)
        for level in due:
            if level >= 1:
                oracle.downsample(w_rad, R, o_regs[level - 1, 0:3], level, 1)
        torch.cuda.synchronize()
        assert np.array_equal(_np_regions(state), o_regs), k
        g_op = op.cpu().numpy().view(np.uint32)
        g_rad = rad.cpu().numpy().view(np.uint32)
        assert np.array_equal(g_op, w_op), f"frame {k}: opacity {np.count_nonzero(g_op != w_op)} texels differ"
        assert np.array_equal(g_rad, w_rad), f"frame {k}: radiance {np.count_nonzero(g_rad != w_rad)} texels differ"
    assert np.array_equal(sh.cpu().numpy().view(np.uint32), w_sh.view(np.uint32))
    # the toroidal mode without its region state is refused
    with pytest.raises(capi.VctError):
        passes.clipmap_frame(ds, PATH[0], R, op, rad, sh, light, lsd, ws, revoxelization=capi.REVOX_TOROIDAL)


@pytest.mark.parametrize("seed", [1, 2])
def test_random_walk_slabs_bit_exact(cuda, oracle, seed):
    """A random camera walk (small steps, a few jumps past level extents) through the slab pass."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    R = 32
    rng = np.random.default_rng(seed)
    sc = room_scene(seed=seed, n_random=2000)
    ds, ws = passes.DeviceScene(sc), passes.Workspace()
    cam = np.float32([0.3, 2.0, -0.5])
    regs = clipmap.clip_regions(tuple(cam.tolist()), R)
    o_regs = oracle.clip_regions(cam, R).astype(np.int32).copy()
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity(ds, regs, R, atlas, ws)
    want = oracle.voxelize_opacity(sc, R, o_regs)
    for k in range(8):
        step = rng.normal(0, 0.8, 3) if k % 4 else rng.normal(0, 12.0, 3)
        cam = (cam + step).astype(np.float32)
        slabs, levels = passes.update_clip_regions(regs, cam.tolist(), R)
        o_slabs, o_levels = oracle.update_clip_regions(o_regs, cam, R)
        passes.voxelize_opacity_slabs(ds, regs, R, atlas, slabs, levels, ws)
        oracle.voxelize_opacity_slabs(sc, R, o_regs, want, o_slabs, o_levels)
    torch.cuda.synchronize()
    got = atlas.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"
