"""GPU parity of the conservative voxelisation mode (vct_voxelize_opacity_conservative) against the oracle:
the same triangle / box overlap arithmetic, so every atlas word is compared bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(cuda, oracle, sc, cam, R, mask=0x3F):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    ds = passes.DeviceScene(sc)
    regs = clipmap.clip_regions(cam, R)
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity_conservative(ds, regs, R, atlas, level_mask=mask)
    torch.cuda.synchronize()
    got = atlas.cpu().numpy().view(np.uint32)
    want = oracle.voxelize_conservative(sc, R, oracle.clip_regions(cam, R), level_mask=mask)
    return got, want


@pytest.mark.parametrize("R,cam,mask", [(32, (0.3, 2.0, -0.5), 0x3F), (64, (-4.0, 5.5, 2.0), 0x2D)])
def test_room_scene_bit_exact(cuda, oracle, R, cam, mask):
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    got, want = _run(cuda, oracle, room_scene(seed=2, n_random=3000), cam, R, mask)
    assert np.count_nonzero(want) > 1000
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} words differ"


def test_hall_scene_bit_exact(cuda, oracle):
    from vk_voxel_cone_tracing_gb300.scene import hall_scene
    got, want = _run(cuda, oracle, hall_scene(seed=2, target=40_000), (0.0, 5.0, 0.0), 64)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} words differ"


def test_superset_of_the_msaa_voxels_on_large_triangles(cuda, oracle):
    """On a scene of large triangles well inside level 0, the voxels the MSAA voxeliser marks are marked by
    the conservative mode too (the MSAA position lies on the triangle)."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import _pack
    rng = np.random.default_rng(3)
    tris = rng.uniform(-3.0, 3.0, (1, 3)) + rng.uniform(-2.5, 2.5, (40, 3, 3))
    sc = _pack(tris, rng)
    R, cam = 64, (0.0, 0.0, 0.0)
    got, want = _run(cuda, oracle, sc, cam, R, mask=1)
    assert np.array_equal(got, want)
    ws = passes.Workspace()
    msaa = clipmap.new_atlas(R)
    passes.voxelize_opacity(passes.DeviceScene(sc), clipmap.clip_regions(cam, R), R, msaa, ws, level_mask=1)
    torch.cuda.synchronize()
    m = msaa.cpu().numpy().view(np.uint32)
    rb = R + 2
    inner = (slice(2, R), slice(2, R), slice(2, R))  # away from the region's clamp band
    mm, cc = m[:, :rb, :rb][inner] != 0, got[:, :rb, :rb][inner] != 0
    assert mm.sum() > 100 and cc.sum() >= mm.sum()
    # an MSAA sample within rounding of a voxel face can land in the neighbouring voxel (its index comes
    # from fract(p / extent) * R, not from the region's integer corner)
    assert np.mean(cc[mm]) > 0.999, f"{np.count_nonzero(mm & ~cc)} MSAA voxels not marked"


def test_bad_arguments(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    ds = passes.DeviceScene(room_scene(seed=1, n_random=100))
    regs = clipmap.clip_regions((0.0, 0.0, 0.0), 32)
    with pytest.raises(capi.VctError):
        passes.voxelize_opacity_conservative(ds, regs, 32, clipmap.new_atlas(32), level_mask=0x40)
    with pytest.raises(capi.VctError):
        passes.voxelize_opacity_conservative(ds, regs, 24, clipmap.new_atlas(32))
