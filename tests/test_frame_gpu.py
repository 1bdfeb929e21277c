"""One full frame of the clipmap method on the GPU (vct_clipmap_frame) against
the oracle running the same passes in Application::run's order, then the
cone trace of that frame's radiance clipmap."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAM = (0.35, 2.1, -0.7)
LIGHT_DIR = (0.3, -1.0, 0.2)


def _origin(center=(0.0, 4.0, 0.0), dist=15.0):
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - dist * d).astype(np.float32).tolist())


def oracle_frame(oracle, scene, R, shadow_res):
    regions = oracle.clip_regions(CAM, R)
    opacity = oracle.voxelize_opacity(scene, R, regions)
    for level in range(1, 6):
        oracle.downsample(opacity, R, regions[level - 1, 0:3], level, 0)
    oracle.wrap_border(opacity, R)
    sd = oracle.light_shadow_desc(_origin(), LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd, shadow_res, shadow_res)
    radiance = np.zeros_like(opacity)
    radiance = oracle.inject_radiance(scene, R, regions, shadow, sd, atlas=radiance)
    for level in range(6):
        oracle.copy_alpha(radiance, opacity, R, level)
    for level in range(1, 6):
        oracle.downsample(radiance, R, regions[level - 1, 0:3], level, 1)
    return regions, opacity, shadow, radiance, sd


@pytest.mark.parametrize("R", [32, 64])
def test_clipmap_frame_bit_exact(cuda, oracle, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    scene = room_scene(seed=1, n_random=3000)
    regions, w_op, w_sh, w_rad, sd_o = oracle_frame(oracle, scene, R, 256)
    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    op = clipmap.new_atlas(R)
    rad = clipmap.new_atlas(R)
    sh = torch.empty((256, 256), dtype=torch.float32, device="cuda")
    passes.clipmap_frame(ds, CAM, R, op, rad, sh, passes.light_desc(LIGHT_DIR),
                         passes.light_shadow_desc(_origin(), LIGHT_DIR), ws)
    torch.cuda.synchronize()
    assert np.array_equal(sh.cpu().numpy().view(np.uint32), w_sh.view(np.uint32))
    g_op = op.cpu().numpy().view(np.uint32)
    g_rad = rad.cpu().numpy().view(np.uint32)
    assert np.array_equal(g_op, w_op), f"opacity: {np.count_nonzero(g_op != w_op)} texels differ"
    assert np.array_equal(g_rad, w_rad), f"radiance: {np.count_nonzero(g_rad != w_rad)} texels differ"
    assert np.count_nonzero(g_rad >> 24) > 1000  # copy-alpha carried opacity into radiance.a

    # trace this frame's radiance (fast form) against the FP64 oracle
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, surface_samples
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    samples = surface_samples(scene, 1500, seed=5)
    eye = (0.0, 3.0, -3.0)
    sd_bytes = sd_o
    d64, s64, _, _ = oracle.cone_trace(64, bytes(desc), eye, w_rad, R, samples, shadow=w_sh,
                                       shadow_desc_bytes=sd_bytes)
    tex = clipmap.RadianceTexture(R).update(rad)
    d, s = clipmap.cone_trace_fast(desc, eye, tex, clipmap.samples_to_device(samples),
                                   light=passes.light_desc(LIGHT_DIR), shadow=sh,
                                   shadow_desc=passes.light_shadow_desc(_origin(), LIGHT_DIR))
    torch.cuda.synchronize()
    for got, want in ((d.cpu().numpy()[:, :3], d64[:, :3]), (s.cpu().numpy()[:, :3], s64[:, :3])):
        rel = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-12)
        assert rel < 1e-2, rel
    tex.close()


def test_frame_keeps_the_radiance_texture_equal_to_the_atlas(cuda):
    """With vct_frame_desc.radiance_texture set, the frame's copy-alpha and mip
    passes also store their texels into the texture: after a full frame and
    after a frame that refreshes level 0 only (frame_index 1), the texture read
    back equals the radiance atlas on every texel, borders included."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    R = 32
    scene = room_scene(seed=2, n_random=2000)
    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((256, 256), dtype=torch.float32, device="cuda")
    tex = clipmap.RadianceTexture(R)
    back = clipmap.new_atlas(R)
    for frame_index, cam in ((0, CAM), (1, (CAM[0] + 0.7, CAM[1], CAM[2] - 0.4))):
        passes.clipmap_frame(ds, cam, R, op, rad, sh, passes.light_desc(LIGHT_DIR),
                             passes.light_shadow_desc(_origin(), LIGHT_DIR), ws, frame_index=frame_index,
                             texture=tex)
        tex.read(back)
        torch.cuda.synchronize()
        a = rad.cpu().numpy().view(np.uint32)
        b = back.cpu().numpy().view(np.uint32)
        assert np.count_nonzero(a) > 1000
        assert np.array_equal(a, b), f"frame {frame_index}: {np.count_nonzero(a != b)} texels differ"
    # a texture of another resolution is refused before any work
    other = clipmap.RadianceTexture(16)
    with pytest.raises(RuntimeError, match="radiance texture"):
        passes.clipmap_frame(ds, CAM, R, op, rad, sh, passes.light_desc(LIGHT_DIR),
                             passes.light_shadow_desc(_origin(), LIGHT_DIR), ws, texture=other)
    tex.close()
    other.close()


def test_second_frame_refreshes_level_zero_only_bit_exact(cuda, oracle):
    """Frame 0 then frame 1 with a moved camera: frame 1 revoxelises every
    level but clears, injects and copies alpha into radiance level 0 only
    (cadence 2^level) -- the fused voxelise + count pass must count only the
    due level's samples.  Compared with the oracle running the reference's
    passes in order, bit for bit."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    R = 32
    scene = room_scene(seed=3, n_random=2000)
    cam1 = (CAM[0] + 1.3, CAM[1] - 0.4, CAM[2] + 0.9)
    _, w_op, w_sh, w_rad, sd_o = oracle_frame(oracle, scene, R, 256)
    regions1 = oracle.clip_regions(cam1, R)
    w_op1 = oracle.voxelize_opacity(scene, R, regions1)
    for level in range(1, 6):
        oracle.downsample(w_op1, R, regions1[level - 1, 0:3], level, 0)
    oracle.wrap_border(w_op1, R)
    w_rad1 = w_rad.copy()
    oracle.clear_region(w_rad1, R, (0, 0, 0), (R, R, R), 0)
    w_rad1 = oracle.inject_radiance(scene, R, regions1, w_sh, sd_o, level_mask=1, atlas=w_rad1)
    oracle.copy_alpha(w_rad1, w_op1, R, 0)
    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((256, 256), dtype=torch.float32, device="cuda")
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(_origin(), LIGHT_DIR)
    passes.clipmap_frame(ds, CAM, R, op, rad, sh, light, lsd, ws, frame_index=0)
    passes.clipmap_frame(ds, cam1, R, op, rad, sh, light, lsd, ws, frame_index=1)
    torch.cuda.synchronize()
    g_op = op.cpu().numpy().view(np.uint32)
    g_rad = rad.cpu().numpy().view(np.uint32)
    assert np.array_equal(g_op, w_op1), f"opacity: {np.count_nonzero(g_op != w_op1)} texels differ"
    assert np.array_equal(g_rad, w_rad1), f"radiance: {np.count_nonzero(g_rad != w_rad1)} texels differ"
    assert np.count_nonzero(g_rad != w_rad) > 100  # level 0 did change
