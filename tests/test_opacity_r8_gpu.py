"""The one-byte opacity form of a frame (vct_frame_desc.opacity_format =
VCT_OPACITY_R8): the frame with an R8 opacity atlas against the same frame
with the reference's RGBA8 atlas (Voxelizer.cpp:159), which the frame tests
hold bit-exact to the oracle.  The radiance atlas and its texture must be
equal bit for bit, and every R8 opacity byte must equal the alpha byte of
the RGBA8 atlas (the byte copy-alpha, the mips and the border wrap read)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)


def _origin(center=(0.0, 4.0, 0.0), dist=15.0):
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - dist * d).astype(np.float32).tolist())


@pytest.mark.parametrize("R,scene_kind,cam", [(32, "room", (0.35, 2.1, -0.7)), (64, "room", (1.2, 3.0, 0.4)),
                                              (128, "hall", (0.0, 5.0, 0.0))])
def test_r8_opacity_frame_equals_rgba8(cuda, R, scene_kind, cam):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import hall_scene, room_scene
    scene = room_scene(seed=1, n_random=3000) if scene_kind == "room" else hall_scene(seed=2, target=200000)
    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(_origin(), LIGHT_DIR)
    sh = torch.empty((512, 512), dtype=torch.float32, device="cuda")
    out = {}
    for fmt in (capi.OPACITY_RGBA8, capi.OPACITY_R8):
        op = clipmap.new_atlas(R) if fmt == capi.OPACITY_RGBA8 else clipmap.new_atlas_r8(R)
        op.fill_(0x5A)  # stale contents: the frame's clear must cover every texel
        rad = clipmap.new_atlas(R)
        tex = clipmap.RadianceTexture(R)
        for frame_index in (0, 1, 2):  # all levels due, then the cadence's partial refreshes
            passes.clipmap_frame(ds, cam, R, op, rad, sh, light, lsd, ws, frame_index=frame_index, texture=tex,
                                 opacity_format=fmt)
        back = tex.read(clipmap.new_atlas(R))
        torch.cuda.synchronize()
        out[fmt] = (op.cpu().numpy(), rad.cpu().numpy(), back.cpu().numpy())
        tex.close()
    op32, rad32, tex32 = out[capi.OPACITY_RGBA8]
    op8, rad8, tex8 = out[capi.OPACITY_R8]
    assert np.array_equal(op8, (op32.view(np.uint32) >> 24).astype(np.uint8))
    assert np.array_equal(rad8, rad32) and np.array_equal(tex8, tex32)
    assert np.count_nonzero(rad32.view(np.uint32) >> 24) > 1000


def test_r8_opacity_rejects_toroidal_and_atomic(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    R = 32
    ds = passes.DeviceScene(room_scene(seed=1, n_random=500))
    ws = passes.Workspace()
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(_origin(), LIGHT_DIR)
    op, rad = clipmap.new_atlas_r8(R), clipmap.new_atlas(R)
    sh = torch.empty((128, 128), dtype=torch.float32, device="cuda")
    state = (capi.ClipmapRegion * 6)()
    with pytest.raises(capi.VctError, match="R8 opacity"):
        passes.clipmap_frame(ds, (0.0, 1.0, 0.0), R, op, rad, sh, light, lsd, ws, revoxelization=capi.REVOX_TOROIDAL,
                             regions_state=state, opacity_format=capi.OPACITY_R8)
    with pytest.raises(capi.VctError, match="R8 opacity"):
        passes.clipmap_frame(ds, (0.0, 1.0, 0.0), R, op, rad, sh, light, lsd, ws, inject_mode=capi.INJECT_ATOMIC,
                             opacity_format=capi.OPACITY_R8)
