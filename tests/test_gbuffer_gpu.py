"""GPU parity of the G-buffer producer (vct_gbuffer) against the oracle.

Visibility (closest centre sample, earlier triangle on ties), the clipped
sub-triangles, the perspective-correct attributes and the attachment texels are
all FP32 arithmetic of one pinned order, so every field of every record is
compared bit for bit -- except the emission of a material with an emission
texture, whose pow(texel, 2.2) is the device's powf against the host's
(documented within 2 ulp) and is compared to one RGBA16F step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ws(cuda):
    from vk_voxel_cone_tracing_gb300.passes import Workspace
    return Workspace()


def _run(cuda, sc, cam, W, H, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    ds = passes.DeviceScene(sc)
    c = capi.CamMatrix.from_buffer_copy(np.ascontiguousarray(cam, np.float32).tobytes())
    out = passes.gbuffer(ds, c, W, H, ws)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _compare(got, want, emission_tol=False):
    assert got.shape == want.shape
    exact = np.ones(20, bool)
    if emission_tol:
        exact[16:19] = False
    g, w = got[:, exact].view(np.uint32), want[:, exact].view(np.uint32)
    bad = np.nonzero((g != w).any(1))[0]
    assert bad.size == 0, f"{bad.size} pixels differ, first {bad[:5]}: {got[bad[0]]} vs {want[bad[0]]}"
    if emission_tol:
        e_g, e_w = got[:, 16:19], want[:, 16:19]
        assert np.all(np.abs(e_g - e_w) <= np.maximum(np.abs(e_w), 6.1e-5) * 2.0 ** -10)


@pytest.mark.parametrize("W,H,pos,dirn", [
    (160, 96, (0.3, 2.0, -4.0), (0.2, -0.1, 1.0)),
    (203, 117, (-6.0, 7.5, 3.0), (0.9, -0.5, -0.4)),   # odd size, looking down into the room
    (128, 128, (9.7, 0.2, 4.6), (-1.0, 0.05, -0.6)),   # close to a wall: triangles cross the near plane
])
def test_room_scene_bit_exact(cuda, oracle, ws, W, H, pos, dirn):
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    sc = room_scene(seed=1, n_random=3000)
    cam = oracle.camera_matrix(pos, dirn, aspect=W / H)
    want = oracle.gbuffer(sc, cam, W, H)
    got = _run(cuda, sc, cam, W, H, ws)
    assert (want[:, 3] < 1.0).mean() > 0.9
    _compare(got, want)


def test_floor_through_the_near_plane_bit_exact(cuda, oracle, ws):
    from tests.test_gbuffer_oracle import _floor, _quads_scene
    sc = _quads_scene([_floor(half=50.0)], [0xFFFFFFFF])
    cam = oracle.camera_matrix((0.0, 1.0, 0.0), (0.0, -1.0, 0.6), aspect=1.5)
    want = oracle.gbuffer(sc, cam, 96, 64)
    _compare(_run(cuda, sc, cam, 96, 64, ws), want)


def test_materials_discard_and_ties_bit_exact(cuda, oracle, ws):
    from tests.test_gbuffer_oracle import _quads_scene, _wall
    from vk_voxel_cone_tracing_gb300.scene import _materials_for
    tex = np.asarray([0x20FFFFFF, 0xFF4080C0, 0xFFC08040, 0xFF80FF00, 0xFF00FFFF], np.uint32)
    m = _materials_for(tex)
    m["alpha_mode"][0] = 1
    m["alpha_cutoff"][0] = 0.5
    m["pbr_metallic_factor"] = (0.0, 0.3, 0.9, 0.5, 0.0)
    m["pbr_roughness_factor"] = (1.0, 0.01, 0.6, 0.2, 0.5)
    m["pbr_metallic_roughness_texture"][3] = 4
    m["emissive_factor"][2] = (0.5, 2.0, 0.25)
    m["emissive_texture"][2] = 3
    quads = [_wall(0.0, 1.0), _wall(0.5, 1.5), _wall(0.5, 2.0), _wall(1.0, 3.0), _wall(2.0, 4.0)]
    sc = _quads_scene(quads, tex, m)
    cam = oracle.camera_matrix((0.3, -0.2, -5.0), (0.05, 0.02, 1.0), aspect=1.25)
    want = oracle.gbuffer(sc, cam, 120, 96)
    got = _run(cuda, sc, cam, 120, 96, ws)
    _compare(got, want, emission_tol=True)
    assert (np.abs(want[:, 16:19]).sum(1) > 0).any()


def test_hall_scene_bit_exact(cuda, oracle, ws):
    from vk_voxel_cone_tracing_gb300.scene import hall_scene
    sc = hall_scene(seed=2, target=60_000)
    cam = oracle.camera_matrix((1.0, 4.0, -20.0), (0.1, -0.15, 1.0), aspect=16 / 9)
    want = oracle.gbuffer(sc, cam, 256, 144)
    _compare(_run(cuda, sc, cam, 256, 144, ws), want)


def test_empty_and_bad_arguments(cuda, oracle, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    from tests.test_gbuffer_oracle import _quads_scene, _wall
    sc = _quads_scene([_wall(0.0)], [0xFFFFFFFF])
    ds = passes.DeviceScene(sc)
    cam = passes.camera_matrix((0.0, 0.0, 5.0), (0.0, 0.0, 1.0), aspect=1.0)  # the wall is behind the camera
    out = passes.gbuffer(ds, cam, 32, 32, ws)
    torch.cuda.synchronize()
    g = out.cpu().numpy()
    assert (g[:, 3] == 1.0).all()
    want = oracle.gbuffer(sc, np.frombuffer(bytes(cam), np.float32), 32, 32)
    _compare(g, want)
    with pytest.raises(capi.VctError):
        passes.gbuffer(ds, cam, 0, 32, ws)
    with pytest.raises(ValueError):
        passes.gbuffer(ds, cam, 32, 32, ws, out=torch.empty((10, 20), device="cuda"))


@pytest.mark.parametrize("seed", range(6))
def test_random_cameras_bit_exact(cuda, oracle, ws, seed):
    """Random cameras in and around the room (random field of view, aspect and odd image sizes): every
    record equal to the oracle's."""
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    rng = np.random.default_rng(100 + seed)
    sc = room_scene(seed=seed % 3, n_random=1500)
    W, H = int(rng.integers(40, 200)), int(rng.integers(30, 150))
    pos = rng.uniform([-14, -3, -9], [14, 12, 9]).astype(np.float32)
    d = rng.normal(size=3).astype(np.float32)
    d[1] *= 0.4
    cam = oracle.camera_matrix(tuple(pos.tolist()), tuple(d.tolist()), fovy_degrees=float(rng.uniform(30, 100)),
                               aspect=float(W) / H)
    want = oracle.gbuffer(sc, cam, W, H)
    _compare(_run(cuda, sc, cam, W, H, ws), want)
