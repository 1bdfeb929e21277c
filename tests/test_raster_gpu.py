"""GPU parity of the rasterisation-driven passes against the oracle.

Opacity voxelisation, shadow depth, deterministic radiance injection and the
SVO fragment list are integer / RGBA8 / float-exact outputs of one pinned
rasteriser and are compared bit for bit.  The atomic injection mode (the
reference's CAS loop, order-dependent) is compared statistically."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAM = (0.35, 2.1, -0.7)
LIGHT_DIR = (0.3, -1.0, 0.2)


def _light_origin(center, d=LIGHT_DIR, dist=15.0):
    d = np.asarray(d, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - dist * d).astype(np.float32).tolist())


@pytest.fixture(scope="module")
def scene():
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    return room_scene(seed=1, n_random=3000)


@pytest.fixture(scope="module")
def dscene(cuda, scene):
    from vk_voxel_cone_tracing_gb300.passes import DeviceScene
    return DeviceScene(scene)


@pytest.fixture(scope="module")
def ws(cuda):
    from vk_voxel_cone_tracing_gb300.passes import Workspace
    return Workspace()


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("R", [32, 64])
def test_voxelize_opacity_bit_exact(cuda, oracle, scene, dscene, ws, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    want = oracle.voxelize_opacity(scene, R, oracle.clip_regions(CAM, R))
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity(dscene, clipmap.clip_regions(CAM, R), R, atlas, ws)
    torch.cuda.synchronize()
    got = _u32(atlas)
    assert np.count_nonzero(want) > 1000
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"


def test_shadow_depth_bit_exact(cuda, oracle, scene, dscene, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import passes
    origin = _light_origin((0.0, 4.0, 0.0))
    sd_o = oracle.light_shadow_desc(origin, LIGHT_DIR)
    want = oracle.shadow_depth(scene, sd_o, 512, 512)
    sd = passes.light_shadow_desc(origin, LIGHT_DIR)
    assert bytes(sd) == sd_o
    depth = torch.empty((512, 512), dtype=torch.float32, device="cuda")
    passes.shadow_depth(dscene, sd, depth, ws)
    torch.cuda.synchronize()
    got = depth.cpu().numpy()
    assert (want < 1.0).sum() > 10000
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("R", [32, 64])
def test_inject_radiance_deterministic_bit_exact(cuda, oracle, scene, dscene, ws, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    origin = _light_origin((0.0, 4.0, 0.0))
    sd_o = oracle.light_shadow_desc(origin, LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd_o, 256, 256)
    want = oracle.inject_radiance(scene, R, oracle.clip_regions(CAM, R), shadow, sd_o)
    sd = passes.light_shadow_desc(origin, LIGHT_DIR)
    dshadow = torch.from_numpy(shadow).cuda()
    atlas = clipmap.new_atlas(R)
    passes.inject_radiance(dscene, clipmap.clip_regions(CAM, R), R, dshadow, passes.light_desc(LIGHT_DIR), sd, atlas,
                           ws, mode=capi.INJECT_DETERMINISTIC)
    torch.cuda.synchronize()
    got = _u32(atlas)
    assert np.count_nonzero(want) > 1000
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"
    # the atomic (reference CAS-loop) mode touches exactly the same texels; its
    # running averages differ only where the fold order differs
    atom = clipmap.new_atlas(R)
    passes.inject_radiance(dscene, clipmap.clip_regions(CAM, R), R, dshadow, passes.light_desc(LIGHT_DIR), sd, atom,
                           ws, mode=capi.INJECT_ATOMIC)
    torch.cuda.synchronize()
    a = _u32(atom)
    assert np.array_equal(a != 0, want != 0)
    nz = want != 0
    same = np.mean(a[nz] == want[nz])
    diff = np.abs((a[nz][:, None] >> np.array([0, 8, 16, 24], np.uint32)) & 0xFF).astype(int) - \
        ((want[nz][:, None] >> np.array([0, 8, 16, 24], np.uint32)) & 0xFF).astype(int)
    assert same > 0.5, same
    # the alpha channel is the fragment count (mod 256): order-independent
    assert (diff[:, 3] == 0).all()


def test_inject_long_runs_into_prefilled_atlas_bit_exact(cuda, oracle):
    """400 stacked quads inside one level-0 voxel layer put about 800 face
    records on most texels they touch (far past the 256-step alpha wrap of the
    running average), and the atlas starts from random texels (random alpha
    counters), so the per-texel fold meets every starting phase."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import _pack
    R = 32
    rng = np.random.default_rng(5)
    quads = []
    for i in range(400):
        x = np.float32(-2.0 + 0.001 * i)
        a, b, c, d = [x, -4, -6], [x, 8, -6], [x, 8, 6], [x, -4, 6]
        quads += [[a, c, b], [a, d, c]]
    stack = _pack(np.array(quads, np.float32), rng)
    dstack = passes.DeviceScene(stack)
    ws = passes.Workspace()
    regions = oracle.clip_regions(CAM, R)
    start = rng.integers(0, 2 ** 32, size=(R + 2, 6 * (R + 2), 6 * (R + 2)), dtype=np.uint64).astype(np.uint32)
    want = oracle.inject_radiance(stack, R, regions, None, bytes(capi.DirectionalLightShadowDesc()),
                                  atlas=start.copy())
    atlas = torch.from_numpy(start.view(np.int32).copy()).cuda()
    passes.inject_radiance(dstack, clipmap.clip_regions(CAM, R), R, None, passes.light_desc(LIGHT_DIR),
                           capi.DirectionalLightShadowDesc(), atlas, ws, mode=capi.INJECT_DETERMINISTIC)
    torch.cuda.synchronize()
    got = _u32(atlas)
    assert np.count_nonzero(want != start) > 1000
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"
    # from a zero atlas the alpha byte is the record count mod 256: 800 -> 32
    zero = oracle.inject_radiance(stack, R, regions, None, bytes(capi.DirectionalLightShadowDesc()))
    assert np.count_nonzero(((zero >> 24) & 0xFF) == 32) > 1000


def test_svo_fragments_bit_exact(cuda, oracle, scene, dscene, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import passes
    origin = _light_origin((0.0, 4.0, 0.0))
    sd_o = oracle.light_shadow_desc(origin, LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd_o, 256, 256)
    bmin, bmax = dscene.bb_min, dscene.bb_max
    want, n = oracle.svo_fragments(scene, 6, bmin, bmax, shadow, sd_o)
    frags = passes.svo_fragments(dscene, 6, torch.from_numpy(shadow).cuda(), passes.light_desc(LIGHT_DIR),
                                 passes.light_shadow_desc(origin, LIGHT_DIR), ws)
    torch.cuda.synchronize()
    got = frags.cpu().numpy().view(np.uint32)
    assert n > 1000 and got.shape[0] == n
    assert np.array_equal(got, want)
