"""GPU parity of the sparse-voxel-octree build against the oracle.

The deterministic build (scan allocation in breadth-first order, leaf colours
folded in fragment order) is compared bit for bit with the oracle's
restatement of the six node shaders.  The atomic build (the reference's racy
atomicAdd allocation and CAS loops) is canonicalised and must then have the
same structure and mips of the same structure; leaf colours may differ only
where several fragments average into one leaf in another order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)


@pytest.fixture(scope="module")
def setup(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    scene = room_scene(seed=3, n_random=3000)
    d = np.array(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    origin = tuple((np.array([0.0, 4.0, 0.0]) - 15.0 * d).astype(np.float32).tolist())
    sd_o = oracle.light_shadow_desc(origin, LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd_o, 256, 256)
    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    return scene, ds, ws, origin, sd_o, shadow


@pytest.mark.parametrize("level", [5, 7])
def test_svo_build_deterministic_bit_exact(cuda, oracle, setup, level):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    scene, ds, ws, origin, sd_o, shadow = setup
    frags_np, F = oracle.svo_fragments(scene, level, ds.bb_min, ds.bb_max, shadow, sd_o)
    want, n_want = oracle.svo_build(frags_np, level)
    frags = torch.from_numpy(frags_np.view(np.int32).copy()).cuda()
    pool, n = passes.svo_build(frags, level, ws, mode=capi.SVO_DETERMINISTIC)
    torch.cuda.synchronize()
    assert n == n_want and n > 64
    got = pool[:n].cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} words differ"
    # canonicalising a breadth-first pool is the identity
    canon = passes.svo_canonicalize(pool, n, level, ws)
    torch.cuda.synchronize()
    assert np.array_equal(canon.cpu().numpy().view(np.uint32), want)


def test_svo_build_atomic_canonicalises_to_deterministic(cuda, oracle, setup):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    scene, ds, ws, origin, sd_o, shadow = setup
    level = 7
    frags_np, F = oracle.svo_fragments(scene, level, ds.bb_min, ds.bb_max, shadow, sd_o)
    want, n_want = oracle.svo_build(frags_np, level)
    frags = torch.from_numpy(frags_np.view(np.int32).copy()).cuda()
    pool, n = passes.svo_build(frags, level, ws, mode=capi.SVO_ATOMIC)
    canon = passes.svo_canonicalize(pool, n, level, ws)
    torch.cuda.synchronize()
    assert n == n_want
    c = canon.cpu().numpy().view(np.uint32)
    assert np.array_equal(c[:, 0], want[:, 0]), "node structure differs after canonicalisation"
    same = np.mean(c[:, 1] == want[:, 1])
    assert same > 0.9, same


def test_svo_overflow_is_reported(cuda, oracle, setup):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    scene, ds, ws, origin, sd_o, shadow = setup
    frags_np, F = oracle.svo_fragments(scene, 7, ds.bb_min, ds.bb_max, shadow, sd_o)
    frags = torch.from_numpy(frags_np.view(np.int32).copy()).cuda()
    with pytest.raises(capi.VctError) as e:
        passes.svo_build(frags, 7, ws, capacity=64)
    assert e.value.code == capi.VCT_E_OVERFLOW


def test_svo_cone_trace_matches_oracle(cuda, oracle, setup):
    """voxelConeTracing_Octree.frag over the deterministic pool of the room scene at level 8
    (volume dimension 256, the pass's value); the scene box is the room's own."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_samples
    scene, ds, ws, origin, sd_o, shadow = setup
    level = 8
    frags_np, F = oracle.svo_fragments(scene, level, ds.bb_min, ds.bb_max, shadow, sd_o)
    pool_np, n = oracle.svo_build(frags_np, level)
    regions = oracle.clip_regions((0.3, 2.0, -0.5), 128)
    kw = default_trace_desc(regions, 128)
    kw.update(volume_dimension=256.0, indirect_diffuse_intensity=15.0, occlusion_decay=3.0)
    desc = clipmap.trace_desc(**kw)
    samples = random_samples(1500, (0.0, 3.0, 0.0), 4.0, seed=31)
    eye = (0.0, 3.0, -4.0)
    bmin, bmax = tuple(ds.bb_min.tolist()), tuple(ds.bb_max.tolist())
    d32, s32, st32 = oracle.svo_trace(32, bytes(desc), eye, pool_np, samples, bmin, bmax)
    d64, s64, st64 = oracle.svo_trace(64, bytes(desc), eye, pool_np, samples, bmin, bmax)
    pool = torch.from_numpy(pool_np.view(np.int32).copy()).cuda()
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    d, s = passes.svo_cone_trace(desc, eye, pool, n, clipmap.samples_to_device(samples), bmin, bmax, steps=steps)
    torch.cuda.synchronize()
    d = d.cpu().numpy().astype(np.float64)
    s = s.cpu().numpy().astype(np.float64)
    for got, want in ((d, d32), (s, s32)):
        err = np.abs(got - want).max(1) / np.maximum(np.abs(want).max(1), 1e-3)
        assert np.mean(err < 1e-4) > 0.99, np.sort(err)[-8:]
    for got, want in ((d[:, :3], d64[:, :3]), (s[:, :3], s64[:, :3])):
        assert np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-12) < 1e-2
    assert abs(int(steps.item()) - st32) <= max(8, 0.002 * st32)


def test_fragment_list_into_a_given_buffer(cuda, setup):
    """svo_fragments(out=...) writes the list in one call when the buffer is
    large enough, and repeats into a new buffer when it is too small; both
    equal the two-step (count, then write) list bit for bit."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import passes
    scene, ds, ws, origin, sd_o, shadow = setup
    sh = torch.from_numpy(shadow).cuda()
    light, sd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(origin, LIGHT_DIR)
    want = passes.svo_fragments(ds, 6, sh, light, sd, ws).cpu().numpy()
    big = torch.full((want.shape[0] + 100, 2), -1, dtype=torch.int32, device="cuda")
    got = passes.svo_fragments(ds, 6, sh, light, sd, ws, out=big)
    assert got.data_ptr() == big.data_ptr() and np.array_equal(got.cpu().numpy(), want)
    small = torch.empty((want.shape[0] // 2, 2), dtype=torch.int32, device="cuda")
    got2 = passes.svo_fragments(ds, 6, sh, light, sd, ws, out=small)
    assert np.array_equal(got2.cpu().numpy(), want)


def test_terrain_level9_chain_bit_exact(cuda, oracle):
    """The large-octree workload's scene (gradient-noise terrain + boxes) at its level 9 (512^3), reduced to
    about 40k triangles: the fragment list and the deterministic build equal the oracle's word for word, and
    the octree trace over the built pool follows the oracle's FP32 mirror."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, surface_samples, terrain_scene
    scene = terrain_scene(seed=3, target=40000, boxes=250)
    ds, ws = passes.DeviceScene(scene), passes.Workspace()
    d = np.array(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    origin = tuple((np.array([0.0, 1.5, 0.0]) - 15.0 * d).astype(np.float32).tolist())
    sd_o = oracle.light_shadow_desc(origin, LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd_o, 512, 512)
    level = 9
    want_f, F = oracle.svo_fragments(scene, level, ds.bb_min, ds.bb_max, shadow, sd_o)
    frags = passes.svo_fragments(ds, level, torch.from_numpy(shadow).cuda(), passes.light_desc(LIGHT_DIR),
                                 passes.light_shadow_desc(origin, LIGHT_DIR), ws)
    torch.cuda.synchronize()
    assert F > 500000 and frags.shape[0] == F
    assert np.array_equal(frags.cpu().numpy().view(np.uint32), want_f)
    want, n_want = oracle.svo_build(want_f, level)
    pool, n = passes.svo_build(frags, level, ws, mode=capi.SVO_DETERMINISTIC)
    torch.cuda.synchronize()
    assert n == n_want
    assert np.array_equal(pool[:n].cpu().numpy().view(np.uint32), want)
    # the trace over the octree: the scene's own box, volume dimension 512
    regions = oracle.clip_regions((0.0, 3.0, 0.0), 512)
    desc = clipmap.trace_desc(**default_trace_desc(regions, 512))
    samples = surface_samples(scene, 1024, seed=3)
    eye = (0.0, 6.0, -20.0)
    bmin, bmax = tuple(ds.bb_min.tolist()), tuple(ds.bb_max.tolist())
    d32, s32, st32 = oracle.svo_trace(32, bytes(desc), eye, want, samples, bmin, bmax)
    dg, sg = passes.svo_cone_trace(desc, eye, pool, n, clipmap.samples_to_device(samples), bmin, bmax)
    torch.cuda.synchronize()
    for got, ref in ((dg.cpu().numpy().astype(np.float64), d32), (sg.cpu().numpy().astype(np.float64), s32)):
        err = np.abs(got - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-3)
        assert np.mean(err < 1e-4) > 0.99, np.sort(err)[-8:]
    assert np.abs(d32[:, :3]).sum() > 0
