"""GPU parity of the clipmap passes and the exact cone tracer against the oracle.

Integer / RGBA8 passes are compared bit for bit.  Traced radiance is compared
with the FP32 mirror (per-sample tolerance, allowing the few samples where a
level or step boundary flips on a last-ulp difference of log2/exp2/tan/pow)
and with the FP64 oracle (relative L2 error <= 1e-2, the bar of the spec)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _to_dev(torch, a):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


def _from_dev(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("R", [16, 32, 64])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("cam", [(0.0, 0.0, 0.0), (3.7, -1.2, 6.4)])
def test_downsample_all_levels_bit_exact(cuda, oracle, R, mode, cam):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import random_atlas
    atlas = random_atlas(R, seed=R + mode, fill=0.4)
    regions = oracle.clip_regions(cam, R)
    want = atlas.copy()
    for level in range(1, 6):
        oracle.downsample(want, R, regions[level - 1, 0:3], level, mode)
    dev = _to_dev(torch, atlas)
    clipmap.cmd_downsample_all(dev, R, clipmap.clip_regions(cam, R), mode)
    torch.cuda.synchronize()
    got = _from_dev(dev)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"
    assert np.count_nonzero(got != atlas) > 0


@pytest.mark.parametrize("R", [16, 64])
def test_clear_copy_alpha_border_bit_exact(cuda, oracle, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import random_atlas
    a = random_atlas(R, seed=11, fill=0.7)
    b = random_atlas(R, seed=12, fill=0.7)
    # clear: a toroidal sub-region that wraps, and a full level
    wa = a.copy()
    oracle.clear_region(wa, R, (R - 3, 5, R // 2), (7, R - 5, R // 2 + 1), 2)
    oracle.clear_region(wa, R, (0, 0, 0), (R, R, R), 4)
    da = _to_dev(torch, a)
    clipmap.cmd_clear_region(da, R, (R - 3, 5, R // 2), (7, R - 5, R // 2 + 1), 2)
    clipmap.cmd_clear_region(da, R, (0, 0, 0), (R, R, R), 4)
    torch.cuda.synchronize()
    assert np.array_equal(_from_dev(da), wa)
    # copy alpha, every level
    wb = b.copy()
    db = _to_dev(torch, b)
    for lvl in range(6):
        oracle.copy_alpha(wb, wa, R, lvl)
        clipmap.cmd_copy_alpha(db, da, R, lvl)
    torch.cuda.synchronize()
    assert np.array_equal(_from_dev(db), wb)
    # border wrap
    oracle.wrap_border(wb, R)
    clipmap.cmd_wrap_border(db, R)
    torch.cuda.synchronize()
    got = _from_dev(db)
    assert np.array_equal(got, wb)
    # index R+1 of every face block is never written (borderWrapping dispatch covers R indices)
    assert np.array_equal(got[R + 1], b[R + 1])


def _trace_setup(oracle, R, n, seed, fill=0.05, spec=0.5):
    from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = trace_desc(**default_trace_desc(regions, R))
    atlas = random_atlas(R, seed=seed, fill=fill)
    for level in range(1, 6):
        oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
    samples = random_samples(n, (0, 0, 0), 6.0, seed=seed + 1, specular_fraction=spec)
    return desc, atlas, samples


@pytest.mark.parametrize("R,n", [(32, 2048), (64, 1024)])
def test_cone_trace_exact_matches_oracle(cuda, oracle, R, n):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    desc, atlas, samples = _trace_setup(oracle, R, n, seed=R)
    eye = (0.5, 1.0, -4.0)
    d32, s32, steps32, wr = oracle.cone_trace(32, bytes(desc), eye, atlas, R, samples)
    d64, s64, steps64, _ = oracle.cone_trace(64, bytes(desc), eye, atlas, R, samples)
    dev_atlas = _to_dev(torch, atlas)
    dev_s = clipmap.samples_to_device(samples)
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    dout, sout = clipmap.cone_trace(desc, eye, dev_atlas, R, dev_s, steps=steps)
    torch.cuda.synchronize()
    dout = dout.cpu().numpy().astype(np.float64)
    sout = sout.cpu().numpy().astype(np.float64)
    assert np.isfinite(dout).all() and np.isfinite(sout).all()
    # FP32 mirror: per-sample agreement, except rare boundary flips
    for got, want in ((dout, d32), (sout, s32)):
        err = np.abs(got - want).max(1) / np.maximum(np.abs(want).max(1), 1e-3)
        assert np.mean(err < 1e-4) > 0.99, np.sort(err)[-10:]
    # FP64 oracle: relative L2 error of traced radiance within 1e-2
    for got, want in ((dout[:, :3], d64[:, :3]), (sout[:, :3], s64[:, :3])):
        rel = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-12)
        assert rel < 1e-2, rel
    gsteps = int(steps.item())
    assert abs(gsteps - steps32) <= max(8, 0.002 * steps32), (gsteps, steps32)


@pytest.mark.parametrize("R", [16, 32, 64])
@pytest.mark.parametrize("cam", [(0.0, 0.0, 0.0), (3.7, -1.2, 6.4), (-9.3, 4.1, -2.2)])
def test_fused_copy_alpha_downsample_equals_the_two_passes(cuda, oracle, R, cam):
    """vct_copy_alpha_downsample (levels 1..5) after vct_copy_alpha (level 0)
    gives the atlas of copy-alpha on every level then the radiance mips, bit
    for bit (the frame's order), including regions that wrap toroidally."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import random_atlas
    rad = random_atlas(R, seed=R + 7, fill=0.4)
    opa = random_atlas(R, seed=R + 8, fill=0.6)
    regions = oracle.clip_regions(cam, R)
    want = rad.copy()
    for level in range(6):
        oracle.copy_alpha(want, opa, R, level)
    for level in range(1, 6):
        oracle.downsample(want, R, regions[level - 1, 0:3], level, 1)
    dev, dopa = _to_dev(torch, rad), _to_dev(torch, opa)
    clipmap.cmd_copy_alpha(dev, dopa, R, 0)
    for level in range(1, 6):
        clipmap.cmd_copy_alpha_downsample(dev, dopa, R, tuple(int(v) for v in regions[level - 1, 0:3]), level)
    torch.cuda.synchronize()
    got = _from_dev(dev)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} texels differ"
