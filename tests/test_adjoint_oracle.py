"""The FP64 reference gradients of the oracle (CPU only).

oracle.cone_trace_grad_f4 and oracle.downsample_chain_grad_f4 differentiate
the oracle's own restatement of the trace (voxelConeTracing.frag:143-392) and
of the mips (radianceDownSample.comp / opacityDownSample.comp) by reverse-mode
automatic differentiation.  Before the GPU adjoints are held to them, they are
checked here against central finite differences of the FP64 oracle: the
difference quotient of the same function, computed without any derivative
code."""
import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import clipmap
from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_samples, smooth_volume


def _fd(loss, vol, k, eps):
    vp, vm = vol.copy(), vol.copy()
    vp.reshape(-1)[k] += eps
    vm.reshape(-1)[k] -= eps
    h = float(vp.reshape(-1)[k]) - float(vm.reshape(-1)[k])
    return (loss(vp) - loss(vm)) / h


@pytest.mark.parametrize("mode", [8, 7, 6])
def test_trace_reference_gradient_matches_central_differences(oracle, mode):
    R, n = 16, 64
    vol = smooth_volume(R, seed=mode)
    regions = oracle.clip_regions((0.2, 1.1, -0.4), R)
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    desc.rendering_mode = mode
    samples = random_samples(n, (0.2, 1.1, -0.4), 3.0, seed=mode + 1, specular_fraction=0.6)
    samples["emission_texel"] = 0.0
    rng = np.random.default_rng(mode)
    wd = rng.normal(size=(n, 4)).astype(np.float32)
    ws = rng.normal(size=(n, 4)).astype(np.float32)
    eye = (0.0, 3.0, -3.0)
    g = oracle.cone_trace_grad_f4(bytes(desc), eye, vol, R, samples, wd, ws)
    assert g.shape == vol.shape and np.count_nonzero(g) > 1000

    def loss(v):
        d, s, _ = oracle.cone_trace_f4(bytes(desc), eye, v, R, samples)
        return float((d * wd).sum() + (s * ws).sum())

    flat = np.abs(g).reshape(-1)
    scale = float(flat.max())
    pick = np.concatenate([np.argsort(flat)[-10:], rng.choice(np.nonzero(flat)[0], 10, replace=False)])
    for k in pick:
        fd = _fd(loss, vol, k, np.float32(1e-3))
        assert abs(fd - g.reshape(-1)[k]) <= 1e-5 * abs(fd) + 1e-7 * scale, (int(k), g.reshape(-1)[k], fd)


@pytest.mark.parametrize("mode", [1, 0])
def test_mip_chain_reference_adjoint_matches_central_differences(oracle, mode):
    R = 8
    regions = oracle.clip_regions((0.7, -0.3, 1.9), R)
    vol = smooth_volume(R, seed=11, max_alpha=0.9)
    rng = np.random.default_rng(mode)
    W = rng.normal(size=vol.shape)
    G = oracle.downsample_chain_grad_f4(vol, R, regions, W, mode)

    def loss(v):
        v = v.copy()
        for level in range(1, 6):
            oracle.downsample_f4(v, R, regions[level - 1, 0:3], level, mode)
        return float((v.astype(np.float64) * W).sum())

    # the border texels feed nothing and are never written: their adjoint is W itself
    assert np.array_equal(G[0], W[0])
    picks = [(int(rng.integers(1, R + 1)), int(rng.integers(1, R + 1)) + lv * (R + 2),
              int(rng.integers(1, R + 1)) + (R + 2) * int(rng.integers(0, 6)), int(rng.integers(0, 4)))
             for lv in (0, 0, 0, 1, 1, 2, 3) for _ in range(3)]
    scale = float(np.abs(G).max())
    for z, y, x, c in picks:
        k = np.ravel_multi_index((z, y, x, c), vol.shape)
        fd = _fd(loss, vol, k, np.float32(1e-2))
        # the oracle chain stores floats between levels: its difference quotient carries about 1e-6 of the
        # largest entry of rounding noise
        assert abs(fd - G[z, y, x, c]) <= 1e-5 * abs(fd) + 4e-6 * scale, ((z, y, x, c), G[z, y, x, c], fd)
