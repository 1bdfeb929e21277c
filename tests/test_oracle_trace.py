"""Self-consistency of the cone-tracing oracle (CPU only).

The reference ships no tests or golden outputs for this path, so the oracle is
checked (a) against analytic cases of voxelConeTracing.frag's arithmetic and
(b) FP32 mirror against FP64, with the tolerance the build targets."""
import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import capi
from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples

R = 32


@pytest.fixture(scope="module")
def setup(oracle):
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = trace_desc(**default_trace_desc(regions, R))
    return regions, bytes(desc)


def test_empty_volume_gives_full_visibility(oracle, setup):
    """Empty clipmap: every cone returns (0,0,0, 1-occlusion=1).  The accumulator starts at
    vec4(0,0,0,1) (voxelConeTracing.frag:170), so indirect.a = (1 + sum(cos+)) / 16 * AO factor."""
    regions, desc = setup
    atlas = np.zeros((R + 2, 6 * (R + 2), 6 * (R + 2)), np.uint32)
    s = random_samples(64, (0, 0, 0), 1.0, seed=3, specular_fraction=0.0)
    s["emission_texel"] = 0
    d = trace_desc(**{**default_trace_desc(regions, R), "rendering_mode": 7})
    dout, sout, steps, wr = oracle.cone_trace(64, bytes(d), (0, 0, -3), atlas, R, s)
    assert wr.all() and steps > 0
    n = (s["normal_texel"].astype(np.float64) * 2 - 1)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    from oracle.clipmap_oracle_tables import DIRS16
    cos = n @ DIRS16.T
    expect = (1.0 + np.where(cos >= 0, cos, 0).sum(1)) / 16 * 0.5
    np.testing.assert_allclose(dout[:, 0], expect, rtol=1e-6, atol=1e-7)


def test_opaque_volume_occludes(oracle, setup):
    """Fully opaque clipmap: every diffuse cone saturates, so AO is far below the empty-volume value."""
    regions, desc = setup
    atlas = np.full((R + 2, 6 * (R + 2), 6 * (R + 2)), 0xFF808080, np.uint32)
    s = random_samples(32, (0, 0, 0), 1.0, seed=4, specular_fraction=0.0)
    d = trace_desc(**{**default_trace_desc(regions, R), "rendering_mode": 7})
    dout, _, steps, _ = oracle.cone_trace(64, bytes(d), (0, 0, -3), atlas, R, s)
    assert (dout[:, 0] < 0.2).all()


def test_fp32_mirror_matches_fp64(oracle, setup):
    regions, desc = setup
    atlas = random_atlas(R, seed=5, fill=0.05)
    s = random_samples(256, (0, 0, 0), 3.0, seed=6)
    d32, s32, st32, _ = oracle.cone_trace(32, desc, (0.5, 1.0, -4.0), atlas, R, s)
    d64, s64, st64, _ = oracle.cone_trace(64, desc, (0.5, 1.0, -4.0), atlas, R, s)
    for a, b in ((d32, d64), (s32, s64)):
        rel = np.linalg.norm(a[:, :3] - b[:, :3]) / max(np.linalg.norm(b[:, :3]), 1e-12)
        assert rel < 1e-3, rel
    assert abs(st32 - st64) <= 0.01 * st64
