"""Host-side checks of the inverse-fitting driver (no GPU): the target shapes it accepts, and that a loss
without targets is refused before any device call."""
import numpy as np
import pytest
import torch

from vk_voxel_cone_tracing_gb300 import capi, clipmap, fit
from vk_voxel_cone_tracing_gb300.scene import default_trace_desc


def _fit(n=64, R=8):
    regions = np.zeros((6, 7), np.int32)
    regions[:, 3:6] = R
    regions[:, 6] = np.float32(16.0 / R).view(np.int32)
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    cam = clipmap.cam_matrix((0.0, 1.0, -3.0))
    light = capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    samples = torch.zeros((n, 20), dtype=torch.float32)
    return fit.RadianceFit(R, regions, desc, cam, light, samples)


def test_targets_must_match_the_samples():
    f = _fit()
    assert f.param.numel() == 4 * int(capi.lib().vct_atlas_texels(8))
    with pytest.raises(ValueError):
        f.set_targets(torch.zeros((63, 4)), torch.zeros((64, 4)))
    f.set_targets(torch.zeros((64, 4)), torch.zeros((64, 4)))
    assert f.target_d.shape == (64, 4)


def test_loss_without_targets_is_refused():
    f = _fit()
    with pytest.raises(ValueError):
        f._sq_error(grad=True)


def test_downsample_desc_reads_the_finer_level():
    regions = np.arange(42, dtype=np.int32).reshape(6, 7)
    d = fit.downsample_desc(regions, 3, 64)
    assert list(d.prev_region_min_corner) == list(regions[2, 0:3])
    assert (d.clip_level, d.clipmap_resolution, d.downsample_region_size) == (3, 64, capi.DOWNSAMPLE_REGION_SIZE)
