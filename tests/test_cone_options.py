"""The diffuse-aperture option of the trace (vct_trace_options; no
counterpart in the reference, whose shader fixes the aperture constants of
its cone tables): the oracle side, CPU only.  Configuration 1 of the
benchmark set asks for 16 fixed 30-degree cones; the shader's 16-cone set
uses 0.872665 rad (50 degrees)."""
import math

import numpy as np

from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples

R = 16


def _case(oracle):
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = bytes(trace_desc(**default_trace_desc(regions, R)))
    atlas = random_atlas(R, seed=3, fill=0.1)
    samples = random_samples(300, (0, 0, 0), 3.0, seed=4)
    return desc, atlas, samples


def test_the_shaders_aperture_is_the_default(oracle):
    desc, atlas, samples = _case(oracle)
    eye = (0.0, 1.0, -4.0)
    a = oracle.cone_trace(32, desc, eye, atlas, R, samples)
    b = oracle.cone_trace(32, desc, eye, atlas, R, samples, diffuse_aperture=0.872665)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


def test_thirty_degree_cones_march_more_steps(oracle):
    desc, atlas, samples = _case(oracle)
    eye = (0.0, 1.0, -4.0)
    wide = oracle.cone_trace(64, desc, eye, atlas, R, samples)
    narrow = oracle.cone_trace(64, desc, eye, atlas, R, samples, diffuse_aperture=math.radians(30.0))
    # a narrower cone grows its steps by 1 + 2 tan(15 deg) instead of 1 + 2 tan(25 deg): more of them
    assert narrow[2] > wide[2]
    assert not np.allclose(narrow[0][:, :3], wide[0][:, :3])
    # the specular cone does not depend on the diffuse aperture
    assert np.array_equal(narrow[1], wide[1])
