"""Pins the oracle to the reference: golden vectors produced from the
reference's own vendored glm (with the reference's defines) and constants
parsed from its shader source by tests/golden/make_golden.py.  CPU only."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _f(bits):
    return np.array(bits, dtype=np.uint32).view(np.float32)


@pytest.fixture(scope="module")
def host_math():
    return json.loads((GOLDEN / "glm_host_math.json").read_text())


def test_clip_regions_bit_exact(oracle, host_math):
    seen = 0
    for rec in host_math["regions"]:
        cam = _f(rec["cam"])
        regions = oracle.clip_regions(cam, rec["R"])
        lvl = rec["level"]
        assert list(regions[lvl, 0:3]) == rec["min_corner"], rec
        assert regions[lvl, 6:7].view(np.uint32)[0] == rec["voxel_size"]
        seen += 1
    assert seen == 4 * 3 * 6


def test_voxelizer_view_proj_bit_exact(oracle, host_math):
    for rec in host_math["regions"]:
        regions = oracle.clip_regions(_f(rec["cam"]), rec["R"])
        vp = oracle.voxel_view_proj(regions[rec["level"]])
        want = np.array(rec["view_proj"], np.uint32).reshape(3, 16)
        assert np.array_equal(vp.view(np.uint32), want), rec["level"]


def test_library_clip_regions_match_golden(vct_lib, host_math):
    from vk_voxel_cone_tracing_gb300.clipmap import clip_regions, regions_to_numpy
    for rec in host_math["regions"][::6]:
        got = regions_to_numpy(clip_regions(_f(rec["cam"]).tolist(), rec["R"]))
        assert list(got[0, 0:3]) == rec["min_corner"]


def test_light_matrices_bit_exact(oracle, host_math):
    for rec in host_math["lights"]:
        sd = np.frombuffer(oracle.light_shadow_desc(_f(rec["origin"]), _f(rec["direction"])), np.float32)
        assert np.array_equal(sd[0:16].view(np.uint32), np.array(rec["view"], np.uint32))
        assert np.array_equal(sd[16:32].view(np.uint32), np.array(rec["proj"], np.uint32))


def test_cone_tables_match_shader():
    from oracle.clipmap_oracle_tables import APERTURE16, APERTURE32, DIRS16
    t = json.loads((GOLDEN / "cone_tables.json").read_text())
    assert np.array_equal(np.array(t["DIFFUSE_CONE_DIRECTIONS_16"], np.float32).astype(np.float64), DIRS16)
    assert len(t["DIFFUSE_CONE_DIRECTIONS_32"]) == 32
    assert np.float32(t["DIFFUSE_CONE_APERTURE_16"]) == np.float32(APERTURE16)
    assert np.float32(t["DIFFUSE_CONE_APERTURE_32"]) == np.float32(APERTURE32)
    # the C++ oracle and the CUDA constant tables carry the same literals
    src = (Path(__file__).resolve().parents[1] / "oracle" / "clipmap_oracle.hpp").read_text()
    cu = (Path(__file__).resolve().parents[1] / "vk_voxel_cone_tracing_gb300" / "csrc" / "trace_common.cuh").read_text()
    for d in t["DIFFUSE_CONE_DIRECTIONS_32"] + t["DIFFUSE_CONE_DIRECTIONS_16"]:
        lit = "{" + ", ".join(f"{x:g}f" for x in d) + "}"
        assert lit.replace(" ", "") in src.replace(" ", ""), lit
        assert lit.replace(" ", "") in cu.replace(" ", ""), lit
    assert t["MAX_TRACE_DISTANCE"] == 30.0 and t["MIN_TRACE_STEP_FACTOR"] == 0.2


def _cam_inputs(rec):
    v = _f(rec["in"])
    return v[0:3], v[3:6], v[6:9], float(v[9]), float(v[10])


def test_camera_matrix_bit_exact(oracle, host_math):
    """Camera::updateCamera: perspective, lookAt and glm::inverse against glm itself."""
    assert len(host_math["cameras"]) == 4
    for rec in host_math["cameras"]:
        pos, d, up, fovy, aspect = _cam_inputs(rec)
        cam = oracle.camera_matrix(pos, d, up, fovy, aspect)
        assert np.array_equal(cam[0:16].view(np.uint32), np.array(rec["view_proj"], np.uint32))
        assert np.array_equal(cam[16:32].view(np.uint32), np.array(rec["view_proj_inv"], np.uint32))
        assert np.array_equal(cam[32:35], pos)


def test_inverse4_bit_exact(oracle, host_math):
    """glm::inverse restated: the view and projection inverses, entry by entry."""
    for rec in host_math["cameras"]:
        for m, inv in (("view", "view_inv"), ("proj", "proj_inv")):
            src = np.array(rec[m], np.uint32).view(np.float32)
            got = oracle.inverse4(src)
            assert np.array_equal(got.view(np.uint32), np.array(rec[inv], np.uint32)), m
