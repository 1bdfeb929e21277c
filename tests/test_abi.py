"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol include/vct_capi.h declares, the ctypes structs match the header's
byte layouts, host-side entry points agree with the oracle, and bad
arguments are rejected before any device work is enqueued."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import capi
from vk_voxel_cone_tracing_gb300.scene import MATERIAL_DTYPE, SAMPLE_DTYPE

from .conftest import ROOT


def test_library_exports_every_declared_symbol(vct_lib):
    declared = capi.declared_symbols()
    assert "vct_cone_trace" in declared and "vct_downsample" in declared
    missing = [s for s in declared if not hasattr(vct_lib, s)]
    assert not missing, f"symbols declared in vct_capi.h but not exported: {missing}"
    nm = subprocess.run(["nm", "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True, text=True).stdout
    for s in declared:
        assert f" {s}" in nm


def test_bindings_cover_header():
    declared = set(capi.declared_symbols())
    assert declared == set(capi._SIGS), declared ^ set(capi._SIGS)


def test_struct_sizes_match_header():
    for cls, size in capi.STRUCT_SIZES.items():
        assert C.sizeof(cls) == size, cls.__name__
    assert SAMPLE_DTYPE.itemsize == 80 and MATERIAL_DTYPE.itemsize == 80


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "vct_capi.h"\nint main(void){return 0;}\n')
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-fsyntax-only", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_version_and_texels(vct_lib):
    assert b"sm_103a" in vct_lib.vct_version()
    assert vct_lib.vct_atlas_texels(128) == 130 * 6 * 130 * 6 * 130
    assert vct_lib.vct_atlas_texels(100) == -1


@pytest.mark.parametrize("cam", [(0, 0, 0), (1.3, 2.7, -5.1), (-40.2, 3.3, 17.9)])
@pytest.mark.parametrize("R", [64, 128, 256])
def test_clip_regions_match_oracle(vct_lib, oracle, cam, R):
    from vk_voxel_cone_tracing_gb300.clipmap import clip_regions, regions_to_numpy
    got = regions_to_numpy(clip_regions(cam, R))
    want = oracle.clip_regions(cam, R)
    assert np.array_equal(got, want)
    # camera at the origin: every level is centred, min corner -R/2
    if cam == (0, 0, 0):
        assert (got[:, 0:3] == -(R // 2)).all()


def test_bad_arguments_rejected_without_gpu(vct_lib):
    d = capi.DownSampleDesc(capi.i3(0, 0, 0), 0, 128, 10)  # level 0 is invalid
    rc = vct_lib.vct_downsample(C.c_void_p(16), capi.ref(d), 0, None)
    assert rc == capi.VCT_E_BAD_ARG
    assert b"clip level" in vct_lib.vct_last_error()
    d = capi.DownSampleDesc(capi.i3(0, 0, 0), 1, 100, 10)  # not a power of two
    assert vct_lib.vct_downsample(C.c_void_p(16), capi.ref(d), 0, None) == capi.VCT_E_BAD_ARG
    c = capi.ImageCleaningDesc(capi.i3(-1, 0, 0), 0, capi.u3(8, 8, 8), 128, 6)
    assert vct_lib.vct_clear_region(C.c_void_p(16), capi.ref(c), None) == capi.VCT_E_BAD_ARG
    w = capi.BorderWrappingDesc(128, 3, 6, 6)
    assert vct_lib.vct_wrap_border(C.c_void_p(16), capi.ref(w), None) == capi.VCT_E_BAD_ARG
    assert vct_lib.vct_cone_trace(None, None, None, 128, None, None, None, None, 1, None, None, None, None) == \
        capi.VCT_E_BAD_ARG
    # an empty trace is a no-op, not an error
    assert vct_lib.vct_cone_trace(None, None, C.c_void_p(16), 128, None, None, None, None, 0, None, None, None,
                                  None) == capi.VCT_OK


def test_new_entry_points_reject_bad_arguments(vct_lib):
    """The entry points of the G-buffer, filter, toroidal, instance, batch and gradient paths validate their
    arguments on the host before any device work (these calls need no GPU)."""
    P = C.c_void_p
    bad = [
        ("vct_gbuffer", (None, None, 16, 16, None, None, None)),
        ("vct_specular_filter", (None, None, None, 16, 16, None, None)),
        ("vct_present_srgb8", (P(16), 0, 16, P(16), None)),
        ("vct_cone_trace_f32", (None, None, P(16), 48, None, None, None, None, 0, None, None, None, None)),
        ("vct_cone_trace_backward", (None, None, P(16), 48, None, None, None, None, 0, None, None, P(16), None)),
        ("vct_downsample_f32", (P(16), None, 1, None)),
        ("vct_downsample_backward", (P(16), P(16), None, 1, None)),
        ("vct_batch_submit", (None, 1, 4)),
        ("vct_atlas_alloc", (48, capi.TEX_RGBA8, C.byref(C.c_void_p()))),
        ("vct_create", (None, C.byref(C.c_void_p()))),
        ("vct_context_frame", (None, None, None, None, None, 0, None)),
        ("vct_voxelize_opacity_slabs", (None, None, 32, None, None, None, 0, None, None)),
        ("vct_update_clip_regions", (None, None, 32, 16, None, None, None)),
    ]
    for name, args in bad:
        with pytest.raises(capi.VctError):
            capi.call(name, *args)
    # the batch's stream count is checked first
    with pytest.raises(capi.VctError, match="streams"):
        capi.call("vct_batch_submit", None, 0, 0)
    # a direction parallel to up has no camera frame
    out = capi.CamMatrix()
    v = lambda *x: C.cast((C.c_float * 3)(*x), C.c_void_p)
    with pytest.raises(capi.VctError, match="parallel"):
        capi.call("vct_camera_matrix", v(0, 0, 0), v(0, 2, 0), v(0, 1, 0), 60.0, 1.0, capi.ref(out))


def test_png_unfilter_rejects_an_unknown_filter(vct_lib):
    raw = np.array([7, 1, 2, 3], np.uint8)  # filter type 7
    out = np.zeros(3, np.uint8)
    with pytest.raises(capi.VctError, match="filter"):
        capi.call("vct_png_unfilter", raw.ctypes.data_as(C.c_void_p), 3, 1, 1, out.ctypes.data_as(C.c_void_p))
