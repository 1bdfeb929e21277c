"""The specular filter / tone map / present oracle (CPU) and the library's
Gaussian stencil against it."""
import ctypes as C

import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import capi


def test_gaussian_stencil_library_matches_oracle(vct_lib, oracle):
    out = (C.c_float * 9)()
    capi.call("vct_specular_filter_stencil", C.cast(out, C.c_void_p))
    lib_w = np.frombuffer(bytes(out), np.float32)
    assert np.array_equal(lib_w.view(np.uint32), oracle.gaussian_stencil().view(np.uint32))


def test_gaussian_stencil_shape(oracle):
    """257 taps within 0.01 texel, normalised by 241: a near-identity that brightens by 257 / 241."""
    w = oracle.gaussian_stencil().astype(np.float64).reshape(3, 3)
    assert abs(w.sum() - 257.0 / 241.0) < 1e-6
    assert w[1, 1] > 1.05 and w[1, 1] < 257.0 / 241.0
    assert np.allclose(w, w[::-1, :], atol=1e-9) and np.allclose(w, w[:, ::-1], atol=1e-9)
    assert np.allclose(w, w.T, atol=1e-9)
    assert 1e-3 < w[0, 1] < 3e-3 and w[0, 0] < 1e-5


def _img(rng, H, W, hdr=2.0):
    a = rng.uniform(0.0, hdr, size=(H, W, 4)).astype(np.float32)
    a[..., 3] = 1.0
    return a


def test_gaussian_path_is_the_stencil(oracle):
    rng = np.random.default_rng(3)
    d, s = _img(rng, 9, 13), _img(rng, 9, 13)
    out = oracle.specular_filter(d, s, method=1)
    w = oracle.gaussian_stencil().reshape(3, 3).astype(np.float64)
    pad = np.pad(s[..., :3].astype(np.float64), ((1, 1), (1, 1), (0, 0)), mode="edge")
    blur = sum(w[r, c] * pad[r:r + 9, c:c + 13] for r in range(3) for c in range(3))
    assert np.allclose(out[..., :3], d[..., :3] + blur, rtol=1e-6, atol=1e-6)
    assert np.array_equal(out[..., 3], d[..., 3])


def test_bilateral_constant_and_delta(oracle):
    H, W = 31, 33
    d = np.zeros((H, W, 4), np.float32)
    s = np.full((H, W, 4), 0.25, np.float32)
    out = oracle.specular_filter(d, s, method=0)
    assert np.allclose(out[..., :3], 0.25, rtol=1e-6)
    # a small delta: the range weight is ~1 (sigma 10), so the spread is the spatial KERNEL x KERNEL
    s[:] = 0.0
    s[15, 16, :3] = 0.01
    out = oracle.specular_filter(d, s, method=0)
    k = np.array([0.031225216, 0.033322271, 0.035206333, 0.036826804, 0.038138565, 0.039104044, 0.039695028,
                  0.039894000, 0.039695028, 0.039104044, 0.038138565, 0.036826804, 0.035206333, 0.033322271,
                  0.031225216])
    kk = np.outer(k, k) / np.outer(k, k).sum()
    got = out[8:23, 9:24, 0]
    assert np.allclose(got, 0.01 * kk, rtol=1e-4)
    assert out[0, 0, 0] == 0.0


def test_filter_method_other_values_run_bilateral(oracle):
    rng = np.random.default_rng(5)
    d, s = _img(rng, 12, 10), _img(rng, 12, 10)
    b0 = oracle.specular_filter(d, s, method=0)
    assert np.array_equal(oracle.specular_filter(d, s, method=7), b0)
    assert not np.array_equal(oracle.specular_filter(d, s, method=1), b0)


def test_tonemap_white_point(oracle):
    """Uncharted2 normalised by its value at 11.2: colour * exposure == 11.2 maps to 1."""
    d = np.zeros((1, 3, 4), np.float32)
    d[0, :, :3] = np.float32([0.0, 11.2 / 0.1, 5.0])[:, None]
    d[..., 3] = 1.0
    s = np.zeros_like(d)
    out = oracle.specular_filter(d, s, tonemap=1, method=1)
    assert abs(out[0, 1, 0] - 1.0) < 1e-6
    assert 0.0 < out[0, 2, 0] < 1.0 and out[0, 1, 3] == 1.0


def test_present_srgb8(oracle):
    rgba = np.array([[[0.0, 0.5, 1.0, 1.0], [2.0, -1.0, 0.002, 0.5]]], np.float32)
    px = oracle.present_srgb8(rgba)
    b = px.view(np.uint8).reshape(1, 2, 4)  # bytes B, G, R, A
    assert list(b[0, 0]) == [255, 188, 0, 255]
    assert list(b[0, 1]) == [int(np.floor(0.002 * 12.92 * 255 + 0.5)), 0, 255, 128]
