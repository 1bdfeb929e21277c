"""GPU parity of the fast cone tracer (texture-sampled, Morton-ordered,
warp-compacted) and of the FP16-storage mips.

Tolerances: traced radiance within a relative L2 error of 1e-2 of the FP64
oracle (the spec's bar for the hardware-filtered forms: the texture unit uses
8-bit sub-texel weights); integer-exact properties (order invariance,
repeatability) bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-2


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)


def _setup(oracle, R, n, seed, fill=0.05, spec=0.5, mode=8, cones32=0):
    from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = trace_desc(**{**default_trace_desc(regions, R), "rendering_mode": mode, "enable_32_cones": cones32})
    atlas = random_atlas(R, seed=seed, fill=fill)
    for level in range(1, 6):
        oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
    samples = random_samples(n, (0, 0, 0), 6.0, seed=seed + 1, specular_fraction=spec)
    return regions, desc, atlas, samples


def _dev(torch, a):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


@pytest.mark.parametrize("R,n", [(32, 3000), (64, 2000)])
def test_fast_rgba8_matches_fp64_oracle(cuda, oracle, R, n):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    regions, desc, atlas, samples = _setup(oracle, R, n, seed=R + 1)
    eye = (0.5, 1.0, -4.0)
    d64, s64, steps64, _ = oracle.cone_trace(64, bytes(desc), eye, atlas, R, samples)
    tex = clipmap.RadianceTexture(R).update(_dev(torch, atlas))
    dev_s = clipmap.samples_to_device(samples)
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    d, s = clipmap.cone_trace_fast(desc, eye, tex, dev_s, steps=steps)
    torch.cuda.synchronize()
    d = d.cpu().numpy().astype(np.float64)
    s = s.cpu().numpy().astype(np.float64)
    assert np.isfinite(d).all() and np.isfinite(s).all()
    assert _rel(d[:, :3], d64[:, :3]) < TOL_FP64
    assert _rel(s[:, :3], s64[:, :3]) < TOL_FP64
    assert _rel(d[:, 3], d64[:, 3]) < TOL_FP64
    assert abs(int(steps.item()) - steps64) <= 0.01 * steps64
    tex.close()


@pytest.mark.parametrize("mode", list(range(9)))
def test_fast_all_rendering_modes_match_exact(cuda, oracle, mode):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    R = 32
    regions, desc, atlas, samples = _setup(oracle, R, 1000, seed=5, mode=mode)
    eye = (0.0, 2.0, -5.0)
    da = _dev(torch, atlas)
    tex = clipmap.RadianceTexture(R).update(da)
    dev_s = clipmap.samples_to_device(samples)
    de, se = clipmap.cone_trace(desc, eye, da, R, dev_s)
    df, sf = clipmap.cone_trace_fast(desc, eye, tex, dev_s)
    torch.cuda.synchronize()
    for a, b in ((df, de), (sf, se)):
        a = a.cpu().numpy().astype(np.float64)
        b = b.cpu().numpy().astype(np.float64)
        assert _rel(a, b) < TOL_FP64, (mode, _rel(a, b))
    tex.close()


def test_fast_32_cones_and_discarded_samples(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    R = 32
    regions, desc, atlas, samples = _setup(oracle, R, 800, seed=9, cones32=1)
    samples["depth"][::7] = 1.0  # sky texels: the shader discards them, outputs stay untouched
    eye = (0.0, 2.0, -5.0)
    d64, s64, _, written = oracle.cone_trace(64, bytes(desc), eye, atlas, R, samples)
    tex = clipmap.RadianceTexture(R).update(_dev(torch, atlas))
    dev_s = clipmap.samples_to_device(samples)
    sentinel = torch.full((800, 4), -7.0, device="cuda")
    d, s = clipmap.cone_trace_fast(desc, eye, tex, dev_s, diffuse=sentinel.clone(), specular=sentinel.clone())
    torch.cuda.synchronize()
    d = d.cpu().numpy()
    s = s.cpu().numpy()
    skip = written == 0
    assert skip.sum() == len(range(0, 800, 7))
    assert (d[skip] == -7.0).all() and (s[skip] == -7.0).all()
    assert _rel(d[~skip][:, :3], d64[~skip][:, :3]) < TOL_FP64
    assert _rel(s[~skip][:, :3], s64[~skip][:, :3]) < TOL_FP64
    tex.close()


def test_fast_order_invariant_and_repeatable(cuda, oracle):
    """Each sample's outputs depend only on that sample: a permuted input gives bitwise the same results."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    R = 32
    regions, desc, atlas, samples = _setup(oracle, R, 4096, seed=13)
    eye = (0.0, 2.0, -5.0)
    tex = clipmap.RadianceTexture(R).update(_dev(torch, atlas))
    perm = np.random.default_rng(0).permutation(samples.shape[0])
    a_d, a_s = clipmap.cone_trace_fast(desc, eye, tex, clipmap.samples_to_device(samples))
    b_d, b_s = clipmap.cone_trace_fast(desc, eye, tex, clipmap.samples_to_device(samples[perm]))
    c_d, c_s = clipmap.cone_trace_fast(desc, eye, tex, clipmap.samples_to_device(samples))
    torch.cuda.synchronize()
    assert torch.equal(a_d, c_d) and torch.equal(a_s, c_s)
    assert torch.equal(a_d[torch.from_numpy(perm).cuda()], b_d)
    assert torch.equal(a_s[torch.from_numpy(perm).cuda()], b_s)
    tex.close()


@pytest.mark.parametrize("R", [16, 32])
def test_rgba16f_mips_match_fp64(cuda, oracle, R):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import random_atlas
    atlas = random_atlas(R, seed=R, fill=0.4)
    regions = oracle.clip_regions((1.5, -0.5, 2.5), R)
    want = oracle.rgba8_to_f4(atlas)
    for mode in (1,):
        for level in range(1, 6):
            oracle.downsample_f4(want, R, regions[level - 1, 0:3], level, mode)
    creg = clipmap.clip_regions((1.5, -0.5, 2.5), R)
    a16 = clipmap.to_rgba16f(_dev(torch, atlas), R)
    clipmap.cmd_downsample_rgba16f_all(a16, R, creg, 1)
    torch.cuda.synchronize()
    got = a16.cpu().numpy().view(np.float16).astype(np.float32).reshape(want.shape)
    err = np.abs(got - want)
    # FP16 storage: each level rounds to 11 significant bits (relative 2^-11 per level)
    assert err.max() < 4e-3, err.max()


def test_fp16_form_trace_matches_fp64(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    R = 32
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = trace_desc(**default_trace_desc(regions, R))
    atlas = random_atlas(R, seed=21, fill=0.05)
    ref4 = oracle.rgba8_to_f4(atlas)
    for level in range(1, 6):
        oracle.downsample_f4(ref4, R, regions[level - 1, 0:3], level, 1)
    samples = random_samples(2000, (0, 0, 0), 6.0, seed=22)
    eye = (0.5, 1.0, -4.0)
    d64, s64, _ = oracle.cone_trace_f4(bytes(desc), eye, ref4, R, samples)
    a16 = clipmap.to_rgba16f(_dev(torch, atlas), R)
    clipmap.cmd_downsample_rgba16f_all(a16, R, clipmap.clip_regions((0.0, 0.0, 0.0), R), 1)
    tex = clipmap.RadianceTexture(R, capi.TEX_RGBA16F).update(a16)
    d, s = clipmap.cone_trace_fast(desc, eye, tex, clipmap.samples_to_device(samples))
    torch.cuda.synchronize()
    d = d.cpu().numpy().astype(np.float64)
    s = s.cpu().numpy().astype(np.float64)
    assert _rel(d[:, :3], d64[:, :3]) < TOL_FP64
    assert _rel(s[:, :3], s64[:, :3]) < TOL_FP64
    tex.close()


def test_fp16_passes_keep_their_texture_current(cuda, oracle):
    """The FP16 conversion and mips with a mirror texture leave the texture equal to the FP16 atlas, texel for
    texel, with no vct_texture_update (a texture refreshed by a copy is the reference); a mirror of the wrong
    format or resolution is refused."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import random_atlas
    R = 32
    atlas = _dev(torch, random_atlas(R, seed=5, fill=0.3))
    creg = clipmap.clip_regions((0.7, 0.2, -1.1), R)
    mirrored = clipmap.RadianceTexture(R, capi.TEX_RGBA16F)
    a16 = clipmap.to_rgba16f(atlas, R, mirror=mirrored)
    clipmap.cmd_downsample_rgba16f_all(a16, R, creg, 1, mirror=mirrored)
    back = mirrored.read(torch.empty_like(a16))
    copied = clipmap.RadianceTexture(R, capi.TEX_RGBA16F).update(a16)
    back2 = copied.read(torch.empty_like(a16))
    torch.cuda.synchronize()
    assert torch.equal(back, a16) and torch.equal(back2, a16)
    assert (a16 != 0).any()
    with pytest.raises(capi.VctError):
        clipmap.to_rgba16f(atlas, R, out=a16, mirror=clipmap.RadianceTexture(R, capi.TEX_RGBA8))
    with pytest.raises(capi.VctError):
        clipmap.cmd_downsample_rgba16f(a16, R, (0, 0, 0), 1, 1, mirror=clipmap.RadianceTexture(16, capi.TEX_RGBA16F))
    mirrored.close()
    copied.close()


def test_gather_probe_reports_a_finite_rate_and_checks_arguments(cuda, oracle):
    """The roofline probe (no reference counterpart) runs the fetch pattern of
    one cone sample per step and reports a positive rate; bad arguments are
    rejected before any launch."""
    torch = cuda
    import ctypes as C
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    R = 32
    regions, desc, atlas, _ = _setup(oracle, R, 16, seed=9)
    tex = clipmap.RadianceTexture(R).update(_dev(torch, atlas))
    rate = clipmap.gather_probe(desc, tex, cones=2048, steps_per_cone=64)
    assert np.isfinite(rate) and rate > 1e6
    out = C.c_double(0.0)
    rc = capi.lib().vct_gather_probe(capi.ref(desc), tex.handle, 0, 64, C.byref(out), None)
    assert rc == capi.VCT_E_BAD_ARG
    tex.close()


def test_diffuse_aperture_option_thirty_degree_cones(cuda, oracle):
    """vct_cone_trace_opt / vct_cone_trace_fast_opt with 16 fixed 30-degree cones: the exact form follows the
    oracle's FP32 mirror per sample, both forms stay within the FP64 bar; bad options are rejected."""
    import ctypes as C
    import math
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    R = 32
    regions, desc, atlas, samples = _setup(oracle, R, 2000, seed=31)
    ap = math.radians(30.0)
    eye = (0.5, 1.0, -4.0)
    d32, s32, st32, _ = oracle.cone_trace(32, bytes(desc), eye, atlas, R, samples, diffuse_aperture=ap)
    d64, s64, _, _ = oracle.cone_trace(64, bytes(desc), eye, atlas, R, samples, diffuse_aperture=ap)
    da = _dev(torch, atlas)
    dev_s = clipmap.samples_to_device(samples)
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    de, se = clipmap.cone_trace(desc, eye, da, R, dev_s, steps=steps, diffuse_aperture=ap)
    tex = clipmap.RadianceTexture(R).update(da)
    df, sf = clipmap.cone_trace_fast(desc, eye, tex, dev_s, diffuse_aperture=ap)
    torch.cuda.synchronize()
    de = de.cpu().numpy().astype(np.float64)
    err = np.abs(de - d32).max(1) / np.maximum(np.abs(d32).max(1), 1e-3)
    assert np.mean(err < 1e-4) > 0.99, np.sort(err)[-8:]
    assert abs(int(steps.item()) - st32) <= max(8, 0.002 * st32)
    for got in (de, df.cpu().numpy().astype(np.float64)):
        assert _rel(got[:, :3], d64[:, :3]) < TOL_FP64
    bad = capi.TraceOptions(4.0)
    out = torch.zeros((2000, 4), device="cuda")
    cam = clipmap.cam_matrix(eye)
    light = capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    rc = capi.lib().vct_cone_trace_opt(capi.ref(desc), capi.ref(cam), C.c_void_p(da.data_ptr()), R, None,
                                       capi.ref(light), None, C.c_void_p(dev_s.data_ptr()), 2000,
                                       C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None, capi.ref(bad),
                                       None)
    assert rc == capi.VCT_E_BAD_ARG
    tex.close()
