"""GPU parity of the specular filter / tone map / present kernels against the
oracle, and one whole frame through ``render.Renderer``.

Tolerances: the Gaussian path without tone mapping is FP32 multiply / add
only and is compared bit for bit.  The bilateral filter's weights use exp and
the tone map / sRGB encode use pow; CUDA's expf / powf are within 2 ulp of
the exact value and the host's within 1, so those outputs are compared to a
relative 1e-5 (and the sRGB bytes to one step, nearly all exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _img(rng, H, W, hdr=2.0):
    a = rng.uniform(0.0, hdr, size=(H, W, 4)).astype(np.float32)
    a[..., 3] = rng.uniform(0.5, 1.0, size=(H, W)).astype(np.float32)
    return a


def _gpu_filter(torch, d, s, **kw):
    from vk_voxel_cone_tracing_gb300 import render
    H, W = d.shape[:2]
    dd = torch.from_numpy(d.reshape(-1, 4)).cuda()
    ss = torch.from_numpy(s.reshape(-1, 4)).cuda()
    out = render.specular_filter(dd, ss, W, H, render.filter_desc(**kw))
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(H, W, 4)


@pytest.mark.parametrize("H,W", [(197, 333), (8, 8), (1, 37)])
def test_gaussian_bit_exact(cuda, oracle, H, W):
    rng = np.random.default_rng(H * 1000 + W)
    d, s = _img(rng, H, W), _img(rng, H, W)
    got = _gpu_filter(cuda, d, s, method=1)
    want = oracle.specular_filter(d, s, method=1)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("method", [0, 5])
def test_bilateral_matches(cuda, oracle, method):
    rng = np.random.default_rng(11)
    d, s = _img(rng, 70, 101), _img(rng, 70, 101, hdr=30.0)  # contrasts above sigma 10 engage the range weight
    got = _gpu_filter(cuda, d, s, method=method)
    want = oracle.specular_filter(d, s, method=method)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-6)
    assert np.array_equal(got[..., 3], want[..., 3])


@pytest.mark.parametrize("method", [0, 1])
def test_tonemap_matches(cuda, oracle, method):
    rng = np.random.default_rng(12)
    d, s = _img(rng, 41, 67, hdr=40.0), _img(rng, 41, 67, hdr=5.0)
    got = _gpu_filter(cuda, d, s, method=method, tonemap=True, gamma=2.2, exposure=0.1)
    want = oracle.specular_filter(d, s, method=method, tonemap=1, gamma=2.2, exposure=0.1)
    assert np.isfinite(want).all()
    assert np.allclose(got, want, rtol=1e-5, atol=1e-6)


def test_present_srgb8(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import render
    rng = np.random.default_rng(13)
    rgba = rng.uniform(-0.1, 1.2, size=(123, 77, 4)).astype(np.float32)
    rgba[0, :5, 0] = [0.0, 0.0031308, 0.5, 1.0, 0.04045]
    got = render.present_srgb8(torch.from_numpy(rgba.reshape(-1, 4)).cuda(), 77, 123)
    torch.cuda.synchronize()
    g = got.cpu().numpy().view(np.uint32)
    w = oracle.present_srgb8(rgba)
    gb, wb = g.view(np.uint8).astype(int), w.view(np.uint8).astype(int)
    assert np.abs(gb - wb).max() <= 1
    assert (gb == wb).mean() > 0.999


def test_bad_arguments(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, render
    a = torch.zeros((16, 4), device="cuda")
    with pytest.raises(capi.VctError):
        render.specular_filter(a, a, 4, 4, out=a)  # the output aliases the specular image
    with pytest.raises(ValueError):
        render.specular_filter(a, a, 5, 4)


def test_renderer_frame(cuda, oracle):
    """A whole frame: the G-buffer equals the oracle's, the output equals the oracle's filter over the
    trace's own contribution images, and the image shows the lit room."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import render
    from vk_voxel_cone_tracing_gb300.scene import room_scene
    sc = room_scene(seed=1, n_random=2000)
    W, H = 160, 96
    r = render.Renderer(sc, R=64, width=W, height=H, shadow_res=512)
    pos, d = (0.3, 3.0, -3.5), (0.3, -0.25, 1.0)
    out = r.render(pos, d)
    torch.cuda.synchronize()
    cam = np.frombuffer(bytes(r.camera), np.float32)
    want_g = oracle.gbuffer(sc, cam, W, H)
    assert np.array_equal(r.samples.cpu().numpy().view(np.uint32), want_g.view(np.uint32))
    dif = r.diffuse.cpu().numpy().reshape(H, W, 4)
    spe = r.specular.cpu().numpy().reshape(H, W, 4)
    want = oracle.specular_filter(dif, spe, method=1)
    assert np.array_equal(out.cpu().numpy().reshape(H, W, 4).view(np.uint32), want.view(np.uint32))
    img = r.image.cpu().numpy().view(np.uint8).reshape(H, W, 4)
    assert np.isfinite(want).all()
    assert img[..., :3].mean() > 5 and img[..., :3].std() > 2  # lit, with structure
    r.close()


@pytest.mark.parametrize("seed", range(4))
def test_random_sizes_gaussian_bit_exact(cuda, oracle, seed):
    rng = np.random.default_rng(seed)
    H, W = int(rng.integers(1, 90)), int(rng.integers(1, 130))
    d, s = _img(rng, H, W, hdr=float(rng.uniform(0.5, 20))), _img(rng, H, W, hdr=float(rng.uniform(0.5, 20)))
    got = _gpu_filter(cuda, d, s, method=1)
    want = oracle.specular_filter(d, s, method=1)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
