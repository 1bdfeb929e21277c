"""Inverse radiance fitting on the GPU: the Adam step bit for bit against a
float32 restatement, the squared-error kernel against numpy, and a small
fit (R = 32, 4 x 64^2 samples) that recovers a hidden smooth volume's images
through the trace and mip adjoints."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def adam_reference(p, g, m, v, step, lr, betas, eps, rgb, alpha):
    """vct_adam_step in float32 numpy, one rounding per operation in the kernel's order; the bias
    corrections in double from the float32 betas, as the library computes them."""
    f = np.float32
    b1, b2 = f(betas[0]), f(betas[1])
    omb1, omb2 = f(1.0) - b1, f(1.0) - b2
    c1 = f(1.0 / (1.0 - float(b1) ** step))
    c2 = f(1.0 / (1.0 - float(b2) ** step))
    p, g, m, v = (np.asarray(x, np.float32).reshape(-1, 4) for x in (p, g, m, v))
    m = b1 * m + omb1 * g
    v = b2 * v + (omb2 * g) * g
    upd = (f(lr) * (m * c1)) / (np.sqrt(v * c2) + f(eps))
    lo = np.array([rgb[0]] * 3 + [alpha[0]], np.float32)
    hi = np.array([rgb[1]] * 3 + [alpha[1]], np.float32)
    return np.minimum(np.maximum(p - upd, lo), hi).reshape(-1), m.reshape(-1), v.reshape(-1)


def test_adam_step_bit_exact(cuda):
    torch = cuda
    import ctypes as C
    from vk_voxel_cone_tracing_gb300 import capi
    rng = np.random.default_rng(0)
    n = 4 * 10007
    p = rng.uniform(-0.2, 1.2, n).astype(np.float32)
    m = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    tp, tm, tv = (torch.from_numpy(x.copy()).cuda() for x in (p, m, v))
    desc = capi.AdamDesc(0.03, 0.9, 0.999, 1e-8, 0, 1, 0.0, 1.0, 0.0, 0.95)
    for step in range(1, 6):
        g = rng.normal(0, 0.1 * step, n).astype(np.float32)
        g[::7] = 0.0
        tg = torch.from_numpy(g.copy()).cuda()
        desc.step = step
        capi.call("vct_adam_step", C.c_void_p(tp.data_ptr()), C.c_void_p(tg.data_ptr()), C.c_void_p(tm.data_ptr()),
                  C.c_void_p(tv.data_ptr()), n, capi.ref(desc), None)
        p, m, v = adam_reference(p, g, m, v, step, 0.03, (0.9, 0.999), 1e-8, (0.0, 1.0), (0.0, 0.95))
        torch.cuda.synchronize()
        for got, want in ((tp, p), (tm, m), (tv, v)):
            assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32)), step
        assert not tg.any().item()  # zero_grad
    with pytest.raises(capi.VctError):
        desc.step = 0
        capi.call("vct_adam_step", C.c_void_p(tp.data_ptr()), C.c_void_p(tg.data_ptr()), C.c_void_p(tm.data_ptr()),
                  C.c_void_p(tv.data_ptr()), n, capi.ref(desc), None)
    with pytest.raises(capi.VctError):
        desc.step = 1
        capi.call("vct_adam_step", C.c_void_p(tp.data_ptr()), C.c_void_p(tg.data_ptr()), C.c_void_p(tm.data_ptr()),
                  C.c_void_p(tv.data_ptr()), n - 2, capi.ref(desc), None)


def test_sq_error(cuda):
    torch = cuda
    import ctypes as C
    from vk_voxel_cone_tracing_gb300 import capi
    rng = np.random.default_rng(1)
    n = 300001
    o = rng.normal(size=(n, 4)).astype(np.float32)
    t = rng.normal(size=(n, 4)).astype(np.float32)
    to, tt = torch.from_numpy(o).cuda(), torch.from_numpy(t).cuda()
    g = torch.empty_like(to)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    scale = 1.0 / (4 * n)
    capi.call("vct_sq_error", C.c_void_p(to.data_ptr()), C.c_void_p(tt.data_ptr()), n, scale,
              C.c_void_p(g.data_ptr()), C.c_void_p(loss.data_ptr()), None)
    torch.cuda.synchronize()
    d = o - t
    assert np.array_equal(g.cpu().numpy(), np.float32(2.0 * np.float32(scale)) * d)
    want = float((d.astype(np.float64) ** 2).sum() * np.float32(scale))
    assert abs(loss.item() - want) <= 1e-12 * abs(want)
    first = loss.item()
    capi.call("vct_sq_error", C.c_void_p(to.data_ptr()), C.c_void_p(tt.data_ptr()), n, scale, None,
              C.c_void_p(loss.data_ptr()), None)
    torch.cuda.synchronize()
    assert loss.item() == first  # fixed reduction order


def test_fit_recovers_hidden_volume(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, fit
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_samples, smooth_volume
    R = 32
    centre = (0.2, 1.1, -0.4)
    regions = clipmap.regions_to_numpy(clipmap.clip_regions(centre, R))
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    cam = clipmap.cam_matrix((0.0, 3.0, -3.0))
    light = capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    smp = random_samples(4 * 64 * 64, centre, 3.0, seed=9, specular_fraction=0.6)
    smp["emission_texel"] = 0.0
    samples = clipmap.samples_to_device(smp)
    hidden = torch.from_numpy(np.ascontiguousarray(smooth_volume(R, seed=4)).reshape(-1)).cuda()
    f = fit.RadianceFit(R, regions, desc, cam, light, samples, lr=0.05)
    td, ts = f.render(hidden.clone())
    f.set_targets(td, ts)
    losses = [f.step() for _ in range(40)]
    final = f.loss()
    assert np.all(np.isfinite(losses)) and losses[0] > 0
    assert final < 0.2 * losses[0], (losses[0], losses[-1], final)
    # the hidden volume itself has zero loss
    g = fit.RadianceFit(R, regions, desc, cam, light, samples, td, ts, init=hidden)
    assert g.loss() == 0.0
