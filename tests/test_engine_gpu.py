"""The instance API (vct_create / vct_context_frame / vct_context_trace) and the
batched submission (vct_batch_submit) on the GPU: an instance reproduces the
pass-by-pass path bit for bit, and a batch over several streams reproduces the
same jobs run one at a time."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)


def _light(center):
    from vk_voxel_cone_tracing_gb300 import passes
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    origin = tuple((np.asarray(center, np.float64) - 15.0 * d).astype(np.float32).tolist())
    return passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(origin, LIGHT_DIR)


def test_atlas_alloc_and_errors(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, engine
    for fmt, words in ((capi.TEX_RGBA8, 1), (capi.TEX_RGBA16F, 2)):
        p = C.c_void_p()
        capi.call("vct_atlas_alloc", 32, fmt, C.byref(p))
        n = capi.lib().vct_atlas_texels(32) * words
        view = engine._device_view(p.value, (n,))
        torch.cuda.synchronize()
        assert int(view.abs().sum().item()) == 0  # created cleared
        del view
        capi.call("vct_atlas_free", p)
    with pytest.raises(capi.VctError):
        capi.call("vct_atlas_alloc", 33, capi.TEX_RGBA8, C.byref(C.c_void_p()))
    with pytest.raises(capi.VctError):
        capi.call("vct_create", capi.ref(capi.Config(48, 0, 0, 0, 0)), C.byref(C.c_void_p()))


def test_instance_matches_the_pass_path(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, engine, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, room_scene, surface_samples
    R, S = 32, 256
    sc = room_scene(seed=6, n_random=2500)
    ds = passes.DeviceScene(sc)
    cam0, cam1 = (0.35, 2.1, -0.7), (0.9, 2.4, -1.1)
    light, lsd = _light(cam0)
    samples = clipmap.samples_to_device(surface_samples(sc, 3000, seed=9))
    eye = (0.0, 3.0, -3.0)
    # the instance: two frames (the second toroidal) and a trace
    ctx = engine.Context(R, shadow_size=S)
    ctx.frame(ds, cam0, light, lsd)
    ctx.frame(ds, cam1, light, lsd, revoxelization=1)  # VCT_REVOX_TOROIDAL
    td = clipmap.trace_desc(**default_trace_desc(np.zeros((6, 7), np.int32), R))  # volume fields are replaced
    d1, s1 = ctx.trace(td, eye, samples, light, lsd)
    # the pass path with the same steps
    ws = passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((S, S), dtype=torch.float32, device="cuda")
    tex = clipmap.RadianceTexture(R)
    from vk_voxel_cone_tracing_gb300 import capi
    state = (capi.ClipmapRegion * 6)()
    passes.clipmap_frame(ds, cam0, R, op, rad, sh, light, lsd, ws, frame_index=0, texture=tex, regions_state=state)
    regs = passes.clipmap_frame(ds, cam1, R, op, rad, sh, light, lsd, ws, frame_index=1, texture=tex,
                                revoxelization=capi.REVOX_TOROIDAL, regions_state=state)
    td2 = clipmap.trace_desc(**default_trace_desc(clipmap.regions_to_numpy(regs), R))
    d2, s2 = clipmap.cone_trace_fast(td2, eye, tex, samples, light=light, shadow=sh, shadow_desc=lsd)
    torch.cuda.synchronize()
    b = ctx.buffers()
    assert b.frame_index == 2
    assert np.array_equal(np.frombuffer(bytes(b.regions), np.int32), np.frombuffer(bytes(state), np.int32))
    assert np.array_equal(ctx.atlas("opacity").cpu().numpy(), op.cpu().numpy())
    assert np.array_equal(ctx.atlas("radiance").cpu().numpy(), rad.cpu().numpy())
    assert np.array_equal(d1.cpu().numpy().view(np.uint32), d2.cpu().numpy().view(np.uint32))
    assert np.array_equal(s1.cpu().numpy().view(np.uint32), s2.cpu().numpy().view(np.uint32))
    ctx.reset()
    assert ctx.buffers().frame_index == 0
    ctx.close()
    tex.close()


def _jobs(torch, n_jobs=6):
    from vk_voxel_cone_tracing_gb300 import clipmap, engine, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, room_scene, surface_samples
    ctxs = [engine.Context(32, shadow_size=256), engine.Context(64, shadow_size=256), engine.Context(32, shadow_size=256)]
    jobs, outs, keep = [], [], []
    for i in range(n_jobs):
        sc = room_scene(seed=20 + i, n_random=1000 + 700 * i)
        ds = passes.DeviceScene(sc)
        ctx = ctxs[i % 3]
        cam = (0.3 * i, 2.0 + 0.1 * i, -0.5)
        light, lsd = _light(cam)
        smp = clipmap.samples_to_device(surface_samples(sc, 1500 + 500 * i, seed=i))
        td = clipmap.trace_desc(**default_trace_desc(np.zeros((6, 7), np.int32), ctx.R))
        d = torch.zeros((smp.shape[0], 4), dtype=torch.float32, device="cuda")
        s = torch.zeros_like(d)
        jobs.append(engine.batch_job(ctx, ds, cam, light, lsd, td, (0.0, 3.0, -3.0), smp, d, s))
        outs.append((d, s))
        keep.append((ds, smp, td, light, lsd))
    return ctxs, jobs, outs, keep


def test_batch_over_streams_equals_one_at_a_time(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import engine
    ctxs, jobs, outs, keep = _jobs(torch)
    engine.batch_submit(jobs, streams=1)
    torch.cuda.synchronize()
    want = [(d.cpu().numpy().copy(), s.cpu().numpy().copy()) for d, s in outs]
    for d, s in outs:
        d.zero_()
        s.zero_()
    engine.batch_submit(jobs, streams=3)
    torch.cuda.synchronize()
    for (d, s), (wd, wsp) in zip(outs, want):
        assert np.abs(wd).sum() > 0
        assert np.array_equal(d.cpu().numpy().view(np.uint32), wd.view(np.uint32))
        assert np.array_equal(s.cpu().numpy().view(np.uint32), wsp.view(np.uint32))
    for c in ctxs:
        c.close()
