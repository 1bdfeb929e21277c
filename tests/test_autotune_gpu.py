"""The fast trace's launch-shape autotuner (vct_cone_trace_fast_autotune) and
the instance flags (vct_config.flags): a tuned shape changes the time, not the
results -- every shape the tuner tries and the one it keeps give the default
shape's outputs bit for bit -- and a context that tunes on its first trace, or
keeps its opacity atlas one byte per texel, gives the outputs of a plain
context on the same frames."""
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


def test_tuned_shape_gives_the_default_results(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    R = 64
    cam = (0.2, -0.1, 0.3)
    regions = oracle.clip_regions(cam, R)
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    atlas = random_atlas(R, seed=5, fill=0.07)
    for level in range(1, 6):
        oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
    tex = clipmap.RadianceTexture(R).update(torch.from_numpy(atlas.view(np.int32).copy()).cuda())
    samples = clipmap.samples_to_device(random_samples(20000, cam, 3.0, seed=8, specular_fraction=0.5))
    eye = (0.7, 1.0, -4.0)
    capi.call("vct_trace_tuning_reset")
    assert clipmap.trace_tuning(R) == {"diffuse_blocks_per_sm": 8, "specular_blocks_per_sm": 64, "tuned": False}
    d0, s0 = clipmap.cone_trace_fast(desc, eye, tex, samples)
    # the tuner's own outputs come from the last shape it tried
    d1, s1 = torch.full_like(d0, -1.0), torch.full_like(s0, -1.0)
    t = clipmap.autotune_fast(desc, eye, tex, samples, diffuse=d1, specular=s1)
    torch.cuda.synchronize()
    assert torch.equal(d1, d0) and torch.equal(s1, s0)
    assert t["specular_blocks_per_sm"] in (16, 32, 64, 128) and t["diffuse_blocks_per_sm"] in (4, 8, 16)
    assert 0.0 < t["trace_ms"] <= t["default_ms"]
    got = clipmap.trace_tuning(R)
    assert got["tuned"] and got["specular_blocks_per_sm"] == t["specular_blocks_per_sm"]
    d2, s2 = clipmap.cone_trace_fast(desc, eye, tex, samples)
    torch.cuda.synchronize()
    assert torch.equal(d2, d0) and torch.equal(s2, s0)
    assert not clipmap.trace_tuning(2 * R)["tuned"]  # kept per resolution
    capi.call("vct_trace_tuning_reset")
    assert not clipmap.trace_tuning(R)["tuned"]
    tex.close()


def test_context_flags_autotune_and_r8_opacity(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, engine, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, room_scene, surface_samples
    R, S = 32, 256
    sc = room_scene(seed=6, n_random=2500)
    ds = passes.DeviceScene(sc)
    cam = (0.35, 2.1, -0.7)
    light, lsd = _light(cam)
    samples = clipmap.samples_to_device(surface_samples(sc, 3000, seed=9))
    td = clipmap.trace_desc(**default_trace_desc(np.zeros((6, 7), np.int32), R))
    eye = (0.0, 3.0, -3.0)
    capi.call("vct_trace_tuning_reset")
    out = {}
    for flags in (0, capi.CONTEXT_AUTOTUNE, capi.CONTEXT_OPACITY_R8, capi.CONTEXT_AUTOTUNE | capi.CONTEXT_OPACITY_R8):
        ctx = engine.Context(R, shadow_size=S, flags=flags)
        for _ in range(2):
            ctx.frame(ds, cam, light, lsd)
        d, s = ctx.trace(td, eye, samples, light, lsd)
        torch.cuda.synchronize()
        out[flags] = (ctx.atlas("opacity").clone(), ctx.atlas("radiance").clone(), d, s)
        if flags & capi.CONTEXT_AUTOTUNE:
            assert clipmap.trace_tuning(R)["tuned"]
        ctx.close()
    op32, rad32, d32, s32 = out[0]
    for flags, (op, rad, d, s) in out.items():
        assert torch.equal(rad, rad32) and torch.equal(d, d32) and torch.equal(s, s32), flags
        if flags & capi.CONTEXT_OPACITY_R8:
            assert op.dtype == torch.uint8
            assert torch.equal(op.to(torch.int32), (op32 >> 24) & 0xFF)
    with pytest.raises(capi.VctError, match="flags"):
        engine.Context(R, shadow_size=S, flags=8)
    capi.call("vct_trace_tuning_reset")
