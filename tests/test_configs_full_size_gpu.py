"""Parity at the sizes that are benchmarked, not only at small test sizes.

1. The benchmark's own workload: the seeded hall of 1,000,000 triangles
   (hall_scene(seed=2)), clip resolution 256 -- two RGBA8 atlases of 2.47 GB,
   so texel byte offsets pass 2^31 and the tile plans hold millions of items
   -- camera (0, 5, 0), light (0.3, -1, 0.2) with a 2048^2 shadow map.  The
   GPU frame (vct_clipmap_frame: voxelise, opacity mips, border wrap, shadow
   depth, injection, copy-alpha, radiance mips, in Application.cpp:171-221's
   order, keeping the RGBA8 radiance texture current) is compared with the
   oracle's pass-by-pass frame bit for bit, and so is the octree at 256^3
   (fragment list and deterministic node pool).  Every trace form then runs on
   a seeded subset of 16,384 of the benchmark's 1920x1080 samples.
2. Configuration 1 at its stated size: room_scene(seed=1) (about 34k
   triangles), R = 128, 65,536 area-uniform samples, octree depth 7.

Bars: RGBA8 / integer stages bit-exact; the exact FP32 trace within 1e-4 of
the oracle's FP32 mirror per sample for >= 99 % of samples; every form's
traced outputs within relative L2 1e-2 of the FP64 oracle (on RGBA8 storage
for the RGBA8 forms, on float storage with FP64 mips for the FP16 and float
forms, on the node pool for the octree trace); FP16 mips within 4e-3 of the
FP64 mips.  The measured errors (relative L2 and max abs, per form and per
output: indirect diffuse + direct RGB, ambient occlusion, specular RGB) are
written as JSON to the path in $VCT_ERROR_REPORT when it is set.
"""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)
TOL_FP64 = 1e-2
SUBSET = 16384


def _origin(center):
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - 15.0 * d).astype(np.float32).tolist())


def _f4(atlas):
    """RGBA8 words -> float RGBA (c / 255 in FP32, as oracle.rgba8_to_f4), a few depth slices at a time."""
    out = np.empty(atlas.shape + (4,), np.float32)
    for z in range(0, atlas.shape[0], 8):
        a = atlas[z:z + 8]
        for c in range(4):
            out[z:z + 8, ..., c] = ((a >> np.uint32(8 * c)) & np.uint32(0xFF)).astype(np.float32) / np.float32(255.0)
    return out


def _stats(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return {"rel_l2": float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-12)),
            "max_abs": float(np.abs(got - want).max()) if got.size else 0.0,
            "ref_rms": float(np.sqrt(np.mean(want ** 2))) if want.size else 0.0}


def _report(config, rows):
    path = os.environ.get("VCT_ERROR_REPORT")
    if not path:
        return
    data = json.loads(open(path).read()) if os.path.exists(path) else {}
    data[config] = rows
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def _outputs(mode8, mode7):
    """(diffuse rgb, specular rgb) of the default mode and the AO of mode 7."""
    (d8, s8), (d7, _) = mode8, mode7
    return {"diffuse_rgb": np.asarray(d8)[:, :3], "specular_rgb": np.asarray(s8)[:, :3], "ao": np.asarray(d7)[:, 0]}


def _check_form(rows, form, got, want):
    rows[form] = {k: _stats(got[k], want[k]) for k in want}
    for k, st in rows[form].items():
        assert st["rel_l2"] < TOL_FP64, (form, k, st)


def _desc_mode(base, mode):
    from vk_voxel_cone_tracing_gb300 import capi
    d = capi.ConeTracingDesc.from_buffer_copy(bytes(base))
    d.rendering_mode = mode
    return d


def _trace_all_forms(torch, oracle, rows, R, regions_np, rad_np, rad_dev, tex8, sh_np, sh_dev, samples, eye,
                     light, lsd, sd_bytes, fp16_regions):
    """Every clipmap trace form on `samples`, against the FP64 oracle; appends to `rows`."""
    import ctypes as C

    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc
    base = clipmap.trace_desc(**default_trace_desc(regions_np, R))
    dev_s = clipmap.samples_to_device(samples)
    n = samples.shape[0]
    ref8, mirror32, exact, fast = {}, {}, {}, {}
    for mode in (8, 7):
        desc = _desc_mode(base, mode)
        d64, s64, _, wr = oracle.cone_trace(64, bytes(desc), eye, rad_np, R, samples, shadow=sh_np,
                                            shadow_desc_bytes=sd_bytes)
        assert wr.all()
        ref8[mode] = (d64, s64)
        mirror32[mode] = oracle.cone_trace(32, bytes(desc), eye, rad_np, R, samples, shadow=sh_np,
                                           shadow_desc_bytes=sd_bytes)[:2]
        de, se = clipmap.cone_trace(desc, eye, rad_dev, R, dev_s, light=light, shadow=sh_dev, shadow_desc=lsd)
        dx, sx = clipmap.cone_trace_tex(desc, eye, tex8, dev_s, light=light, shadow=sh_dev, shadow_desc=lsd)
        df, sf = clipmap.cone_trace_fast(desc, eye, tex8, dev_s, light=light, shadow=sh_dev, shadow_desc=lsd)
        torch.cuda.synchronize()
        # the exact arithmetic with its texels read through the texture: the same results, bit for bit
        assert torch.equal(dx, de) and torch.equal(sx, se), mode
        exact[mode] = (de.cpu().numpy(), se.cpu().numpy())
        fast[mode] = (df.cpu().numpy(), sf.cpu().numpy())
        # the exact form follows the FP32 restatement sample by sample
        for got, want in zip(exact[mode], mirror32[mode]):
            err = np.abs(got - want).max(1) / np.maximum(np.abs(want).max(1), 1e-3)
            assert np.mean(err < 1e-4) > 0.99, (mode, np.sort(err)[-8:])
    want8 = _outputs(ref8[8], ref8[7])
    assert np.abs(want8["diffuse_rgb"]).sum() > 1.0 and np.abs(want8["specular_rgb"]).sum() > 0.1
    _check_form(rows, "exact_rgba8", _outputs(exact[8], exact[7]), want8)
    _check_form(rows, "texture_rgba8", _outputs(fast[8], fast[7]), want8)
    rows["fp32_mirror"] = {k: _stats(v, want8[k]) for k, v in _outputs(mirror32[8], mirror32[7]).items()}

    # float storage: the FP64 reference mips the float image of the RGBA8 radiance (levels 1-5 recomputed)
    ref4 = _f4(rad_np)
    for level in range(1, 6):
        oracle.downsample_f4(ref4, R, regions_np[level - 1, 0:3], level, 1)
    a16 = clipmap.to_rgba16f(rad_dev, R)
    tex16 = clipmap.RadianceTexture(R, capi.TEX_RGBA16F)
    clipmap.to_rgba16f(rad_dev, R, out=a16, mirror=tex16)
    clipmap.cmd_downsample_rgba16f_all(a16, R, fp16_regions, 1, mirror=tex16)
    torch.cuda.synchronize()
    worst = 0.0
    for z in range(0, ref4.shape[0], 16):
        got = a16[z:z + 16].cpu().numpy().view(np.float16).astype(np.float32).reshape(ref4[z:z + 16].shape)
        worst = max(worst, float(np.abs(got - ref4[z:z + 16]).max()))
    del a16
    rows["fp16_mips_max_abs"] = worst
    assert worst < 4e-3, worst
    # the float form: level 0 uploaded, the float mips run on the GPU
    vol = torch.from_numpy(_f4(rad_np).reshape(-1)).cuda()
    for level in range(1, 6):
        d = capi.DownSampleDesc(capi.i3(*[int(v) for v in regions_np[level - 1, 0:3]]), level, R,
                                capi.DOWNSAMPLE_REGION_SIZE)
        capi.call("vct_downsample_f32", C.c_void_p(vol.data_ptr()), capi.ref(d), 1, None)
    ref4_64, fp16, f32 = {}, {}, {}
    sm = capi.ShadowMap(sh_dev.data_ptr(), sh_dev.shape[1], sh_dev.shape[0])
    cam = clipmap.cam_matrix(eye)
    for mode in (8, 7):
        desc = _desc_mode(base, mode)
        ref4_64[mode] = oracle.cone_trace_f4(bytes(desc), eye, ref4, R, samples, shadow=sh_np,
                                             shadow_desc_bytes=sd_bytes)[:2]
        dh, sh_ = clipmap.cone_trace_fast(desc, eye, tex16, dev_s, light=light, shadow=sh_dev, shadow_desc=lsd)
        d32 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        s32 = torch.zeros_like(d32)
        capi.call("vct_cone_trace_f32", capi.ref(desc), capi.ref(cam), C.c_void_p(vol.data_ptr()), R,
                  capi.ref(sm), capi.ref(light), capi.ref(lsd), C.c_void_p(dev_s.data_ptr()), n,
                  C.c_void_p(d32.data_ptr()), C.c_void_p(s32.data_ptr()), None, None)
        torch.cuda.synchronize()
        fp16[mode] = (dh.cpu().numpy(), sh_.cpu().numpy())
        f32[mode] = (d32.cpu().numpy(), s32.cpu().numpy())
    tex16.close()
    del vol
    want4 = _outputs(ref4_64[8], ref4_64[7])
    _check_form(rows, "texture_rgba16f", _outputs(fp16[8], fp16[7]), want4)
    _check_form(rows, "exact_f32", _outputs(f32[8], f32[7]), want4)
    return base


def _svo_chain(torch, oracle, rows, scene, ds, ws, level, sh_np, sh_dev, sd_bytes, light, lsd, base_desc, samples,
               eye):
    """Fragment list and deterministic pool at `level` bit for bit, then the octree trace against FP64."""
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    want_f, F = oracle.svo_fragments(scene, level, ds.bb_min, ds.bb_max, sh_np, sd_bytes)
    frags = passes.svo_fragments(ds, level, sh_dev, light, lsd, ws)
    torch.cuda.synchronize()
    assert frags.shape[0] == F and F > 100000
    assert np.array_equal(frags.cpu().numpy().view(np.uint32), want_f)
    want_pool, n_want = oracle.svo_build(want_f, level)
    pool, n = passes.svo_build(frags, level, ws, mode=capi.SVO_DETERMINISTIC)
    torch.cuda.synchronize()
    assert n == n_want
    assert np.array_equal(pool[:n].cpu().numpy().view(np.uint32), want_pool)
    bmin, bmax = tuple(ds.bb_min.tolist()), tuple(ds.bb_max.tolist())
    dev_s = clipmap.samples_to_device(samples)
    ref, got, mirror = {}, {}, {}
    for mode in (8, 7):
        desc = _desc_mode(base_desc, mode)
        ref[mode] = oracle.svo_trace(64, bytes(desc), eye, want_pool, samples, bmin, bmax, shadow=sh_np,
                                     shadow_desc_bytes=sd_bytes)[:2]
        mirror[mode] = oracle.svo_trace(32, bytes(desc), eye, want_pool, samples, bmin, bmax, shadow=sh_np,
                                        shadow_desc_bytes=sd_bytes)[:2]
        dg, sg = passes.svo_cone_trace(desc, eye, pool, n, dev_s, bmin, bmax, light=light, shadow=sh_dev,
                                       shadow_desc=lsd)
        torch.cuda.synchronize()
        got[mode] = (dg.cpu().numpy(), sg.cpu().numpy())
        for g, w in zip(got[mode], mirror[mode]):
            err = np.abs(g - w).max(1) / np.maximum(np.abs(w).max(1), 1e-3)
            assert np.mean(err < 1e-4) > 0.99, (mode, np.sort(err)[-8:])
    _check_form(rows, f"svo_l{level}", _outputs(got[8], got[7]), _outputs(ref[8], ref[7]))
    rows[f"svo_l{level}_nodes"] = int(n)
    rows[f"svo_l{level}_fragments"] = int(F)


def _frame_bit_exact(torch, oracle, scene, R, cam, shadow_res):
    """The GPU frame (with its RGBA8 texture) against the oracle's passes; returns both sides' buffers."""
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    origin = _origin(cam)
    regions = oracle.clip_regions(cam, R)
    w_op = oracle.voxelize_opacity(scene, R, regions)
    for level in range(1, 6):
        oracle.downsample(w_op, R, regions[level - 1, 0:3], level, 0)
    oracle.wrap_border(w_op, R)
    sd_bytes = oracle.light_shadow_desc(origin, LIGHT_DIR)
    w_sh = oracle.shadow_depth(scene, sd_bytes, shadow_res, shadow_res)
    w_rad = oracle.inject_radiance(scene, R, regions, w_sh, sd_bytes)
    for level in range(6):
        oracle.copy_alpha(w_rad, w_op, R, level)
    for level in range(1, 6):
        oracle.downsample(w_rad, R, regions[level - 1, 0:3], level, 1)

    ds = passes.DeviceScene(scene)
    ws = passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((shadow_res, shadow_res), dtype=torch.float32, device="cuda")
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(origin, LIGHT_DIR)
    tex = clipmap.RadianceTexture(R)
    regs = passes.clipmap_frame(ds, cam, R, op, rad, sh, light, lsd, ws, texture=tex)
    torch.cuda.synchronize()
    assert np.array_equal(clipmap.regions_to_numpy(regs), regions)
    assert np.array_equal(sh.cpu().numpy().view(np.uint32), w_sh.view(np.uint32))
    g_op = op.cpu().numpy().view(np.uint32)
    assert np.array_equal(g_op, w_op), f"opacity: {np.count_nonzero(g_op != w_op)} texels differ"
    del g_op, op
    g_rad = rad.cpu().numpy().view(np.uint32)
    assert np.array_equal(g_rad, w_rad), f"radiance: {np.count_nonzero(g_rad != w_rad)} texels differ"
    assert np.count_nonzero(g_rad >> np.uint32(24)) > 10000
    del g_rad
    back = tex.read(clipmap.new_atlas(R))
    assert torch.equal(back, rad), "the frame's radiance texture differs from its atlas"
    del back
    torch.cuda.synchronize()
    return dict(regions=regions, rad_np=w_rad, sh_np=w_sh, sd_bytes=sd_bytes, ds=ds, ws=ws, rad=rad, sh=sh,
                light=light, lsd=lsd, tex=tex, regs=regs)


def test_benchmark_workload_hall_r256(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300.scene import hall_scene, surface_samples
    R, cam, eye = 256, (0.0, 5.0, 0.0), (0.0, 5.0, -12.0)
    scene = hall_scene(seed=2)
    assert scene.triangle_count >= 1_000_000
    f = _frame_bit_exact(torch, oracle, scene, R, cam, 2048)
    full = surface_samples(scene, 1920 * 1080, seed=12)  # the benchmark's samples
    pick = np.sort(np.random.default_rng(2).choice(full.shape[0], SUBSET, replace=False))
    samples = np.ascontiguousarray(full[pick])
    del full
    rows = {"samples": SUBSET, "of": 1920 * 1080, "R": R, "triangles": scene.triangle_count}
    base = _trace_all_forms(torch, oracle, rows, R, f["regions"], f["rad_np"], f["rad"], f["tex"], f["sh_np"],
                            f["sh"], samples, eye, f["light"], f["lsd"], f["sd_bytes"], f["regs"])
    f["tex"].close()
    del f["rad"], f["rad_np"]
    _svo_chain(torch, oracle, rows, scene, f["ds"], f["ws"], 8, f["sh_np"], f["sh"], f["sd_bytes"], f["light"],
               f["lsd"], base, samples, eye)
    _report("hall_1M_r256_bench_workload", rows)


def test_configuration_1_room_at_stated_size(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import room_scene, surface_samples
    R, cam, eye = 128, (0.0, 4.0, 0.0), (0.0, 4.0, -4.5)
    scene = room_scene(seed=1)
    assert 30000 < scene.triangle_count < 40000
    f = _frame_bit_exact(torch, oracle, scene, R, cam, 2048)
    samples = surface_samples(scene, 65536, seed=1)
    rows = {"samples": 65536, "R": R, "triangles": scene.triangle_count}
    base = _trace_all_forms(torch, oracle, rows, R, f["regions"], f["rad_np"], f["rad"], f["tex"], f["sh_np"],
                            f["sh"], samples, eye, f["light"], f["lsd"], f["sd_bytes"], f["regs"])
    # the configuration's own cone set: 16 fixed 30-degree cones (the shader's aperture constant is 50 degrees)
    ap = math.radians(30.0)
    want, got_t, got_e = {}, {}, {}
    dev_s = clipmap.samples_to_device(samples)
    for mode in (8, 7):
        desc = _desc_mode(base, mode)
        want[mode] = oracle.cone_trace(64, bytes(desc), eye, f["rad_np"], R, samples, shadow=f["sh_np"],
                                       shadow_desc_bytes=f["sd_bytes"], diffuse_aperture=ap)[:2]
        got_t[mode] = [t.cpu().numpy() for t in clipmap.cone_trace_fast(
            desc, eye, f["tex"], dev_s, light=f["light"], shadow=f["sh"], shadow_desc=f["lsd"], diffuse_aperture=ap)]
        got_e[mode] = [t.cpu().numpy() for t in clipmap.cone_trace(
            desc, eye, f["rad"], R, dev_s, light=f["light"], shadow=f["sh"], shadow_desc=f["lsd"],
            diffuse_aperture=ap)]
    w30 = _outputs(want[8], want[7])
    _check_form(rows, "texture_rgba8_30deg_cones", _outputs(got_t[8], got_t[7]), w30)
    _check_form(rows, "exact_rgba8_30deg_cones", _outputs(got_e[8], got_e[7]), w30)
    f["tex"].close()
    _svo_chain(torch, oracle, rows, scene, f["ds"], f["ws"], 7, f["sh_np"], f["sh"], f["sd_bytes"], f["light"],
               f["lsd"], base, samples, eye)
    _report("room_34k_r128_configuration_1", rows)
