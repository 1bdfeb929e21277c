#!/usr/bin/env python3
"""Headline benchmark of the voxel cone tracing core on one GPU.

Workload (configuration 2 of the reference's benchmark set, at the headline
clipmap resolution 256): a seeded procedural hall of 1,000,000 fp32 triangles
(instanced columns, arches, clutter; one RGBA8 albedo per triangle), camera at
(0, 5, 0), 6 clip levels x 6 faces of 256^3 (RGBA8 opacity and radiance
atlases, 2.47 GB each -- larger than L2), a directional light (0.3, -1, 0.2)
with a 2048^2 shadow map, and 1920x1080 area-uniform G-buffer samples with
face normals, roughness U(0.1, 0.9) and metallic U(0, 1): 16 diffuse cones,
one specular cone and VXAO per sample.

Metric: cone samples/s of the cone-tracing pass (one cone sample = one
iteration of traceCone's marching loop, voxelConeTracing.frag:361-389).  The
line also reports the frame time of voxelise + shadow + inject + mips and of
the SVO build (fragments + subdivide + leaf + mips) at 256^3.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--form tex|fp16|exact]

``--impl reference`` runs the CPU restatement of the reference's shaders (the
reference itself is GLSL under Vulkan, which this machine cannot run) on the
same workload: it builds the same clipmap on the host cores and times the
trace over a bounded prefix of the samples.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

R_DEFAULT = 256
N_SAMPLES = 1920 * 1080
SVO_LEVEL = 8
CAMERA = (0.0, 5.0, 0.0)
VIEW_DIR = (0.6, -0.2, 0.77)
EYE = (0.0, 5.0, -12.0)
LIGHT_DIR = (0.3, -1.0, 0.2)
SHADOW_RES = 2048
SCENE_SEED, SAMPLE_SEED = 2, 12
BYTES_PER_CONE_SAMPLE = {"exact": 192, "tex": 192, "fp16": 384}
METRIC = "cone samples/s (clipmap cone trace @256^3, 16 diffuse + specular cones)"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def light_origin():
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(CAMERA) - 15.0 * d).astype(np.float32).tolist())


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        num = lambda s: s.replace(".", "", 1).isdigit()
        sm = [float(r[1]) for r in rows if num(r[1])]
        mx = [float(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def aggregate(units: float, ms: float, world: int, device="cpu") -> tuple[float, float]:
    """The whole job's units (summed over the ranks) and the slowest rank's time (max over the ranks), over
    the job's process group (NCCL on the GPUs; any backend works); one rank returns its own values."""
    if world == 1:
        return float(units), float(ms)
    import torch
    import torch.distributed as dist
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item())


def make_inputs(n_samples: int, sample_seed: int):
    from vk_voxel_cone_tracing_gb300.scene import hall_scene, surface_samples
    scene = hall_scene(seed=SCENE_SEED)
    samples = surface_samples(scene, n_samples, seed=sample_seed)
    return scene, samples


def trace_desc_for(regions_np: np.ndarray, R: int):
    from vk_voxel_cone_tracing_gb300.clipmap import trace_desc
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc
    return trace_desc(**default_trace_desc(regions_np, R))


def cpu_trace_rate(R, desc, radiance, shadow, sd_bytes, samples, target_s):
    """Cone samples/s of the FP32 CPU restatement over a bounded prefix of `samples`."""
    from oracle import oracle
    n_probe = min(1024, samples.shape[0])
    t0 = time.perf_counter()
    oracle.cone_trace(32, bytes(desc), EYE, radiance, R, samples, shadow=shadow, shadow_desc_bytes=sd_bytes,
                      end=n_probe)
    dt = time.perf_counter() - t0
    n = int(min(samples.shape[0], max(n_probe, n_probe * target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    _, _, steps, _ = oracle.cone_trace(32, bytes(desc), EYE, radiance, R, samples, shadow=shadow,
                                       shadow_desc_bytes=sd_bytes, end=n)
    dt = time.perf_counter() - t0
    return steps / dt, n, steps, dt, oracle.num_threads()


def run_reference(args, world, rank):
    """The reference's path on the host cores: the C++ restatement of its shaders."""
    if rank != 0:
        return
    from oracle import oracle
    R = args.R
    scene, samples = make_inputs(N_SAMPLES, SAMPLE_SEED)
    t0 = time.perf_counter()
    regions = oracle.clip_regions(CAMERA, R)
    opacity = oracle.voxelize_opacity(scene, R, regions)
    for level in range(1, 6):
        oracle.downsample(opacity, R, regions[level - 1, 0:3], level, 0)
    oracle.wrap_border(opacity, R)
    sd = oracle.light_shadow_desc(light_origin(), LIGHT_DIR)
    shadow = oracle.shadow_depth(scene, sd, SHADOW_RES, SHADOW_RES)
    radiance = oracle.inject_radiance(scene, R, regions, shadow, sd)
    for level in range(6):
        oracle.copy_alpha(radiance, opacity, R, level)
    for level in range(1, 6):
        oracle.downsample(radiance, R, regions[level - 1, 0:3], level, 1)
    frame_s = time.perf_counter() - t0
    desc = trace_desc_for(regions, R)
    rates, info = [], None
    for i in range(args.warmup + args.steps):
        rate, n, steps, dt, cores = cpu_trace_rate(R, desc, radiance, shadow, sd, samples,
                                                   args.cpu_seconds / max(1, args.steps))
        if i >= args.warmup:
            rates.append(rate)
            info = (n, steps, dt, cores)
    v = float(statistics.median(rates))
    n, steps, dt, cores = info
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cone samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"hall scene 1M triangles, clipmap R={R}, 1920x1080 G-buffer samples "
                               f"(trace timed over a bounded prefix)", "samples_traced": n, "cone_samples": steps,
                   "frame_ms_cpu": frame_s * 1e3},
        "cpu_baseline": {"value": v, "unit": "cone samples/s", "cores": cores, "kind": "port",
                         "sample": f"first {n} of {N_SAMPLES} samples, FP32 C++ restatement of "
                                   "voxelConeTracing.frag; frame built by the restated passes"},
        "e2e": {"value": v, "unit": "cone samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's passes are GLSL under Vulkan, which this machine cannot run; the CPU "
                "restatement of its shaders is timed on all host threads",
    }
    print(json.dumps(line), flush=True)


def events_ms(stream, fn, reps):
    import torch
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(reps + 1)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for i in range(reps):
        fn()
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    return [ev[i].elapsed_time(ev[i + 1]) for i in range(reps)], ev[0].elapsed_time(ev[-1])


def run_ours(args, world, rank, local):
    import torch
    import torch.distributed as dist

    from vk_voxel_cone_tracing_gb300 import build, capi, clipmap, passes

    build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    R = args.R
    log(f"[bench] generating the scene and {args.samples} samples")
    scene, samples_np = make_inputs(args.samples, SAMPLE_SEED + rank)  # weak scaling: one frame per rank
    ds = passes.DeviceScene(scene, dev)
    ws = passes.Workspace()
    opacity = clipmap.new_atlas(R, dev)
    radiance = clipmap.new_atlas(R, dev)
    shadow = torch.empty((SHADOW_RES, SHADOW_RES), dtype=torch.float32, device=dev)
    light = passes.light_desc(LIGHT_DIR)
    lsd = passes.light_shadow_desc(light_origin(), LIGHT_DIR)
    stream = torch.cuda.current_stream()

    # the texture forms sample a texture the frame keeps equal to the atlas they trace: the RGBA8 form's
    # through the frame's copy-alpha and mip passes, the FP16 form's through its conversion and FP16 mip
    # passes (each texel those passes write is stored into the texture too)
    tex = clipmap.RadianceTexture(R, capi.TEX_RGBA8 if args.form != "fp16" else capi.TEX_RGBA16F) \
        if args.form in ("tex", "fp16") else None
    frame_tex = tex if args.form == "tex" else None
    atlas16 = clipmap.new_atlas_rgba16f(R, dev) if args.form == "fp16" else None

    def frame(frame_index: int = 0):
        regs = passes.clipmap_frame(ds, CAMERA, R, opacity, radiance, shadow, light, lsd, ws, texture=frame_tex,
                                    frame_index=frame_index)
        if atlas16 is not None:  # FP16 form: RGBA16F radiance with FP16 mips, mirrored into its texture
            clipmap.to_rgba16f(radiance, R, out=atlas16, mirror=tex)
            clipmap.cmd_downsample_rgba16f_all(atlas16, R, regs, 1, mirror=tex)
        return regs

    regs = frame()
    torch.cuda.synchronize()
    regions_np = clipmap.regions_to_numpy(regs)
    desc = trace_desc_for(regions_np, R)

    samples = clipmap.samples_to_device(samples_np, dev)
    n = samples.shape[0]
    dout = torch.empty((n, 4), dtype=torch.float32, device=dev)
    sout = torch.empty((n, 4), dtype=torch.float32, device=dev)
    steps_ctr = torch.zeros(1, dtype=torch.int64, device=dev)
    tex_src, scratch = (atlas16 if atlas16 is not None else radiance), None
    if tex is not None:
        scratch = clipmap.fast_scratch(n, dev)

    def trace(inp, counter=None):
        if tex is None:
            clipmap.cone_trace(desc, EYE, radiance, R, inp, light=light, shadow=shadow, shadow_desc=lsd,
                               diffuse=dout, specular=sout, steps=counter)
        else:
            clipmap.cone_trace_fast(desc, EYE, tex, inp, light=light, shadow=shadow, shadow_desc=lsd, diffuse=dout,
                                    specular=sout, steps=counter, scratch=scratch)

    trace(samples, steps_ctr)
    torch.cuda.synchronize()
    cone_samples = int(steps_ctr.item())
    # the launch-shape autotuner (result-neutral shapes) on these inputs, before the timed steps
    tuning = clipmap.autotune_fast(desc, EYE, tex, samples, light=light, shadow=shadow, shadow_desc=lsd,
                                   diffuse=dout, specular=sout, scratch=scratch) if tex is not None else None
    for _ in range(args.warmup):
        trace(samples)
    if world > 1:
        dist.barrier()
    with Clocks(local) as clocks:
        per, total_ms = events_ms(stream, lambda: trace(samples), args.steps)
    total_cone_samples, total_ms = aggregate(cone_samples, total_ms, world, dev)
    ms = total_ms / args.steps
    value = total_cone_samples / (ms * 1e-3)
    # the trace's speed of light: the same fetches per cone sample with nothing else (vct_gather_probe)
    gather_peak = clipmap.gather_probe(desc, tex) if tex is not None else None
    # what a full clipmap -> texture array copy (vct_texture_update) costs; the texture forms need none per step
    refresh_ms = statistics.median(events_ms(stream, lambda: tex.update(tex_src), 5)[0]) if tex is not None else None
    if tex is not None:
        frame()  # the measurement above overwrote the texture with the same atlas; keep the frame's state

    # voxelise + shadow + inject + mips of one frame, and the SVO build at 256^3
    for _ in range(2):
        frame()
    frame_per, _ = events_ms(stream, frame, max(3, args.steps))
    frags = passes.svo_fragments(ds, SVO_LEVEL, shadow, light, lsd, ws)
    pool_cap = passes.svo_pool_capacity(frags.shape[0])
    pool = torch.empty((pool_cap, 2), dtype=torch.int32, device=dev)
    import ctypes as C
    nodes = C.c_int64(0)

    svo_buf = torch.empty((int(frags.shape[0] * 1.25) + 1024, 2), dtype=torch.int32, device=dev)

    def svo():  # one fragment-list call per build: the buffer is sized from the first frame's count
        f = passes.svo_fragments(ds, SVO_LEVEL, shadow, light, lsd, ws, out=svo_buf)
        capi.call("vct_svo_build", f.data_ptr(), f.shape[0], SVO_LEVEL, pool.data_ptr(), pool_cap,
                  capi.SVO_DETERMINISTIC, C.byref(nodes), ws.handle, C.c_void_p(stream.cuda_stream))

    svo()
    svo_per, _ = events_ms(stream, svo, max(3, args.steps))
    frame_ms = statistics.median(frame_per)
    opacity_r8 = frame_r8_opacity(dev, stream, ds, R, shadow, light, lsd, ws, radiance, frame_tex, args.steps) \
        if args.form == "tex" else None
    # the conservative voxelisation mode over the same levels (into the opacity atlas; the frame after the
    # moving-camera runs below restores it)
    cons = lambda: passes.voxelize_opacity_conservative(ds, regs, R, opacity)
    passes.clear_atlas(opacity, R)
    cons()
    cons_voxels = int((opacity != 0).sum().item()) // 6
    cons_ms = statistics.median(events_ms(stream, cons, 3)[0])
    svo_ms = statistics.median(svo_per)
    # the SVO cone trace (voxelConeTracing_Octree.frag) over the first 262144 samples of the octree just built,
    # with the scene's bounding box (the reference's hard-coded Sponza box does not fit the hall scene)
    svo_n = min(n, 262144)
    svo_steps = torch.zeros(1, dtype=torch.int64, device=dev)
    svo_trace = lambda counter=None: passes.svo_cone_trace(desc, EYE, pool, int(nodes.value), samples[:svo_n],
                                                          bb_min=ds.bb_min, bb_max=ds.bb_max, light=light,
                                                          shadow=shadow, shadow_desc=lsd, steps=counter)
    svo_trace(svo_steps)
    torch.cuda.synchronize()
    svo_trace_ms = statistics.median(events_ms(stream, svo_trace, 3)[0])
    svo_trace_rate = int(svo_steps.item()) / (svo_trace_ms * 1e-3)

    # a moving camera over the 32-frame radiance cadence (level l refreshed every 2^l frames): the mean
    # frame time with full revoxelisation every frame (the reference as shipped) and with the toroidal
    # update (only the slabs the move uncovers are revoxelised)
    import ctypes as C
    path = [(CAMERA[0] + 0.05 * k, CAMERA[1], CAMERA[2] + 0.03 * k) for k in range(33)]
    walk_ms = {}
    for mode in (capi.REVOX_FULL, capi.REVOX_TOROIDAL):
        state = (capi.ClipmapRegion * 6)()
        passes.clipmap_frame(ds, path[0], R, opacity, radiance, shadow, light, lsd, ws, frame_index=0,
                             texture=frame_tex, regions_state=state)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for k in range(1, 33):
            passes.clipmap_frame(ds, path[k], R, opacity, radiance, shadow, light, lsd, ws, frame_index=k,
                                 texture=frame_tex, revoxelization=mode, regions_state=state)
        t1.record(stream)
        torch.cuda.synchronize()
        walk_ms["full" if mode == capi.REVOX_FULL else "toroidal"] = t0.elapsed_time(t1) / 32
    frame()  # back to the bench camera's clipmap for what follows

    # the camera's view: G-buffer at 1920x1080 for a camera in the hall, the trace over its pixels, the
    # specular filter and the sRGB present -- the passes of a rendered frame after the clipmap frame
    from vk_voxel_cone_tracing_gb300 import render
    GW, GH = 1920, 1080
    cam = passes.camera_matrix(CAMERA, VIEW_DIR, (0.0, 1.0, 0.0), 60.0, GW / GH)
    gb = torch.empty((GW * GH, 20), dtype=torch.float32, device=dev)
    cd = torch.empty((GW * GH, 4), dtype=torch.float32, device=dev)
    cs = torch.empty((GW * GH, 4), dtype=torch.float32, device=dev)
    img = torch.empty((GW * GH, 4), dtype=torch.float32, device=dev)
    srgb = torch.empty((GH, GW), dtype=torch.int32, device=dev)
    clear = torch.tensor([0.0, 0.0, 0.0, 1.0], device=dev)
    fdesc = render.filter_desc()
    bdesc = render.filter_desc(method=capi.FILTER_BILATERAL)
    cam_scratch = clipmap.fast_scratch(GW * GH, dev) if tex is not None else None

    def cam_trace():
        cd.copy_(clear.expand_as(cd))
        cs.copy_(clear.expand_as(cs))
        if tex is None:
            clipmap.cone_trace(desc, CAMERA, radiance, R, gb, light=light, shadow=shadow, shadow_desc=lsd,
                               diffuse=cd, specular=cs)
        else:
            clipmap.cone_trace_fast(desc, CAMERA, tex, gb, light=light, shadow=shadow, shadow_desc=lsd,
                                    diffuse=cd, specular=cs, scratch=cam_scratch)

    stages = {
        "gbuffer": lambda: passes.gbuffer(ds, cam, GW, GH, ws, out=gb),
        "trace": cam_trace,
        "filter_gaussian": lambda: render.specular_filter(cd, cs, GW, GH, fdesc, out=img),
        "filter_bilateral": lambda: render.specular_filter(cd, cs, GW, GH, bdesc, out=img),
        "present": lambda: render.present_srgb8(img, GW, GH, out=srgb),
    }
    cam_ms = {}
    for name, fn in stages.items():
        for _ in range(2):
            fn()
        cam_ms[name] = statistics.median(events_ms(stream, fn, max(3, args.steps))[0])
    cam_steps = torch.zeros(1, dtype=torch.int64, device=dev)
    if tex is None:
        clipmap.cone_trace(desc, CAMERA, radiance, R, gb, light=light, shadow=shadow, shadow_desc=lsd,
                           diffuse=cd, specular=cs, steps=cam_steps)
    else:
        clipmap.cone_trace_fast(desc, CAMERA, tex, gb, light=light, shadow=shadow, shadow_desc=lsd, diffuse=cd,
                                specular=cs, steps=cam_steps, scratch=cam_scratch)
    covered = int((gb[:, 3] < 1.0).sum().item())

    def rendered_frame():
        frame()
        stages["gbuffer"]()
        cam_trace()
        stages["filter_gaussian"]()
        stages["present"]()

    for _ in range(2):
        rendered_frame()
    rendered_ms = statistics.median(events_ms(stream, rendered_frame, max(3, args.steps))[0])
    filter_bytes = GW * GH * 48  # diffuse + specular texel read, output written (RGBA32F)

    forms = other_forms(dev, stream, R, regs, desc, radiance, samples, light, shadow, lsd, max(3, args.steps)) \
        if args.form == "tex" and not args.no_batch and world == 1 else None
    if forms is not None:
        rate_tex = cone_samples / (ms * 1e-3)
        forms["texture_rgba8"] = {"trace_ms": ms, "cone_samples_per_s": rate_tex}
        forms["ratio_fp16_vs_exact_fp32"] = forms["texture_rgba16f"]["cone_samples_per_s"] / \
            forms["exact_rgba8"]["cone_samples_per_s"]
        forms["ratio_rgba8_texture_vs_exact_fp32"] = rate_tex / forms["exact_rgba8"]["cone_samples_per_s"]
        frame()  # restore the RGBA8 texture the frame keeps (the FP16 section used its own)
    batch = batched_scenes(dev) if not args.no_batch and world == 1 else None
    diff = differentiable_volume(dev) if not args.no_batch and world == 1 else None
    svo_large = large_svo(dev, max(3, args.steps)) if not args.no_batch and world == 1 else None

    # end to end: host G-buffer -> device, frame, trace, outputs -> host
    h_samples = samples.cpu().pin_memory()
    h_d = torch.empty(dout.shape, dtype=torch.float32).pin_memory()
    h_s = torch.empty(sout.shape, dtype=torch.float32).pin_memory()
    d_in = torch.empty_like(samples)

    copy_stream = torch.cuda.Stream(device=dev)
    uploaded, traced, read_back = torch.cuda.Event(), torch.cuda.Event(), torch.cuda.Event()

    frame_counter = [0]

    def e2e_step():
        # one frame of the reference's loop: full opacity revoxelisation, radiance level l refreshed every
        # 2^l frames (the frame index advances per step), then the trace.  The copies run on a copy stream:
        # the G-buffer upload overlaps the frame (which does not read it) after the previous step's trace
        # has read d_in; the outputs' readback overlaps the next step's frame, whose trace waits for it
        # before writing the outputs again
        copy_stream.wait_event(traced)
        with torch.cuda.stream(copy_stream):
            d_in.copy_(h_samples, non_blocking=True)
            uploaded.record(copy_stream)
        frame(frame_counter[0])
        frame_counter[0] += 1
        stream.wait_event(uploaded)
        stream.wait_event(read_back)
        trace(d_in)
        traced.record(stream)
        copy_stream.wait_event(traced)
        with torch.cuda.stream(copy_stream):
            h_d.copy_(dout, non_blocking=True)
            h_s.copy_(sout, non_blocking=True)
            read_back.record(copy_stream)

    traced.record(stream)
    read_back.record(copy_stream)
    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    stream.wait_event(read_back)  # the last step's outputs are on the host inside the timed region
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_total = e0.elapsed_time(e1)
    _, e2e_total = aggregate(cone_samples, e2e_total, world, dev)
    e2e_ms = e2e_total / args.steps

    if rank == 0:
        peak, peak_kind = measured_peaks()
        bpcs = BYTES_PER_CONE_SAMPLE[args.form]
        achieved = cone_samples * bpcs / (statistics.mean(per) * 1e-3) / 1e9
        traffic = None
        prof = ROOT / "profiles" / f"cone_trace_{args.form}_r{R}.txt"
        if prof.exists():
            for line in prof.read_text().splitlines():
                if line.startswith("dram_bytes_per_launch_full:"):
                    traffic = float(line.split(":")[1])
        log(f"[bench] cone samples/step={cone_samples} trace ms={ms:.3f} frame ms={frame_ms:.3f} "
            f"svo ms={svo_ms:.3f} e2e ms={e2e_ms:.3f}")
        cpu = None
        if not args.no_cpu:
            rad_np = radiance.cpu().numpy().view(np.uint32)
            sh_np = shadow.cpu().numpy()
            rate, ncpu, st, dt, cores = cpu_trace_rate(R, desc, rad_np, sh_np, bytes(lsd), samples_np, args.cpu_seconds)
            cpu = {"value": rate, "unit": "cone samples/s", "cores": cores, "kind": "port",
                   "sample": f"first {ncpu} of {n} samples ({st} cone samples, {dt:.1f} s) traced by the FP32 C++ "
                             "restatement on the same clipmap"}
        # kernels launched per trace step: Morton keys, cub radix sort of 30 bits (histogram, exclusive sum,
        # 4 onesweep passes), specular keys, cub radix pass on 1 bit (histogram, exclusive sum, onesweep),
        # diffuse, specular (the texture refresh is a memcpy, not a kernel)
        launches = 1 if tex is None else 13
        line = {
            "metric": METRIC, "value": value, "unit": "cone samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"hall scene ({scene.triangle_count} fp32 triangles), clipmap R={R} "
                                   "(6 levels x 6 faces, RGBA8 opacity + radiance atlases of 2.47 GB), "
                                   "1920x1080 G-buffer samples, 16 diffuse + 1 specular cone + VXAO",
                       "form": args.form, "R": R, "samples_per_step": n, "cone_samples_per_step": cone_samples,
                       "l2": "inputs larger than L2 (2.47 GB clipmap)",
                       "texture_full_copy_ms": refresh_ms, "trace_tuning": tuning,
                       "texture": "kept current by the frame's copy-alpha and mip passes" if frame_tex is not None
                       else ("kept current by the frame's FP16 conversion and FP16 mip passes" if tex is not None
                             else "none (linear atlas)"),
                       "voxelize_inject_mip_ms": frame_ms, "frame_r8_opacity": opacity_r8,
                       "svo_ms": svo_ms, "svo_level": SVO_LEVEL,
                       "conservative_voxelize": {"ms": cons_ms, "voxels": cons_voxels,
                                                 "note": "triangle/box overlap mode (Schwarz & Seidel 2010), "
                                                         "6 levels of 256^3; voxels marked over all levels"},
                       "svo_fragments": int(frags.shape[0]), "svo_nodes": int(nodes.value),
                       "svo_trace": {"samples": svo_n, "ms": svo_trace_ms, "cone_samples_per_s": svo_trace_rate},
                       "voxelize_svo_mip_ms": frame_ms + svo_ms,
                       "forms": forms,
                       "batched_scenes": batch,
                       "differentiable": diff,
                       "svo_large": svo_large,
                       "moving_camera_frame_ms": walk_ms,
                       "moving_camera": "32 frames (the whole radiance cadence) along a path of 0.06 per frame; "
                                        "mean frame time, full revoxelisation vs the toroidal update",
                       "camera_view": {
                           "resolution": [GW, GH], "camera": list(CAMERA), "direction": list(VIEW_DIR),
                           "covered_pixels": covered, "cone_samples": int(cam_steps.item()),
                           "stage_ms": cam_ms,
                           "trace_cone_samples_per_s": int(cam_steps.item()) / (cam_ms["trace"] * 1e-3),
                           "filter_gaussian_gbs": filter_bytes / (cam_ms["filter_gaussian"] * 1e-3) / 1e9,
                           "rendered_frame_ms": rendered_ms,
                           "rendered_frame": "clipmap frame + G-buffer + trace + Gaussian specular filter + "
                                             "sRGB present, all on the device"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": f"{bpcs} B of algorithmic texel reads per cone sample over the {peak_kind} HBM "
                                 "copy peak, per trace step (CUDA events around the step: Morton sort, specular "
                                 "partition, diffuse and specular kernels; the specular kernel is about 71 % of it "
                                 "in the ncu launch list); the taps are served mostly from L1/TEX and L2, so the "
                                 "figure exceeds the HBM peak; traffic = ncu DRAM bytes of one step"},
            "gather_roofline": None if gather_peak is None else {
                "bound": "l1tex/l2 gather", "achieved": cone_samples / (statistics.mean(per) * 1e-3),
                "peak": gather_peak, "unit": "cone samples/s",
                "frac": cone_samples / (statistics.mean(per) * 1e-3) / gather_peak,
                "note": "peak = vct_gather_probe: the texture fetches of one cone sample (3 faces x 2 levels, "
                        "trilinear) per step of warp-coherent synthetic cones, measured on this GPU with the same "
                        "texture; achieved = the whole trace step (Morton sort, specular partition, diffuse and "
                        "specular kernels)"},
            "cpu_baseline": cpu,
            "e2e": {"value": total_cone_samples / (e2e_ms * 1e-3), "unit": "cone samples/s",
                    "h2d_bytes_per_step": int(samples.numel() * 4),
                    "d2h_bytes_per_step": int((dout.numel() + sout.numel()) * 4),
                    "step": "G-buffer upload (overlapping the frame) + one frame of the reference's loop "
                            "(full opacity revoxelisation, shadow, radiance levels due at the frame index: level "
                            "l every 2^l frames) + trace + output readback (on a copy stream, overlapping the "
                            "next step's frame; the last step's readback inside the timed region)",
                    "frames": f"frame indices {args.warmup}..{args.warmup + args.steps - 1} timed after "
                              f"{args.warmup} warm-up frames"},
            "gpu_launches": args.steps * launches,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if tex is not None:
        tex.close()
    if world > 1:
        dist.destroy_process_group()


def frame_r8_opacity(dev, stream, ds, R, shadow, light, lsd, ws, radiance, tex, steps):
    """The same frame with the one-byte opacity atlas (vct_frame_desc.opacity_format = R8): CUDA events,
    median; its radiance atlas is compared bit for bit with the RGBA8 frame's (`radiance`, current)."""
    import torch
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    ref = radiance.clone()
    op8, rad8 = clipmap.new_atlas_r8(R, dev), clipmap.new_atlas(R, dev)
    tex8 = clipmap.RadianceTexture(R)

    def frame8():
        passes.clipmap_frame(ds, CAMERA, R, op8, rad8, shadow, light, lsd, ws, texture=tex8 if tex is not None else None,
                             opacity_format=capi.OPACITY_R8)

    for _ in range(2):
        frame8()
    per, _ = events_ms(stream, frame8, max(3, steps))
    torch.cuda.synchronize()
    equal = bool(torch.equal(rad8, ref))
    tex8.close()
    del op8, rad8, ref
    return {"frame_ms": statistics.median(per), "radiance_bit_equal": equal,
            "opacity_bytes": int(atlas_bytes(R) // 4),
            "note": "opacity stored one byte per texel (alpha only): a quarter of the RGBA8 opacity atlas's clear, "
                    "voxelisation, mip, border and copy-alpha traffic; radiance atlas and texture unchanged"}


def atlas_bytes(R: int) -> int:
    return 4 * (R + 2) * 36 * (R + 2) * (R + 2)


def other_forms(dev, stream, R, regs, desc, radiance, samples, light, shadow, lsd, reps):
    """The two other forms of the trace on the benchmark's frame and samples: the FP16-storage form (the
    frame's radiance converted to RGBA16F with FP16 mips, written into an RGBA16F texture as the passes run;
    FP32 compositing) and the exact FP32 drop-in (software trilinear over the linear RGBA8 atlas, the
    shader's arithmetic).  CUDA events on the launching stream, median over `reps`."""
    import torch

    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    n = samples.shape[0]
    dout = torch.empty((n, 4), dtype=torch.float32, device=dev)
    sout = torch.empty((n, 4), dtype=torch.float32, device=dev)
    out = {}
    tex16 = clipmap.RadianceTexture(R, capi.TEX_RGBA16F)
    a16 = clipmap.new_atlas_rgba16f(R, dev)

    def fp16_passes():
        clipmap.to_rgba16f(radiance, R, out=a16, mirror=tex16)
        clipmap.cmd_downsample_rgba16f_all(a16, R, regs, 1, mirror=tex16)

    scratch = clipmap.fast_scratch(n, dev)

    def fp16_trace(counter=None):
        clipmap.cone_trace_fast(desc, EYE, tex16, samples, light=light, shadow=shadow, shadow_desc=lsd, diffuse=dout,
                                specular=sout, steps=counter, scratch=scratch)

    for _ in range(2):
        fp16_passes()
    passes_ms = statistics.median(events_ms(stream, fp16_passes, reps)[0])
    ctr = torch.zeros(1, dtype=torch.int64, device=dev)
    fp16_trace(ctr)
    for _ in range(2):
        fp16_trace()
    t16 = statistics.median(events_ms(stream, fp16_trace, reps)[0])
    c16 = int(ctr.item())
    out["texture_rgba16f"] = {"trace_ms": t16, "cone_samples": c16, "cone_samples_per_s": c16 / (t16 * 1e-3),
                              "conversion_and_fp16_mips_ms": passes_ms,
                              "note": "radiance mips recomputed in FP16 from level 0, FP32 compositing"}
    tex16.close()
    del a16, scratch

    def exact_trace(counter=None):
        clipmap.cone_trace(desc, EYE, radiance, R, samples, light=light, shadow=shadow, shadow_desc=lsd,
                           diffuse=dout, specular=sout, steps=counter)

    ctr.zero_()
    exact_trace(ctr)
    exact_trace()
    te = statistics.median(events_ms(stream, exact_trace, reps)[0])
    ce = int(ctr.item())
    out["exact_rgba8"] = {"trace_ms": te, "cone_samples": ce, "cone_samples_per_s": ce / (te * 1e-3),
                          "note": "the plain FP32 drop-in: software trilinear over the linear RGBA8 atlas"}
    # the same exact arithmetic with its texels read through a texture holding the atlas (vct_cone_trace_tex);
    # its outputs are compared bit for bit with the linear-atlas trace's
    tex8 = clipmap.RadianceTexture(R).update(radiance)
    ref_d, ref_s = dout.clone(), sout.clone()

    def exact_tex_trace(counter=None):
        clipmap.cone_trace_tex(desc, EYE, tex8, samples, light=light, shadow=shadow, shadow_desc=lsd,
                               diffuse=dout, specular=sout, steps=counter)

    ctr.zero_()
    exact_tex_trace(ctr)
    torch.cuda.synchronize()
    equal = bool(torch.equal(dout, ref_d) and torch.equal(sout, ref_s))
    exact_tex_trace()
    tx = statistics.median(events_ms(stream, exact_tex_trace, reps)[0])
    upd = statistics.median(events_ms(stream, lambda: tex8.update(radiance), reps)[0])
    cx = int(ctr.item())
    out["exact_rgba8_texel_reads"] = {
        "trace_ms": tx, "cone_samples": cx, "cone_samples_per_s": cx / (tx * 1e-3), "texture_update_ms": upd,
        "outputs_bit_equal_to_exact_rgba8": equal, "speedup_vs_exact_rgba8": te / tx,
        "note": "vct_cone_trace_tex: the exact FP32 arithmetic, each texel one point-sampled texture fetch "
                "(decoded exactly by the texture unit) from a texture holding the atlas (the one a frame keeps "
                "current, or vct_texture_update: texture_update_ms)"}
    tex8.close()
    return out


def batched_trace_phase(dev, jobs, keep, ctxs, streams, grids):
    """The traces of the batch on their own: every scene's clipmap is rebuilt by its frame and copied into a
    texture of its own, then the 64 traces run (a) as 64 vct_cone_trace_fast calls back to back on one stream
    and (b) as one vct_cone_trace_fast_batch call (one launch per stage over the work queue of all jobs).
    CUDA events, median of 5; the outputs of (a) and (b) are compared bit for bit."""
    import torch
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, engine
    stream = torch.cuda.current_stream()
    texes, descs, outs, records = [], [], [], []
    for i, j in enumerate(jobs):
        engine.batch_submit([j], 1)
        ctx = ctxs[(i % streams, int(grids[i]))]
        b = ctx.buffers()
        R = int(grids[i])
        tex = clipmap.RadianceTexture(R).update(ctx.atlas("radiance"))
        r0 = b.regions[0]
        d = capi.ConeTracingDesc.from_buffer_copy(bytes(keep[i][3]))
        for a in range(3):
            d.volume_center[a] = float(np.float32(r0.min_corner[a]) * np.float32(r0.voxel_size) +
                                       (np.float32(r0.extent[a]) * np.float32(r0.voxel_size)) * np.float32(0.5))
        d.voxel_size = r0.voxel_size
        d.volume_dimension = float(R)
        smp = keep[i][2]
        n = smp.shape[0]
        o = (torch.empty((n, 4), device=dev), torch.empty((n, 4), device=dev),
             torch.empty((n, 4), device=dev), torch.empty((n, 4), device=dev))
        shadow = engine._device_view(b.shadow_depth, (1024, 1024)).view(torch.float32).clone()
        texes.append(tex)
        descs.append(d)
        outs.append((o, shadow, j.light, j.light_shadow))
        records.append(clipmap.trace_job(d, keep[i][6], tex, smp, o[2], o[3], light=j.light, shadow=shadow,
                                         shadow_desc=j.light_shadow))
    torch.cuda.synchronize()
    scratch_one = clipmap.fast_scratch(max(k[2].shape[0] for k in keep), dev)

    def separate():
        for i in range(len(jobs)):
            o, shadow, light, lsd = outs[i]
            clipmap.cone_trace_fast(descs[i], keep[i][6], texes[i], keep[i][2], light=light, shadow=shadow,
                                    shadow_desc=lsd, diffuse=o[0], specular=o[1], scratch=scratch_one)

    arr = (capi.TraceJob * len(records))(*records)
    need = capi.lib().vct_cone_trace_fast_batch_scratch_bytes(ctypes_void(arr), len(records))
    scratch_all = torch.empty(need + 256, dtype=torch.uint8, device=dev)

    def batched():
        clipmap.cone_trace_fast_batch(records, scratch_all)

    separate()
    batched()
    torch.cuda.synchronize()
    equal = all(torch.equal(o[0], o[2]) and torch.equal(o[1], o[3]) for o, *_ in outs)
    sep_ms = statistics.median(events_ms(stream, separate, 5)[0])
    bat_ms = statistics.median(events_ms(stream, batched, 5)[0])
    for t in texes:
        t.close()
    return {"separate_calls_ms": sep_ms, "one_batched_call_ms": bat_ms, "outputs_bit_equal": equal,
            "note": "trace phase only: the 64 scenes' traces as 64 vct_cone_trace_fast calls on one stream vs one "
                    "vct_cone_trace_fast_batch call; CUDA events, median of 5"}


def ctypes_void(arr):
    import ctypes as C
    return C.cast(arr, C.c_void_p)


def batched_scenes(dev, streams: int = 4, n_scenes: int = 64, seed: int = 4):
    """Configuration 4: independent scenes (triangles log-uniform 10k-500k, clipmap R in {64, 128, 256},
    G-buffer samples log-uniform 4k-256k), one full frame + one trace each, submitted as one batch over
    `streams` streams (vct_batch_submit) and one scene at a time; host wall clock around each submission
    (it returns when the work is done)."""
    import torch
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, engine, passes
    from vk_voxel_cone_tracing_gb300.scene import room_scene, surface_samples, default_trace_desc
    rng = np.random.default_rng(seed)
    tris = np.exp(rng.uniform(np.log(1e4), np.log(5e5), n_scenes)).astype(int)
    grids = rng.choice([64, 128, 256], n_scenes)
    nsamp = np.exp(rng.uniform(np.log(4096), np.log(262144), n_scenes)).astype(int)
    ctxs = {(t, int(R)): engine.Context(int(R), shadow_size=1024) for t in range(streams) for R in set(grids.tolist())}
    jobs, keep, steps = [], [], []
    for i in range(n_scenes):
        sc = room_scene(seed=1000 + i, n_random=max(int(tris[i]) - 14000, 1000))
        ds = passes.DeviceScene(sc, dev)
        R = int(grids[i])
        cam = (float(rng.uniform(-5, 5)), float(rng.uniform(1, 6)), float(rng.uniform(-3, 3)))
        d = np.asarray(LIGHT_DIR, np.float64)
        d /= np.linalg.norm(d)
        light = passes.light_desc(LIGHT_DIR)
        lsd = passes.light_shadow_desc(tuple((np.asarray(cam) - 15.0 * d).astype(np.float32).tolist()), LIGHT_DIR)
        smp = clipmap.samples_to_device(surface_samples(sc, int(nsamp[i]), seed=i), dev)
        td = clipmap.trace_desc(**default_trace_desc(np.zeros((6, 7), np.int32), R))
        dout = torch.empty((smp.shape[0], 4), dtype=torch.float32, device=dev)
        sout = torch.empty_like(dout)
        st = torch.zeros(1, dtype=torch.int64, device=dev)
        jobs.append(engine.batch_job(ctxs[(i % streams, R)], ds, cam, light, lsd, td, cam, smp, dout, sout, st))
        keep.append((sc, ds, smp, td, dout, sout, cam))
        steps.append(st)
    engine.batch_submit(jobs, streams)  # warm-up: workspaces and trace scratch reach their sizes
    torch.cuda.synchronize()
    cone_samples = int(sum(int(st.item()) for st in steps))
    t0 = time.perf_counter()
    engine.batch_submit(jobs, streams)
    batched = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    engine.batch_submit(jobs, 1)
    sequential = (time.perf_counter() - t0) * 1e3
    per = []
    for j in jobs:
        t0 = time.perf_counter()
        engine.batch_submit([j], 1)
        per.append((time.perf_counter() - t0) * 1e3)
    trace_phase = batched_trace_phase(dev, jobs, keep, ctxs, streams, grids)
    ref_out = [(k[4].clone(), k[5].clone()) for k in keep]
    for c in ctxs.values():
        c.close()
    # the same batch with contexts that keep their opacity atlas one byte per texel (VCT_CONTEXT_OPACITY_R8)
    ctx8 = {(t, int(R)): engine.Context(int(R), shadow_size=1024, flags=capi.CONTEXT_OPACITY_R8)
            for t in range(streams) for R in set(grids.tolist())}
    jobs8 = [engine.batch_job(ctx8[(i % streams, int(grids[i]))], k[1], k[6], j.light, j.light_shadow, k[3], k[6],
                              k[2], k[4], k[5]) for i, (j, k) in enumerate(zip(jobs, keep))]
    engine.batch_submit(jobs8, streams)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.batch_submit(jobs8, streams)
    batched_r8 = (time.perf_counter() - t0) * 1e3
    torch.cuda.synchronize()
    r8_equal = all(torch.equal(k[4], a) and torch.equal(k[5], b) for k, (a, b) in zip(keep, ref_out))
    for c in ctx8.values():
        c.close()
    return {"scenes": n_scenes, "triangles": int(tris.sum()), "samples": int(nsamp.sum()),
            "grids": {str(k): int((grids == k).sum()) for k in (64, 128, 256)}, "streams": streams,
            "cone_samples": cone_samples, "batched_ms": batched, "one_at_a_time_ms": sequential,
            "batched_cone_samples_per_s": cone_samples / (batched * 1e-3),
            "per_scene_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
            "trace_phase": trace_phase,
            "batched_r8_opacity_ms": batched_r8, "r8_outputs_bit_equal": r8_equal,
            "note": "each job: a full clipmap frame (voxelise, shadow, inject, mips) + the fast trace of its "
                    "samples; host wall clock, the submission synchronises"}


def large_svo(dev, reps: int, level: int = 9, n_samples: int = 4 << 20, seed: int = 3):
    """Configuration 3: the sparse-voxel-octree chain at 512^3 (level 9) over the 4M-triangle terrain scene
    (gradient-noise terrain + 10k boxes): the fragment list (vct_svo_fragments), the octree build
    (vct_svo_build: subdivision, leaf fold, mips) and the octree cone trace (vct_svo_cone_trace) of
    `n_samples` area-uniform surface samples with 16 diffuse cones + the specular cone.  CUDA events on the
    stream, median of `reps`."""
    import ctypes as C

    import torch
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, surface_samples, terrain_scene
    stream = torch.cuda.current_stream()
    sc = terrain_scene(seed=seed)
    ds = passes.DeviceScene(sc, dev)
    ws = passes.Workspace()
    light = passes.light_desc(LIGHT_DIR)
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    lsd = passes.light_shadow_desc(tuple((np.array([0.0, 1.5, 0.0]) - 15.0 * d).astype(np.float32).tolist()),
                                   LIGHT_DIR)
    shadow = torch.empty((SHADOW_RES, SHADOW_RES), dtype=torch.float32, device=dev)
    passes.shadow_depth(ds, lsd, shadow, ws)
    frags = passes.svo_fragments(ds, level, shadow, light, lsd, ws)
    F = int(frags.shape[0])
    buf = torch.empty((int(F * 1.25) + 1024, 2), dtype=torch.int32, device=dev)
    pool_cap = passes.svo_pool_capacity(F)
    pool = torch.empty((pool_cap, 2), dtype=torch.int32, device=dev)
    nodes = C.c_int64(0)
    del frags
    holder = [None]

    def fragments():
        holder[0] = passes.svo_fragments(ds, level, shadow, light, lsd, ws, out=buf)

    def build():
        f = holder[0]
        capi.call("vct_svo_build", f.data_ptr(), f.shape[0], level, pool.data_ptr(), pool_cap,
                  capi.SVO_DETERMINISTIC, C.byref(nodes), ws.handle, C.c_void_p(stream.cuda_stream))

    for _ in range(2):
        fragments()
        build()
    frag_ms = statistics.median(events_ms(stream, fragments, reps)[0])
    build_ms = statistics.median(events_ms(stream, build, reps)[0])
    # octree trace: volume dimension 2^level over the scene's own box (the reference hard-codes Sponza's)
    regions = clipmap.regions_to_numpy(clipmap.clip_regions((0.0, 3.0, 0.0), 1 << level))
    kw = default_trace_desc(regions, 1 << level)
    desc = clipmap.trace_desc(**kw)
    samples = clipmap.samples_to_device(surface_samples(sc, n_samples, seed=seed), dev)
    steps = torch.zeros(1, dtype=torch.int64, device=dev)
    eye = (0.0, 6.0, -20.0)
    bmin, bmax = tuple(ds.bb_min.tolist()), tuple(ds.bb_max.tolist())

    def trace(counter=None):
        passes.svo_cone_trace(desc, eye, pool, int(nodes.value), samples, bb_min=bmin, bb_max=bmax, light=light,
                              shadow=shadow, shadow_desc=lsd, steps=counter)

    trace(steps)
    torch.cuda.synchronize()
    cone_samples = int(steps.item())
    trace_ms = statistics.median(events_ms(stream, trace, reps)[0])
    # algorithmic bytes of the build: the fragment (8 B) + every node on its root-to-leaf path (8 B per
    # level, summed over the L flag passes: 8 L (L + 1) / 2) + the leaf read-modify-write (8 B)
    build_bytes = F * (8 + 8 * level * (level + 1) // 2 + 8)
    return {"scene": f"terrain ({sc.triangle_count} fp32 triangles: gradient-noise heightfield + 10000 boxes)",
            "level": level, "resolution": 1 << level, "fragments": F, "nodes": int(nodes.value),
            "pool_capacity_nodes": pool_cap, "fragments_ms": frag_ms, "build_ms": build_ms,
            "fragments_build_ms": frag_ms + build_ms,
            "build_algorithmic_gbs": build_bytes / (build_ms * 1e-3) / 1e9,
            "trace": {"samples": n_samples, "cone_samples": cone_samples, "ms": trace_ms,
                      "cone_samples_per_s": cone_samples / (trace_ms * 1e-3)},
            "note": "deterministic build (scan allocation, fragment-order leaf fold); CUDA events, median"}


def differentiable_volume(dev, R: int = 128, views: int = 16, res: int = 512, seed: int = 5, fit_iterations: int = 8):
    """Configuration 5: a hidden float RGBA clipmap (R = 128, smooth noise, alpha <= 0.3) seen through
    `views` x res^2 G-buffer samples: one forward trace of the float atlas (vct_cone_trace_f32), its adjoint
    (vct_cone_trace_backward, dL/d atlas for a unit upstream gradient on every output), and the five-level
    float mip chain with its adjoint, then `fit_iterations` Adam iterations of the inverse fit from a zero
    volume.  CUDA events on the stream; the adjoint synchronises."""
    import ctypes as C
    import torch
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_samples, smooth_volume
    regs = clipmap.clip_regions((0.0, 0.0, 0.0), R)
    regions = clipmap.regions_to_numpy(regs)
    vol = smooth_volume(R, seed=seed, xp=torch, device=dev).reshape(-1)
    n = views * res * res
    smp = clipmap.samples_to_device(random_samples(n, (0.0, 0.0, 0.0), 6.0, seed=seed, specular_fraction=0.5), dev)
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    cam = clipmap.cam_matrix((0.0, 2.0, -9.0))
    light = capi.DirectionalLightDesc(capi.f3(*LIGHT_DIR), 1.0, capi.f3(1, 1, 1), 0)
    dout = torch.empty((n, 4), dtype=torch.float32, device=dev)
    sout = torch.empty_like(dout)
    gd = torch.ones_like(dout)
    gs = torch.ones_like(dout)
    G = torch.zeros_like(vol)
    steps = torch.zeros(1, dtype=torch.int64, device=dev)
    st = torch.cuda.current_stream()
    p = lambda t: C.c_void_p(t.data_ptr())

    def fwd(counter=None):
        capi.call("vct_cone_trace_f32", capi.ref(desc), capi.ref(cam), p(vol), R, None, capi.ref(light), None, p(smp), n,
                  p(dout), p(sout), p(counter) if counter is not None else None, C.c_void_p(st.cuda_stream))

    def bwd():
        capi.call("vct_cone_trace_backward", capi.ref(desc), capi.ref(cam), p(vol), R, None, capi.ref(light), None,
                  p(smp), n, p(gd), p(gs), p(G), C.c_void_p(st.cuda_stream))

    fwd(steps)
    torch.cuda.synchronize()
    cone_samples = int(steps.item())
    fwd_ms = statistics.median(events_ms(st, fwd, 3)[0])
    bwd()
    bwd_ms = statistics.median(events_ms(st, bwd, 2)[0])

    def ds_desc(level):
        d = capi.DownSampleDesc()
        d.prev_region_min_corner = capi.i3(*[int(x) for x in regions[level - 1, 0:3]])
        d.clip_level, d.clipmap_resolution, d.downsample_region_size = level, R, capi.DOWNSAMPLE_REGION_SIZE
        return d

    def mips():
        for level in range(1, 6):
            capi.call("vct_downsample_f32", p(vol), capi.ref(ds_desc(level)), 1, C.c_void_p(st.cuda_stream))

    def mips_bwd():
        for level in range(5, 0, -1):
            capi.call("vct_downsample_backward", p(vol), p(G), capi.ref(ds_desc(level)), 1, C.c_void_p(st.cuda_stream))

    mips()
    mips_ms = statistics.median(events_ms(st, mips, 3)[0])
    mips_bwd_ms = statistics.median(events_ms(st, mips_bwd, 3)[0])
    # inverse radiance fitting: Adam from a zero volume towards the hidden volume's images, each iteration
    # = mips + trace + squared error + trace adjoint + mip adjoint + Adam (host clock: the adjoint synchronises)
    from vk_voxel_cone_tracing_gb300 import fit
    del G
    fit_result = None
    if fit_iterations > 0:
        f = fit.RadianceFit(R, regions, desc, cam, light, smp, lr=0.005)
        f.set_targets(*f.render(vol))
        losses, iter_ms = [], []
        for _ in range(fit_iterations):
            t0 = time.perf_counter()
            losses.append(f.step())
            iter_ms.append((time.perf_counter() - t0) * 1e3)
        losses.append(f.loss())
        fit_result = {"iterations": fit_iterations, "iteration_ms": statistics.median(iter_ms), "loss": losses,
                      "optimiser": "Adam (lr 0.005, betas 0.9 / 0.999), from zero"}
    return {"R": R, "views": views, "resolution": res, "samples": n, "cone_samples": cone_samples,
            "forward_ms": fwd_ms, "backward_ms": bwd_ms, "forward_cone_samples_per_s": cone_samples / (fwd_ms * 1e-3),
            "mips_ms": mips_ms, "mips_backward_ms": mips_bwd_ms,
            "fit": fit_result,
            "note": "float RGBA atlas (16 B per texel, 1.27 GB at R = 128), software trilinear; the adjoint "
                    "marches each cone once, keeping its first 128 steps' records in device scratch (later segments "
                    "recomputed from 32-step checkpoints), and scatters float4 atomics"}


def profile_case(args):
    """A small case for the ncu captures under profiles/ (no JSON line): the hall scene with `--triangles`
    triangles at clipmap `--R`, the bench camera and light.
      frame      two frames keeping the radiance texture current
      frames     3 + 3 timed frames with the texture, without it, and with the R8 opacity form
      trace      one frame, then three fast traces of `--samples` area-uniform samples
      exact      one frame, then two exact traces on the linear atlas
      exact_tex  one frame, then two exact traces reading the texels through the texture
      adjoint    the differentiable workload at R = 64, one view (forward + adjoint)"""
    import torch

    from vk_voxel_cone_tracing_gb300 import build, capi, clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import hall_scene, surface_samples
    build.build()
    if args.profile_case == "adjoint":
        print(json.dumps(differentiable_volume(torch.device("cuda"), R=64, views=1, res=512, fit_iterations=0)))
        return
    R = args.R
    scene = hall_scene(seed=2, target=args.triangles)
    ds, ws = passes.DeviceScene(scene), passes.Workspace()
    op, rad = clipmap.new_atlas(R), clipmap.new_atlas(R)
    sh = torch.empty((SHADOW_RES, SHADOW_RES), dtype=torch.float32, device="cuda")
    light, lsd = passes.light_desc(LIGHT_DIR), passes.light_shadow_desc(light_origin(), LIGHT_DIR)
    tex = clipmap.RadianceTexture(R)
    frame = lambda **kw: passes.clipmap_frame(ds, CAMERA, R, op, rad, sh, light, lsd, ws, **kw)
    if args.profile_case == "frames":
        op8 = clipmap.new_atlas_r8(R)
        for kw in ({"texture": tex}, {}):
            for _ in range(6):
                frame(**kw)
        for _ in range(6):
            passes.clipmap_frame(ds, CAMERA, R, op8, rad, sh, light, lsd, ws, texture=tex,
                                 opacity_format=capi.OPACITY_R8)
        torch.cuda.synchronize()
        return
    for _ in range(2):
        regs = frame(texture=tex)
    if args.profile_case == "frame":
        torch.cuda.synchronize()
        return
    desc = trace_desc_for(clipmap.regions_to_numpy(regs), R)
    smp = clipmap.samples_to_device(surface_samples(scene, args.samples, seed=1))
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    for k in range(3 if args.profile_case == "trace" else 2):
        kw = dict(light=light, shadow=sh, shadow_desc=lsd, steps=steps if k == 0 else None)
        if args.profile_case == "trace":
            clipmap.cone_trace_fast(desc, EYE, tex, smp, **kw)
        elif args.profile_case == "exact":
            clipmap.cone_trace(desc, EYE, rad, R, smp, **kw)
        else:
            clipmap.cone_trace_tex(desc, EYE, tex, smp, **kw)
    torch.cuda.synchronize()
    print("cone samples per trace", int(steps.item()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="tex", choices=["exact", "tex", "fp16"])
    ap.add_argument("--samples", type=int, default=N_SAMPLES)
    ap.add_argument("--R", type=int, default=R_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched multi-scene, differentiable-form and large-SVO measurements")
    ap.add_argument("--profile-case", choices=["frame", "frames", "trace", "exact", "exact_tex", "adjoint"],
                    help="run a small case for an ncu capture instead of the benchmark (see profile_case)")
    ap.add_argument("--triangles", type=int, default=1_000_000, help="hall scene size of --profile-case")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
