"""The batched form of the fast trace (vct_cone_trace_fast_batch): many
clipmaps and sample sets of uneven size in one launch per stage over a
work queue.  Each job's outputs and cone-step count must equal, bit for bit,
those of vct_cone_trace_fast on that job alone (per-sample results do not
depend on the visiting order), and the first job's against the FP64 oracle
within the texture form's 1e-2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(torch, oracle, spec):
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    out = []
    for k, (R, n, mode, cones32) in enumerate(spec):
        cam = (0.3 * k, -0.2 * k, 0.1 * k)
        regions = oracle.clip_regions(cam, R)
        desc = clipmap.trace_desc(**{**default_trace_desc(regions, R), "rendering_mode": mode,
                                     "enable_32_cones": cones32})
        atlas = random_atlas(R, seed=50 + k, fill=0.06)
        for level in range(1, 6):
            oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
        tex = clipmap.RadianceTexture(R).update(torch.from_numpy(atlas.view(np.int32).copy()).cuda())
        samples = random_samples(n, cam, 0.4 * R / 8, seed=60 + k)
        eye = (cam[0] + 0.5, cam[1] + 1.0, cam[2] - 4.0)
        out.append(dict(R=R, desc=desc, tex=tex, atlas=atlas, samples=samples, eye=eye,
                        dev=clipmap.samples_to_device(samples) if n else torch.zeros((0, 20), device="cuda")))
    return out


def test_batched_trace_equals_each_job_alone(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    # uneven sizes: an empty job, a single sample, a count off the 32 grid, several resolutions and modes
    spec = [(32, 3000, 8, 0), (16, 0, 8, 0), (64, 1, 8, 0), (32, 33, 6, 0), (16, 1000, 7, 1), (64, 2500, 8, 0),
            (32, 777, 5, 0)]
    J = _jobs(torch, oracle, spec)
    want, records, got = [], [], []
    for j in J:
        n = j["dev"].shape[0]
        st = torch.zeros(1, dtype=torch.int64, device="cuda")
        d, s = clipmap.cone_trace_fast(j["desc"], j["eye"], j["tex"], j["dev"], steps=st) if n else (None, None)
        want.append((d, s, st))
        gd = torch.full((n, 4), -3.0, device="cuda")
        gs = torch.full((n, 4), -3.0, device="cuda")
        gst = torch.zeros(1, dtype=torch.int64, device="cuda")
        got.append((gd, gs, gst))
        records.append(clipmap.trace_job(j["desc"], j["eye"], j["tex"], j["dev"], gd, gs, steps=gst))
    clipmap.cone_trace_fast_batch(records)
    torch.cuda.synchronize()
    for k, ((d, s, st), (gd, gs, gst)) in enumerate(zip(want, got)):
        if d is None:
            continue
        assert torch.equal(gd, d) and torch.equal(gs, s), k
        assert int(gst.item()) == int(st.item()), k
    # the first job against the FP64 oracle
    j = J[0]
    d64, s64, _, _ = oracle.cone_trace(64, bytes(j["desc"]), j["eye"], j["atlas"], j["R"], j["samples"])
    gd = got[0][0].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gd[:, :3] - d64[:, :3]) / np.linalg.norm(d64[:, :3]) < 1e-2
    for j in J:
        j["tex"].close()


def test_batched_trace_more_jobs_than_one_table(cuda, oracle):
    """More jobs than one kernel-parameter table holds: the call runs them in chunks, same results."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    spec = [(16, 50 + 7 * k, 8, 0) for k in range(70)]
    J = _jobs(torch, oracle, spec)
    records, pairs = [], []
    for j in J:
        n = j["dev"].shape[0]
        d, s = clipmap.cone_trace_fast(j["desc"], j["eye"], j["tex"], j["dev"])
        gd, gs = torch.empty((n, 4), device="cuda"), torch.empty((n, 4), device="cuda")
        records.append(clipmap.trace_job(j["desc"], j["eye"], j["tex"], j["dev"], gd, gs))
        pairs.append((d, s, gd, gs))
    clipmap.cone_trace_fast_batch(records)
    torch.cuda.synchronize()
    for d, s, gd, gs in pairs:
        assert torch.equal(gd, d) and torch.equal(gs, s)
    for j in J:
        j["tex"].close()


def test_batched_trace_rejects_bad_jobs(cuda, oracle):
    import ctypes as C
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    J = _jobs(torch, oracle, [(16, 64, 8, 0)])
    j = J[0]
    out = torch.empty((64, 4), device="cuda")
    rec = clipmap.trace_job(j["desc"], j["eye"], j["tex"], j["dev"], out, out)
    rec.desc.volume_dimension = 32.0  # not the texture's resolution
    arr = (capi.TraceJob * 1)(rec)
    scratch = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    rc = capi.lib().vct_cone_trace_fast_batch(C.cast(arr, C.c_void_p), 1, C.c_void_p(clipmap._aligned(scratch)),
                                              (1 << 20) - 256, None)
    assert rc == capi.VCT_E_BAD_ARG
    assert capi.lib().vct_cone_trace_fast_batch_scratch_bytes(None, -1) < 0
    j["tex"].close()
