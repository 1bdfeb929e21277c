"""Failure paths on the GPU that fault nothing: an allocation the device cannot
satisfy, scenes with out-of-range indices, a batch whose job fails, and the
library's state after each (the next call works)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT_DIR = (0.3, -1.0, 0.2)


def test_allocation_failure_is_reported_and_recoverable(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    h = C.c_void_p()
    with pytest.raises(capi.VctError) as e:
        capi.call("vct_workspace_create", 1 << 52, C.byref(h))  # 4 PB: cudaMalloc refuses
    assert e.value.code == capi.VCT_E_CUDA
    torch.cuda.synchronize()  # the context is intact, and the next launches are not blamed for it
    ws = passes.Workspace(1 << 20)
    assert ws.nbytes >= 1 << 20
    from vk_voxel_cone_tracing_gb300 import clipmap
    atlas = clipmap.new_atlas(16)
    clipmap.cmd_clear_region(atlas, 16, (0, 0, 0), (16, 16, 16), 0)
    torch.cuda.synchronize()
    ws.close()


def test_out_of_range_indices_read_the_last_entry(cuda, oracle):
    """Vertex and instance indices past the arrays are clamped to the last entry on the device (the
    reference would read out of bounds); the oracle clamps the same way, so the passes still agree."""
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    from vk_voxel_cone_tracing_gb300.scene import Scene, room_scene
    base = room_scene(seed=8, n_random=1500)
    idx = base.indices.copy()
    idx[5] = [0xFFFFFFF0, 1, 2]  # one bad vertex index
    idx[9] = [3, 0x7FFFFFFF, 4]
    inst = np.zeros(base.triangle_count, np.uint32)
    inst[11] = 1000  # past the single instance
    eye = np.concatenate([np.eye(4, dtype=np.float32).reshape(16)] * 2)[None, :]
    sc = Scene(base.positions, base.normals, idx, base.tri_material, base.materials, base.textures,
               node_matrices=eye, tri_instance=inst)
    R = 32
    cam = (0.35, 2.1, -0.7)
    want = oracle.voxelize_opacity(sc, R, oracle.clip_regions(cam, R))
    ds = passes.DeviceScene(sc)
    ws = passes.Workspace()
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity(ds, clipmap.clip_regions(cam, R), R, atlas, ws)
    torch.cuda.synchronize()
    assert np.array_equal(atlas.cpu().numpy().view(np.uint32), want)


def test_a_failing_batch_job_reports_and_the_others_finish(cuda):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap, engine, passes
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, room_scene, surface_samples
    good = room_scene(seed=30, n_random=800)
    ds_good = passes.DeviceScene(good)
    ds_bad = passes.DeviceScene(good)
    ds_bad.desc.material_count = 0  # check_scene refuses a scene without materials
    ctxs = [engine.Context(32, shadow_size=128) for _ in range(3)]
    light = passes.light_desc(LIGHT_DIR)
    lsd = passes.light_shadow_desc((5.0, 14.0, 3.0), LIGHT_DIR)
    td = clipmap.trace_desc(**default_trace_desc(np.zeros((6, 7), np.int32), 32))
    smp = clipmap.samples_to_device(surface_samples(good, 500, seed=1))
    outs = [(torch.zeros((500, 4), device="cuda"), torch.zeros((500, 4), device="cuda")) for _ in range(3)]
    jobs = [engine.batch_job(c, d, (0.3, 2.0, -0.5), light, lsd, td, (0, 3, -3), smp, o[0], o[1])
            for c, d, o in zip(ctxs, (ds_good, ds_bad, ds_good), outs)]
    with pytest.raises(capi.VctError, match="material"):
        engine.batch_submit(jobs, streams=3)
    torch.cuda.synchronize()
    assert outs[0][0].abs().sum().item() > 0 and outs[2][0].abs().sum().item() > 0
    # the library keeps working
    engine.batch_submit([jobs[0]], streams=1)
    for c in ctxs:
        c.close()
