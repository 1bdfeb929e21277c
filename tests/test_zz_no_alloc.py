"""vct_cone_trace_fast_noalloc: the fast cone tracer for callers that cannot
allocate device memory (hosts whose own allocator owns the GPU, frame loops
that must not call cudaMalloc).  Its scratch is a static device array inside
the library, so this test calls it through the C ABI with only inputs and
outputs, twice in a row on different sample sets (the array keeps the first
call's contents), and checks each result against vct_cone_trace_fast with
caller-provided scratch.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-2  # relative L2 tolerance the fast-trace tests use


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12))


def test_noalloc_matches_fast_trace_on_two_calls(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    R = 32
    regions = oracle.clip_regions((0.0, 0.0, 0.0), R)
    desc = clipmap.trace_desc(**default_trace_desc(regions, R))
    atlas = random_atlas(R, seed=41, fill=0.05)
    for level in range(1, 6):
        oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
    tex = clipmap.RadianceTexture(R).update(torch.from_numpy(atlas.view(np.int32).copy()).cuda())
    eye = (0.5, 1.0, -4.0)
    cam = clipmap.cam_matrix(eye)
    light = capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    sm = capi.ShadowMap(None, 0, 0)
    sd = capi.DirectionalLightShadowDesc()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    need = capi.lib().vct_cone_trace_fast_scratch_bytes(capi.NOALLOC_MAX_SAMPLES)
    assert 0 < need <= capi.NOALLOC_SCRATCH_BYTES
    for call, (seed, n) in enumerate(((42, 3000), (43, 1200))):
        samples = clipmap.samples_to_device(random_samples(n, (0, 0, 0), 6.0, seed=seed))
        want_d, want_s = clipmap.cone_trace_fast(desc, eye, tex, samples)
        got_d = torch.full((n, 4), -1.0, device="cuda")
        got_s = torch.full((n, 4), -1.0, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        capi.call("vct_cone_trace_fast_noalloc", capi.ref(desc), capi.ref(cam), tex.handle, capi.ref(sm),
                  capi.ref(light), capi.ref(sd), C.c_void_p(samples.data_ptr()), n, C.c_void_p(got_d.data_ptr()),
                  C.c_void_p(got_s.data_ptr()), None, stream)
        torch.cuda.synchronize()
        if call > 0:
            # the first call may commit the static array (lazy module loading); later calls take no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        wd, ws = want_d.cpu().numpy(), want_s.cpu().numpy()
        gd, gs = got_d.cpu().numpy(), got_s.cpu().numpy()
        assert _rel(gd, wd) < TOL and _rel(gs, ws) < TOL
        assert np.array_equal(gd, wd) and np.array_equal(gs, ws)
    tex.close()


def test_noalloc_rejects_too_many_samples(cuda):
    from vk_voxel_cone_tracing_gb300 import capi
    L = capi.lib()
    dummy = C.c_void_p(256)  # never dereferenced: the size check comes first
    rc = L.vct_cone_trace_fast_noalloc(dummy, dummy, dummy, None, dummy, None, dummy, capi.NOALLOC_MAX_SAMPLES + 1,
                                       dummy, dummy, None, None)
    assert rc == capi.VCT_E_BAD_ARG
    assert b"VCT_NOALLOC_MAX_SAMPLES" in L.vct_last_error()
