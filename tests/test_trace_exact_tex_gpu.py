"""The exact FP32 trace reading its texels through the radiance texture
(vct_cone_trace_tex) against the same trace on the linear RGBA8 atlas
(vct_cone_trace, itself held to the FP32 restatement of
voxelConeTracing.frag:143-392 at 1e-4 per sample): outputs and cone-step
counts equal bit for bit, over atlases whose texels take every byte value,
every rendering mode that traces, both cone sets and a 30-degree aperture."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R,mode,cones32,aperture", [(32, 8, 0, 0.0), (64, 8, 1, 0.0), (32, 7, 0, 0.0),
                                                     (64, 6, 0, 0.0), (32, 5, 0, 0.0), (64, 8, 0, 0.523599)])
def test_texel_read_trace_equals_atlas_trace(cuda, oracle, R, mode, cones32, aperture):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_atlas, random_samples
    cam = (0.4, -0.3, 0.2)
    regions = oracle.clip_regions(cam, R)
    desc = clipmap.trace_desc(**{**default_trace_desc(regions, R), "rendering_mode": mode,
                                 "enable_32_cones": cones32})
    atlas = random_atlas(R, seed=R + mode, fill=0.08)
    for level in range(1, 6):
        oracle.downsample(atlas, R, regions[level - 1, 0:3], level, 1)
    assert len(np.unique(atlas.view(np.uint8))) == 256
    rad = torch.from_numpy(atlas.view(np.int32).copy()).cuda()
    tex = clipmap.RadianceTexture(R).update(rad)
    samples = clipmap.samples_to_device(random_samples(4096, cam, 0.4 * R / 8, seed=mode, specular_fraction=0.6))
    eye = (cam[0] + 0.5, cam[1] + 1.0, cam[2] - 4.0)
    st_a = torch.zeros(1, dtype=torch.int64, device="cuda")
    st_t = torch.zeros(1, dtype=torch.int64, device="cuda")
    da, sa = clipmap.cone_trace(desc, eye, rad, R, samples, steps=st_a, diffuse_aperture=aperture)
    dt, stx = clipmap.cone_trace_tex(desc, eye, tex, samples, steps=st_t, diffuse_aperture=aperture)
    torch.cuda.synchronize()
    assert torch.equal(dt, da) and torch.equal(stx, sa)
    assert int(st_t.item()) == int(st_a.item()) > 0
    tex.close()


def test_texel_read_trace_rejects_fp16_texture_and_wrong_resolution(cuda, oracle):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, clipmap
    from vk_voxel_cone_tracing_gb300.scene import default_trace_desc, random_samples
    R = 16
    desc = clipmap.trace_desc(**default_trace_desc(oracle.clip_regions((0.0, 0.0, 0.0), R), R))
    smp = clipmap.samples_to_device(random_samples(64, (0.0, 0.0, 0.0), 1.0))
    t16 = clipmap.RadianceTexture(R, capi.TEX_RGBA16F)
    with pytest.raises(capi.VctError, match="RGBA8"):
        clipmap.cone_trace_tex(desc, (0.0, 1.0, -3.0), t16, smp)
    t16.close()
    t8 = clipmap.RadianceTexture(2 * R)
    with pytest.raises(capi.VctError, match="resolution"):
        clipmap.cone_trace_tex(desc, (0.0, 1.0, -3.0), t8, smp)
    t8.close()
