"""GPU parity of the raster passes on instanced scenes (NodeMatrix per triangle),
the layout the glTF loader produces: the device transforms every vertex by its
instance's model matrix and every normal by its itModel, as the oracle does."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAM = (0.35, 2.1, -0.7)
LIGHT_DIR = (0.3, -1.0, 0.2)


def _instanced_room():
    from vk_voxel_cone_tracing_gb300 import gltf
    from vk_voxel_cone_tracing_gb300.scene import Scene, room_scene
    base = room_scene(seed=3, n_random=800)
    T = base.triangle_count
    mats = []
    for i, (ang, t, s) in enumerate(((0.0, (0, 0, 0), 1.0), (0.6, (1.5, 0.2, -0.5), 0.5),
                                     (-1.1, (-2.0, 1.0, 1.0), 0.3))):
        q = (0.0, np.sin(ang / 2), 0.0, np.cos(ang / 2))
        world = gltf.node_local({"translation": list(t), "rotation": list(q), "scale": [s, s, s]})
        mats.append(np.concatenate([world, gltf.transpose(gltf.inverse(world))]))
    idx = np.concatenate([base.indices] * 3)
    return Scene(base.positions, base.normals, idx, np.concatenate([base.tri_material] * 3), base.materials,
                 base.textures, node_matrices=np.stack(mats).astype(np.float32),
                 tri_instance=np.repeat(np.arange(3, dtype=np.uint32), T))


@pytest.fixture(scope="module")
def scene():
    return _instanced_room()


@pytest.fixture(scope="module")
def dscene(cuda, scene):
    from vk_voxel_cone_tracing_gb300.passes import DeviceScene
    return DeviceScene(scene)


@pytest.fixture(scope="module")
def ws(cuda):
    from vk_voxel_cone_tracing_gb300.passes import Workspace
    return Workspace()


def _light(center=(0.0, 4.0, 0.0)):
    d = np.asarray(LIGHT_DIR, np.float64)
    d /= np.linalg.norm(d)
    return tuple((np.asarray(center) - 15.0 * d).astype(np.float32).tolist())


def test_instanced_voxelize_shadow_inject_bit_exact(cuda, oracle, scene, dscene, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import clipmap, passes
    R = 64
    want = oracle.voxelize_opacity(scene, R, oracle.clip_regions(CAM, R))
    atlas = clipmap.new_atlas(R)
    passes.voxelize_opacity(dscene, clipmap.clip_regions(CAM, R), R, atlas, ws)
    sd = passes.light_shadow_desc(_light(), LIGHT_DIR)
    depth = torch.empty((512, 512), dtype=torch.float32, device="cuda")
    passes.shadow_depth(dscene, sd, depth, ws)
    torch.cuda.synchronize()
    assert np.count_nonzero(want) > 1000
    assert np.array_equal(atlas.cpu().numpy().view(np.uint32), want)
    want_d = oracle.shadow_depth(scene, bytes(sd), 512, 512)
    assert np.array_equal(depth.cpu().numpy().view(np.uint32), want_d.view(np.uint32))
    rad = clipmap.new_atlas(R)
    light = passes.light_desc(LIGHT_DIR)
    passes.inject_radiance(dscene, clipmap.clip_regions(CAM, R), R, depth, light, sd, rad, ws)
    torch.cuda.synchronize()
    want_r = oracle.inject_radiance(scene, R, oracle.clip_regions(CAM, R), want_d, bytes(sd), bytes(light))
    assert np.count_nonzero(want_r) > 1000
    assert np.array_equal(rad.cpu().numpy().view(np.uint32), want_r)


def test_instanced_gbuffer_bit_exact(cuda, oracle, scene, dscene, ws):
    torch = cuda
    from vk_voxel_cone_tracing_gb300 import capi, passes
    W, H = 192, 108
    cam = oracle.camera_matrix((0.5, 2.5, -4.0), (0.1, -0.3, 1.0), aspect=W / H)
    c = capi.CamMatrix.from_buffer_copy(cam.tobytes())
    got = passes.gbuffer(dscene, c, W, H, ws)
    torch.cuda.synchronize()
    want = oracle.gbuffer(scene, cam, W, H)
    assert (want[:, 3] < 1.0).mean() > 0.9
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_gltf_document_gbuffer_bit_exact(cuda, oracle, ws, tmp_path):
    torch = cuda
    from tests.test_gltf import _doc, _png_fixture, _write_glb
    from vk_voxel_cone_tracing_gb300 import capi, gltf, passes
    png, _ = _png_fixture()
    doc, buf = _doc(png)
    sc = gltf.load_gltf(_write_glb(tmp_path, doc, buf)).scene
    ds = passes.DeviceScene(sc)
    cam = oracle.camera_matrix((1.0, 4.0, -6.0), (0.0, -0.5, 1.0), aspect=1.5)
    got = passes.gbuffer(ds, capi.CamMatrix.from_buffer_copy(cam.tobytes()), 96, 64, ws)
    torch.cuda.synchronize()
    want = oracle.gbuffer(sc, cam, 96, 64)
    assert (want[:, 3] < 1.0).sum() > 100
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))
