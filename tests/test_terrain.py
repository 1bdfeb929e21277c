"""The terrain scene of the large-octree workload (configuration 3) on the CPU: the gradient noise's
defining properties, the triangle count and orientation, and determinism."""
import numpy as np

from vk_voxel_cone_tracing_gb300.scene import _box_triangles, gradient_noise2, terrain_height, terrain_scene


def _perm(seed=0):
    p = np.random.default_rng(seed).permutation(256)
    return np.concatenate([p, p])


def test_noise_is_zero_on_the_lattice_and_bounded():
    perm = _perm()
    i = np.arange(-20, 20, dtype=np.float64)
    xx, yy = np.meshgrid(i, i)
    assert np.all(gradient_noise2(xx, yy, perm) == 0.0)  # every corner ramp vanishes at its own corner
    x = np.random.default_rng(1).uniform(-300, 300, size=(2, 200000))
    n = gradient_noise2(x[0], x[1], perm)
    assert np.abs(n).max() <= 1.0 and n.std() > 0.1


def test_noise_is_continuous_and_periodic():
    perm = _perm(3)
    x = np.random.default_rng(2).uniform(-50, 50, size=(2, 10000))
    a = gradient_noise2(x[0], x[1], perm)
    assert np.abs(gradient_noise2(x[0] + 1e-6, x[1], perm) - a).max() < 1e-5
    assert np.allclose(gradient_noise2(x[0] + 256.0, x[1] - 512.0, perm), a, atol=1e-9)  # the lattice hash wraps at 256


def test_boxes_are_closed_and_outward():
    lo = np.array([[0.0, 0.0, 0.0], [-2.0, 1.0, 3.0]])
    hi = np.array([[1.0, 2.0, 3.0], [-1.5, 1.25, 4.0]])
    t = _box_triangles(lo, hi)
    assert t.shape == (2, 12, 3, 3)
    for b in range(2):
        c = 0.5 * (lo[b] + hi[b])
        n = np.cross(t[b, :, 1] - t[b, :, 0], t[b, :, 2] - t[b, :, 0])
        assert np.all(((t[b].mean(1) - c) * n).sum(1) > 0)
        area = 0.5 * np.linalg.norm(n, axis=1).sum()
        e = hi[b] - lo[b]
        assert np.isclose(area, 2 * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]))


def test_terrain_scene_layout_and_determinism():
    sc = terrain_scene(seed=3, target=30000, boxes=200)
    T = sc.triangle_count
    assert 29000 <= T <= 30000 and T == sc.tri_material.shape[0]
    t = sc.triangles()
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    assert np.all(n[: T - 200 * 12, 1] > 0)  # terrain cells face up
    assert np.all(np.abs(t[..., 0]) <= 15.0) and np.all(np.abs(t[..., 2]) <= 15.0)
    assert sc.tri_material.max() < sc.materials.shape[0] == sc.textures.shape[0]
    # heights follow the fractal sum at the grid's vertices
    perm = np.random.default_rng(3).permutation(256)
    perm = np.concatenate([perm, perm])
    v = t[: T - 200 * 12].reshape(-1, 3)
    assert np.allclose(v[:, 1], terrain_height(v[:, 0].astype(np.float64), v[:, 2].astype(np.float64), perm),
                       atol=1e-5)
    again = terrain_scene(seed=3, target=30000, boxes=200)
    assert np.array_equal(again.positions, sc.positions) and np.array_equal(again.tri_material, sc.tri_material)
