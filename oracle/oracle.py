"""ctypes binding of the CPU oracle (libvct_oracle.so) -- TEST INFRASTRUCTURE ONLY.

The oracle is a C++ restatement of the reference's shader arithmetic
(clipmap_oracle.hpp and friends).  Only ``tests/``, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg import this module; the CUDA product path
never does.  ``build()`` compiles the oracle with g++ (-ffp-contract=off so
no multiply-add is fused, -fopenmp for the timed CPU baseline).

Parity pinning: the host math (clip regions, the voxeliser / light / camera /
glTF-node matrices with glm::inverse) is pinned bit for bit against the
reference's vendored glm, and the cone tables and trace constants against its
shader source (tests/golden).  The shader arithmetic itself is a restatement:
its parity with the GLSL is unpinned, because the reference's passes need
Vulkan, which is unavailable on this machine, and the reference ships no tests or
fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libvct_oracle.so"
SOURCES = ["vct_oracle.cpp"]
HEADERS = ["ad_tape.hpp", "adjoint_oracle.hpp", "oracle_common.hpp", "clipmap_oracle.hpp", "raster_oracle.hpp", "svo_oracle.hpp", "gbuffer_oracle.hpp",
           "composite_oracle.hpp"]

P = C.c_void_p


def _deps():
    return [HERE / s for s in SOURCES] + [HERE / h for h in HEADERS if (HERE / h).exists()] + [Path(__file__)]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in _deps()):
        return LIB
    BUILD.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           *[str(HERE / s) for s in SOURCES], "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_L = None


def lib():
    global _L
    if _L is None:
        build()
        L = C.CDLL(str(LIB))
        L.vcto_num_threads.restype = C.c_int
        L.vcto_set_threads.argtypes = [C.c_int]
        L.vcto_clip_regions.argtypes = [P, C.c_int, C.c_int, P]
        L.vcto_clear_region.argtypes = [P, C.c_int, P, P, C.c_int, C.c_int]
        L.vcto_copy_alpha.argtypes = [P, P, C.c_int, C.c_int, C.c_int]
        L.vcto_wrap_border.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int]
        L.vcto_downsample.argtypes = [P, C.c_int, P, C.c_int, C.c_int, C.c_int]
        L.vcto_cone_trace_opt.restype = C.c_uint64
        L.vcto_cone_trace_opt.argtypes = [C.c_int, P, P, P, C.c_int, P, C.c_int, C.c_int, P, P, P, C.c_int64,
                                          C.c_int64, P, P, P, C.c_float]
        L.vcto_cone_trace.restype = C.c_uint64
        L.vcto_cone_trace.argtypes = [C.c_int, P, P, P, C.c_int, P, C.c_int, C.c_int, P, P, P, C.c_int64,
                                      C.c_int64, P, P, P]
        L.vcto_cone_trace_f4.restype = C.c_uint64
        L.vcto_cone_trace_f4.argtypes = [P, P, P, C.c_int, P, C.c_int, C.c_int, P, P, P, C.c_int64, C.c_int64,
                                         P, P]
        L.vcto_downsample_f4.argtypes = [P, C.c_int, P, C.c_int, C.c_int, C.c_int]
        L.vcto_cone_trace_grad_f4.argtypes = [P, P, P, C.c_int, P, C.c_int, C.c_int, P, P, P, C.c_int64, C.c_int64,
                                              P, P, P]
        L.vcto_downsample_chain_grad_f4.argtypes = [P, C.c_int, P, C.c_int, C.c_int, C.c_int, P]
        L.vcto_voxel_view_proj.argtypes = [P, P]
        L.vcto_voxelization_desc.argtypes = [P, C.c_int, C.c_int, P]
        L.vcto_light_shadow_desc.argtypes = [P, P, C.c_float, C.c_float, P]
        L.vcto_voxelize_opacity.argtypes = [P, C.c_int, P, P, C.c_int]
        L.vcto_voxelize_conservative.argtypes = [P, C.c_int, P, P, C.c_int]
        L.vcto_cons_overlap.restype = C.c_int
        L.vcto_cons_overlap.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int]
        L.vcto_shadow_depth.argtypes = [P, P, P, C.c_int, C.c_int]
        L.vcto_camera_matrix.argtypes = [P, P, P, C.c_float, C.c_float, P]
        L.vcto_inverse4.argtypes = [P, P]
        L.vcto_gbuffer.argtypes = [P, P, C.c_int, C.c_int, P]
        L.vcto_update_clip_regions.restype = C.c_int
        L.vcto_update_clip_regions.argtypes = [P, P, C.c_int, C.c_int, P, P]
        L.vcto_voxelize_opacity_slabs.argtypes = [P, C.c_int, P, P, P, P, C.c_int]
        L.vcto_gaussian_stencil.argtypes = [P]
        L.vcto_specular_filter.argtypes = [P, P, P, C.c_int, C.c_int, P]
        L.vcto_present_srgb8.argtypes = [P, C.c_int64, P]
        L.vcto_inject_radiance.argtypes = [P, C.c_int, P, P, C.c_int, C.c_int, P, P, P, C.c_int]
        L.vcto_svo_fragments.restype = C.c_int64
        L.vcto_svo_fragments.argtypes = [P, C.c_int, P, P, P, C.c_int, C.c_int, P, P, P, C.c_int64]
        L.vcto_svo_build.restype = C.c_int
        L.vcto_svo_build.argtypes = [P, C.c_int64, C.c_int, P, C.c_int64, P]
        L.vcto_svo_trace.restype = C.c_uint64
        L.vcto_svo_trace.argtypes = [C.c_int, P, P, P, P, P, P, C.c_int, C.c_int, P, P, P, C.c_int64, C.c_int64,
                                     P, P]
        L.vcto_procedural_atlas.argtypes = [P, C.c_int64, C.c_uint32, C.c_double]
        _L = L
    return _L


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n: int) -> None:
    lib().vcto_set_threads(int(n))


def num_threads() -> int:
    return int(lib().vcto_num_threads())


def clip_regions(cam, R: int, extent_l0: int = 16) -> np.ndarray:
    """6 regions as an int/float record array: min_corner(3 i32), extent(3 u32), voxel_size(f32)."""
    out = np.zeros(6 * 7, dtype=np.int32)
    cam = np.asarray(cam, dtype=np.float32)
    lib().vcto_clip_regions(_p(cam), R, extent_l0, _p(out))
    return out.reshape(6, 7)


def region_voxel_size(regions: np.ndarray, level: int) -> float:
    return float(regions[level, 6:7].view(np.float32)[0])


def clear_region(atlas: np.ndarray, R: int, region_min, extent, level: int, faces: int = 6) -> None:
    lib().vcto_clear_region(_p(atlas), R, _p(np.asarray(region_min, np.int32)), _p(np.asarray(extent, np.uint32)),
                            level, faces)


def copy_alpha(dst: np.ndarray, src: np.ndarray, R: int, level: int, faces: int = 6) -> None:
    lib().vcto_copy_alpha(_p(dst), _p(src), R, level, faces)


def wrap_border(atlas: np.ndarray, R: int, border_width_desc: int = 2, faces: int = 6, regions: int = 6) -> None:
    lib().vcto_wrap_border(_p(atlas), R, border_width_desc, faces, regions)


def downsample(atlas: np.ndarray, R: int, prev_min, level: int, mode: int, band: int = 10) -> None:
    lib().vcto_downsample(_p(atlas), R, _p(np.asarray(prev_min, np.int32)), level, band, mode)


def procedural_atlas(R: int, seed: int = 3, fill: float = 0.05) -> np.ndarray:
    """The benchmark's hash-random atlas (identical to scene.procedural_atlas_torch) built in C++."""
    shape = (R + 2, 6 * (R + 2), 6 * (R + 2))
    out = np.empty(shape, np.uint32)
    lib().vcto_procedural_atlas(_p(out), out.size, seed & 0xFFFFFFFF, fill)
    return out


def downsample_f4(atlas4: np.ndarray, R: int, prev_min, level: int, mode: int, band: int = 10) -> None:
    """One level on float4 storage with FP64 arithmetic (reference for the RGBA16F mips)."""
    assert atlas4.dtype == np.float32
    lib().vcto_downsample_f4(_p(atlas4), R, _p(np.asarray(prev_min, np.int32)), level, band, mode)


def rgba8_to_f4(atlas: np.ndarray) -> np.ndarray:
    a = atlas.astype(np.uint32)
    return (np.stack([(a >> (8 * c)) & 0xFF for c in range(4)], -1).astype(np.float32) / np.float32(255.0))


def default_light_bytes() -> bytes:
    """DirectionalLightDesc{direction (0.3,-1,0.2), intensity 1, colour 1}: the configurations' light."""
    return np.array([0.3, -1.0, 0.2, 1.0, 1.0, 1.0, 1.0, 0.0], np.float32).tobytes()


def cone_trace(precision: int, desc_bytes: bytes, eye, atlas: np.ndarray, R: int, samples: np.ndarray,
               shadow: np.ndarray | None = None, shadow_desc_bytes: bytes | None = None,
               light_bytes: bytes | None = None, begin: int = 0, end: int | None = None,
               diffuse_aperture: float = 0.0):
    """Trace samples [begin, end) with the FP32 (precision=32) or FP64 (64) restatement; a non-zero
    `diffuse_aperture` (radians) replaces the shader's diffuse cone aperture.

    Returns (diffuse[n,4] f64, specular[n,4] f64, steps, written[n] u8)."""
    n = samples.shape[0]
    end = n if end is None else end
    dout = np.zeros((n, 4), np.float64)
    sout = np.zeros((n, 4), np.float64)
    written = np.zeros(n, np.uint8)
    desc = np.frombuffer(desc_bytes, np.uint8).copy()
    sd = np.frombuffer(shadow_desc_bytes or bytes(136), np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    eye = np.asarray(eye, np.float32)
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    steps = lib().vcto_cone_trace_opt(precision, _p(desc), _p(eye), _p(atlas), R, _p(shadow), sw, sh, _p(sd),
                                      _p(light), _p(samples), begin, end, _p(dout), _p(sout), _p(written),
                                      float(diffuse_aperture))
    return dout, sout, int(steps), written


def cone_trace_f4(desc_bytes: bytes, eye, atlas4: np.ndarray, R: int, samples: np.ndarray,
                  shadow: np.ndarray | None = None, shadow_desc_bytes: bytes | None = None,
                  light_bytes: bytes | None = None, begin: int = 0, end: int | None = None):
    n = samples.shape[0]
    end = n if end is None else end
    dout = np.zeros((n, 4), np.float64)
    sout = np.zeros((n, 4), np.float64)
    desc = np.frombuffer(desc_bytes, np.uint8).copy()
    sd = np.frombuffer(shadow_desc_bytes or bytes(136), np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    eye = np.asarray(eye, np.float32)
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    steps = lib().vcto_cone_trace_f4(_p(desc), _p(eye), _p(atlas4), R, _p(shadow), sw, sh, _p(sd), _p(light),
                                     _p(samples), begin, end, _p(dout), _p(sout))
    return dout, sout, int(steps)


def cone_trace_grad_f4(desc_bytes: bytes, eye, atlas4: np.ndarray, R: int, samples: np.ndarray,
                       grad_diffuse: np.ndarray, grad_specular: np.ndarray, shadow: np.ndarray | None = None,
                       shadow_desc_bytes: bytes | None = None, light_bytes: bytes | None = None) -> np.ndarray:
    """FP64 reference gradient (reverse-mode AD of the restated trace) of
    sum(grad_diffuse * diffuse + grad_specular * specular) with respect to the float atlas: an array of the
    atlas's shape, float64."""
    assert atlas4.dtype == np.float32 and atlas4.flags["C_CONTIGUOUS"]
    n = samples.shape[0]
    gd = np.ascontiguousarray(grad_diffuse, np.float32).reshape(n, 4)
    gs = np.ascontiguousarray(grad_specular, np.float32).reshape(n, 4)
    out = np.zeros(atlas4.shape, np.float64)
    desc = np.frombuffer(desc_bytes, np.uint8).copy()
    sd = np.frombuffer(shadow_desc_bytes or bytes(136), np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    lib().vcto_cone_trace_grad_f4(_p(desc), _p(np.asarray(eye, np.float32)), _p(atlas4), R, _p(shadow), sw, sh,
                                  _p(sd), _p(light), _p(samples), 0, n, _p(gd), _p(gs), _p(out))
    return out


def downsample_chain_grad_f4(atlas4: np.ndarray, R: int, regions: np.ndarray, grad_out: np.ndarray, mode: int,
                             first: int = 1, band: int = 10) -> np.ndarray:
    """FP64 reference adjoint of the float mips, levels first..5: given dL/d(atlas after the chain), returns
    dL/d(atlas before it) (float64, the atlas's shape)."""
    assert atlas4.dtype == np.float32 and atlas4.flags["C_CONTIGUOUS"]
    pm = np.ascontiguousarray(np.asarray(regions)[0:5, 0:3], np.int32).reshape(15)
    G = np.ascontiguousarray(grad_out, np.float64).copy()
    lib().vcto_downsample_chain_grad_f4(_p(atlas4), R, _p(pm), first, band, mode, _p(G))
    return G


# ------------------------------------------------------------ raster passes

class SceneView(C.Structure):
    """Mirror of vcto::SceneView / vct_scene (host pointers)."""
    _fields_ = [("positions", P), ("normals", P), ("indices", P), ("vertex_count", C.c_int64),
                ("triangle_count", C.c_int64), ("triangle_material", P), ("materials", P),
                ("material_count", C.c_int32), ("textures", P), ("texture_count", C.c_int32),
                ("node_matrices", P), ("triangle_instance", P), ("instance_count", C.c_int32)]


def scene_view(scene):
    """SceneView over a vk_voxel_cone_tracing_gb300.scene.Scene (arrays kept alive on the returned object)."""
    keep = [np.ascontiguousarray(scene.positions, np.float32), np.ascontiguousarray(scene.normals, np.float32),
            np.ascontiguousarray(scene.indices, np.uint32), np.ascontiguousarray(scene.tri_material, np.uint32),
            np.ascontiguousarray(scene.materials), np.ascontiguousarray(scene.textures, np.uint32)]
    nm, ti, ninst = None, None, 0
    if getattr(scene, "node_matrices", None) is not None:
        keep += [np.ascontiguousarray(scene.node_matrices, np.float32), np.ascontiguousarray(scene.tri_instance, np.uint32)]
        nm, ti, ninst = _p(keep[6]), _p(keep[7]), keep[6].shape[0]
    sv = SceneView(_p(keep[0]), _p(keep[1]), _p(keep[2]), keep[0].shape[0], keep[2].shape[0], _p(keep[3]),
                   _p(keep[4]), keep[4].shape[0], _p(keep[5]), keep[5].shape[0], nm, ti, ninst)
    sv._keep = keep
    return sv


def _regions_arg(regions: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(regions, np.int32)


def voxel_view_proj(region_row: np.ndarray) -> np.ndarray:
    out = np.zeros(48, np.float32)
    lib().vcto_voxel_view_proj(_p(np.ascontiguousarray(region_row, np.int32)), _p(out))
    return out.reshape(3, 16)


def voxelization_desc(regions: np.ndarray, level: int, R: int) -> bytes:
    out = np.zeros(16, np.int32)
    lib().vcto_voxelization_desc(_p(_regions_arg(regions)), level, R, _p(out))
    return out.tobytes()


def light_shadow_desc(origin, direction, z_near: float = 0.1, z_far: float = 30.0) -> bytes:
    out = np.zeros(34, np.float32)
    lib().vcto_light_shadow_desc(_p(np.asarray(origin, np.float32)), _p(np.asarray(direction, np.float32)),
                                 z_near, z_far, _p(out))
    return out.tobytes()


def voxelize_opacity(scene, R: int, regions: np.ndarray, level_mask: int = 0x3F,
                     atlas: np.ndarray | None = None) -> np.ndarray:
    if atlas is None:
        atlas = np.zeros((R + 2, 6 * (R + 2), 6 * (R + 2)), np.uint32)
    sv = scene_view(scene)
    lib().vcto_voxelize_opacity(C.byref(sv), R, _p(_regions_arg(regions)), _p(atlas), level_mask)
    return atlas


def voxelize_conservative(scene, R: int, regions: np.ndarray, level_mask: int = 0x3F,
                          atlas: np.ndarray | None = None) -> np.ndarray:
    """The conservative voxelisation mode (triangle / box overlap, Schwarz & Seidel 2010) into an opacity
    atlas: every voxel of each level's region that a triangle touches."""
    if atlas is None:
        atlas = np.zeros((R + 2, 6 * (R + 2), 6 * (R + 2)), np.uint32)
    sv = scene_view(scene)
    lib().vcto_voxelize_conservative(C.byref(sv), R, _p(_regions_arg(regions)), _p(atlas), level_mask)
    return atlas


def cons_overlap(tri, region_row, R: int, i: int, j: int, k: int) -> bool:
    """One overlap decision of the conservative mode: triangle (3 x 3 world floats) against voxel (i, j, k)
    of the region given as one clip_regions row."""
    t = np.ascontiguousarray(tri, np.float32).reshape(9)
    rg = np.ascontiguousarray(region_row, np.int32).reshape(7)
    return bool(lib().vcto_cons_overlap(_p(t), _p(rg), R, i, j, k))


def shadow_depth(scene, shadow_desc_bytes: bytes, W: int, H: int) -> np.ndarray:
    depth = np.empty((H, W), np.float32)
    sd = np.frombuffer(shadow_desc_bytes, np.uint8).copy()
    sv = scene_view(scene)
    lib().vcto_shadow_depth(C.byref(sv), _p(sd), _p(depth), W, H)
    return depth


def update_clip_regions(regions: np.ndarray, cam, R: int, extent_l0: int = 16):
    """Toroidal region update: moves `regions` ((6, 7) int32 records, in place) and returns the slabs
    ((n, 7) records) and their levels."""
    assert regions.dtype == np.int32 and regions.flags["C_CONTIGUOUS"]
    slabs = np.zeros((18, 7), np.int32)
    levels = np.zeros(18, np.int32)
    c = np.asarray(cam, np.float32)
    n = lib().vcto_update_clip_regions(_p(regions), _p(c), R, extent_l0, _p(slabs), _p(levels))
    return slabs[:n].copy(), levels[:n].copy()


def voxelize_opacity_slabs(scene, R: int, regions: np.ndarray, atlas: np.ndarray, slabs: np.ndarray,
                           levels: np.ndarray) -> None:
    sv = scene_view(scene)
    lib().vcto_voxelize_opacity_slabs(C.byref(sv), R, _p(_regions_arg(regions)), _p(atlas),
                                      _p(np.ascontiguousarray(slabs, np.int32)),
                                      _p(np.ascontiguousarray(levels, np.int32)), len(levels))


def camera_matrix(position, direction, up=(0.0, 1.0, 0.0), fovy_degrees=60.0, aspect=16.0 / 9.0) -> np.ndarray:
    """Camera::updateCamera's CamMatrix block as 36 float32 (view_proj, view_proj_inv, eye, padding)."""
    out = np.zeros(36, np.float32)
    v = [np.asarray(x, np.float32) for x in (position, direction, up)]
    lib().vcto_camera_matrix(_p(v[0]), _p(v[1]), _p(v[2]), fovy_degrees, aspect, _p(out))
    return out


def inverse4(m: np.ndarray) -> np.ndarray:
    """glm::inverse of a column-major 4x4 (16 float32)."""
    out = np.zeros(16, np.float32)
    lib().vcto_inverse4(_p(np.ascontiguousarray(m, np.float32)), _p(out))
    return out


def gbuffer(scene, cam: np.ndarray, W: int, H: int) -> np.ndarray:
    """GBufferPass at one centre sample per pixel: (H * W, 20) float32 vct_surface_sample rows."""
    out = np.zeros((W * H, 20), np.float32)
    sv = scene_view(scene)
    lib().vcto_gbuffer(C.byref(sv), _p(np.ascontiguousarray(cam, np.float32)), W, H, _p(out))
    return out


def gaussian_stencil() -> np.ndarray:
    """The Gaussian blur's 3 x 3 stencil (row-major dy, dx = -1..1), divided by 241."""
    w = np.zeros(9, np.float32)
    lib().vcto_gaussian_stencil(_p(w))
    return w


def specular_filter(diffuse: np.ndarray, specular: np.ndarray, gamma=2.2, exposure=0.1, tonemap=0,
                    method=1) -> np.ndarray:
    """specularFilter.frag over (H, W, 4) float32 images -> (H, W, 4) float32."""
    H, W = diffuse.shape[:2]
    fd = np.array([gamma, exposure], np.float32).tobytes() + np.array([tonemap, method], np.int32).tobytes()
    fd = np.frombuffer(fd, np.uint8).copy()
    out = np.zeros((H, W, 4), np.float32)
    lib().vcto_specular_filter(_p(fd), _p(np.ascontiguousarray(diffuse, np.float32)),
                               _p(np.ascontiguousarray(specular, np.float32)), W, H, _p(out))
    return out


def present_srgb8(rgba: np.ndarray) -> np.ndarray:
    """FinalPass into B8G8R8A8_SRGB: uint32 per pixel (bytes B, G, R, A)."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(rgba.shape[:-1], np.uint32)
    lib().vcto_present_srgb8(_p(rgba), out.size, _p(out))
    return out


def inject_radiance(scene, R: int, regions: np.ndarray, shadow: np.ndarray | None, shadow_desc_bytes: bytes,
                    light_bytes: bytes | None = None, level_mask: int = 0x3F,
                    atlas: np.ndarray | None = None) -> np.ndarray:
    if atlas is None:
        atlas = np.zeros((R + 2, 6 * (R + 2), 6 * (R + 2)), np.uint32)
    sd = np.frombuffer(shadow_desc_bytes, np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    sv = scene_view(scene)
    lib().vcto_inject_radiance(C.byref(sv), R, _p(_regions_arg(regions)), _p(shadow), sw, sh, _p(sd), _p(light),
                               _p(atlas), level_mask)
    return atlas


def svo_fragments(scene, level: int, bb_min, bb_max, shadow: np.ndarray | None, shadow_desc_bytes: bytes,
                  light_bytes: bytes | None = None, capacity: int | None = None):
    sd = np.frombuffer(shadow_desc_bytes, np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    sv = scene_view(scene)
    bmin = np.asarray(bb_min, np.float32)
    bmax = np.asarray(bb_max, np.float32)
    if capacity is None:
        capacity = int(lib().vcto_svo_fragments(C.byref(sv), level, _p(bmin), _p(bmax), _p(shadow), sw, sh, _p(sd),
                                                _p(light), None, 0))
    frags = np.zeros((max(capacity, 1), 2), np.uint32)
    n = int(lib().vcto_svo_fragments(C.byref(sv), level, _p(bmin), _p(bmax), _p(shadow), sw, sh, _p(sd), _p(light),
                                     _p(frags), capacity))
    return frags[:min(n, capacity)], n


def svo_build(frags: np.ndarray, level: int, capacity: int | None = None):
    F = frags.shape[0]
    if capacity is None:
        capacity = min(max(8 * F, 1_000_000), 500_000_000)
    pool = np.zeros((capacity, 2), np.uint32)
    nodes = np.zeros(1, np.int64)
    rc = lib().vcto_svo_build(_p(np.ascontiguousarray(frags, np.uint32)), F, level, _p(pool), capacity, _p(nodes))
    if rc != 0:
        raise RuntimeError("oracle svo_build: node pool capacity exceeded")
    return pool[:int(nodes[0])], int(nodes[0])


SPONZA_BB_MIN = (-15.367, -1.011, -9.462)   # voxelConeTracing_Octree.frag:321
SPONZA_BB_MAX = (14.399, 11.43, 8.84)       # voxelConeTracing_Octree.frag:322


def svo_trace(precision: int, desc_bytes: bytes, eye, pool: np.ndarray, samples: np.ndarray,
              bb_min=SPONZA_BB_MIN, bb_max=SPONZA_BB_MAX, shadow: np.ndarray | None = None,
              shadow_desc_bytes: bytes | None = None, light_bytes: bytes | None = None):
    """voxelConeTracing_Octree.frag over a node pool ((n, 2) uint32); returns (diffuse, specular, steps)."""
    n = samples.shape[0]
    dout = np.zeros((n, 4), np.float64)
    sout = np.zeros((n, 4), np.float64)
    desc = np.frombuffer(desc_bytes, np.uint8).copy()
    sd = np.frombuffer(shadow_desc_bytes or bytes(136), np.uint8).copy()
    light = np.frombuffer(light_bytes or default_light_bytes(), np.uint8).copy()
    sh, sw = (shadow.shape if shadow is not None else (0, 0))
    steps = lib().vcto_svo_trace(precision, _p(desc), _p(np.asarray(eye, np.float32)),
                                 _p(np.ascontiguousarray(pool, np.uint32)), _p(np.asarray(bb_min, np.float32)),
                                 _p(np.asarray(bb_max, np.float32)), _p(shadow), sw, sh, _p(sd), _p(light),
                                 _p(samples), 0, n, _p(dout), _p(sout))
    return dout, sout, int(steps)
