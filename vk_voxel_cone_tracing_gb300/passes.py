"""Python face of the rasterisation-driven passes (voxelise, shadow depth,
radiance injection, SVO fragment list) over torch device tensors.

``DeviceScene`` uploads a ``scene.Scene`` into the vct_scene layout;
``Workspace`` owns the device scratch arena the raster passes use.  Every
function calls the CUDA library through the C ABI on the current stream.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import capi
from .clipmap import _ptr, _stream
from .scene import world_positions


class Workspace:
    """vct_workspace: device scratch arena grown on demand by the raster passes."""

    def __init__(self, initial_bytes: int = 0):
        h = C.c_void_p()
        capi.call("vct_workspace_create", initial_bytes, C.byref(h))
        self.handle = h

    @property
    def nbytes(self) -> int:
        return int(capi.lib().vct_workspace_bytes(self.handle))

    def close(self):
        if self.handle:
            capi.call("vct_workspace_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceScene:
    """A scene.Scene resident on the GPU, with its vct_scene descriptor."""

    def __init__(self, scene, device="cuda"):
        self.positions = torch.from_numpy(np.ascontiguousarray(scene.positions, np.float32)).to(device)
        self.normals = torch.from_numpy(np.ascontiguousarray(scene.normals, np.float32)).to(device)
        self.indices = torch.from_numpy(np.ascontiguousarray(scene.indices, np.uint32).view(np.int32)).to(device)
        self.tri_material = torch.from_numpy(np.ascontiguousarray(scene.tri_material, np.uint32).view(np.int32)).to(device)
        self.materials = torch.from_numpy(np.ascontiguousarray(scene.materials).view(np.uint8)).to(device)
        self.textures = torch.from_numpy(np.ascontiguousarray(scene.textures, np.uint32).view(np.int32)).to(device)
        nm, ti, ninst = None, None, 0
        if getattr(scene, "node_matrices", None) is not None:
            self.node_matrices = torch.from_numpy(np.ascontiguousarray(scene.node_matrices, np.float32)).to(device)
            self.tri_instance = torch.from_numpy(
                np.ascontiguousarray(scene.tri_instance, np.uint32).view(np.int32)).to(device)
            nm, ti, ninst = self.node_matrices.data_ptr(), self.tri_instance.data_ptr(), scene.node_matrices.shape[0]
        self.desc = capi.Scene(self.positions.data_ptr(), self.normals.data_ptr(), self.indices.data_ptr(),
                               scene.positions.shape[0], scene.indices.shape[0], self.tri_material.data_ptr(),
                               self.materials.data_ptr(), scene.materials.shape[0], self.textures.data_ptr(),
                               scene.textures.shape[0], nm, ti, ninst)
        p = world_positions(scene)
        self.bb_min = p.min(0).astype(np.float32)
        self.bb_max = p.max(0).astype(np.float32)

    @property
    def triangle_count(self) -> int:
        return int(self.desc.triangle_count)


def light_desc(direction=(0.3, -1.0, 0.2), intensity=1.0, color=(1.0, 1.0, 1.0)) -> capi.DirectionalLightDesc:
    return capi.DirectionalLightDesc(capi.f3(*direction), intensity, capi.f3(*color), 0)


def light_shadow_desc(origin, direction, z_near=0.1, z_far=30.0) -> capi.DirectionalLightShadowDesc:
    out = capi.DirectionalLightShadowDesc()
    o = (C.c_float * 3)(*origin)
    d = (C.c_float * 3)(*direction)
    capi.call("vct_directional_light_shadow", C.cast(o, C.c_void_p), C.cast(d, C.c_void_p), z_near, z_far,
              capi.ref(out))
    return out


def camera_matrix(position, direction, up=(0.0, 1.0, 0.0), fovy_degrees=60.0, aspect=16.0 / 9.0) -> capi.CamMatrix:
    """Camera::updateCamera's CamMatrix block (view-projection, its inverse, eye)."""
    out = capi.CamMatrix()
    vecs = [(C.c_float * 3)(*v) for v in (position, direction, up)]
    capi.call("vct_camera_matrix", *[C.cast(v, C.c_void_p) for v in vecs], fovy_degrees, aspect, capi.ref(out))
    return out


def gbuffer(dscene: DeviceScene, cam: capi.CamMatrix, width: int, height: int, ws: Workspace,
            out: torch.Tensor | None = None) -> torch.Tensor:
    """GBufferPass: the camera's per-pixel surface records, an (height * width, 20) float32 tensor
    (vct_surface_sample rows, row-major pixels; depth 1 where nothing was drawn)."""
    n = width * height
    if out is None:
        out = torch.empty((n, 20), dtype=torch.float32, device=dscene.positions.device)
    if out.shape != (n, 20) or out.dtype != torch.float32 or not out.is_contiguous():
        raise ValueError("gbuffer: out must be a contiguous (width * height, 20) float32 tensor")
    capi.call("vct_gbuffer", capi.ref(dscene.desc), capi.ref(cam), width, height, _ptr(out), ws.handle, _stream())
    return out


def clear_atlas(atlas: torch.Tensor, R: int) -> None:
    capi.call("vct_clear_atlas", _ptr(atlas), R, _stream())


def voxelize_opacity(dscene: DeviceScene, regions, R: int, atlas: torch.Tensor, ws: Workspace,
                     level_mask: int = 0x3F) -> None:
    capi.call("vct_voxelize_opacity", capi.ref(dscene.desc), C.cast(regions, C.c_void_p), R, _ptr(atlas),
              level_mask, ws.handle, _stream())


def voxelize_opacity_conservative(dscene: DeviceScene, regions, R: int, atlas: torch.Tensor,
                                  level_mask: int = 0x3F) -> None:
    """The conservative voxelisation mode: every voxel of each level's region a triangle touches (triangle /
    box overlap, Schwarz & Seidel 2010), stored like voxelize_opacity."""
    capi.call("vct_voxelize_opacity_conservative", capi.ref(dscene.desc), C.cast(regions, C.c_void_p), R,
              _ptr(atlas), level_mask, _stream())


def shadow_depth(dscene: DeviceScene, sd: capi.DirectionalLightShadowDesc, depth: torch.Tensor, ws: Workspace) -> None:
    H, W = depth.shape
    capi.call("vct_shadow_depth", capi.ref(dscene.desc), capi.ref(sd), _ptr(depth), W, H, ws.handle, _stream())


def _shadow_map(depth: torch.Tensor | None) -> capi.ShadowMap:
    if depth is None:
        return capi.ShadowMap(None, 0, 0)
    return capi.ShadowMap(depth.data_ptr(), depth.shape[1], depth.shape[0])


def inject_radiance(dscene: DeviceScene, regions, R: int, depth: torch.Tensor | None,
                    light: capi.DirectionalLightDesc, sd: capi.DirectionalLightShadowDesc, atlas: torch.Tensor,
                    ws: Workspace, level_mask: int = 0x3F, mode: int = capi.INJECT_DETERMINISTIC) -> None:
    sm = _shadow_map(depth)
    capi.call("vct_inject_radiance", capi.ref(dscene.desc), C.cast(regions, C.c_void_p), R, capi.ref(sm),
              capi.ref(light), capi.ref(sd), _ptr(atlas), level_mask, mode, ws.handle, _stream())


def svo_fragments(dscene: DeviceScene, level: int, depth: torch.Tensor | None, light: capi.DirectionalLightDesc,
                  sd: capi.DirectionalLightShadowDesc, ws: Workspace, bb_min=None, bb_max=None,
                  out: torch.Tensor | None = None):
    """The SVO fragment list as an (F, 2) int32 tensor (a view of `out` when it is large enough).

    Without `out` this is the reference's two-step shape: a count-only call, then the write into a buffer
    of that size.  With `out` (for instance the previous frame's list) it is one call; when `out` is too
    small the call reports the count and is repeated into a new buffer."""
    bmin = (C.c_float * 3)(*(dscene.bb_min if bb_min is None else bb_min))
    bmax = (C.c_float * 3)(*(dscene.bb_max if bb_max is None else bb_max))
    sm = _shadow_map(depth)
    count = C.c_int64(0)

    def run(buf, cap):
        return capi.lib().vct_svo_fragments(capi.ref(dscene.desc), level, C.cast(bmin, C.c_void_p),
                                            C.cast(bmax, C.c_void_p), capi.ref(sm), capi.ref(light), capi.ref(sd),
                                            _ptr(buf) if buf is not None else None, cap, C.byref(count),
                                            ws.handle, _stream())

    if out is not None and out.shape[0] > 0:
        rc = run(out, out.shape[0])
        if rc == capi.VCT_OK:
            return out[:count.value]
        if rc != capi.VCT_E_OVERFLOW:
            capi.check("vct_svo_fragments", rc)
    else:
        capi.check("vct_svo_fragments", run(None, 0))
    frags = torch.empty((max(count.value, 1), 2), dtype=torch.int32, device=dscene.positions.device)
    capi.check("vct_svo_fragments", run(frags, count.value))
    return frags[:count.value]


def svo_pool_capacity(fragment_count: int) -> int:
    return int(capi.lib().vct_svo_pool_capacity(fragment_count))


def svo_build(frags: torch.Tensor, level: int, ws: Workspace, mode: int = capi.SVO_DETERMINISTIC,
              capacity: int | None = None):
    """OctreeBuilder::cmdBuild over an (F, 2) fragment tensor; returns (pool[(n, 2) int32], n)."""
    F = frags.shape[0]
    cap = svo_pool_capacity(F) if capacity is None else capacity
    pool = torch.empty((cap, 2), dtype=torch.int32, device=frags.device)
    n = C.c_int64(0)
    capi.call("vct_svo_build", _ptr(frags) if F else None, F, level, _ptr(pool), cap, mode, C.byref(n), ws.handle,
              _stream())
    return pool, int(n.value)


def svo_canonicalize(pool: torch.Tensor, node_count: int, level: int, ws: Workspace) -> torch.Tensor:
    out = torch.zeros((node_count, 2), dtype=torch.int32, device=pool.device)
    capi.call("vct_svo_canonicalize", _ptr(pool), node_count, level, _ptr(out), ws.handle, _stream())
    return out


SPONZA_BB_MIN = (-15.367, -1.011, -9.462)   # voxelConeTracing_Octree.frag:321
SPONZA_BB_MAX = (14.399, 11.43, 8.84)       # voxelConeTracing_Octree.frag:322


def svo_cone_trace(desc: capi.ConeTracingDesc, eye, pool: torch.Tensor, node_count: int, samples: torch.Tensor,
                   bb_min=SPONZA_BB_MIN, bb_max=SPONZA_BB_MAX, light: capi.DirectionalLightDesc | None = None,
                   shadow: torch.Tensor | None = None, shadow_desc: capi.DirectionalLightShadowDesc | None = None,
                   steps: torch.Tensor | None = None):
    from .clipmap import cam_matrix
    n = samples.shape[0]
    dout = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    sout = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    light = light or light_desc()
    sd = shadow_desc or capi.DirectionalLightShadowDesc()
    sm = _shadow_map(shadow)
    bmin = (C.c_float * 3)(*bb_min)
    bmax = (C.c_float * 3)(*bb_max)
    capi.call("vct_svo_cone_trace", capi.ref(desc), capi.ref(cam_matrix(eye)), _ptr(pool), node_count,
              C.cast(bmin, C.c_void_p), C.cast(bmax, C.c_void_p), capi.ref(sm), capi.ref(light), capi.ref(sd),
              _ptr(samples), n, _ptr(dout), _ptr(sout), _ptr(steps), _stream())
    return dout, sout


def clipmap_frame(dscene: DeviceScene, camera_pos, R: int, opacity: torch.Tensor, radiance: torch.Tensor,
                  shadow: torch.Tensor | None, light: capi.DirectionalLightDesc,
                  light_shadow: capi.DirectionalLightShadowDesc, ws: Workspace, frame_index: int = 0,
                  inject_mode: int = capi.INJECT_DETERMINISTIC, texture=None, revoxelization: int = capi.REVOX_FULL,
                  regions_state=None, opacity_format: int = capi.OPACITY_RGBA8):
    """vct_clipmap_frame: voxelise, mips, border, shadow depth, inject, copy alpha, radiance mips; `texture`
    (an RGBA8 RadianceTexture of resolution R) is kept equal to the radiance atlas's written texels.
    `regions_state` ((ClipmapRegion * 6), kept by the caller) persists the regions between frames: a FULL
    frame writes them, a TOROIDAL frame moves them and revoxelises only the uncovered slabs.  With
    `opacity_format` OPACITY_R8, `opacity` is a uint8 atlas (clipmap.new_atlas_r8) holding the alpha only."""
    f = capi.FrameDesc()
    f.camera_pos = capi.f3(*camera_pos)
    f.clipmap_resolution = R
    f.frame_index = frame_index
    f.inject_mode = inject_mode
    f.shadow_width = shadow.shape[1] if shadow is not None else 0
    f.shadow_height = shadow.shape[0] if shadow is not None else 0
    f.light = light
    f.light_shadow = light_shadow
    f.radiance_texture = texture.handle if texture is not None else None
    f.revoxelization = revoxelization
    f.opacity_format = opacity_format
    f.regions_state = C.cast(regions_state, C.c_void_p) if regions_state is not None else None
    regs = (capi.ClipmapRegion * 6)()
    capi.call("vct_clipmap_frame", capi.ref(dscene.desc), capi.ref(f), _ptr(opacity), _ptr(radiance),
              _ptr(shadow), C.cast(regs, C.c_void_p), ws.handle, _stream())
    return regs


def update_clip_regions(regions, camera_pos, R: int, extent_l0: int = capi.VOXEL_EXTENT_L0):
    """vct_update_clip_regions: moves `regions` ((ClipmapRegion * 6), in place) toward the camera and returns
    the uncovered slabs as (ClipmapRegion * n, [level per slab])."""
    slabs = (capi.ClipmapRegion * 18)()
    levels = (C.c_int32 * 18)()
    n = C.c_int32(0)
    cam = (C.c_float * 3)(*camera_pos)
    capi.call("vct_update_clip_regions", C.cast(regions, C.c_void_p), C.cast(cam, C.c_void_p), R, extent_l0,
              C.cast(slabs, C.c_void_p), C.cast(levels, C.c_void_p), C.byref(n))
    return slabs, list(levels[:n.value])


def voxelize_opacity_slabs(dscene: DeviceScene, regions, R: int, atlas: torch.Tensor, slabs, levels,
                           ws: Workspace) -> None:
    """vct_voxelize_opacity_slabs: clear and revoxelise the listed slabs (toroidal update)."""
    lv = (C.c_int32 * max(1, len(levels)))(*levels)
    capi.call("vct_voxelize_opacity_slabs", capi.ref(dscene.desc), C.cast(regions, C.c_void_p), R, _ptr(atlas),
              C.cast(slabs, C.c_void_p), C.cast(lv, C.c_void_p), len(levels), ws.handle, _stream())
