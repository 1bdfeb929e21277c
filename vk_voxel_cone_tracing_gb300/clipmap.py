"""Python face of the clipmap passes over torch device tensors.

Thin wrappers that validate tensors and call the C ABI (libvct_gb300.so) on
the current torch CUDA stream.  Names follow the reference's recorders
(ClipmapCleaner::cmdClear*, CopyAlpha::cmdImageCopyAlpha,
DownSampler::cmdDownSample*, BorderWrapper::cmdWrapping*Border,
VoxelConeTracingPass::onUpdate).  There is no CPU path: every call runs the
CUDA kernels and raises ``capi.VctError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import capi
from .scene import SAMPLE_DTYPE, atlas_shape


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor | None) -> C.c_void_p | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("tensor must live on the GPU")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return C.c_void_p(t.data_ptr())


def new_atlas(R: int, device="cuda") -> torch.Tensor:
    """Zeroed RGBA8 atlas (uint32 words as int32) in the reference's layout, shape (R+2, 6(R+2), 6(R+2))."""
    return torch.zeros(atlas_shape(R), dtype=torch.int32, device=device)


def clip_regions(camera_pos, R: int, extent_l0: int = capi.VOXEL_EXTENT_L0):
    regs = (capi.ClipmapRegion * 6)()
    cam = (C.c_float * 3)(*[float(x) for x in camera_pos])
    capi.call("vct_clip_regions", C.cast(cam, C.c_void_p), R, extent_l0, C.cast(regs, C.c_void_p))
    return regs


def regions_to_numpy(regs) -> np.ndarray:
    return np.frombuffer(bytes(regs), np.int32).reshape(6, 7).copy()


def cmd_clear_region(atlas: torch.Tensor, R: int, region_min, extent, level: int, faces: int = 6) -> None:
    d = capi.ImageCleaningDesc(capi.i3(*region_min), level, capi.u3(*extent), R, faces)
    capi.call("vct_clear_region", _ptr(atlas), capi.ref(d), _stream())


def cmd_copy_alpha(dst: torch.Tensor, src: torch.Tensor, R: int, level: int, faces: int = 6) -> None:
    d = capi.CopyAlphaDesc(level, R, faces)
    capi.call("vct_copy_alpha", _ptr(dst), _ptr(src), capi.ref(d), _stream())


def cmd_downsample(atlas: torch.Tensor, R: int, prev_region_min, level: int, mode: int,
                   band: int = capi.DOWNSAMPLE_REGION_SIZE) -> None:
    d = capi.DownSampleDesc(capi.i3(*prev_region_min), level, R, band)
    capi.call("vct_downsample", _ptr(atlas), capi.ref(d), mode, _stream())


def cmd_downsample_all(atlas: torch.Tensor, R: int, regions, mode: int) -> None:
    capi.call("vct_downsample_all", _ptr(atlas), C.cast(regions, C.c_void_p), R, mode, _stream())


def cmd_wrap_border(atlas: torch.Tensor, R: int, faces: int = 6, regions: int = 6) -> None:
    d = capi.BorderWrappingDesc(R, capi.VOXEL_BORDER, faces, regions)
    capi.call("vct_wrap_border", _ptr(atlas), capi.ref(d), _stream())


def trace_desc(**kw) -> capi.ConeTracingDesc:
    d = capi.ConeTracingDesc()
    for k, v in kw.items():
        if k == "volume_center":
            d.volume_center = capi.f3(*v)
        else:
            setattr(d, k, v)
    return d


def cam_matrix(eye) -> capi.CamMatrix:
    c = capi.CamMatrix()
    c.eye_pos = capi.f3(*[float(x) for x in eye])
    return c


def samples_to_device(samples: np.ndarray, device="cuda") -> torch.Tensor:
    assert samples.dtype == SAMPLE_DTYPE
    return torch.from_numpy(samples.view(np.float32).reshape(-1, 20).copy()).to(device)


def cone_trace(desc: capi.ConeTracingDesc, eye, radiance: torch.Tensor, R: int, samples: torch.Tensor,
               light: capi.DirectionalLightDesc | None = None, shadow: torch.Tensor | None = None,
               shadow_desc: capi.DirectionalLightShadowDesc | None = None, diffuse: torch.Tensor | None = None,
               specular: torch.Tensor | None = None, steps: torch.Tensor | None = None):
    """VoxelConeTracingPass over `samples` ((n, 20) float32 vct_surface_sample records)."""
    n = samples.shape[0]
    if diffuse is None:
        diffuse = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    if specular is None:
        specular = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    cam = cam_matrix(eye)
    light = light or capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    sm = capi.ShadowMap(None, 0, 0)
    if shadow is not None:
        sm = capi.ShadowMap(shadow.data_ptr(), shadow.shape[1], shadow.shape[0])
    sd = shadow_desc or capi.DirectionalLightShadowDesc()
    capi.call("vct_cone_trace", capi.ref(desc), capi.ref(cam), _ptr(radiance), R, capi.ref(sm), capi.ref(light),
              capi.ref(sd), _ptr(samples), n, _ptr(diffuse), _ptr(specular), _ptr(steps), _stream())
    return diffuse, specular
