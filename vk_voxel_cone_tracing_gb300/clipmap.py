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


def new_atlas_r8(R: int, device="cuda") -> torch.Tensor:
    """A zeroed one-byte-per-texel opacity atlas (vct_frame_desc.opacity_format = OPACITY_R8), [D, H, W]."""
    D, H, W = R + 2, 6 * (R + 2), 6 * (R + 2)
    return torch.zeros((D, H, W), dtype=torch.uint8, device=device)


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


def cmd_copy_alpha_downsample(radiance: torch.Tensor, opacity: torch.Tensor, R: int, prev_region_min, level: int,
                              band: int = capi.DOWNSAMPLE_REGION_SIZE, mirror=None) -> None:
    """vct_copy_alpha (level) + vct_downsample (radiance, level) fused into one pass; `mirror` (a
    RadianceTexture) receives every texel written."""
    d = capi.DownSampleDesc(capi.i3(*prev_region_min), level, R, band)
    capi.call("vct_copy_alpha_downsample", _ptr(radiance), _ptr(opacity), capi.ref(d),
              mirror.handle if mirror is not None else None, _stream())


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
               specular: torch.Tensor | None = None, steps: torch.Tensor | None = None,
               diffuse_aperture: float = 0.0):
    """VoxelConeTracingPass over `samples` ((n, 20) float32 vct_surface_sample records); a non-zero
    `diffuse_aperture` (radians) replaces the shader's diffuse cone aperture (vct_cone_trace_opt)."""
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
    opt = capi.TraceOptions(diffuse_aperture)
    capi.call("vct_cone_trace_opt", capi.ref(desc), capi.ref(cam), _ptr(radiance), R, capi.ref(sm), capi.ref(light),
              capi.ref(sd), _ptr(samples), n, _ptr(diffuse), _ptr(specular), _ptr(steps), capi.ref(opt), _stream())
    return diffuse, specular


# ----------------------------------------------------------------- fast form

def cone_trace_tex(desc: capi.ConeTracingDesc, eye, tex: "RadianceTexture", samples: torch.Tensor,
                   light: capi.DirectionalLightDesc | None = None, shadow: torch.Tensor | None = None,
                   shadow_desc: capi.DirectionalLightShadowDesc | None = None, diffuse: torch.Tensor | None = None,
                   specular: torch.Tensor | None = None, steps: torch.Tensor | None = None,
                   diffuse_aperture: float = 0.0):
    """cone_trace (the exact FP32 arithmetic, same results bit for bit) reading the texels through the RGBA8
    texture `tex`, which must hold the atlas's texels (vct_cone_trace_tex)."""
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
    opt = capi.TraceOptions(diffuse_aperture)
    capi.call("vct_cone_trace_tex", capi.ref(desc), capi.ref(cam), tex.handle, capi.ref(sm), capi.ref(light),
              capi.ref(sd), _ptr(samples), n, _ptr(diffuse), _ptr(specular), _ptr(steps), capi.ref(opt), _stream())
    return diffuse, specular


class RadianceTexture:
    """Hardware-filtered copy of a radiance atlas (vct_texture_*): RGBA8 or RGBA16F."""

    def __init__(self, R: int, fmt: int = capi.TEX_RGBA8):
        self.R = R
        self.fmt = fmt
        h = C.c_void_p()
        capi.call("vct_texture_create", R, fmt, C.byref(h))
        self.handle = h

    def update(self, atlas: torch.Tensor) -> "RadianceTexture":
        capi.call("vct_texture_update", self.handle, _ptr(atlas), _stream())
        return self

    def read(self, out: torch.Tensor) -> torch.Tensor:
        """Copy the texture back into a linear atlas of its format."""
        capi.call("vct_texture_read", self.handle, _ptr(out), _stream())
        return out

    def close(self) -> None:
        if self.handle:
            capi.call("vct_texture_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def new_atlas_rgba16f(R: int, device="cuda") -> torch.Tensor:
    """Zeroed RGBA16F atlas: 4 halves per texel, shape (R+2, 6(R+2), 6(R+2)*4) as int16."""
    d, h, w = atlas_shape(R)
    return torch.zeros((d, h, w * 4), dtype=torch.int16, device=device)


def _mirror(tex: "RadianceTexture | None"):
    return None if tex is None else tex.handle


def to_rgba16f(atlas: torch.Tensor, R: int, out: torch.Tensor | None = None,
               mirror: "RadianceTexture | None" = None) -> torch.Tensor:
    """The RGBA8 atlas as RGBA16F; `mirror` (an RGBA16F RadianceTexture) receives every texel too."""
    out = new_atlas_rgba16f(R, atlas.device) if out is None else out
    capi.call("vct_atlas_rgba8_to_rgba16f", _ptr(atlas), _ptr(out), R, _mirror(mirror), _stream())
    return out


def cmd_downsample_rgba16f(atlas16: torch.Tensor, R: int, prev_region_min, level: int, mode: int,
                           band: int = capi.DOWNSAMPLE_REGION_SIZE, mirror: "RadianceTexture | None" = None) -> None:
    d = capi.DownSampleDesc(capi.i3(*prev_region_min), level, R, band)
    capi.call("vct_downsample_rgba16f", _ptr(atlas16), capi.ref(d), mode, _mirror(mirror), _stream())


def cmd_downsample_rgba16f_all(atlas16: torch.Tensor, R: int, regions, mode: int,
                               mirror: "RadianceTexture | None" = None) -> None:
    for level in range(1, 6):
        prev = regions[level - 1].min_corner
        cmd_downsample_rgba16f(atlas16, R, (prev[0], prev[1], prev[2]), level, mode, mirror=mirror)


def fast_scratch(n: int, device="cuda") -> torch.Tensor:
    nbytes = capi.lib().vct_cone_trace_fast_scratch_bytes(n)
    if nbytes < 0:
        raise ValueError(f"sample count {n} out of range")
    return torch.empty(nbytes + 256, dtype=torch.uint8, device=device)


def _aligned(t: torch.Tensor, align: int = 256) -> int:
    p = t.data_ptr()
    return (p + align - 1) // align * align


def cone_trace_fast(desc: capi.ConeTracingDesc, eye, tex: RadianceTexture, samples: torch.Tensor,
                    light: capi.DirectionalLightDesc | None = None, shadow: torch.Tensor | None = None,
                    shadow_desc: capi.DirectionalLightShadowDesc | None = None,
                    diffuse: torch.Tensor | None = None, specular: torch.Tensor | None = None,
                    steps: torch.Tensor | None = None, scratch: torch.Tensor | None = None,
                    diffuse_aperture: float = 0.0):
    """GB300 form of VoxelConeTracingPass: same inputs/outputs as cone_trace, sampling `tex`; a non-zero
    `diffuse_aperture` (radians) replaces the shader's diffuse cone aperture (vct_cone_trace_fast_opt)."""
    n = samples.shape[0]
    if diffuse is None:
        diffuse = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    if specular is None:
        specular = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    if scratch is None:
        scratch = fast_scratch(n, samples.device)
    base = _aligned(scratch)
    avail = scratch.data_ptr() + scratch.numel() - base
    cam = cam_matrix(eye)
    light = light or capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    sm = capi.ShadowMap(None, 0, 0)
    if shadow is not None:
        sm = capi.ShadowMap(shadow.data_ptr(), shadow.shape[1], shadow.shape[0])
    sd = shadow_desc or capi.DirectionalLightShadowDesc()
    opt = capi.TraceOptions(diffuse_aperture)
    capi.call("vct_cone_trace_fast_opt", capi.ref(desc), capi.ref(cam), tex.handle, capi.ref(sm), capi.ref(light),
              capi.ref(sd), _ptr(samples), n, _ptr(diffuse), _ptr(specular), _ptr(steps), capi.ref(opt),
              C.c_void_p(base), avail, _stream())
    return diffuse, specular


def autotune_fast(desc: capi.ConeTracingDesc, eye, tex: RadianceTexture, samples: torch.Tensor,
                  light: capi.DirectionalLightDesc | None = None, shadow: torch.Tensor | None = None,
                  shadow_desc: capi.DirectionalLightShadowDesc | None = None, diffuse: torch.Tensor | None = None,
                  specular: torch.Tensor | None = None, scratch: torch.Tensor | None = None) -> dict:
    """vct_cone_trace_fast_autotune: times the fast trace of these inputs under a few launch shapes (the results
    are the same under every shape) and keeps the fastest for this device and the texture's resolution."""
    n = samples.shape[0]
    if diffuse is None:
        diffuse = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    if specular is None:
        specular = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
    if scratch is None:
        scratch = fast_scratch(n, samples.device)
    base = _aligned(scratch)
    cam = cam_matrix(eye)
    light = light or capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    sm = capi.ShadowMap(shadow.data_ptr(), shadow.shape[1], shadow.shape[0]) if shadow is not None else \
        capi.ShadowMap(None, 0, 0)
    sd = shadow_desc or capi.DirectionalLightShadowDesc()
    t = capi.TraceTuning()
    capi.call("vct_cone_trace_fast_autotune", capi.ref(desc), capi.ref(cam), tex.handle, capi.ref(sm), capi.ref(light),
              capi.ref(sd), _ptr(samples), n, _ptr(diffuse), _ptr(specular), C.c_void_p(base),
              scratch.data_ptr() + scratch.numel() - base, capi.ref(t), _stream())
    return {"diffuse_blocks_per_sm": t.diffuse_blocks_per_sm, "specular_blocks_per_sm": t.specular_blocks_per_sm,
            "trace_ms": t.trace_ms, "default_ms": t.default_ms}


def trace_tuning(R: int) -> dict:
    """vct_trace_tuning_get: the launch shape the fast trace uses at resolution R on the current device."""
    t = capi.TraceTuning()
    capi.call("vct_trace_tuning_get", R, capi.ref(t))
    return {"diffuse_blocks_per_sm": t.diffuse_blocks_per_sm, "specular_blocks_per_sm": t.specular_blocks_per_sm,
            "tuned": bool(t.tuned)}


def trace_job(desc: capi.ConeTracingDesc, eye, tex: RadianceTexture, samples: torch.Tensor,
              diffuse: torch.Tensor, specular: torch.Tensor, light: capi.DirectionalLightDesc | None = None,
              shadow: torch.Tensor | None = None, shadow_desc: capi.DirectionalLightShadowDesc | None = None,
              steps: torch.Tensor | None = None) -> capi.TraceJob:
    """One vct_trace_job record (the tensors must outlive the batched call)."""
    j = capi.TraceJob()
    j.desc = desc
    j.eye = capi.f3(*[float(x) for x in eye])
    j.radiance = tex.handle
    j.shadow = capi.ShadowMap(shadow.data_ptr(), shadow.shape[1], shadow.shape[0]) if shadow is not None else \
        capi.ShadowMap(None, 0, 0)
    j.light = light or capi.DirectionalLightDesc(capi.f3(0.3, -1.0, 0.2), 1.0, capi.f3(1, 1, 1), 0)
    j.light_shadow = shadow_desc or capi.DirectionalLightShadowDesc()
    j.samples = samples.data_ptr() if samples.numel() else None
    j.sample_count = samples.shape[0]
    j.diffuse_out = diffuse.data_ptr() if diffuse.numel() else None
    j.specular_out = specular.data_ptr() if specular.numel() else None
    j.cone_steps = steps.data_ptr() if steps is not None else None
    return j


def cone_trace_fast_batch(jobs: list, scratch: torch.Tensor | None = None) -> None:
    """vct_cone_trace_fast_batch over a list of trace_job records (one launch per stage for every job)."""
    arr = (capi.TraceJob * max(1, len(jobs)))(*jobs)
    need = capi.lib().vct_cone_trace_fast_batch_scratch_bytes(C.cast(arr, C.c_void_p), len(jobs))
    if need < 0:
        raise ValueError("too many samples for one batched trace")
    if scratch is None or scratch.numel() < need + 256:
        scratch = torch.empty(need + 256, dtype=torch.uint8, device="cuda")
    base = _aligned(scratch)
    capi.call("vct_cone_trace_fast_batch", C.cast(arr, C.c_void_p), len(jobs), C.c_void_p(base),
              scratch.data_ptr() + scratch.numel() - base, _stream())


def gather_probe(desc: capi.ConeTracingDesc, tex: RadianceTexture, cones: int = 152 * 1024, steps_per_cone: int = 64) -> float:
    """Measured cone-sample rate of the pure fetch pattern (vct_gather_probe): the trace's speed of light."""
    rate = C.c_double(0.0)
    capi.call("vct_gather_probe", capi.ref(desc), tex.handle, cones, steps_per_cone, C.byref(rate), _stream())
    return rate.value
