"""A headless clipmap VCT instance (vct_context) and batched submission.

``Context`` owns an instance's atlases, depth map, radiance texture,
workspace and trace scratch (vct_create); ``frame`` runs Application::run's
pre-passes on it and ``trace`` the cone-tracing pass.  ``batch_submit`` runs
many (frame + trace) jobs over several streams at once (vct_batch_submit).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import capi
from .clipmap import _ptr, _stream


class Context:
    def __init__(self, R: int, shadow_size: int = 2048, workspace_bytes: int = 0, flags: int = 0):
        """`flags`: capi.CONTEXT_AUTOTUNE (tune the fast trace's launch shape on the first trace),
        capi.CONTEXT_OPACITY_R8 (one-byte opacity atlas)."""
        cfg = capi.Config(R, shadow_size, shadow_size, flags, workspace_bytes)
        h = C.c_void_p()
        capi.call("vct_create", capi.ref(cfg), C.byref(h))
        self.handle = h
        self.R = R
        self.flags = flags

    def buffers(self) -> capi.ContextBuffers:
        b = capi.ContextBuffers()
        capi.call("vct_context_buffers_get", self.handle, capi.ref(b))
        return b

    def atlas(self, which: str) -> torch.Tensor:
        """A torch view of the instance's opacity or radiance atlas (int32, [D, H, W]; a CONTEXT_OPACITY_R8
        context's opacity atlas as uint8)."""
        b = self.buffers()
        ptr = b.opacity if which == "opacity" else b.radiance
        D, H, W = self.R + 2, 6 * (self.R + 2), 6 * (self.R + 2)
        if which == "opacity" and self.flags & capi.CONTEXT_OPACITY_R8:
            return _device_view(ptr, (D, H, W), "|u1")
        return _device_view(ptr, (D, H, W))

    def reset(self) -> None:
        capi.call("vct_context_reset", self.handle)

    def frame(self, dscene, camera_pos, light: capi.DirectionalLightDesc,
              light_shadow: capi.DirectionalLightShadowDesc, revoxelization: int = capi.REVOX_FULL) -> None:
        cam = (C.c_float * 3)(*camera_pos)
        capi.call("vct_context_frame", self.handle, capi.ref(dscene.desc), C.cast(cam, C.c_void_p), capi.ref(light),
                  capi.ref(light_shadow), revoxelization, _stream())

    def trace(self, desc: capi.ConeTracingDesc, eye, samples: torch.Tensor, light: capi.DirectionalLightDesc,
              light_shadow: capi.DirectionalLightShadowDesc, diffuse: torch.Tensor | None = None,
              specular: torch.Tensor | None = None, steps: torch.Tensor | None = None):
        n = samples.shape[0]
        if diffuse is None:
            diffuse = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
        if specular is None:
            specular = torch.zeros((n, 4), dtype=torch.float32, device=samples.device)
        cam = capi.CamMatrix()
        cam.eye_pos = capi.f3(*[float(x) for x in eye])
        capi.call("vct_context_trace", self.handle, capi.ref(desc), capi.ref(cam), capi.ref(light),
                  capi.ref(light_shadow), _ptr(samples), n, _ptr(diffuse), _ptr(specular), _ptr(steps), _stream())
        return diffuse, specular

    def close(self) -> None:
        if self.handle:
            capi.call("vct_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _device_view(ptr: int, shape, typestr: str = "<i4") -> torch.Tensor:
    """A torch tensor (int32 unless `typestr` says otherwise) over device memory owned by the library (no copy)."""
    import numpy as np
    n = int(np.prod(shape))

    class _Iface:
        __cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                    "version": 2, "strides": None}
    t = torch.as_tensor(_Iface(), device="cuda")
    assert t.numel() == n
    return t


def batch_job(ctx: Context, dscene, camera_pos, light, light_shadow, desc: capi.ConeTracingDesc, eye,
              samples: torch.Tensor, diffuse: torch.Tensor, specular: torch.Tensor,
              steps: torch.Tensor | None = None, reset: bool = True, revoxelization: int = capi.REVOX_FULL):
    """A vct_batch_job (the structs it points at are kept alive on the returned object)."""
    j = capi.BatchJob()
    j.context = ctx.handle
    j.scene = C.cast(C.pointer(dscene.desc), C.c_void_p)
    j.camera_pos = capi.f3(*camera_pos)
    j.revoxelization = revoxelization
    j.reset = 1 if reset else 0
    j.light = light
    j.light_shadow = light_shadow
    cam = capi.CamMatrix()
    cam.eye_pos = capi.f3(*[float(x) for x in eye])
    j._keep = (desc, cam, dscene)
    j.trace_desc = C.cast(C.pointer(desc), C.c_void_p)
    j.cam = C.cast(C.pointer(cam), C.c_void_p)
    j.samples = samples.data_ptr()
    j.sample_count = samples.shape[0]
    j.diffuse_out = diffuse.data_ptr()
    j.specular_out = specular.data_ptr()
    j.cone_steps = steps.data_ptr() if steps is not None else None
    return j


def batch_submit(jobs, streams: int = 4) -> None:
    arr = (capi.BatchJob * len(jobs))(*jobs)
    capi.call("vct_batch_submit", C.cast(arr, C.c_void_p), len(jobs), streams)
