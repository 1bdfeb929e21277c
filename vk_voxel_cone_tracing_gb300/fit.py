"""Inverse radiance fitting through the hand-written adjoints.

A float RGBA clipmap (the parameter) is rendered the way the reference's frame
renders its radiance clipmap -- the anisotropic radiance mips of levels 1..5
recomputed from the finer level (DownSampler::cmdDownSampleRadiance,
VFS/RenderPass/Clipmap/DownSampler.cpp:115-168) and then
voxelConeTracing.frag over G-buffer samples -- and fitted to target images
with Adam.  One iteration:

    work  = mips(param)              vct_downsample_f32, levels 1..5 (radiance mode)
    out   = trace(work)              vct_cone_trace_f32 (diffuse and specular images)
    loss  = mean (out - target)^2    vct_sq_error, both images
    grad  = trace^T(dL/d out)        vct_cone_trace_backward (one march, its steps kept)
    grad  = mips^T(grad)             vct_downsample_backward, levels 5..1
    param = adam(param, grad)        vct_adam_step (RGB kept >= 0, alpha in [0, alpha_max])

Every step runs in the library's kernels on the caller's stream; torch only
holds the buffers.  The reference renders forward only, so this is a
build-only capability over the same pass semantics.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import capi
from .clipmap import regions_to_numpy


def _p(t: torch.Tensor | None) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def downsample_desc(regions, level: int, R: int) -> capi.DownSampleDesc:
    """DownSampleDesc of `level` (reads the finer level's region, DownSampler.cpp:115-168)."""
    regs = regions if isinstance(regions, np.ndarray) else regions_to_numpy(regions)
    d = capi.DownSampleDesc()
    d.prev_region_min_corner = capi.i3(*[int(x) for x in regs[level - 1, 0:3]])
    d.clip_level, d.clipmap_resolution, d.downsample_region_size = level, R, capi.DOWNSAMPLE_REGION_SIZE
    return d


class RadianceFit:
    """Fits a float RGBA clipmap of resolution R to target diffuse / specular images of `samples`."""

    def __init__(self, R: int, regions, desc: capi.ConeTracingDesc, cam: capi.CamMatrix,
                 light: capi.DirectionalLightDesc, samples: torch.Tensor, target_diffuse: torch.Tensor | None = None,
                 target_specular: torch.Tensor | None = None, lr: float = 0.02, betas=(0.9, 0.999), eps: float = 1e-8,
                 alpha_max: float = 0.95, init: torch.Tensor | None = None):
        dev = samples.device
        self.R, self.desc, self.cam, self.light = R, desc, cam, light
        self.ds = [None] + [downsample_desc(regions, l, R) for l in range(1, capi.CLIP_LEVEL_COUNT)]
        self.samples = samples
        self.n = samples.shape[0]
        self.target_d = self.target_s = None
        if target_diffuse is not None:
            self.set_targets(target_diffuse, target_specular)
        floats = 4 * int(capi.lib().vct_atlas_texels(R))
        self.param = torch.zeros(floats, dtype=torch.float32, device=dev) if init is None else init.clone()
        self.work = torch.empty_like(self.param)
        self.grad = torch.zeros_like(self.param)
        self.m = torch.zeros_like(self.param)
        self.v = torch.zeros_like(self.param)
        self.dout = torch.empty((self.n, 4), dtype=torch.float32, device=dev)
        self.sout = torch.empty_like(self.dout)
        self.gd = torch.empty_like(self.dout)
        self.gs = torch.empty_like(self.dout)
        self.loss_parts = torch.zeros(2, dtype=torch.float64, device=dev)
        self.adam = capi.AdamDesc(lr, betas[0], betas[1], eps, 0, 1, 0.0, 3.0e38, 0.0, alpha_max)
        self.step_count = 0

    def set_targets(self, diffuse: torch.Tensor, specular: torch.Tensor) -> None:
        if diffuse.shape != (self.n, 4) or specular.shape != (self.n, 4):
            raise ValueError("targets must be (samples, 4) float tensors")
        self.target_d, self.target_s = diffuse.contiguous(), specular.contiguous()

    # -------------------------------------------------------------- forward
    def mips(self, vol: torch.Tensor) -> None:
        for level in range(1, capi.CLIP_LEVEL_COUNT):
            capi.call("vct_downsample_f32", _p(vol), capi.ref(self.ds[level]), 1, _stream())

    def trace(self, vol: torch.Tensor, dout: torch.Tensor, sout: torch.Tensor, steps: torch.Tensor | None = None):
        capi.call("vct_cone_trace_f32", capi.ref(self.desc), capi.ref(self.cam), _p(vol), self.R, None,
                  capi.ref(self.light), None, _p(self.samples), self.n, _p(dout), _p(sout), _p(steps), _stream())

    def render(self, vol: torch.Tensor, steps: torch.Tensor | None = None):
        """(diffuse, specular) images of `vol` (its mips are recomputed in place)."""
        self.mips(vol)
        d = torch.empty_like(self.dout)
        s = torch.empty_like(self.sout)
        self.trace(vol, d, s, steps)
        return d, s

    def loss(self) -> float:
        """The current parameter's loss (mean squared error over both images), without a step."""
        self.work.copy_(self.param)
        self.mips(self.work)
        self.trace(self.work, self.dout, self.sout)
        self._sq_error(grad=False)
        return float(self.loss_parts.sum().item())

    def _sq_error(self, grad: bool) -> None:
        if self.target_d is None:
            raise ValueError("RadianceFit: no targets (set_targets)")
        scale = 1.0 / (8.0 * self.n)
        lp = self.loss_parts.data_ptr()
        capi.call("vct_sq_error", _p(self.dout), _p(self.target_d), self.n, scale, _p(self.gd) if grad else None,
                  C.c_void_p(lp), _stream())
        capi.call("vct_sq_error", _p(self.sout), _p(self.target_s), self.n, scale, _p(self.gs) if grad else None,
                  C.c_void_p(lp + 8), _stream())

    # ---------------------------------------------------------- one step
    def step(self) -> float:
        """One Adam iteration; returns the loss of the parameter before the update."""
        self.work.copy_(self.param)
        self.mips(self.work)
        self.trace(self.work, self.dout, self.sout)
        self._sq_error(grad=True)
        # self.grad is zero here: the previous Adam step cleared it
        capi.call("vct_cone_trace_backward", capi.ref(self.desc), capi.ref(self.cam), _p(self.work), self.R, None,
                  capi.ref(self.light), None, _p(self.samples), self.n, _p(self.gd), _p(self.gs), _p(self.grad),
                  _stream())
        for level in range(capi.CLIP_LEVEL_COUNT - 1, 0, -1):
            capi.call("vct_downsample_backward", _p(self.work), _p(self.grad), capi.ref(self.ds[level]), 1,
                      _stream())
        self.step_count += 1
        self.adam.step = self.step_count
        capi.call("vct_adam_step", _p(self.param), _p(self.grad), _p(self.m), _p(self.v), self.param.numel(),
                  capi.ref(self.adam), _stream())
        return float(self.loss_parts.sum().item())

