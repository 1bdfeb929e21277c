"""The passes after the trace and a whole clipmap frame, camera to image.

``specular_filter`` and ``present_srgb8`` wrap SpecularFilterPass and
FinalPass (vct_specular_filter, vct_present_srgb8).  ``Renderer`` chains the
reference's per-frame pass order (VFS/Renderer.cpp, Application.cpp) on device
buffers: the clipmap frame (voxelise, shadow, inject, mips, border), the
G-buffer for the camera, the cone trace over its pixels, the specular filter
and the swapchain image -- headless, the swapchain being a device buffer that
``write_ppm`` can store.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi, clipmap, passes
from .clipmap import _ptr, _stream
from .scene import default_trace_desc


def filter_desc(gamma: float = 2.2, exposure: float = 0.1, tonemap: bool = False,
                method: int = capi.FILTER_GAUSSIAN) -> capi.SpecularFilterDesc:
    """SpecularFilterPass push constants; the defaults are the reference's (SpecularFilterPass.h:48-51)."""
    return capi.SpecularFilterDesc(gamma, exposure, int(tonemap), method)


def specular_filter(diffuse: torch.Tensor, specular: torch.Tensor, width: int, height: int,
                    desc: capi.SpecularFilterDesc | None = None, out: torch.Tensor | None = None) -> torch.Tensor:
    """SpecularFilterPass over (width * height, 4) float32 contribution images -> the RGBA32F output image."""
    n = width * height
    for t in (diffuse, specular):
        if t.shape != (n, 4) or t.dtype != torch.float32 or not t.is_contiguous():
            raise ValueError("specular_filter: images must be contiguous (width * height, 4) float32")
    if out is None:
        out = torch.empty((n, 4), dtype=torch.float32, device=diffuse.device)
    capi.call("vct_specular_filter", capi.ref(desc or filter_desc()), _ptr(diffuse), _ptr(specular), width, height,
              _ptr(out), _stream())
    return out


def present_srgb8(rgba: torch.Tensor, width: int, height: int, out: torch.Tensor | None = None) -> torch.Tensor:
    """FinalPass: the B8G8R8A8_SRGB swapchain image as (height, width) int32 (bytes B, G, R, A)."""
    if out is None:
        out = torch.empty((height, width), dtype=torch.int32, device=rgba.device)
    capi.call("vct_present_srgb8", _ptr(rgba), width, height, _ptr(out), _stream())
    return out


def write_ppm(path, bgra8: np.ndarray) -> None:
    """Store a (height, width) B8G8R8A8 image as binary PPM, top row = framebuffer row 0."""
    px = np.ascontiguousarray(bgra8).view(np.uint8).reshape(bgra8.shape[0], bgra8.shape[1], 4)
    rgb = px[..., [2, 1, 0]]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]))
        f.write(rgb.tobytes())


class Renderer:
    """A device-resident clipmap VCT frame: camera -> G-buffer -> cone trace -> filter -> image.

    Buffers (atlases, shadow map, radiance texture, G-buffer records, contribution and output images)
    are allocated once; ``render`` runs one frame on the current stream."""

    def __init__(self, scene, R: int = 256, width: int = 1280, height: int = 720, fovy: float = 60.0,
                 light_dir=(0.3, -1.0, 0.2), light_distance: float = 15.0, shadow_res: int = 2048,
                 device="cuda"):
        self.R, self.width, self.height, self.fovy = R, width, height, fovy
        self.light_dir = tuple(float(x) for x in light_dir)
        self.light_distance = light_distance
        self.ds = passes.DeviceScene(scene, device)
        self.ws = passes.Workspace()
        self.opacity = clipmap.new_atlas(R, device)
        self.radiance = clipmap.new_atlas(R, device)
        self.shadow = torch.empty((shadow_res, shadow_res), dtype=torch.float32, device=device)
        self.light = passes.light_desc(self.light_dir)
        self.tex = clipmap.RadianceTexture(R, capi.TEX_RGBA8)
        n = width * height
        self.samples = torch.empty((n, 20), dtype=torch.float32, device=device)
        self.diffuse = torch.empty((n, 4), dtype=torch.float32, device=device)
        self.specular = torch.empty((n, 4), dtype=torch.float32, device=device)
        self.output = torch.empty((n, 4), dtype=torch.float32, device=device)
        self.image = torch.empty((height, width), dtype=torch.int32, device=device)
        self.scratch = clipmap.fast_scratch(n, device)
        self.clear = torch.tensor([0.0, 0.0, 0.0, 1.0], dtype=torch.float32, device=device)
        self.regions = None
        self.regions_state = (capi.ClipmapRegion * 6)()  # persists between frames (toroidal mode)
        self.camera = None

    def light_shadow(self, center) -> capi.DirectionalLightShadowDesc:
        d = np.asarray(self.light_dir, np.float64)
        d /= np.linalg.norm(d)
        origin = (np.asarray(center, np.float64) - self.light_distance * d).astype(np.float32)
        return passes.light_shadow_desc(tuple(origin.tolist()), self.light_dir)

    def render(self, position, direction, up=(0.0, 1.0, 0.0), frame_index: int = 0,
               desc: capi.SpecularFilterDesc | None = None, revoxelization: int = capi.REVOX_FULL) -> torch.Tensor:
        """One frame from camera `position` looking along `direction`; returns the RGBA32F output image.
        `revoxelization` VCT_REVOX_TOROIDAL updates the opacity atlas from the previous frame's regions."""
        lsd = self.light_shadow(position)
        self.regions = passes.clipmap_frame(self.ds, position, self.R, self.opacity, self.radiance, self.shadow,
                                            self.light, lsd, self.ws, frame_index=frame_index, texture=self.tex,
                                            revoxelization=revoxelization, regions_state=self.regions_state)
        self.camera = passes.camera_matrix(position, direction, up, self.fovy, self.width / self.height)
        passes.gbuffer(self.ds, self.camera, self.width, self.height, self.ws, out=self.samples)
        # the cone-tracing pass's attachments clear to (0, 0, 0, 1); the trace leaves sky pixels untouched
        self.diffuse.copy_(self.clear.expand_as(self.diffuse))
        self.specular.copy_(self.clear.expand_as(self.specular))
        td = clipmap.trace_desc(**default_trace_desc(clipmap.regions_to_numpy(self.regions), self.R))
        clipmap.cone_trace_fast(td, position, self.tex, self.samples, light=self.light, shadow=self.shadow,
                                shadow_desc=lsd, diffuse=self.diffuse, specular=self.specular, scratch=self.scratch)
        specular_filter(self.diffuse, self.specular, self.width, self.height, desc, out=self.output)
        present_srgb8(self.output, self.width, self.height, out=self.image)
        return self.output

    def close(self) -> None:
        self.tex.close()
        self.ws.close()


def main(argv=None) -> None:
    """Render frames of a scene to PPM images: python -m vk_voxel_cone_tracing_gb300.render --out frame.ppm"""
    import argparse
    import time

    from .scene import hall_scene, room_scene
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--scene", default="hall", help="hall, room, or a .gltf / .glb path")
    ap.add_argument("--R", type=int, default=256)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=1, help="frames along a short camera path")
    ap.add_argument("--toroidal", action="store_true", help="toroidal revoxelisation after the first frame")
    ap.add_argument("--position", type=float, nargs=3, default=(0.0, 5.0, 0.0))
    ap.add_argument("--direction", type=float, nargs=3, default=(0.6, -0.2, 0.77))
    ap.add_argument("--out", default="frame.ppm", help="image of the last frame (binary PPM)")
    a = ap.parse_args(argv)
    if a.scene == "hall":
        sc = hall_scene()
    elif a.scene == "room":
        sc = room_scene()
    else:
        from .gltf import load_gltf
        sc = load_gltf(a.scene).scene
    r = Renderer(sc, R=a.R, width=a.width, height=a.height)
    from . import capi
    times = []
    for k in range(a.frames):
        pos = (a.position[0] + 0.05 * k, a.position[1], a.position[2] + 0.03 * k)
        t0 = time.perf_counter()
        r.render(pos, a.direction, frame_index=k,
                 revoxelization=capi.REVOX_TOROIDAL if (a.toroidal and k > 0) else capi.REVOX_FULL)
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t0) * 1e3)
    write_ppm(a.out, r.image.cpu().numpy())
    print(f"{sc.triangle_count} triangles, R={a.R}, {a.width}x{a.height}: frame ms " +
          " ".join(f"{t:.2f}" for t in times) + f" -> {a.out}")
    r.close()


if __name__ == "__main__":
    main()
