"""ctypes binding of ``include/vct_capi.h`` (libvct_gb300.so).

Struct classes mirror the C structs byte for byte (their sizes are asserted
against the header's static asserts in the tests).  ``lib()`` loads the
in-tree CUDA library and raises if it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libvct_gb300.so"

VCT_OK = 0
VCT_E_BAD_ARG = -1
VCT_E_CUDA = -2
VCT_E_OVERFLOW = -3
VCT_E_TIMEOUT = -4
VCT_E_UNSUPPORTED = -5

FACE_COUNT = 6
CLIP_LEVEL_COUNT = 6
VOXEL_BORDER = 2
DOWNSAMPLE_REGION_SIZE = 10
VOXEL_EXTENT_L0 = 16

DOWNSAMPLE_OPACITY = 0
DOWNSAMPLE_RADIANCE = 1

MODE_GI_OUTPUT = 8

FILTER_BILATERAL = 0
FILTER_GAUSSIAN = 1

INJECT_DETERMINISTIC = 0
INJECT_ATOMIC = 1

REVOX_FULL = 0
REVOX_TOROIDAL = 1
CONTEXT_AUTOTUNE = 1
CONTEXT_OPACITY_R8 = 2
OPACITY_RGBA8 = 0
OPACITY_R8 = 1

SVO_DETERMINISTIC = 0
SVO_ATOMIC = 1

NOALLOC_MAX_SAMPLES = 1048576
NOALLOC_SCRATCH_BYTES = 48 << 20

TEX_RGBA8 = 0
TEX_RGBA16F = 1

f3 = C.c_float * 3
f4 = C.c_float * 4
f16 = C.c_float * 16
i3 = C.c_int32 * 3
u3 = C.c_uint32 * 3


class ClipmapRegion(C.Structure):
    _fields_ = [("min_corner", i3), ("extent", u3), ("voxel_size", C.c_float)]


class VoxelizationDesc(C.Structure):
    _fields_ = [("region_min_corner", f3), ("clip_level", C.c_uint32), ("region_max_corner", f3),
                ("clip_max_extent", C.c_float), ("prev_region_min_corner", f3), ("voxel_size", C.c_float),
                ("prev_region_max_corner", f3), ("clipmap_resolution", C.c_int32)]


class DownSampleDesc(C.Structure):
    _fields_ = [("prev_region_min_corner", i3), ("clip_level", C.c_int32), ("clipmap_resolution", C.c_int32),
                ("downsample_region_size", C.c_int32)]


class ImageCleaningDesc(C.Structure):
    _fields_ = [("region_min_corner", i3), ("clip_level", C.c_int32), ("clip_max_extent", u3),
                ("clipmap_resolution", C.c_int32), ("face_count", C.c_uint32)]


class CopyAlphaDesc(C.Structure):
    _fields_ = [("clip_level", C.c_int32), ("clipmap_resolution", C.c_int32), ("face_count", C.c_int32)]


class BorderWrappingDesc(C.Structure):
    _fields_ = [("clipmap_resolution", C.c_uint32), ("clip_border_width", C.c_uint32), ("face_count", C.c_uint32),
                ("clip_region_count", C.c_uint32)]


class ConeTracingDesc(C.Structure):
    _fields_ = [("volume_center", f3), ("rendering_mode", C.c_uint32), ("voxel_size", C.c_float),
                ("volume_dimension", C.c_float), ("trace_start_offset", C.c_float),
                ("indirect_diffuse_intensity", C.c_float), ("ambient_occlusion_factor", C.c_float),
                ("min_trace_step_factor", C.c_float), ("indirect_specular_intensity", C.c_float),
                ("occlusion_decay", C.c_float), ("enable_32_cones", C.c_int32)]


class TraceOptions(C.Structure):
    """vct_trace_options: diffuse_aperture (radians, 0 = the shader's constant), reserved zeros."""
    _fields_ = [("diffuse_aperture", C.c_float), ("reserved", C.c_float * 3)]


class CamMatrix(C.Structure):
    _fields_ = [("view_proj", f16), ("view_proj_inv", f16), ("eye_pos", f3), ("padding", C.c_int32)]


class DirectionalLightDesc(C.Structure):
    _fields_ = [("direction", f3), ("intensity", C.c_float), ("color", f3), ("padding", C.c_int32)]


class DirectionalLightShadowDesc(C.Structure):
    _fields_ = [("view", f16), ("proj", f16), ("z_near", C.c_float), ("z_far", C.c_float)]


class GltfShadeMaterial(C.Structure):
    _fields_ = [("pbr_base_color_factor", f4), ("pbr_base_color_texture", C.c_int32),
                ("pbr_metallic_factor", C.c_float), ("pbr_roughness_factor", C.c_float),
                ("pbr_metallic_roughness_texture", C.c_int32), ("emissive_texture", C.c_int32),
                ("alpha_mode", C.c_int32), ("alpha_cutoff", C.c_float), ("double_sided", C.c_int32),
                ("emissive_factor", f3), ("normal_texture", C.c_int32), ("normal_texture_scale", C.c_float),
                ("occlusion_texture", C.c_int32), ("occlusion_texture_strength", C.c_float),
                ("padding", C.c_int32)]


class SpecularFilterDesc(C.Structure):
    _fields_ = [("tonemap_gamma", C.c_float), ("tonemap_exposure", C.c_float), ("tonemap_enable", C.c_int32),
                ("filter_method", C.c_int32)]


class AdamDesc(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("step", C.c_int32), ("zero_grad", C.c_int32), ("rgb_lo", C.c_float), ("rgb_hi", C.c_float),
                ("alpha_lo", C.c_float), ("alpha_hi", C.c_float)]


class Scene(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("indices", C.c_void_p),
                ("vertex_count", C.c_int64), ("triangle_count", C.c_int64), ("triangle_material", C.c_void_p),
                ("materials", C.c_void_p), ("material_count", C.c_int32), ("textures", C.c_void_p),
                ("texture_count", C.c_int32), ("node_matrices", C.c_void_p), ("triangle_instance", C.c_void_p),
                ("instance_count", C.c_int32)]


class FrameDesc(C.Structure):
    _fields_ = [("camera_pos", f3), ("clipmap_resolution", C.c_int32), ("frame_index", C.c_int32),
                ("inject_mode", C.c_int32), ("shadow_width", C.c_int32), ("shadow_height", C.c_int32),
                ("light", DirectionalLightDesc), ("light_shadow", DirectionalLightShadowDesc),
                ("radiance_texture", C.c_void_p), ("revoxelization", C.c_int32), ("opacity_format", C.c_int32),
                ("regions_state", C.c_void_p)]


class ShadowMap(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("clipmap_resolution", C.c_int32), ("shadow_width", C.c_int32), ("shadow_height", C.c_int32),
                ("flags", C.c_int32), ("workspace_bytes", C.c_size_t)]


class TraceTuning(C.Structure):
    _fields_ = [("diffuse_blocks_per_sm", C.c_int32), ("specular_blocks_per_sm", C.c_int32), ("trace_ms", C.c_float),
                ("default_ms", C.c_float), ("tuned", C.c_int32), ("reserved", C.c_int32)]


class ContextBuffers(C.Structure):
    _fields_ = [("opacity", C.c_void_p), ("radiance", C.c_void_p), ("shadow_depth", C.c_void_p),
                ("radiance_texture", C.c_void_p), ("workspace", C.c_void_p), ("regions", ClipmapRegion * 6),
                ("frame_index", C.c_int32), ("reserved", C.c_int32)]


class BatchJob(C.Structure):
    _fields_ = [("context", C.c_void_p), ("scene", C.c_void_p), ("camera_pos", f3), ("revoxelization", C.c_int32),
                ("reset", C.c_int32), ("reserved", C.c_int32), ("light", DirectionalLightDesc),
                ("light_shadow", DirectionalLightShadowDesc), ("trace_desc", C.c_void_p), ("cam", C.c_void_p),
                ("samples", C.c_void_p), ("sample_count", C.c_int64), ("diffuse_out", C.c_void_p),
                ("specular_out", C.c_void_p), ("cone_steps", C.c_void_p)]


class TraceJob(C.Structure):
    """vct_trace_job: one trace of a vct_cone_trace_fast_batch call."""
    _fields_ = [("desc", ConeTracingDesc), ("eye", f3), ("radiance", C.c_void_p), ("shadow", ShadowMap),
                ("light", DirectionalLightDesc), ("light_shadow", DirectionalLightShadowDesc),
                ("samples", C.c_void_p), ("sample_count", C.c_int64), ("diffuse_out", C.c_void_p),
                ("specular_out", C.c_void_p), ("cone_steps", C.c_void_p)]


STRUCT_SIZES = {
    ClipmapRegion: 28, VoxelizationDesc: 64, DownSampleDesc: 24, ImageCleaningDesc: 36, CopyAlphaDesc: 12,
    BorderWrappingDesc: 16, ConeTracingDesc: 52, CamMatrix: 144, DirectionalLightDesc: 32,
    DirectionalLightShadowDesc: 136, GltfShadeMaterial: 80, Scene: 104, SpecularFilterDesc: 16, Config: 24,
    ContextBuffers: 216, BatchJob: 264, AdamDesc: 40, TraceOptions: 16, TraceJob: 296, TraceTuning: 24,
}

# Every entry point of include/vct_capi.h: name -> (restype, argtypes).
P = C.c_void_p
_SIGS: dict[str, tuple] = {
    "vct_last_error": (C.c_char_p, []),
    "vct_version": (C.c_char_p, []),
    "vct_atlas_texels": (C.c_int64, [C.c_int32]),
    "vct_clip_regions": (C.c_int, [P, C.c_int32, C.c_int32, P]),
    "vct_update_clip_regions": (C.c_int, [P, P, C.c_int32, C.c_int32, P, P, P]),
    "vct_voxelize_opacity_slabs": (C.c_int, [P, P, C.c_int32, P, P, P, C.c_int32, P, P]),
    "vct_clear_region": (C.c_int, [P, P, P]),
    "vct_copy_alpha": (C.c_int, [P, P, P, P]),
    "vct_downsample": (C.c_int, [P, P, C.c_int32, P]),
    "vct_copy_alpha_downsample": (C.c_int, [P, P, P, P, P]),
    "vct_downsample_all": (C.c_int, [P, P, C.c_int32, C.c_int32, P]),
    "vct_wrap_border": (C.c_int, [P, P, P]),
    "vct_cone_trace": (C.c_int, [P, P, P, C.c_int32, P, P, P, P, C.c_int64, P, P, P, P]),
    "vct_cone_trace_opt": (C.c_int, [P, P, P, C.c_int32, P, P, P, P, C.c_int64, P, P, P, P, P]),
    "vct_cone_trace_tex": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P, P]),
    "vct_cone_trace_fast_autotune": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P, P, P, C.c_size_t, P, P]),
    "vct_trace_tuning_get": (C.c_int, [C.c_int32, P]),
    "vct_trace_tuning_reset": (C.c_int, []),
    "vct_cone_trace_f32": (C.c_int, [P, P, P, C.c_int32, P, P, P, P, C.c_int64, P, P, P, P]),
    "vct_cone_trace_backward": (C.c_int, [P, P, P, C.c_int32, P, P, P, P, C.c_int64, P, P, P, P]),
    "vct_downsample_f32": (C.c_int, [P, P, C.c_int32, P]),
    "vct_downsample_backward": (C.c_int, [P, P, P, C.c_int32, P]),
    "vct_sq_error": (C.c_int, [P, P, C.c_int64, C.c_float, P, P, P]),
    "vct_adam_step": (C.c_int, [P, P, P, P, C.c_int64, P, P]),
    "vct_texture_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "vct_texture_update": (C.c_int, [P, P, P]),
    "vct_texture_read": (C.c_int, [P, P, P]),
    "vct_texture_destroy": (C.c_int, [P]),
    "vct_atlas_rgba8_to_rgba16f": (C.c_int, [P, P, C.c_int32, P, P]),
    "vct_downsample_rgba16f": (C.c_int, [P, P, C.c_int32, P, P]),
    "vct_cone_trace_fast_scratch_bytes": (C.c_int64, [C.c_int64]),
    "vct_cone_trace_fast": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P, C.c_size_t, P]),
    "vct_cone_trace_fast_opt": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P, P, C.c_size_t, P]),
    "vct_cone_trace_fast_batch_scratch_bytes": (C.c_int64, [P, C.c_int32]),
    "vct_cone_trace_fast_batch": (C.c_int, [P, C.c_int32, P, C.c_size_t, P]),
    "vct_gather_probe": (C.c_int, [P, P, C.c_int64, C.c_int32, P, P]),
    "vct_workspace_create": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "vct_workspace_destroy": (C.c_int, [P]),
    "vct_workspace_bytes": (C.c_int64, [P]),
    "vct_voxelization_view_proj": (C.c_int, [P, P]),
    "vct_voxelization_desc_for": (C.c_int, [P, C.c_int32, C.c_int32, P]),
    "vct_directional_light_shadow": (C.c_int, [P, P, C.c_float, C.c_float, P]),
    "vct_camera_matrix": (C.c_int, [P, P, P, C.c_float, C.c_float, P]),
    "vct_gbuffer": (C.c_int, [P, P, C.c_int32, C.c_int32, P, P, P]),
    "vct_specular_filter": (C.c_int, [P, P, P, C.c_int32, C.c_int32, P, P]),
    "vct_specular_filter_stencil": (C.c_int, [P]),
    "vct_present_srgb8": (C.c_int, [P, C.c_int32, C.c_int32, P, P]),
    "vct_png_unfilter": (C.c_int, [P, C.c_int64, C.c_int64, C.c_int32, P]),
    "vct_atlas_alloc": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "vct_atlas_free": (C.c_int, [P]),
    "vct_create": (C.c_int, [P, C.POINTER(C.c_void_p)]),
    "vct_destroy": (C.c_int, [P]),
    "vct_context_buffers_get": (C.c_int, [P, P]),
    "vct_context_reset": (C.c_int, [P]),
    "vct_context_frame": (C.c_int, [P, P, P, P, P, C.c_int32, P]),
    "vct_context_trace": (C.c_int, [P, P, P, P, P, P, C.c_int64, P, P, P, P]),
    "vct_batch_submit": (C.c_int, [P, C.c_int32, C.c_int32]),
    "vct_clear_atlas": (C.c_int, [P, C.c_int32, P]),
    "vct_voxelize_opacity": (C.c_int, [P, P, C.c_int32, P, C.c_uint32, P, P]),
    "vct_voxelize_opacity_conservative": (C.c_int, [P, P, C.c_int32, P, C.c_uint32, P]),
    "vct_shadow_depth": (C.c_int, [P, P, P, C.c_int32, C.c_int32, P, P]),
    "vct_inject_radiance": (C.c_int, [P, P, C.c_int32, P, P, P, P, C.c_uint32, C.c_int32, P, P]),
    "vct_svo_fragments": (C.c_int, [P, C.c_int32, P, P, P, P, P, P, C.c_int64, C.POINTER(C.c_int64), P, P]),
    "vct_svo_pool_capacity": (C.c_int64, [C.c_int64]),
    "vct_svo_build": (C.c_int, [P, C.c_int64, C.c_int32, P, C.c_int64, C.c_int32, C.POINTER(C.c_int64), P, P]),
    "vct_svo_canonicalize": (C.c_int, [P, C.c_int64, C.c_int32, P, P, P]),
    "vct_svo_cone_trace": (C.c_int, [P, P, P, C.c_int64, P, P, P, P, P, P, C.c_int64, P, P, P, P]),
    "vct_clipmap_frame": (C.c_int, [P, P, P, P, P, P, P, P]),
    "vct_cone_trace_fast_noalloc": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P]),
}


class VctError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


_LIB: C.CDLL | None = None


def declared_symbols() -> list[str]:
    """Function names declared in include/vct_capi.h (parsed from the header)."""
    import re
    text = (PKG.parent / "include" / "vct_capi.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z0-9_]+\s*\*?\s*(vct_[a-z0-9_]+)\s*\(", text, re.M)))


def lib() -> C.CDLL:
    """Load libvct_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(fn: str, rc: int) -> None:
    if rc != VCT_OK:
        raise VctError(fn, rc, lib().vct_last_error().decode())


def call(fn: str, *args) -> None:
    check(fn, getattr(lib(), fn)(*args))


def ref(s: C.Structure) -> C.c_void_p:
    return C.cast(C.pointer(s), C.c_void_p)
