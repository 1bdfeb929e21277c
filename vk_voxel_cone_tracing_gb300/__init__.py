"""GB300-native (sm_103a) voxel cone tracing core.

The package is a drop-in for the data-parallel passes of
Snowapril/vk_voxel_cone_tracing: clipmap voxelisation, radiance injection,
anisotropic mips, 16-cone tracing and the sparse-voxel-octree build.  The
compute lives in hand-written CUDA kernels behind the C ABI of
``include/vct_capi.h`` (``libvct_gb300.so``); this Python package only
builds, loads and calls that library.
"""
from . import capi  # noqa: F401

__all__ = ["capi", "build_library"]


def build_library(force: bool = False):
    from .build import build
    return build(force=force)
