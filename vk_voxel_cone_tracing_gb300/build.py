"""Build the CUDA library (libvct_gb300.so) in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc and
linked into one shared library next to this file.  Translation units whose
RGBA8 / integer results must be bit-identical to the FP32 evaluation of the
reference's GLSL are built with ``-fmad=false`` (no fused multiply-add).
A build is skipped when the library is newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvct_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is built with -ffp-contract=off: the host math (glm matrices, clip regions) must
# round like the reference's on every host ISA (aarch64 g++ fuses multiply-adds by default).
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xptxas", "-O3",
          "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
# Units that mirror FP32 shader arithmetic op for op, and the texture-form trace: its device functions are
# inlined into the single and the batched kernels, and with multiply-add contraction left to the compiler the
# two could round a sample's diffuse sum differently (by one unit in the last place) from the same inputs.
NO_FMA = {"clipmap_passes.cu", "trace_exact.cu", "raster.cu", "svo.cu", "svo_trace.cu", "composite.cu", "trace_grad.cu",
          "trace_fast.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvct_gb300.so")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    flags = list(COMMON) + list(extra)
    if src.name in NO_FMA:
        flags.append("-fmad=false")
    cmd = [nvcc(), *ARCH, *flags, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every CUDA translation unit and link libvct_gb300.so."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or []), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
