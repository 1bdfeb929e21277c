#!/usr/bin/env python3
"""Generate the golden vectors that pin the oracle's host math to the reference.

Run in a container that has the reference checkout (it reads the reference
tree, which does not travel with the tests):

    python tests/golden/make_golden.py /path/to/vk_voxel_cone_tracing

1. Compiles glm_golden.cpp (this directory) against the reference's vendored
   glm 0.9.9 (Dependencies/glm) with the reference's own defines
   (GLM_FORCE_LEFT_HANDED, GLM_FORCE_DEPTH_ZERO_TO_ONE, GLM_FORCE_SIZE_T_LENGTH,
   VFS/pch.h:33-35) and records, for a set of cameras / resolutions / lights:
     * the clip regions of VoxelizationPass::createVoxelClipmap,
     * the three view-projection matrices of Voxelizer::setViewProjection,
     * the view / projection of DirectionalLight::setTransform,
     * the CamMatrix block of Camera::updateCamera (glm::perspective, glm::inverse),
     * the node matrices of the glTF loader (translate * mat4_cast(quat) * scale, parent chains,
       transpose(inverse(world))).
2. Parses the fixed cone tables and trace constants out of
   VFS/Shaders/voxelConeTracing.frag.
Writes glm_host_math.json and cone_tables.json next to this script.
"""
from __future__ import annotations

import json
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent


def build_and_run(ref: Path) -> dict:
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "glm_golden"
        cmd = ["g++", "-std=c++17", "-O0", "-ffp-contract=off", "-I", str(ref / "Dependencies"),
               str(HERE / "glm_golden.cpp"), "-o", str(exe)]
        subprocess.run(cmd, check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def cone_tables(ref: Path) -> dict:
    text = (ref / "VFS" / "Shaders" / "voxelConeTracing.frag").read_text()
    def table(name):
        m = re.search(name + r"\[\d+\]\s*=\s*\{(.*?)\};", text, re.S)
        vecs = re.findall(r"vec3\(\s*([-0-9.e]+)\s*,\s*([-0-9.e]+)\s*,\s*([-0-9.e]+)\s*\)", m.group(1))
        return [[float(a), float(b), float(c)] for a, b, c in vecs]
    def const(name):
        return float(re.search(r"const\s+float\s+" + name + r"\s*=\s*([-0-9.e]+)\s*;", text).group(1))
    return {
        "source": "VFS/Shaders/voxelConeTracing.frag",
        "DIFFUSE_CONE_DIRECTIONS_16": table("DIFFUSE_CONE_DIRECTIONS_16"),
        "DIFFUSE_CONE_DIRECTIONS_32": table("DIFFUSE_CONE_DIRECTIONS_32"),
        "DIFFUSE_CONE_APERTURE_16": const("DIFFUSE_CONE_APERTURE_16"),
        "DIFFUSE_CONE_APERTURE_32": const("DIFFUSE_CONE_APERTURE_32"),
        "MIN_TRACE_STEP_FACTOR": const("MIN_TRACE_STEP_FACTOR"),
        "MAX_TRACE_DISTANCE": const("MAX_TRACE_DISTANCE"),
        "MIN_SPECULAR_APERTURE": const("MIN_SPECULAR_APERTURE"),
    }


def main():
    if len(sys.argv) > 1:
        ref = Path(sys.argv[1])
    else:  # the reference checkout named in the repository's benchmark spec
        ref = Path(json.loads((HERE.parents[1] / "BASELINE.json").read_text())["reference_path"])
    host = build_and_run(ref)
    (HERE / "glm_host_math.json").write_text(json.dumps(host, separators=(",", ":")) + "\n")
    (HERE / "cone_tables.json").write_text(json.dumps(cone_tables(ref), indent=1) + "\n")
    print(f"wrote {HERE / 'glm_host_math.json'} and {HERE / 'cone_tables.json'}")


if __name__ == "__main__":
    main()
