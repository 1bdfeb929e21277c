"""glTF 2.0 scene ingest into the device scene layout.

Follows GLTFLoader (VFS/Util/GLTFLoader.cpp) and GLTFScene (VFS/GLTFScene.cpp):

* every mesh primitive in TRIANGLES mode is appended to one vertex pool --
  separate POSITION / NORMAL streams, uint32 indices local to the primitive
  (``loadScene`` :44-127, ``processMesh`` :128-383); a primitive without
  indices gets 0..n-1, one without normals gets the sum of its triangles'
  normalize(cross(normalize(e0), normalize(e1))) per vertex (not
  renormalised: the shaders normalise);
* the default scene's node tree is flattened depth-first (``processNode``
  :399-491): local = translate(T) * mat4(quat R) * scale(S) * matrix,
  world = parent.world * local, in FP32 with glm's operation order; camera
  and light nodes are not scene nodes and their subtrees are skipped;
* the draw (``GLTFScene::cmdDraw``, VFS/GLTFScene.cpp:458-488) visits the
  scene nodes in order and draws each node's primitives with push constants
  {instanceIndex = the node's position in the flat list, materialIndex};
  the triangles come out in that order, indices rebased onto the pool, with
  one material index and one instance index per triangle;
* materials become GltfShadeMaterial records (``importMaterials`` :566-592,
  defaults of the glTF specification), material -1 -> 0.

Two departures, both forced by the device scene format or by a defect:

* textures are 1x1 (the kernels read one texel per texture): each glTF
  texture becomes the rounded mean of its image's RGBA8 texels.  PNG images
  (8-bit, non-interlaced, every colour type) are decoded here (zlib + the
  library's native scanline unfilter); other image formats become opaque
  white and are listed in ``Gltf.warnings``;
* the reference's matrix buffer (``uploadMatrixBuffer`` :398-420) holds only
  the nodes that have meshes while instanceIndex counts every node, so a
  mesh-less node ahead of a mesh node makes the draw read a wrong matrix
  (or past the buffer).  Here every scene node gets its NodeMatrix {world,
  transpose(inverse(world))}, so instanceIndex selects the node's own
  matrices -- the intended behaviour.
"""
from __future__ import annotations

import base64
import ctypes as C
import json
import struct
import zlib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .scene import MATERIAL_DTYPE, Scene

f32 = np.float32

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


# ----------------------------------------------------------- glm in FP32
def _identity() -> np.ndarray:
    return np.eye(4, dtype=f32).reshape(16)  # column-major [c * 4 + r]; the identity is symmetric


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """glm mat4 * mat4: column i = ((a0 b[i][0] + a1 b[i][1]) + a2 b[i][2]) + a3 b[i][3] (FP32)."""
    a = a.reshape(4, 4)  # a[c] = column c
    b = b.reshape(4, 4)
    out = np.empty((4, 4), f32)
    for i in range(4):
        s = a[0] * b[i, 0]
        s = s + a[1] * b[i, 1]
        s = s + a[2] * b[i, 2]
        s = s + a[3] * b[i, 3]
        out[i] = s
    return out.reshape(16)


def translate(t) -> np.ndarray:
    """glm::translate(mat4(1), t): column 3 = ((c0 t0 + c1 t1) + c2 t2) + c3."""
    m = _identity().reshape(4, 4)
    t = np.asarray(t, f32)
    m[3] = ((m[0] * t[0] + m[1] * t[1]) + m[2] * t[2]) + m[3]
    return m.reshape(16)


def scale(s) -> np.ndarray:
    """glm::scale(mat4(1), s)."""
    m = _identity().reshape(4, 4)
    s = np.asarray(s, f32)
    for c in range(3):
        m[c] = m[c] * s[c]
    return m.reshape(16)


def quat_to_mat4(x, y, z, w) -> np.ndarray:
    """glm::mat4_cast(quat(w, x, y, z)) (gtc/quaternion.inl mat3_cast)."""
    x, y, z, w = (f32(v) for v in (x, y, z, w))
    qxx, qyy, qzz = x * x, y * y, z * z
    qxz, qxy, qyz = x * z, x * y, y * z
    qwx, qwy, qwz = w * x, w * y, w * z
    one, two = f32(1), f32(2)
    m = _identity().reshape(4, 4)
    m[0, 0] = one - two * (qyy + qzz)
    m[0, 1] = two * (qxy + qwz)
    m[0, 2] = two * (qxz - qwy)
    m[1, 0] = two * (qxy - qwz)
    m[1, 1] = one - two * (qxx + qzz)
    m[1, 2] = two * (qyz + qwx)
    m[2, 0] = two * (qxz + qwy)
    m[2, 1] = two * (qyz - qwx)
    m[2, 2] = one - two * (qxx + qyy)
    return m.reshape(16)


def inverse(m: np.ndarray) -> np.ndarray:
    """glm::inverse(mat4) in FP32: the adjugate from 2x2 minors of the lower rows, scaled by 1 / det
    (glm 0.9.9 compute_inverse<4, 4>'s evaluation order)."""
    e = np.asarray(m, f32).reshape(4, 4)  # e[c, r]
    rows = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))
    cols = ((2, 3), (2, 3), (1, 3), (1, 2))
    fac = [[e[ca, r0] * e[cb, r1] - e[cb, r0] * e[ca, r1] for (ca, cb) in cols] for (r0, r1) in rows]
    vec = [[e[1, r] if j == 0 else e[0, r] for j in range(4)] for r in range(4)]
    tab = ((1, 0, 2, 1, 3, 2), (0, 0, 2, 3, 3, 4), (0, 1, 1, 3, 3, 5), (0, 2, 1, 4, 2, 5))
    inv = np.empty((4, 4), f32)
    for k, (p, q, s_, t, u, v) in enumerate(tab):
        for j in range(4):
            sgn = f32(-1) if (k + j) & 1 else f32(1)
            val = (vec[p][j] * fac[q][j] - vec[s_][j] * fac[t][j]) + vec[u][j] * fac[v][j]
            inv[k, j] = val * sgn
    det = (e[0, 0] * inv[0, 0] + e[0, 1] * inv[1, 0]) + (e[0, 2] * inv[2, 0] + e[0, 3] * inv[3, 0])
    one_over = f32(1) / det
    return (inv * one_over).astype(f32).reshape(16)


def transpose(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, f32).reshape(4, 4).T).reshape(16)


def node_local(node: dict) -> np.ndarray:
    """GLTFLoader::GetLocalMatrix: ((translate(T) * mat4(R)) * scale(S)) * matrix."""
    t = node.get("translation", [0.0, 0.0, 0.0])
    s = node.get("scale", [1.0, 1.0, 1.0])
    # the reference's default rotation is quat(0, 0, 0, 0), whose mat4_cast is the identity
    r = node.get("rotation", [0.0, 0.0, 0.0, 0.0])
    mat = np.asarray(node.get("matrix", list(_identity())), np.float64).astype(f32)
    return mat_mul(mat_mul(mat_mul(translate(t), quat_to_mat4(*r)), scale(s)), mat)


# ----------------------------------------------------------- PNG
def decode_png(data: bytes) -> np.ndarray:
    """8-bit non-interlaced PNG -> (H, W, 4) uint8 RGBA."""
    from . import capi
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG image")
    pos, idat, plte, trns, hdr = 8, [], None, None, None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0:
        raise ValueError(f"unsupported PNG (bit depth {depth}, interlace {interlace})")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(b"".join(idat))
    row = w * chans
    if len(raw) != h * (row + 1):
        raise ValueError("PNG data size does not match its header")
    out = np.empty(h * row, np.uint8)
    src = np.frombuffer(raw, np.uint8)
    capi.call("vct_png_unfilter", src.ctypes.data_as(C.c_void_p), row, h, chans, out.ctypes.data_as(C.c_void_p))
    px = out.reshape(h, w, chans)
    rgba = np.empty((h, w, 4), np.uint8)
    if ctype == 0:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = 255
    elif ctype == 2:
        rgba[..., :3] = px
        rgba[..., 3] = 255
    elif ctype == 3:
        rgba[..., :3] = plte[px[..., 0]]
        alpha = np.full(len(plte), 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns
        rgba[..., 3] = alpha[px[..., 0]]
    elif ctype == 4:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = px[..., 1]
    else:
        rgba[:] = px
    return rgba


def mean_texel(rgba: np.ndarray) -> int:
    """The 1x1 texel of an image: the rounded mean of each RGBA8 channel, packed R in the low byte."""
    m = np.floor(rgba.reshape(-1, 4).astype(np.float64).mean(0) + 0.5).astype(np.uint32)
    return int(m[0] | (m[1] << 8) | (m[2] << 16) | (m[3] << 24))


# ----------------------------------------------------------- loader
@dataclass
class Gltf:
    scene: Scene
    node_names: list = field(default_factory=list)
    cameras: list = field(default_factory=list)   # (world matrix, glTF camera dict) per camera node
    warnings: list = field(default_factory=list)


def _read_container(path: Path):
    data = path.read_bytes()
    if data[:4] == b"glTF":
        _, _, total = struct.unpack("<III", data[:12])
        pos, doc, bin_chunk = 12, None, None
        while pos < total:
            n, kind = struct.unpack("<II", data[pos:pos + 8])
            chunk = data[pos + 8:pos + 8 + n]
            if kind == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif kind == 0x004E4942:
                bin_chunk = chunk
            pos += 8 + n
        return doc, bin_chunk
    return json.loads(data.decode("utf-8")), None


def _load_uri(uri: str, base: Path) -> bytes:
    if uri.startswith("data:"):
        return base64.b64decode(uri.split(",", 1)[1])
    from urllib.parse import unquote
    return (base / unquote(uri)).read_bytes()


class _Doc:
    def __init__(self, doc: dict, base: Path, bin_chunk: bytes | None):
        self.doc = doc
        self.buffers = []
        for b in doc.get("buffers", []):
            self.buffers.append(_load_uri(b["uri"], base) if "uri" in b else bin_chunk)
        self.base = base

    def view_bytes(self, vi: int) -> tuple[bytes, int]:
        v = self.doc["bufferViews"][vi]
        buf = self.buffers[v["buffer"]]
        off = v.get("byteOffset", 0)
        return buf[off:off + v["byteLength"]], v.get("byteStride", 0)

    def accessor(self, ai: int) -> np.ndarray:
        a = self.doc["accessors"][ai]
        if "sparse" in a:
            raise ValueError("sparse accessors are not supported")
        dt = np.dtype(_COMPONENT[a["componentType"]])
        nc = _NCOMP[a["type"]]
        count = a["count"]
        if "bufferView" not in a:
            return np.zeros((count, nc), dt)
        raw, stride = self.view_bytes(a["bufferView"])
        off = a.get("byteOffset", 0)
        elem = dt.itemsize * nc
        stride = stride or elem
        if stride == elem:
            arr = np.frombuffer(raw, dt, count * nc, off).reshape(count, nc)
        else:
            rows = np.frombuffer(raw, np.uint8, (count - 1) * stride + elem, off)
            arr = np.lib.stride_tricks.as_strided(rows, (count, elem), (stride, 1)).copy().view(dt).reshape(count, nc)
        if a.get("normalized") and dt.kind in "iu":
            info = np.iinfo(dt)
            arr = np.maximum(arr.astype(np.float32) / np.float32(info.max), np.float32(-1.0))
        return arr

    def image_bytes(self, img: dict) -> tuple[bytes, str]:
        if "uri" in img:
            uri = img["uri"]
            mime = img.get("mimeType") or ("image/png" if uri.lower().endswith(".png") or
                                           uri.startswith("data:image/png") else "")
            return _load_uri(uri, self.base), mime
        raw, _ = self.view_bytes(img["bufferView"])
        return raw, img.get("mimeType", "")


def _computed_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """processMesh's missing-normal branch: per vertex, the sum over its triangles of
    normalize(cross(normalize(p1 - p0), normalize(p2 - p0))) (FP32)."""
    def nrm(v):
        d = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
        return v * (np.float32(1) / np.sqrt(d))[:, None]
    t = idx.reshape(-1, 3)
    p0, p1, p2 = pos[t[:, 0]], pos[t[:, 1]], pos[t[:, 2]]
    e0, e1 = nrm(p1 - p0), nrm(p2 - p0)
    c = np.stack([e0[:, 1] * e1[:, 2] - e1[:, 1] * e0[:, 2], e0[:, 2] * e1[:, 0] - e1[:, 2] * e0[:, 0],
                  e0[:, 0] * e1[:, 1] - e1[:, 0] * e0[:, 1]], 1).astype(np.float32)
    n = nrm(c)
    out = np.zeros_like(pos)
    # triangle by triangle, corners 0, 1, 2 (np.add.at applies repeated indices in order)
    np.add.at(out, t.reshape(-1), np.repeat(n, 3, axis=0))
    return out


def load_gltf(path) -> Gltf:
    """Load a .gltf or .glb file into a Scene (draw order, node matrices, 1x1 textures)."""
    path = Path(path)
    doc, bin_chunk = _read_container(path)
    d = _Doc(doc, path.parent, bin_chunk)
    warnings: list[str] = []

    # primitives of every mesh, appended to one pool (mesh order)
    positions, normals, prims, mesh_prims = [], [], [], []
    nverts = 0
    for mesh in doc.get("meshes", []):
        ids = []
        for prim in mesh.get("primitives", []):
            if prim.get("mode", 4) != 4:
                continue
            if "KHR_draco_mesh_compression" in prim.get("extensions", {}):
                raise ValueError(f"{path}: Draco-compressed meshes are not supported")
            pos = d.accessor(prim["attributes"]["POSITION"]).astype(np.float32)
            if "indices" in prim:
                idx = d.accessor(prim["indices"]).reshape(-1).astype(np.uint32)
            else:
                idx = np.arange(pos.shape[0], dtype=np.uint32)
            if "NORMAL" in prim["attributes"]:
                nrm = d.accessor(prim["attributes"]["NORMAL"]).astype(np.float32)
            else:
                nrm = _computed_normals(pos, idx)
            ids.append(len(prims))
            prims.append(dict(first_vertex=nverts, indices=idx, material=max(prim.get("material", -1), 0)))
            positions.append(pos)
            normals.append(nrm)
            nverts += pos.shape[0]
        mesh_prims.append(ids)

    # the default scene's node tree, flattened depth-first
    nodes, node_names, cameras = [], [], []
    gnodes = doc.get("nodes", [])

    def visit(ni: int, parent_world):
        node = gnodes[ni]
        world = mat_mul(parent_world, node_local(node)) if parent_world is not None else mat_mul(_identity(),
                                                                                                 node_local(node))
        if "camera" in node:
            cameras.append((world, doc["cameras"][node["camera"]]))
            return
        if "KHR_lights_punctual" in node.get("extensions", {}):
            return
        nodes.append(dict(world=world, prims=mesh_prims[node["mesh"]] if "mesh" in node else []))
        node_names.append(node.get("name", str(ni)))
        for c in node.get("children", []):
            visit(c, world)

    scenes = doc.get("scenes", [])
    if scenes:
        for ni in scenes[doc.get("scene", 0)].get("nodes", []):
            visit(ni, None)

    # draw order: scene nodes, then their primitives
    tri_idx, tri_mat, tri_inst = [], [], []
    for inst, node in enumerate(nodes):
        for pi in node["prims"]:
            p = prims[pi]
            t = p["indices"][: (p["indices"].size // 3) * 3].reshape(-1, 3).astype(np.uint64) + p["first_vertex"]
            tri_idx.append(t.astype(np.uint32))
            tri_mat.append(np.full(t.shape[0], p["material"], np.uint32))
            tri_inst.append(np.full(t.shape[0], inst, np.uint32))
    if not tri_idx:
        raise ValueError(f"{path}: the default scene draws no triangles")

    node_matrices = np.zeros((max(len(nodes), 1), 32), np.float32)
    for i, node in enumerate(nodes):
        node_matrices[i, :16] = node["world"]
        node_matrices[i, 16:] = transpose(inverse(node["world"]))

    # materials (glTF defaults; the reference maps material -1 to 0, so keep at least one)
    gm = doc.get("materials", []) or [{}]
    mats = np.zeros(len(gm), MATERIAL_DTYPE)
    for i, m in enumerate(gm):
        pbr = m.get("pbrMetallicRoughness", {})
        mats[i]["pbr_base_color_factor"] = pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0])
        mats[i]["pbr_base_color_texture"] = pbr.get("baseColorTexture", {}).get("index", -1)
        mats[i]["pbr_metallic_factor"] = pbr.get("metallicFactor", 1.0)
        mats[i]["pbr_roughness_factor"] = pbr.get("roughnessFactor", 1.0)
        mats[i]["pbr_metallic_roughness_texture"] = pbr.get("metallicRoughnessTexture", {}).get("index", -1)
        mats[i]["emissive_texture"] = m.get("emissiveTexture", {}).get("index", -1)
        mats[i]["alpha_mode"] = {"MASK": 1, "BLEND": 2}.get(m.get("alphaMode", "OPAQUE"), 0)
        mats[i]["alpha_cutoff"] = m.get("alphaCutoff", 0.5)
        mats[i]["double_sided"] = 1 if m.get("doubleSided", False) else 0
        mats[i]["emissive_factor"] = m.get("emissiveFactor", [0.0, 0.0, 0.0])
        mats[i]["normal_texture"] = m.get("normalTexture", {}).get("index", -1)
        mats[i]["normal_texture_scale"] = m.get("normalTexture", {}).get("scale", 1.0)
        mats[i]["occlusion_texture"] = m.get("occlusionTexture", {}).get("index", -1)
        mats[i]["occlusion_texture_strength"] = m.get("occlusionTexture", {}).get("strength", 1.0)

    # textures -> 1x1 texels
    texels = []
    for ti, tex in enumerate(doc.get("textures", [])):
        texel = 0xFFFFFFFF
        src = tex.get("source")
        if src is None:
            warnings.append(f"texture {ti}: no image source; white")
        else:
            raw, mime = d.image_bytes(doc["images"][src])
            if mime == "image/png" or raw[:8] == b"\x89PNG\r\n\x1a\n":
                try:
                    texel = mean_texel(decode_png(raw))
                except ValueError as e:
                    warnings.append(f"texture {ti}: {e}; white")
            else:
                warnings.append(f"texture {ti}: {mime or 'unknown'} image not decoded; white")
        texels.append(texel)
    textures = np.asarray(texels or [0xFFFFFFFF], np.uint32)

    scene = Scene(np.concatenate(positions).astype(np.float32), np.concatenate(normals).astype(np.float32),
                  np.concatenate(tri_idx), np.concatenate(tri_mat), mats, textures,
                  node_matrices=node_matrices, tri_instance=np.concatenate(tri_inst))
    return Gltf(scene=scene, node_names=node_names, cameras=cameras, warnings=warnings)
