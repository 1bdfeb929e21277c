"""glTF ingest (CPU): node matrices pinned against glm, the loader's draw order,
instancing, computed normals, materials and PNG textures, .gltf and .glb."""
import base64
import json
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from vk_voxel_cone_tracing_gb300 import gltf

GOLDEN = Path(__file__).resolve().parent / "golden"


def _u(bits):
    return np.array(bits, np.uint32)


def test_node_matrices_bit_exact_against_glm():
    g = json.loads((GOLDEN / "glm_host_math.json").read_text())
    parent = None
    for rec in g["nodes"]:
        v = _u(rec["trs"]).view(np.float32)
        node = {"translation": v[0:3].tolist(), "rotation": v[3:7].tolist(), "scale": v[7:10].tolist()}
        local = gltf.node_local(node)
        assert np.array_equal(local.view(np.uint32), _u(rec["local"]))
        world = local if parent is None else gltf.mat_mul(parent, local)
        if parent is None:
            world = gltf.mat_mul(np.eye(4, dtype=np.float32).reshape(16), local)
        assert np.array_equal(world.view(np.uint32), _u(rec["world"]))
        it = gltf.transpose(gltf.inverse(world))
        assert np.array_equal(it.view(np.uint32), _u(rec["it_world"]))
        parent = world


def test_inverse_matches_oracle(oracle):
    rng = np.random.default_rng(4)
    for _ in range(20):
        m = rng.normal(size=16).astype(np.float32)
        assert np.array_equal(gltf.inverse(m).view(np.uint32), oracle.inverse4(m).view(np.uint32))


# ------------------------------------------------------------------ PNG
def _png_filter(rows: np.ndarray, bpp: int, types) -> bytes:
    """Forward PNG scanline filters (one type per row)."""
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for r, t in zip(rows.astype(np.int32), types):
        a = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if t == 0:
            f = r
        elif t == 1:
            f = r - a
        elif t == 2:
            f = r - prev
        elif t == 3:
            f = r - (a + prev) // 2
        else:
            p = a + prev - c
            pa, pb, pc = np.abs(p - a), np.abs(p - prev), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, prev, c))
            f = r - pred
        out.append(t)
        out += (f % 256).astype(np.uint8).tobytes()
        prev = r
    return bytes(out)


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def make_png(px: np.ndarray, ctype: int, plte=None, trns=None) -> bytes:
    h, w = px.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    rows = px.reshape(h, w * chans)
    raw = _png_filter(rows, chans, [i % 5 for i in range(h)])
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if plte is not None:
        data += _chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    if trns is not None:
        data += _chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    # split the stream over two IDAT chunks
    z = zlib.compress(raw)
    data += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b"")
    return data


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
def test_png_decode_every_filter_and_colour_type(vct_lib, ctype):
    rng = np.random.default_rng(ctype)
    h, w = 11, 7
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    px = rng.integers(0, 256, size=(h, w, chans), dtype=np.uint8)
    plte = trns = None
    if ctype == 3:
        plte = rng.integers(0, 256, size=(16, 3), dtype=np.uint8)
        trns = rng.integers(0, 256, size=8, dtype=np.uint8)
        px = rng.integers(0, 16, size=(h, w, 1), dtype=np.uint8)
    got = gltf.decode_png(make_png(px, ctype, plte, trns))
    want = np.empty((h, w, 4), np.uint8)
    if ctype == 0:
        want[..., :3], want[..., 3] = px, 255
    elif ctype == 2:
        want[..., :3], want[..., 3] = px, 255
    elif ctype == 3:
        alpha = np.full(16, 255, np.uint8)
        alpha[:8] = trns
        want[..., :3], want[..., 3] = plte[px[..., 0]], alpha[px[..., 0]]
    elif ctype == 4:
        want[..., :3], want[..., 3] = px[..., :1], px[..., 1]
    else:
        want[:] = px
    assert np.array_equal(got, want)


# ------------------------------------------------------------------ a glTF document
def _doc(png: bytes):
    """Two meshes (a u16-indexed quad with normals; a triangle with neither indices nor normals), a node
    tree with a mesh-less root, an instanced mesh, a camera node whose child is skipped, two materials
    and one PNG texture -- all in one buffer."""
    quad_p = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
    quad_n = np.tile(np.float32([0, 1, 0]), (4, 1))
    quad_i = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    tri_p = np.array([[0, 0, 0], [2, 0, 0], [0, 1, 0]], np.float32)
    blobs, views, acc = [], [], []

    def add(arr, ctype, typ, target=None, minmax=False):
        off = sum(len(b) for b in blobs)
        b = arr.tobytes()
        b += b"\0" * (-len(b) % 4)
        blobs.append(b)
        views.append({"buffer": 0, "byteOffset": off, "byteLength": arr.nbytes})
        a = {"bufferView": len(views) - 1, "componentType": ctype, "count": arr.shape[0], "type": typ}
        if minmax:
            a["min"], a["max"] = arr.min(0).tolist(), arr.max(0).tolist()
        acc.append(a)
        return len(acc) - 1

    ap = add(quad_p, 5126, "VEC3", minmax=True)
    an = add(quad_n, 5126, "VEC3")
    ai = add(quad_i, 5123, "SCALAR")
    at = add(tri_p, 5126, "VEC3", minmax=True)
    off = sum(len(b) for b in blobs)
    blobs.append(png + b"\0" * (-len(png) % 4))
    views.append({"buffer": 0, "byteOffset": off, "byteLength": len(png)})
    img_view = len(views) - 1
    buf = b"".join(blobs)
    doc = {
        "asset": {"version": "2.0"},
        "buffers": [{"byteLength": len(buf)}],
        "bufferViews": views, "accessors": acc,
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": ap, "NORMAL": an}, "indices": ai, "material": 0}]},
            {"primitives": [{"attributes": {"POSITION": at}, "material": 1},
                            {"attributes": {"POSITION": at}, "mode": 1}]},  # lines: skipped
        ],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicFactor": 0.25,
                                      "roughnessFactor": 0.6}, "emissiveFactor": [0.5, 0.0, 0.0]},
            {"alphaMode": "MASK", "alphaCutoff": 0.3, "doubleSided": True},
        ],
        "textures": [{"source": 0}],
        "images": [{"bufferView": img_view, "mimeType": "image/png"}],
        "cameras": [{"type": "perspective", "perspective": {"yfov": 1.0, "znear": 0.1}}],
        "nodes": [
            {"name": "root", "translation": [0.0, 1.0, 0.0], "children": [1, 2, 3]},
            {"name": "a", "mesh": 0, "rotation": [0.0, 0.38268343, 0.0, 0.92387953]},
            {"name": "b", "mesh": 0, "scale": [2.0, 1.0, 3.0], "translation": [5.0, 0.0, 0.0]},
            {"name": "cam", "camera": 0, "children": [4]},
            {"name": "hidden", "mesh": 1},
            {"name": "c", "mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, -2, 1]},
        ],
        "scenes": [{"nodes": [0, 5]}], "scene": 0,
    }
    return doc, buf


def _write_gltf(tmp: Path, doc, buf, embed: bool) -> Path:
    doc = json.loads(json.dumps(doc))
    if embed:
        doc["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(buf).decode()
    else:
        (tmp / "scene.bin").write_bytes(buf)
        doc["buffers"][0]["uri"] = "scene.bin"
    p = tmp / "scene.gltf"
    p.write_text(json.dumps(doc))
    return p


def _write_glb(tmp: Path, doc, buf) -> Path:
    j = json.dumps(doc).encode()
    j += b" " * (-len(j) % 4)
    b = buf + b"\0" * (-len(buf) % 4)
    body = struct.pack("<II", len(j), 0x4E4F534A) + j + struct.pack("<II", len(b), 0x004E4942) + b
    p = tmp / "scene.glb"
    p.write_bytes(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
    return p


def _png_fixture():
    px = np.array([[[255, 0, 0, 255], [0, 255, 0, 255]], [[0, 0, 255, 255], [255, 255, 255, 127]]], np.uint8)
    return make_png(px, 6), px


def test_loader_structure(vct_lib, tmp_path):
    png, px = _png_fixture()
    doc, buf = _doc(png)
    g = gltf.load_gltf(_write_gltf(tmp_path, doc, buf, embed=False))
    sc = g.scene
    assert g.node_names == ["root", "a", "b", "c"]  # depth-first; the camera subtree is skipped
    assert len(g.cameras) == 1 and not g.warnings
    # draw order: node a (quad), node b (quad), node c (triangle); the root has no mesh
    assert sc.triangle_count == 5
    assert sc.tri_instance.tolist() == [1, 1, 2, 2, 3]
    assert sc.tri_material.tolist() == [0, 0, 0, 0, 1]
    assert sc.indices.tolist()[:2] == [[0, 1, 2], [0, 2, 3]] and sc.indices.tolist()[2] == [0, 1, 2]
    assert sc.indices.tolist()[4] == [4, 5, 6]  # the triangle mesh's vertices follow the quad's
    # the quad's vertices are shared by the two instances; the triangle's normals are computed
    assert sc.positions.shape == (4 + 3, 3)  # the line primitive adds no vertices
    assert np.allclose(sc.normals[4], [0, 0, 1])
    # node matrices: root translation composes into the children; the camera's child is absent
    m = sc.node_matrices
    assert m.shape == (4, 32)
    b_world = m[2, :16].reshape(4, 4)
    assert np.allclose(b_world[3, :3], [5.0, 1.0, 0.0]) and np.allclose(np.diag(b_world)[:3], [2, 1, 3])
    assert np.allclose(m[3, :16].reshape(4, 4)[3, :3], [0.0, 0.0, -2.0])
    it = m[2, 16:].reshape(4, 4)
    assert np.allclose(it, np.linalg.inv(b_world.astype(np.float64)).T, atol=1e-6)
    # materials and the 1x1 texture (the rounded mean of the image)
    mat = sc.materials
    assert mat["pbr_base_color_texture"].tolist() == [0, -1]
    assert mat["pbr_metallic_factor"][0] == np.float32(0.25) and mat["pbr_metallic_factor"][1] == 1.0
    assert mat["alpha_mode"].tolist() == [0, 1] and mat["alpha_cutoff"][1] == np.float32(0.3)
    assert mat["double_sided"].tolist() == [0, 1] and mat["emissive_factor"][0].tolist() == [0.5, 0.0, 0.0]
    mean = np.floor(px.reshape(-1, 4).mean(0) + 0.5).astype(np.uint32)
    assert sc.textures.tolist() == [int(mean[0] | (mean[1] << 8) | (mean[2] << 16) | (mean[3] << 24))]


def test_gltf_glb_and_embedded_agree(vct_lib, tmp_path):
    png, _ = _png_fixture()
    doc, buf = _doc(png)
    a = gltf.load_gltf(_write_gltf(tmp_path, doc, buf, embed=False)).scene
    b = gltf.load_gltf(_write_gltf(tmp_path, doc, buf, embed=True)).scene
    c = gltf.load_gltf(_write_glb(tmp_path, doc, buf)).scene
    for s in (b, c):
        for f in ("positions", "normals", "indices", "tri_material", "textures", "node_matrices", "tri_instance"):
            assert np.array_equal(getattr(a, f), getattr(s, f)), f
        assert a.materials.tobytes() == s.materials.tobytes()


def test_world_positions_follow_the_node_matrices(vct_lib, tmp_path):
    from vk_voxel_cone_tracing_gb300.scene import world_positions
    png, _ = _png_fixture()
    doc, buf = _doc(png)
    sc = gltf.load_gltf(_write_gltf(tmp_path, doc, buf, embed=False)).scene
    wp = world_positions(sc).reshape(-1, 3, 3)
    # instance b: scale (2, 1, 3) then translate (5, 0, 0) under the root's (0, 1, 0)
    assert np.allclose(wp[2, 0], [5 - 2, 1, -3])
    # node c: translation (0, 0, -2) from its matrix
    assert np.allclose(wp[4], [[0, 0, -2], [2, 0, -2], [0, 1, -2]])


def test_unsupported_image_is_reported(vct_lib, tmp_path):
    png, _ = _png_fixture()
    doc, buf = _doc(png)
    doc["images"][0]["mimeType"] = "image/jpeg"
    bad = bytearray(buf)
    at = bytes(bad).index(png[:8])
    bad[at:at + 8] = b"\xff\xd8\xff\xe0\x00\x10JF"  # a JPEG header in place of the PNG signature
    g = gltf.load_gltf(_write_gltf(tmp_path, doc, bytes(bad), embed=True))
    assert g.scene.textures.tolist() == [0xFFFFFFFF] and "jpeg" in g.warnings[0]
