"""Synthetic glTF 2.0 assets for the import tests, written here from scratch: a textured sphere
(64-vertex hull with normals and tangents), a textured grid plane, an alpha-masked double-sided
material, a node hierarchy with TRS and matrix transforms, and a point light. The same content is
written as .gltf (+ .bin, PNG data URIs) and as .glb (images in buffer views)."""
from __future__ import annotations

import base64
import json
import struct
import zlib

import numpy as np

from glimpsw_gb300 import scenes


def encode_png(words: np.ndarray, color_type: int = 6) -> bytes:
    """RGBA8 words (uint32[h, w]) as a PNG of colour type 6 (RGBA) or 2 (RGB), rows filtered with
    types 0-4 in turn (so a decoder meets every filter)."""
    h, w = words.shape
    ch = np.stack([(words >> (8 * k)) & 255 for k in range(4)], axis=-1).astype(np.int32)
    if color_type == 2:
        ch = ch[..., :3]
    bpp = ch.shape[-1]
    rows = ch.reshape(h, w * bpp)
    out = bytearray()
    prev = np.zeros(w * bpp, np.int32)
    for y in range(h):
        f = y % 5
        line = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int32), line[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if f == 0:
            enc = line
        elif f == 1:
            enc = line - left
        elif f == 2:
            enc = line - prev
        elif f == 3:
            enc = line - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = line - pred
        out.append(f)
        out += (enc & 255).astype(np.uint8).tobytes()
        prev = line

    def chunk(kind, body):
        c = struct.pack(">I", len(body)) + kind + body
        return c + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, 8, color_type, 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b"")


def _sphere():
    p, tris = scenes.meshlet_template()
    pos = p.astype(np.float32)
    nrm = pos / np.linalg.norm(pos, axis=1, keepdims=True)
    up = np.array([0.0, 1.0, 0.0])
    tan = np.cross(up, nrm)
    tan /= np.maximum(np.linalg.norm(tan, axis=1, keepdims=True), 1e-6)
    w = np.where(np.arange(len(pos)) % 2, -1.0, 1.0)[:, None]
    uv = pos[:, [0, 2]] * 0.5 + 0.5
    return pos, tris.astype(np.uint16), uv.astype(np.float32), nrm.astype(np.float32), np.hstack([tan, w]).astype(np.float32)


def _plane(n=20):
    g = np.linspace(-1.0, 1.0, n + 1, dtype=np.float32)
    x, z = np.meshgrid(g, g)
    pos = np.stack([x.ravel(), np.zeros(x.size, np.float32), z.ravel()], axis=1).astype(np.float32)
    uv = (np.stack([x.ravel(), z.ravel()], axis=1) * 2.0 + 2.0).astype(np.float32)
    q = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            q += [a, a + n + 1, a + 1, a + 1, a + n + 1, a + n + 2]
    return pos, np.array(q, dtype=np.uint32).reshape(-1, 3), uv


def build(directory: str, name: str = "model") -> tuple[str, str]:
    """Writes name.gltf (+ name.bin) and name.glb into directory; returns both paths."""
    blob = bytearray()
    views, accessors = [], []

    def add(arr: np.ndarray, comp: int, kind: str, target=None, minmax=False):
        while len(blob) % 4:
            blob.append(0)
        off = len(blob)
        blob.extend(np.ascontiguousarray(arr).tobytes())
        v = {"buffer": 0, "byteOffset": off, "byteLength": arr.nbytes}
        if target:
            v["target"] = target
        views.append(v)
        a = {"bufferView": len(views) - 1, "componentType": comp, "count": int(arr.shape[0]), "type": kind}
        if minmax:
            a["min"], a["max"] = arr.min(axis=0).tolist(), arr.max(axis=0).tolist()
        accessors.append(a)
        return len(accessors) - 1

    sp, st, suv, sn, stan = _sphere()
    pp, pt, puv = _plane()
    sphere = {"attributes": {"POSITION": add(sp, 5126, "VEC3", 34962, True), "TEXCOORD_0": add(suv, 5126, "VEC2", 34962),
                             "NORMAL": add(sn, 5126, "VEC3", 34962), "TANGENT": add(stan, 5126, "VEC4", 34962)},
              "indices": add(st.reshape(-1), 5123, "SCALAR", 34963), "material": 0}
    plane = {"attributes": {"POSITION": add(pp, 5126, "VEC3", 34962, True), "TEXCOORD_0": add(puv, 5126, "VEC2", 34962)},
             "indices": add(pt.reshape(-1), 5125, "SCALAR", 34963), "material": 1}

    size = 64
    base = scenes.value_noise_rgba(size, 21, cells=8, layer=0)
    normal = scenes.value_noise_rgba(size, 22, cells=8, layer=1)
    mr = scenes.value_noise_rgba(size, 23, cells=8, layer=0)
    cut = scenes.value_noise_rgba(size, 24, cells=8, layer=0, cutout=True)
    images = [encode_png(base, 2), encode_png(normal), encode_png(mr, 2), encode_png(cut)]

    doc = {
        "asset": {"version": "2.0", "generator": "glimpsw_gb300 tests"},
        "scene": 0,
        "scenes": [{"nodes": [0, 1, 2, 4]}],
        "nodes": [
            {"mesh": 0, "translation": [0.0, 1.0, 0.0], "rotation": [0.0, 0.38268343, 0.0, 0.92387953], "scale": [1.5, 1.0, 1.5]},
            {"mesh": 1, "matrix": [4, 0, 0, 0, 0, 4, 0, 0, 0, 0, 4, 0, 0, -0.2, 0, 1]},
            {"translation": [2.5, 0.0, 1.0], "children": [3]},
            {"mesh": 0, "translation": [0.0, 0.5, 0.0], "scale": [0.5, 0.5, 0.5]},
            {"translation": [0.0, 4.0, 0.0], "extensions": {"KHR_lights_punctual": {"light": 0}}},
        ],
        "meshes": [{"name": "sphere", "primitives": [sphere]}, {"name": "plane", "primitives": [plane]}],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicRoughnessTexture": {"index": 2}},
             "normalTexture": {"index": 1}},
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 3}}, "alphaMode": "MASK", "alphaCutoff": 0.45,
             "doubleSided": True},
        ],
        "textures": [{"source": i} for i in range(4)],
        "accessors": accessors,
        "bufferViews": views,
        "extensionsUsed": ["KHR_lights_punctual"],
        "extensions": {"KHR_lights_punctual": {"lights": [
            {"type": "point", "color": [1.0, 0.9, 0.8], "intensity": 200.0, "range": 12.0}]}},
    }

    # .gltf: geometry in name.bin, images as data URIs
    gl = json.loads(json.dumps(doc))
    gl["buffers"] = [{"uri": f"{name}.bin", "byteLength": len(blob)}]
    gl["images"] = [{"uri": "data:image/png;base64," + base64.b64encode(im).decode()} for im in images]
    gltf_path = f"{directory}/{name}.gltf"
    open(f"{directory}/{name}.bin", "wb").write(bytes(blob))
    open(gltf_path, "w").write(json.dumps(gl))

    # .glb: images appended to the binary chunk as buffer views
    gb = json.loads(json.dumps(doc))
    bin_blob = bytearray(blob)
    gb["images"] = []
    for im in images:
        while len(bin_blob) % 4:
            bin_blob.append(0)
        gb["bufferViews"].append({"buffer": 0, "byteOffset": len(bin_blob), "byteLength": len(im)})
        bin_blob.extend(im)
        gb["images"].append({"bufferView": len(gb["bufferViews"]) - 1, "mimeType": "image/png"})
    while len(bin_blob) % 4:
        bin_blob.append(0)
    gb["buffers"] = [{"byteLength": len(bin_blob)}]
    js = json.dumps(gb).encode()
    js += b" " * (-len(js) % 4)
    glb = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(bin_blob))
    glb += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bin_blob), 0x004E4942) + bytes(bin_blob)
    glb_path = f"{directory}/{name}.glb"
    open(glb_path, "wb").write(glb)
    return gltf_path, glb_path
