"""glTF 2.0 import (Scene::ImportGltf, Scene.cpp:156-347): .gltf with external or embedded buffers
and .glb; meshes become Meshlet records through the library's meshlet builder
(``swr_build_meshlets``), materials become (texture layers, double-sided, alpha cutoff) the way
``LoadTextures`` (Scene.cpp:71-100) combines them, nodes become (meshlet range, global transform)
instances, and KHR_lights_punctual lights become ``swr_light`` records.

Differences from the reference, all forced by absent libraries or undefined reference behaviour:

* meshlet grouping is the library's own (meshoptimizer is not available);
* images are decoded by a small PNG decoder here; JPEG and other formats are not decoded and leave
  the material's texture out (``Model.warnings`` names them); the reference decodes with stb_image;
* a material without a base colour image has no texture (the reference creates an uninitialised
  4x4 texture);
* a zero tangent packs as octahedral (0.5, 0.5) (the reference's MapOctahedron divides by zero);
* ``MapOctahedron`` runs the reference's rcp14 bit for bit (``approx14.rcp14``) and its fused
  multiply-adds (``approx14.fma32``).

Skins and animations (Scene.cpp:102-153, 304-319) are outside the raster path and not imported.
"""
from __future__ import annotations

import base64
import ctypes as C
import json
import math
import os
import struct
import zlib
from dataclasses import dataclass, field

import numpy as np

from . import scenes
from .approx14 import fma32, rcp14

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NUM = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}


@dataclass
class Instance:
    """A node that draws a mesh: its meshlets [meshlet_offset, meshlet_offset + meshlet_count) and
    its global transform (ModelNode::MeshOffset/MeshCount/GlobalTransform, Scene.h:40-50)."""
    node: int
    name: str
    meshlet_offset: int
    meshlet_count: int
    transform: np.ndarray  # float32[16], column-major (glm layout), like the views' matrices


@dataclass
class Model:
    meshlets: np.ndarray                       # MESHLET_DTYPE[n]
    materials: np.ndarray                      # MATERIAL_DTYPE[m]; texture indexes `textures`
    textures: list                             # per material with a texture: list of RGBA8 layers (uint32[h, w])
    instances: list                            # Instance
    lights: list = field(default_factory=list) # dicts with the swr_light fields
    warnings: list = field(default_factory=list)


# ----------------------------------------------------------------------------- containers
def _read_document(path: str):
    data = open(path, "rb").read()
    if data[:4] == b"glTF":
        version, length = struct.unpack_from("<II", data, 4)
        if version != 2:
            raise ValueError(f"{path}: GLB version {version}")
        pos, doc, bin_chunk = 12, None, None
        while pos + 8 <= min(length, len(data)):
            clen, ctype = struct.unpack_from("<II", data, pos)
            chunk = data[pos + 8:pos + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942 and bin_chunk is None:
                bin_chunk = chunk
            pos += 8 + clen
        if doc is None:
            raise ValueError(f"{path}: GLB without a JSON chunk")
        return doc, bin_chunk
    return json.loads(data.decode("utf-8")), None


def _load_uri(base: str, uri: str) -> bytes:
    if uri.startswith("data:"):
        head, payload = uri.split(",", 1)
        return base64.b64decode(payload) if head.endswith(";base64") else payload.encode()
    from urllib.parse import unquote
    return open(os.path.join(base, unquote(uri)), "rb").read()


def _buffers(doc, base, bin_chunk):
    out = []
    for i, b in enumerate(doc.get("buffers", [])):
        if "uri" in b:
            out.append(_load_uri(base, b["uri"]))
        elif i == 0 and bin_chunk is not None:
            out.append(bin_chunk)
        else:
            raise ValueError("buffer without data")
    return out


def _view_bytes(doc, buffers, view_index):
    v = doc["bufferViews"][view_index]
    off = v.get("byteOffset", 0)
    return buffers[v["buffer"]][off:off + v["byteLength"]], v.get("byteStride", 0)


def read_accessor(doc, buffers, index: int) -> np.ndarray:
    """cgltf_accessor_unpack_floats / _indices: (count, components) in the stored type, with
    normalized integers converted to float as glTF defines."""
    a = doc["accessors"][index]
    dt = np.dtype(_COMPONENT[a["componentType"]]).newbyteorder("<")
    n, count = _NUM[a["type"]], a["count"]
    if "bufferView" in a:
        raw, stride = _view_bytes(doc, buffers, a["bufferView"])
        off = a.get("byteOffset", 0)
        elem = dt.itemsize * n
        stride = stride or elem
        if stride == elem:
            out = np.frombuffer(raw, dt, count * n, off).reshape(count, n).copy()
        else:
            rows = np.lib.stride_tricks.as_strided(np.frombuffer(raw, np.uint8, len(raw) - off, off),
                                                   (count, elem), (stride, 1))
            out = rows.copy().view(dt).reshape(count, n)
    else:
        out = np.zeros((count, n), dt)
    if "sparse" in a:
        sp = a["sparse"]
        idt = np.dtype(_COMPONENT[sp["indices"]["componentType"]]).newbyteorder("<")
        raw, _ = _view_bytes(doc, buffers, sp["indices"]["bufferView"])
        idx = np.frombuffer(raw, idt, sp["count"], sp["indices"].get("byteOffset", 0))
        raw, _ = _view_bytes(doc, buffers, sp["values"]["bufferView"])
        vals = np.frombuffer(raw, dt, sp["count"] * n, sp["values"].get("byteOffset", 0)).reshape(-1, n)
        out[idx.astype(np.int64)] = vals
    if a.get("normalized") and dt.kind in "iu":
        info = np.iinfo(dt)
        f = out.astype(np.float32) / np.float32(info.max)
        out = np.maximum(f, np.float32(-1.0)) if dt.kind == "i" else f
    return out


# ----------------------------------------------------------------------------- images
def decode_png(data: bytes) -> np.ndarray:
    """PNG (8- or 16-bit, grey / grey+alpha / RGB / RGBA / palette, not interlaced) to packed RGBA8
    words, uint32[h, w]."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
    pos, idat, palette, trns = 8, [], None, None
    width = height = depth = ctype = interlace = None
    while pos < len(data):
        ln, kind = struct.unpack_from(">I4s", data, pos)
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if interlace:
        raise ValueError("interlaced PNG")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp_bits = channels * depth
    if depth < 8 and ctype != 3 and ctype != 0:
        raise ValueError("unsupported PNG bit depth")
    stride = (width * bpp_bits + 7) // 8
    bpp = max(1, bpp_bits // 8)
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    rows = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(height):
        f = raw[y * (stride + 1)]
        line = raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)].astype(np.int32)
        if f == 1:  # Sub
            for x in range(bpp, stride, bpp):
                line[x:x + bpp] = (line[x:x + bpp] + line[x - bpp:x]) & 255
        elif f == 2:  # Up
            line = (line + prev) & 255
        elif f == 3:  # Average
            for x in range(stride):
                left = line[x - bpp] if x >= bpp else 0
                line[x] = (line[x] + ((left + prev[x]) >> 1)) & 255
        elif f == 4:  # Paeth
            for x in range(stride):
                a = line[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                line[x] = (line[x] + pred) & 255
        rows[y] = line
        prev = line
    if depth == 16:
        px = rows.reshape(height, width, channels, 2)[..., 0]  # high byte
    elif depth == 8:
        px = rows.reshape(height, width, channels)
    else:  # 1/2/4-bit grey or palette indices
        bits = np.unpackbits(rows, axis=1).reshape(height, -1, depth)
        vals = np.zeros(bits.shape[:2], np.uint8)
        for k in range(depth):
            vals = (vals << 1) | bits[..., k]
        px = vals[:, :width, None]
        if ctype == 0:
            px = (px.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
    if ctype == 3:
        idx = px[..., 0]
        rgb = palette[idx]
        alpha = np.full(idx.shape, 255, np.uint8)
        if trns is not None:
            t = np.frombuffer(trns, np.uint8)
            lut = np.full(256, 255, np.uint8)
            lut[:len(t)] = t
            alpha = lut[idx]
        rgba = np.concatenate([rgb, alpha[..., None]], axis=2)
    elif channels == 1:
        rgba = np.concatenate([px, px, px, np.full_like(px, 255)], axis=2)
    elif channels == 2:
        rgba = np.concatenate([px[..., :1]] * 3 + [px[..., 1:]], axis=2)
    elif channels == 3:
        rgba = np.concatenate([px, np.full(px.shape[:2] + (1,), 255, np.uint8)], axis=2)
    else:
        rgba = px
    rgba = rgba.astype(np.uint32)
    return rgba[..., 0] | (rgba[..., 1] << 8) | (rgba[..., 2] << 16) | (rgba[..., 3] << 24)


def _channels(words: np.ndarray) -> np.ndarray:
    return np.stack([(words >> (8 * k)) & 255 for k in range(4)], axis=-1).astype(np.uint8)


def _pack(ch: np.ndarray) -> np.ndarray:
    c = ch.astype(np.uint32)
    return c[..., 0] | (c[..., 1] << 8) | (c[..., 2] << 16) | (c[..., 3] << 24)


def combine_normal_mr(normal: np.ndarray, mr: np.ndarray | None) -> np.ndarray:
    """CombineNormalMR (Scene.cpp:17-35): renormalised normal XY in RG, metallic (MR.b) and
    roughness (MR.g) in BA."""
    n = _channels(normal)
    v = n[..., :3].astype(np.float32) / np.float32(127.0) - np.float32(1.0)
    v = v / np.sqrt((v * v).sum(axis=-1, keepdims=True)).astype(np.float32)
    v = v * np.float32(127.0) + np.float32(127.0)
    out = n.copy()
    out[..., 0] = np.round(v[..., 0]).astype(np.uint8)
    out[..., 1] = np.round(v[..., 1]).astype(np.uint8)
    if mr is not None:
        m = _channels(mr)
        out[..., 2] = m[..., 2]
        out[..., 3] = m[..., 1]
    return _pack(out)


def insert_emissive_mask(base: np.ndarray, emissive: np.ndarray) -> np.ndarray:
    """InsertEmissiveMask (Scene.cpp:37-48): base alpha 255 where emissive, else at most 254."""
    b, e = _channels(base), _channels(emissive)
    lit = (e[..., :3] > 8).any(axis=-1)
    b[..., 3] = np.where(lit, 255, np.minimum(b[..., 3], 254))
    return _pack(b)


# ----------------------------------------------------------------------------- vertex packing
def pack_half2(uv: np.ndarray) -> np.ndarray:
    """glm::packHalf2x16 of (u, v) per vertex."""
    h = uv.astype(np.float32).astype(np.float16).view(np.uint16).astype(np.uint32)
    return h[:, 0] | (h[:, 1] << 16)


def map_octahedron(n: np.ndarray) -> np.ndarray:
    """texutil::MapOctahedron (Texture.h:282-288) in float32: w = rcp14(|x| + |y| + |z|),
    t = max(-z * w, 0), u = fma(x, w, mulsign(t, x)), v likewise, then * 0.5 + 0.5; a zero vector
    maps to (0.5, 0.5)."""
    n = n.astype(np.float32)
    s = np.abs(n[:, 0]) + np.abs(n[:, 1]) + np.abs(n[:, 2])
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        w = rcp14(s)
        t = np.maximum(-n[:, 2] * w, np.float32(0.0))
        u = fma32(n[:, 0], w, np.copysign(t, n[:, 0]))
        v = fma32(n[:, 1], w, np.copysign(t, n[:, 1]))
    out = np.stack([u, v], axis=1) * np.float32(0.5) + np.float32(0.5)
    return np.where(np.isfinite(out), out, np.float32(0.5)).astype(np.float32)


def pack_unorm4x8(v: np.ndarray) -> np.ndarray:
    """glm::packUnorm4x8: round(clamp(v, 0, 1) * 255) per channel."""
    q = np.floor(np.clip(v, 0.0, 1.0).astype(np.float32) * np.float32(255.0) + np.float32(0.5)).astype(np.uint32)
    return q[:, 0] | (q[:, 1] << 8) | (q[:, 2] << 16) | (q[:, 3] << 24)


# ----------------------------------------------------------------------------- transforms
def _quat_matrix(q):
    x, y, z, w = (float(c) for c in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y), 0],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x), 0],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y), 0],
                     [0, 0, 0, 1]], dtype=np.float64)


def node_local_matrix(node) -> np.ndarray:
    """cgltf_node_transform_local: the node's matrix, or T * R * S (row-major, column vectors)."""
    if "matrix" in node:
        return np.array(node["matrix"], dtype=np.float64).reshape(4, 4).T
    t = np.eye(4)
    t[:3, 3] = node.get("translation", [0, 0, 0])
    r = _quat_matrix(node.get("rotation", [0, 0, 0, 1]))
    s = np.diag(list(node.get("scale", [1, 1, 1])) + [1.0])
    return t @ r @ s


# ----------------------------------------------------------------------------- import
def load(path: str, lib=None) -> Model:
    """Imports a .gltf / .glb file (scene 0, or the document's default scene)."""
    from . import api
    lib = lib or api.load_library()
    doc, bin_chunk = _read_document(path)
    base = os.path.dirname(os.path.abspath(path))
    buffers = _buffers(doc, base, bin_chunk)
    warnings = []

    # materials and their texture layers (LoadTextures, Scene.cpp:71-100)
    image_cache = {}

    def image(tex_ref):
        if not tex_ref:
            return None
        tex = doc["textures"][tex_ref["index"]]
        src = tex.get("source")
        if src is None:
            return None
        if src in image_cache:
            return image_cache[src]
        img = doc["images"][src]
        try:
            if "uri" in img:
                data = _load_uri(base, img["uri"])
            else:
                raw, _ = _view_bytes(doc, buffers, img["bufferView"])
                data = bytes(raw)
            px = decode_png(data)
        except (ValueError, OSError, zlib.error) as e:
            warnings.append(f"image {src} ({img.get('uri', img.get('mimeType', ''))}): {e}")
            px = None
        image_cache[src] = px
        return px

    mats = np.zeros(len(doc.get("materials", [])), dtype=scenes.MATERIAL_DTYPE)
    textures = []
    for i, m in enumerate(doc.get("materials", [])):
        pbr = m.get("pbrMetallicRoughness", {})
        mats[i]["is_double_sided"] = 1 if m.get("doubleSided") else 0
        mats[i]["alpha_cutoff"] = (int(np.float32(m.get("alphaCutoff", 0.5)) * np.float32(255.0) + np.float32(0.5))
                                   if m.get("alphaMode") == "MASK" else 255)
        basecol = image(pbr.get("baseColorTexture"))
        mats[i]["texture"] = 0xFFFFFFFF
        if basecol is None:
            continue
        h, w = basecol.shape
        if w & (w - 1) or h & (h - 1):
            warnings.append(f"material {i}: {w}x{h} base colour is not a power of two; untextured")
            continue
        layers = [basecol]
        normal = image(m.get("normalTexture"))
        emissive = image(m.get("emissiveTexture"))
        has_normal = normal is not None and normal.shape == basecol.shape
        has_emissive = emissive is not None and emissive.shape == basecol.shape
        if has_normal:
            mr = image(pbr.get("metallicRoughnessTexture"))
            layers.append(combine_normal_mr(normal, mr if mr is not None and mr.shape == normal.shape else None))
        if has_emissive:  # three layers; without a normal map the reference leaves layer 1 unset (zero here)
            layers[0] = insert_emissive_mask(basecol, emissive)
            if not has_normal:
                layers.append(np.zeros_like(basecol))
            layers.append(emissive)
        mats[i]["texture"] = len(textures)
        textures.append(layers)

    # meshes -> meshlets (Scene.cpp:196-286)
    records, mesh_ranges = [], []
    total = 0
    for mesh in doc.get("meshes", []):
        first = total
        for prim in mesh["primitives"]:
            if prim.get("mode", 4) != 4:
                warnings.append(f"mesh {mesh.get('name', '')}: primitive mode {prim['mode']} skipped")
                continue
            attrs = prim["attributes"]
            pos = read_accessor(doc, buffers, attrs["POSITION"]).astype(np.float32)
            nv = len(pos)
            idx = (read_accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.uint32) if "indices" in prim
                   else np.arange(nv, dtype=np.uint32))
            idx = idx[: len(idx) // 3 * 3]
            tc = pack_half2(read_accessor(doc, buffers, attrs["TEXCOORD_0"])) if "TEXCOORD_0" in attrs else None
            nt = signs = None
            if "NORMAL" in attrs:
                nrm = read_accessor(doc, buffers, attrs["NORMAL"]).astype(np.float32)
                tan = (read_accessor(doc, buffers, attrs["TANGENT"]).astype(np.float32) if "TANGENT" in attrs
                       else np.zeros((nv, 4), np.float32))
                oct_n, oct_t = map_octahedron(nrm), map_octahedron(tan[:, :3])
                nt = pack_unorm4x8(np.concatenate([oct_n, oct_t], axis=1))
                signs = (tan[:, 3] < 0).astype(np.uint8)
            mat_id = prim.get("material")
            d = api.SwrMeshDesc()
            pos_c = np.ascontiguousarray(pos)
            idx_c = np.ascontiguousarray(idx)
            keep = [pos_c, idx_c]
            d.positions = pos_c.ctypes.data
            d.num_vertices = nv
            d.indices = idx_c.ctypes.data
            d.num_triangles = len(idx_c) // 3
            for name, arr in (("texcoords", tc), ("normal_tangents", nt), ("tangent_signs", signs)):
                if arr is not None:
                    arr = np.ascontiguousarray(arr)
                    keep.append(arr)
                    setattr(d, name, arr.ctypes.data)
            d.material_id = 0xFFFFFFFF if mat_id is None else int(mat_id)
            d.alpha_cutoff = 255 if mat_id is None else int(mats[mat_id]["alpha_cutoff"])
            cap = lib.swr_meshlet_bound(d.num_triangles)
            out = np.zeros(cap, dtype=scenes.MESHLET_DTYPE)
            count = C.c_uint32()
            api._check(lib.swr_build_meshlets(C.byref(d), out.ctypes.data, cap, C.byref(count)))
            records.append(out[: count.value])
            total += count.value
            del keep
        mesh_ranges.append((first, total - first))
    meshlets = np.zeros(total, dtype=scenes.MESHLET_DTYPE)  # (np.concatenate would drop the record's padding)
    pos_ = 0
    for r in records:
        meshlets[pos_:pos_ + len(r)] = r
        pos_ += len(r)

    # nodes (Scene.cpp:288-341)
    instances, lights = [], []
    nodes = doc.get("nodes", [])
    light_defs = doc.get("extensions", {}).get("KHR_lights_punctual", {}).get("lights", [])

    def visit(ni, parent):
        node = nodes[ni]
        g = parent @ node_local_matrix(node)
        if "mesh" in node:
            off, cnt = mesh_ranges[node["mesh"]]
            instances.append(Instance(ni, node.get("name", ""), off, cnt, g.T.reshape(16).astype(np.float32)))
        li = node.get("extensions", {}).get("KHR_lights_punctual", {}).get("light")
        if li is not None:
            lights.append(_light(light_defs[li], g))
        for c in node.get("children", []):
            visit(c, g)

    scene_idx = doc.get("scene", 0)
    if doc.get("scenes"):
        for ni in doc["scenes"][scene_idx].get("nodes", []):
            visit(ni, np.eye(4))
    return Model(meshlets, mats, textures, instances, lights, warnings)


def _light(ld, g):
    """Light::SetRadius / SetSpotAngles (Scene.h:65-75) of a KHR_lights_punctual light, in float32 as
    the reference computes them."""
    f = np.float32
    kind = {"directional": 0, "point": 1, "spot": 2}[ld["type"]]
    radius = f(ld.get("range", 0.0))
    radius = radius if radius > 0 else f(1e6)
    spot = ld.get("spot", {})
    inner, outer = f(spot.get("innerConeAngle", 0.0)), f(spot.get("outerConeAngle", math.pi / 4))
    scale = f(1.0) / max(np.cos(inner) - np.cos(outer), f(1e-4))
    d = -g[:3, 2]
    d = d / max(np.linalg.norm(d), 1e-30)
    return {"type": kind, "position": g[:3, 3].astype(np.float32), "direction": d.astype(np.float32),
            "color": np.array(ld.get("color", [1, 1, 1]), np.float32), "intensity": float(ld.get("intensity", 1.0)),
            "radius": float(radius), "spot_inner": float(inner), "spot_outer": float(outer),
            "inv_radius_sq": float(f(1.0) / (radius * radius)), "spot_scale": float(scale),
            "spot_offset": float(-np.cos(outer) * scale)}


# ----------------------------------------------------------------------------- device upload / draw
def upload(model: Model, max_levels: int = 16):
    """The model's meshlets, textures (mips generated) and materials on the device: returns
    (api.Scene, [api.Texture2D])."""
    from . import api
    texs = []
    for layers in model.textures:
        h, w = layers[0].shape
        t = api.Texture2D(api.FORMAT_RGBA8U, w, h, max_levels, len(layers))
        for i, px in enumerate(layers):
            t.set_pixels(np.ascontiguousarray(px), i)
        t.generate_mips()
        texs.append(t)
    scene = api.Scene()
    if len(model.meshlets):
        scene.upload_meshlets(np.ascontiguousarray(model.meshlets))
    scene.set_materials(model.materials, texs)
    return scene, texs


def draw(model: Model, scene, rast, fb, proj, view, prev_view=None, depth_map=None, bitmaps=None):
    """The frame driver's draw loop (Main.cpp:216-245) for the model's instances: per instance,
    CullMeshlets against the frustum (and depth_map when given) in batches of 65536 meshlets, then
    DrawMeshlets with ObjectToClip = proj * view * instance transform."""
    import torch

    from . import api
    prev_view = view if prev_view is None else prev_view
    w, h = fb.width, fb.height
    for inst in model.instances:
        model_mat = inst.transform
        world_to_clip = scenes.mat_mul(proj, view)
        object_to_clip = scenes.mat_mul(world_to_clip, model_mat)
        for off in range(0, inst.meshlet_count, 65536):
            cnt = min(65536, inst.meshlet_count - off)
            bm = torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda")
            api.cull_meshlets(scene, inst.meshlet_offset + off, cnt, bm, proj, view, model_mat, prev_view, w, h, depth_map)
            rast.draw_meshlets(fb, cnt, api.ShadingContext(scene, object_to_clip, world_to_clip=world_to_clip,
                                                           meshlet_offset=inst.meshlet_offset + off, cull_bitmap=bm))
