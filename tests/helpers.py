"""Shared test helpers: render a scene with the CUDA library and with the CPU oracle."""
from __future__ import annotations

import math

import numpy as np

from glimpsw_gb300 import scenes


def meshlet_from_clip_triangles(tris, material_id=0):
    """One meshlet whose object positions map to the given clip-space vertices through
    CLIP_FROM_OBJECT (x, y, near, z): pass (x, y, w) per vertex."""
    m = np.zeros(1, dtype=scenes.MESHLET_DTYPE)
    tris = np.asarray(tris, dtype=np.float32).reshape(-1, 3, 3)
    n = len(tris)
    assert n <= 21
    pos = tris.reshape(-1, 3)
    m["Positions"][0, :, : len(pos)] = pos.T
    m["NumVertices"] = len(pos)
    m["NumTriangles"] = n
    m["AlphaCutoff"] = 255
    m["MaterialId"] = material_id
    idx = np.zeros((3, 128), dtype=np.uint8)
    idx[:, :n] = np.arange(3 * n).reshape(n, 3).T
    m["Indices"] = idx[None]
    return m


# clip = (x, y, 0.1, z_obj): a projection with f = 1 and NearZ 0.1, so w = object z.
CLIP_FROM_OBJECT = np.array([1, 0, 0, 0,
                             0, 1, 0, 0,
                             0, 0, 0, 1,
                             0, 0, 0.1, 0], dtype=np.float32)


def render_oracle(meshlets, materials, object_to_clip, width, height, count=None, binning=False, clipping=True,
                  guardband=True, meshlet_offset=0, cull_bitmap=None, clear=(0xFF000000, 0.0), fb=None, threads=1,
                  textures=None, shader=0):
    """Oracle frame; with threads > 1 the rows are split over threads and the counters are not kept.
    textures (oracle textures by material texture index) feed the alpha test of alpha-tested materials."""
    from oracle import oracle as O
    if fb is None:
        fb = O.Framebuffer(width, height)
        fb.clear(*clear)
    ctx = O.Context(meshlets, materials, object_to_clip, meshlet_offset=meshlet_offset, cull_bitmap=cull_bitmap,
                    textures=textures)
    n = len(meshlets) - meshlet_offset if count is None else count
    counters = O.draw_meshlets(fb, ctx, n, binning=binning, clipping=clipping, guardband=guardband, threads=threads,
                               shader=shader)
    return fb, counters


class GpuRenderer:
    def __init__(self, meshlets, materials, textures=None):
        from glimpsw_gb300 import api
        self.api = api
        api.load_library()
        self.scene = api.Scene()
        self.scene.upload_meshlets(np.ascontiguousarray(meshlets))
        self.scene.set_materials(materials, textures)
        self.rast = api.Rasterizer()

    def render(self, object_to_clip, width, height, count=None, binning=False, clipping=True, guardband=True,
               meshlet_offset=0, cull_bitmap=None, clear=(0xFF000000, 0.0), fb=None, shader=0):
        api = self.api
        if fb is None:
            fb = api.Framebuffer(width, height)
            fb.clear(*clear)
        self.rast.EnableBinning = binning
        self.rast.EnableClipping = clipping
        self.rast.EnableGuardband = guardband
        ctx = api.ShadingContext(self.scene, object_to_clip, meshlet_offset=meshlet_offset, cull_bitmap=cull_bitmap)
        n = (self._count() - meshlet_offset) if count is None else count
        self.rast.reset_counters()
        self.rast.draw_meshlets(fb, n, ctx, shader)
        return fb, self.rast.counters()

    def _count(self):
        import ctypes as C
        c = C.c_uint32()
        self.api._check(self.api._lib.swr_scene_meshlet_count(self.scene.h, C.byref(c)))
        return c.value


LIGHT_DTYPE = np.dtype([("type", "<u4"), ("position", "<f4", 3), ("direction", "<f4", 3), ("color", "<f4", 3),
                        ("intensity", "<f4"), ("radius", "<f4"), ("spot_inner", "<f4"), ("spot_outer", "<f4"),
                        ("inv_radius_sq", "<f4"), ("spot_scale", "<f4"), ("spot_offset", "<f4")])


def default_lights() -> np.ndarray:
    """The frame driver's fallback light (Main.cpp:192-201): directional, colour 1, 1500 lux."""
    lights = np.zeros(1, dtype=LIGHT_DTYPE)
    d = -np.array([0.589494, 0.684509, 0.428906], dtype=np.float32)
    d = (d * np.float32(1.0 / np.sqrt(np.float64((d * d).sum())))).astype(np.float32)
    lights["direction"] = d
    lights["color"] = 1.0
    lights["intensity"] = 1500.0
    return lights


def make_light(kind: int, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0), color=(1.0, 1.0, 1.0),
               intensity: float = 1.0, radius: float = 0.0, inner: float = 0.0, outer: float = math.pi / 4) -> np.ndarray:
    """One light record as the reference builds it (Scene.h:52-75): a normalised direction, then
    Light::SetRadius (0 or less: 1e6) and Light::SetSpotAngles in float32."""
    f = np.float32
    li = np.zeros(1, dtype=LIGHT_DTYPE)
    li["type"] = kind
    li["position"] = np.asarray(position, f)
    d = np.asarray(direction, f)
    li["direction"] = (d * f(1.0 / np.sqrt(np.float64((d * d).sum())))).astype(f)
    li["color"] = np.asarray(color, f)
    li["intensity"] = f(intensity)
    r = f(radius) if radius > 0 else f(1e6)
    li["radius"] = r
    li["inv_radius_sq"] = f(1.0) / (r * r)
    li["spot_inner"], li["spot_outer"] = f(inner), f(outer)
    scale = f(1.0) / max(np.cos(f(inner)) - np.cos(f(outer)), f(1e-4))
    li["spot_scale"] = scale
    li["spot_offset"] = -np.cos(f(outer)) * scale
    return li


def model_lights(model) -> np.ndarray:
    """An imported glTF model's KHR_lights_punctual lights (gltf.Model.lights) as light records."""
    out = np.zeros(len(model.lights), dtype=LIGHT_DTYPE)
    for i, li in enumerate(model.lights):
        for k in LIGHT_DTYPE.names:
            out[k][i] = li[k]
    return out


def gpu_lights(lights: np.ndarray):
    from glimpsw_gb300 import api
    out = []
    for li in lights:
        s = api.SwrLight()
        s.type = int(li["type"])
        s.position[:] = li["position"].tolist()
        s.direction[:] = li["direction"].tolist()
        s.color[:] = li["color"].tolist()
        s.intensity, s.radius = float(li["intensity"]), float(li["radius"])
        s.spot_inner_angle, s.spot_outer_angle = float(li["spot_inner"]), float(li["spot_outer"])
        s.inv_radius_sq, s.spot_scale, s.spot_offset = float(li["inv_radius_sq"]), float(li["spot_scale"]), float(li["spot_offset"])
        out.append(s)
    return out


class TexturePair:
    """The same texels in an oracle texture and a device texture (mips generated on each side)."""

    def __init__(self, layers, size, fmt=0, max_levels=16, gpu=True):
        from oracle import oracle as O
        self.o = O.Texture(size, size, max_levels, len(layers), fmt=fmt)
        for i, px in enumerate(layers):
            self.o.set_pixels(px, i)
        self.o.generate_mips()
        self.g = None
        if gpu:
            from glimpsw_gb300 import api
            self.g = api.Texture2D(fmt, size, size, max_levels, len(layers))
            for i, px in enumerate(layers):
                self.g.set_pixels(px, i)
            self.g.generate_mips()


def assert_visbuffer_equal(gpu_fb, orc_fb):
    g_ids, o_ids = gpu_fb.get_pixels(0), orc_fb.get_pixels(0)
    g_d, o_d = gpu_fb.get_pixels(1), orc_fb.get_pixels(1)
    bad_d = np.argwhere(g_d != o_d)
    bad_i = np.argwhere(g_ids != o_ids)
    msg = ""
    if len(bad_d) or len(bad_i):
        y, x = (bad_d if len(bad_d) else bad_i)[0]
        msg = (f"{len(bad_d)} depth / {len(bad_i)} id mismatches; first at (x={x}, y={y}): gpu depth "
               f"{g_d[y, x]:#010x} id {g_ids[y, x]} vs oracle depth {o_d[y, x]:#010x} id {o_ids[y, x]}")
    assert not msg, msg
