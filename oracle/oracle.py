"""ctypes binding of the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the CPU-baseline legs
of bench.py, as the checker or the timed CPU baseline; the library under test never uses it.
The oracle restates GLimpSW's CPU code (parity unpinned: the reference cannot be built here and
ships no golden vectors); see swr_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class OrcFramebuffer(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("tile_stride", C.c_uint32),
                ("layer_stride", C.c_uint32), ("num_layers", C.c_uint32), ("data", C.c_void_p)]


class OrcMaterial(C.Structure):
    _fields_ = [("texture", C.c_uint32), ("is_double_sided", C.c_uint8), ("alpha_cutoff", C.c_uint8),
                ("pad", C.c_uint8 * 2)]


class OrcTexture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("mip_levels", C.c_uint32),
                ("num_layers", C.c_uint32), ("row_shift", C.c_uint32), ("layer_stride", C.c_uint32),
                ("scale_u", C.c_float), ("scale_v", C.c_float), ("scale_lerp_u", C.c_float),
                ("scale_lerp_v", C.c_float), ("mask_u", C.c_int32), ("mask_v", C.c_int32),
                ("mask_lerp_u", C.c_int32), ("mask_lerp_v", C.c_int32), ("mip_offsets", C.c_uint32 * 16),
                ("data", C.c_void_p)]


class OrcLight(C.Structure):
    _fields_ = [("type", C.c_uint32), ("position", C.c_float * 3), ("direction", C.c_float * 3),
                ("color", C.c_float * 3), ("intensity", C.c_float), ("radius", C.c_float),
                ("spot_inner", C.c_float), ("spot_outer", C.c_float), ("inv_radius_sq", C.c_float),
                ("spot_scale", C.c_float), ("spot_offset", C.c_float)]


class OrcShadingContext(C.Structure):
    _fields_ = [("meshlets", C.c_void_p), ("materials", C.c_void_p), ("textures", C.c_void_p),
                ("lights", C.c_void_p), ("num_lights", C.c_uint32), ("meshlet_offset", C.c_uint32),
                ("cull_bitmap", C.c_void_p), ("world_to_clip", C.c_float * 16),
                ("object_to_clip", C.c_float * 16), ("object_to_world", C.c_float * 9),
                ("skybox", C.c_void_p), ("view_pos", C.c_float * 3), ("exposure", C.c_float),
                ("num_meshlets", C.c_uint32)]


class OrcRasterFlags(C.Structure):
    _fields_ = [("enable_binning", C.c_int), ("enable_clipping", C.c_int), ("enable_guardband", C.c_int),
                ("shader", C.c_int)]


SHADER_VISBUFFER, SHADER_DEFERRED, SHADER_OVERDRAW, SHADER_TEXCOORD = 0, 1, 2, 3


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        L = _lib
        L.orc_meshlet_size.restype = C.c_uint32
        L.orc_fb_layer_stride.restype = C.c_uint32
        L.orc_cull_meshlets.restype = C.c_uint32
        L.orc_texture_storage_words.restype = C.c_uint64
        L.orc_approx_mode_available.restype = C.c_int
        L.orc_approx14_mismatches.restype = C.c_int64
        L.orc_approx14_mismatches.argtypes = [C.c_int, C.c_uint64, C.c_uint64]
        L.orc_fb_clear.argtypes = [C.c_void_p, C.c_uint32, C.c_float]
        for name in ("orc_ibl_irradiance_texel", "orc_ibl_radiance_texel", "orc_ibl_env_brdf_texel", "orc_debug_lerp16"):
            getattr(L, name).restype = C.c_uint32
        L.orc_debug_calc_mip_level.restype = C.c_int32
        L.orc_debug_calc_mip_level.argtypes = [C.c_float] * 6
        L.orc_cull_meshlets.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_void_p]
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Framebuffer:
    """Host framebuffer in the reference layout (4x4-tiled 32-bit layers)."""

    def __init__(self, width: int, height: int, num_layers: int = 2):
        assert width % 4 == 0 and height % 4 == 0
        L = lib()
        self.layer_stride = L.orc_fb_layer_stride(width, height)
        self.data = np.zeros(self.layer_stride * num_layers + 64, dtype=np.uint32)
        self.s = OrcFramebuffer()
        L.orc_fb_init(C.byref(self.s), width, height, num_layers, _fptr(self.data))
        self.width, self.height, self.num_layers = width, height, num_layers

    def clear(self, color: int, depth: float):
        lib().orc_fb_clear(C.byref(self.s), C.c_uint32(color), C.c_float(depth))

    def clear_layer(self, layer: int, value: int):
        lib().orc_fb_clear_layer(C.byref(self.s), C.c_uint32(layer), C.c_uint32(value))

    def get_pixels(self, layer: int) -> np.ndarray:
        out = np.zeros((self.height, self.width), dtype=np.uint32)
        lib().orc_fb_get_pixels(C.byref(self.s), C.c_uint32(layer), _fptr(out), C.c_uint32(self.width))
        return out


class Texture:
    def __init__(self, width: int, height: int, max_levels: int = 1, num_layers: int = 1, fmt: int = 0):
        L = lib()
        words = L.orc_texture_storage_words(width, height, max_levels, num_layers)
        self.data = np.zeros(words, dtype=np.uint32)
        self.s = OrcTexture()
        self.fmt = fmt
        L.orc_texture_init(C.byref(self.s), width, height, max_levels, num_layers, _fptr(self.data))

    @property
    def mip_levels(self) -> int:
        return self.s.mip_levels

    def set_pixels(self, pixels: np.ndarray, layer: int = 0):
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        lib().orc_texture_set_pixels(C.byref(self.s), _fptr(pixels), C.c_uint32(pixels.shape[1]),
                                     C.c_uint32(layer), C.c_uint32(0))

    def generate_mips(self):
        lib().orc_texture_generate_mips(C.byref(self.s), C.c_uint32(self.fmt))


def _mat(arr, n):
    a = np.ascontiguousarray(arr, dtype=np.float32).reshape(n)
    return (C.c_float * n)(*a.tolist())


class Context:
    """Keeps the numpy buffers referenced by an OrcShadingContext alive."""

    def __init__(self, meshlets: np.ndarray, materials: np.ndarray, object_to_clip, world_to_clip=None,
                 object_to_world=None, meshlet_offset: int = 0, cull_bitmap: np.ndarray | None = None,
                 textures: list | None = None, lights: np.ndarray | None = None, skybox: Texture | None = None,
                 view_pos=(0, 0, 0), exposure: float = 1.0):
        assert meshlets.dtype.itemsize == 1728 and meshlets.flags.c_contiguous, "Meshlet records are 1728 bytes"
        self.meshlets = meshlets
        self.materials = np.ascontiguousarray(materials)
        self.cull_bitmap = cull_bitmap
        self.textures = textures or []
        self.tex_structs = (OrcTexture * max(1, len(self.textures)))(*[t.s for t in self.textures])
        self.skybox = skybox
        self.lights = lights
        s = OrcShadingContext()
        s.meshlets = meshlets.ctypes.data
        s.materials = self.materials.ctypes.data
        s.textures = C.cast(self.tex_structs, C.c_void_p)
        s.lights = lights.ctypes.data if lights is not None else None
        s.num_lights = 0 if lights is None else len(lights)
        s.meshlet_offset = meshlet_offset
        s.cull_bitmap = cull_bitmap.ctypes.data if cull_bitmap is not None else None
        s.object_to_clip = _mat(object_to_clip, 16)
        s.world_to_clip = _mat(world_to_clip if world_to_clip is not None else object_to_clip, 16)
        ow = object_to_world if object_to_world is not None else np.eye(3, dtype=np.float32)
        s.object_to_world = _mat(ow, 9)
        s.skybox = C.cast(C.byref(skybox.s), C.c_void_p) if skybox is not None else None
        s.view_pos = (C.c_float * 3)(*[float(v) for v in view_pos])
        s.exposure = exposure
        s.num_meshlets = len(meshlets)
        self.s = s


def draw_meshlets(fb: Framebuffer, ctx: Context, count: int, binning=False, clipping=True, guardband=True,
                  threads: int = 1, shader: int = SHADER_VISBUFFER) -> np.ndarray:
    flags = OrcRasterFlags(int(binning), int(clipping), int(guardband), int(shader))
    counters = np.zeros(4, dtype=np.uint64)
    if threads > 1:
        lib().orc_draw_meshlets_mt(C.byref(fb.s), C.c_uint32(count), C.byref(ctx.s), C.byref(flags),
                                   C.c_uint32(threads))
    else:
        lib().orc_draw_meshlets(C.byref(fb.s), C.c_uint32(count), C.byref(ctx.s), C.byref(flags), _fptr(counters))
    return counters


def draw_meshlets_binned(fb: Framebuffer, ctx: Context, count: int, threads: int) -> np.ndarray:
    """Rasterizer(threads)::DrawMeshlets with binning on, threaded in the reference's shape (meshlets
    strided over workers, 128x128 bins rasterized by their elected worker); returns the counters."""
    counters = np.zeros(4, dtype=np.uint64)
    lib().orc_draw_meshlets_binned(C.byref(fb.s), C.c_uint32(count), C.byref(ctx.s), C.c_uint32(threads),
                                   _fptr(counters))
    return counters


def ibl_irradiance_texel(env: Texture, x: int, y: int, w: int, h: int) -> int:
    """PrefilterDiffuseIrradiance (Shading.cpp:72-102) of texel (x, y) of a w x h map, packed R11G11B10."""
    return int(lib().orc_ibl_irradiance_texel(C.byref(env.s), x, y, w, h))


def ibl_radiance_texel(env: Texture, level: int, levels: int, x: int, y: int, w0: int, h0: int) -> int:
    """PrefilterEnvMap (Shading.cpp:105-147) of texel (x, y) of mip `level` of a radiance map."""
    return int(lib().orc_ibl_radiance_texel(C.byref(env.s), level, levels, x, y, w0, h0))


def ibl_env_brdf_texel(x: int, y: int, w: int, h: int) -> int:
    """IntegrateBRDF (Shading.cpp:149-175) of texel (x, y) of a w x h table, packed RG16f."""
    return int(lib().orc_ibl_env_brdf_texel(x, y, w, h))


def cull_meshlets(meshlets: np.ndarray, count: int, proj, view, model, prev_view, frame_w, frame_h,
                  depth_map: Texture | None = None):
    bitmap = np.zeros((count + 15) // 16, dtype=np.uint16)
    mats = [np.ascontiguousarray(m, dtype=np.float32).reshape(16) for m in (proj, view, model, prev_view)]
    n = lib().orc_cull_meshlets(_fptr(bitmap), meshlets.ctypes.data_as(C.c_void_p), count,
                                *[_fptr(m) for m in mats], float(frame_w), float(frame_h),
                                C.cast(C.byref(depth_map.s), C.c_void_p) if depth_map is not None else None)
    return bitmap, int(n)


def downsample_depth(fb: Framebuffer, dest: Texture):
    lib().orc_downsample_depth(C.byref(fb.s), C.byref(dest.s))


def resolve(fb: Framebuffer, ctx: Context, threads: int = 1):
    if threads > 1:
        lib().orc_resolve_mt(C.byref(fb.s), C.byref(ctx.s), C.c_uint32(threads))
    else:
        lib().orc_resolve(C.byref(fb.s), C.byref(ctx.s))


def resolve_debug(fb: Framebuffer, ctx: Context, layer: int, threads: int = 1):
    """ShadingContext::ResolveDebug (Shading.cpp:734-773), layer as DebugLayer (Shading.h:8)."""
    lib().orc_resolve_debug_mt(C.byref(fb.s), C.byref(ctx.s), C.c_uint32(layer), C.c_uint32(threads))


def set_approx_mode(mode: int) -> bool:
    """simd::approx_rcp/approx_rsqrt: 0 = exact tables (default), 1 = the AVX-512 instructions
    (x86 hosts with AVX-512 only), 2 = correctly rounded IEEE 1/x and 1/sqrt(x)."""
    if not lib().orc_approx_mode_available(mode):
        return False
    lib().orc_set_approx_mode(mode)
    return True


def approx14_mismatches(which: int, first: int, count: int) -> int:
    """Inputs in [first, first + count) where the tables differ from VRCP14PS (which=0) or
    VRSQRT14PS (which=1); -1 without AVX-512."""
    return int(lib().orc_approx14_mismatches(which, first, count))


def approx_eval(which: int, x: np.ndarray) -> np.ndarray:
    """approx_rcp (which=0) / approx_rsqrt (which=1) of a float32 array in the current mode."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    out = np.empty_like(a)
    lib().orc_approx_eval(C.c_int(which), a.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p),
                          C.c_uint64(a.size))
    return out.view(np.float32)


def hiz_texture_size(width: int, height: int) -> tuple[int, int]:
    """Hi-Z texture dimensions used by the reference frame driver (Main.cpp:54-56)."""
    def half(v):
        x = (v - 1) // 2
        return 1 << (x.bit_length())
    return half(width), half(height)


__all__ = ["Framebuffer", "Texture", "Context", "draw_meshlets", "cull_meshlets", "downsample_depth",
           "resolve", "resolve_debug", "set_approx_mode", "approx14_mismatches", "approx_eval", "hiz_texture_size", "lib", "SHADER_VISBUFFER",
           "SHADER_OVERDRAW"]
_ = os
