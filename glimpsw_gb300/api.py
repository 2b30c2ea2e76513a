"""Python mirror of GLimpSW's renderer API over the C ABI of libswr_gb300.so (ctypes).

Names follow the reference: ``Rasterizer`` (src/SwRast/Rasterizer.h:202-340), ``Framebuffer`` /
``create_framebuffer`` (Rasterizer.h:10-78), ``Texture2D`` / ``create_texture2d`` (Texture.h:314-636),
``ShadingContext`` (Shading.h:12-50) with ``cull_meshlets``, ``resolve`` and ``VisBufferShader``,
and ``downsample_depth`` (Texture.h:243). Errors raise ``SwrError`` carrying the status code and
``swr_last_error()``. The CUDA library is required: importing this module on a machine without
it raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libswr_gb300.so")

SWR_OK, SWR_EINVAL, SWR_ECAPACITY, SWR_ETIMEOUT, SWR_ECUDA, SWR_ENOMEM = range(6)
STATUS_NAMES = {0: "SWR_OK", 1: "SWR_EINVAL", 2: "SWR_ECAPACITY", 3: "SWR_ETIMEOUT", 4: "SWR_ECUDA", 5: "SWR_ENOMEM"}
FORMAT_RGBA8U, FORMAT_R11G11B10F, FORMAT_R32F, FORMAT_RG16F = 0, 1, 2, 3
VisBufferShader = 0
DeferredShader = SHADER_DEFERRED = 1
OverdrawShader = 2
# DebugLayer (Shading.h:8) for ShadingContext.resolve_debug
(DEBUG_NONE, DEBUG_BASE_COLOR, DEBUG_NORMALS, DEBUG_METALLIC_ROUGHNESS, DEBUG_MESHLET_ID, DEBUG_TRIANGLE_ID,
 DEBUG_OVERDRAW_PIXEL, DEBUG_OVERDRAW_QUAD) = range(8)
MAX_RENDER_SIZE = 2896


class SwrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class SwrMaterial(C.Structure):
    _fields_ = [("texture", C.c_void_p), ("is_double_sided", C.c_uint8), ("alpha_cutoff", C.c_uint8)]


class SwrLight(C.Structure):
    _fields_ = [("type", C.c_uint32), ("position", C.c_float * 3), ("direction", C.c_float * 3),
                ("color", C.c_float * 3), ("intensity", C.c_float), ("radius", C.c_float),
                ("spot_inner_angle", C.c_float), ("spot_outer_angle", C.c_float), ("inv_radius_sq", C.c_float),
                ("spot_scale", C.c_float), ("spot_offset", C.c_float)]


class SwrMeshDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("texcoords", C.c_void_p), ("normal_tangents", C.c_void_p),
                ("tangent_signs", C.c_void_p), ("num_vertices", C.c_uint32), ("indices", C.c_void_p),
                ("num_triangles", C.c_uint32), ("material_id", C.c_uint32), ("alpha_cutoff", C.c_uint8)]


class SwrShadingContext(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("meshlet_offset", C.c_uint32), ("cull_bitmap", C.c_void_p),
                ("world_to_clip", C.c_float * 16), ("object_to_clip", C.c_float * 16),
                ("object_to_world", C.c_float * 9), ("skybox", C.c_void_p), ("view_pos", C.c_float * 3),
                ("exposure", C.c_float), ("lights", C.c_void_p), ("num_lights", C.c_uint32)]


_lib = None

# name -> argtypes (all return swr_status unless listed in _RESTYPES)
_SIGS = {
    "swr_last_error": [],
    "swr_set_stream": [C.c_void_p],
    "swr_get_stream": [],
    "swr_synchronize": [],
    "swr_launch_count": [],
    "swr_profile_enable": [C.c_int],
    "swr_profile_collect": [C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_rasterizer_create": [C.c_uint32, C.c_void_p],
    "swr_rasterizer_destroy": [C.c_void_p],
    "swr_rasterizer_set_flags": [C.c_void_p, C.c_int, C.c_int, C.c_int],
    "swr_rasterizer_get_counters": [C.c_void_p, C.c_void_p],
    "swr_rasterizer_set_queue_capacity": [C.c_void_p, C.c_uint32],
    "swr_rasterizer_reset_counters": [C.c_void_p],
    "swr_draw_meshlets": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p],
    "swr_draw_meshlets_noalloc": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_int,
                                  C.c_int],
    "swr_framebuffer_create": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p],
    "swr_framebuffer_destroy": [C.c_void_p],
    "swr_framebuffer_clear": [C.c_void_p, C.c_uint32, C.c_float],
    "swr_framebuffer_clear_layer": [C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_framebuffer_get_pixels": [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32],
    "swr_framebuffer_get_pixels_device": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_framebuffer_layer_data": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_framebuffer_invalidate": [C.c_void_p],
    "swr_framebuffer_size": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_scene_create": [C.c_void_p],
    "swr_scene_destroy": [C.c_void_p],
    "swr_scene_upload_meshlets": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_scene_set_materials": [C.c_void_p, C.c_void_p, C.c_uint32],
    "swr_scene_meshlet_count": [C.c_void_p, C.c_void_p],
    "swr_scene_meshlets_device": [C.c_void_p, C.c_void_p],
    "swr_draw_shaded_meshlets": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p],
    "swr_draw_meshlets_hooked": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int],
    "swr_fragment_source_get": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_texture_create": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p],
    "swr_texture_destroy": [C.c_void_p],
    "swr_texture_set_pixels": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_texture_generate_mips": [C.c_void_p],
    "swr_texture_set_pixels_device": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_texture_info": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_texture_get_data": [C.c_void_p, C.c_void_p, C.c_size_t],
    "swr_texture_set_data": [C.c_void_p, C.c_void_p, C.c_size_t],
    "swr_cull_meshlets": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                          C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p],
    "swr_cull_meshlets_ex": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_uint32],
    "swr_downsample_depth": [C.c_void_p, C.c_void_p],
    "swr_ibl_irradiance_map": [C.c_void_p, C.c_void_p],
    "swr_ibl_radiance_map": [C.c_void_p, C.c_void_p],
    "swr_ibl_env_brdf_lut": [C.c_void_p],
    "swr_resolve": [C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_resolve_debug": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32],
    "swr_batch_create": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p],
    "swr_batch_set_views": [C.c_void_p, C.c_void_p, C.c_uint32],
    "swr_batch_set_tuning": [C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_batch_set_chunk_shape": [C.c_void_p, C.c_uint32, C.c_uint32],
    "swr_batch_render": [C.c_void_p],
    "swr_batch_get_counters": [C.c_void_p, C.c_void_p],
    "swr_batch_reset_counters": [C.c_void_p],
    "swr_batch_destroy": [C.c_void_p],
    "swr_neural_create": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p],
    "swr_neural_destroy": [C.c_void_p],
    "swr_neural_get_info": [C.c_void_p, C.c_void_p],
    "swr_neural_train": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_void_p],
    "swr_neural_gradients": [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_neural_get_params": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_neural_set_params": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_neural_get_latents": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_neural_set_latents": [C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_neural_decode": [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p],
    "swr_resolve_neural": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "swr_neural_set_wait_limit": [C.c_void_p, C.c_uint64],
    "swr_neural_save": [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p],
    "swr_neural_load": [C.c_void_p, C.c_void_p, C.c_size_t],
    "swr_selftest_bounded_wait": [C.c_uint64],
    "swr_meshlet_bound": [C.c_uint32],
    "swr_build_meshlets": [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p],
}


class SwrViewDesc(C.Structure):
    _fields_ = [("fb", C.c_void_p), ("proj", C.c_float * 16), ("view", C.c_float * 16), ("model", C.c_float * 16),
                ("depth_only", C.c_uint32)]
_RESTYPES = {"swr_last_error": C.c_char_p, "swr_get_stream": C.c_void_p, "swr_launch_count": C.c_uint64,
             "swr_meshlet_bound": C.c_uint32}


def load_library(path: str = LIB_PATH):
    """Loads libswr_gb300.so (building it with nvcc first if it is missing). Raises if the CUDA
    library cannot be built or loaded: there is no other implementation to fall back to."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    lib = C.CDLL(path)
    for name, args in _SIGS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def _check(code: int):
    if code != SWR_OK:
        raise SwrError(code, _lib.swr_last_error().decode())


def _ptr(a) -> int:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch tensor (device memory)
        return a.data_ptr()
    return int(a)


def _f16(m) -> C.Array:
    """A 4x4 float32 matrix as a ctypes array (an array made by mat4() passes through unchanged)."""
    if isinstance(m, C.Array):
        return m
    a = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
    return (C.c_float * 16)(*a.tolist())


def mat4(m) -> C.Array:
    """Converts a matrix once for repeated calls (the per-call conversion costs a few microseconds)."""
    return _f16(m)


def set_stream(stream) -> None:
    """Enqueue subsequent work on a CUDA stream (an int handle or a torch.cuda.Stream)."""
    h = getattr(stream, "cuda_stream", stream)
    _check(load_library().swr_set_stream(h))


def synchronize() -> None:
    _check(load_library().swr_synchronize())


def launch_count() -> int:
    """Kernels this library has launched so far (all threads)."""
    return int(load_library().swr_launch_count())


def profile_enable(on: bool = True) -> None:
    _check(load_library().swr_profile_enable(int(on)))


def profile_collect(max_records: int = 4096) -> list[tuple[str, float]]:
    """(kernel name, ms) of every launch recorded since the last collect (synchronises)."""
    names = (C.c_char_p * max_records)()
    ms = (C.c_float * max_records)()
    n = C.c_uint32()
    _check(load_library().swr_profile_collect(max_records, names, ms, C.byref(n)))
    return [(names[i].decode(), float(ms[i])) for i in range(min(n.value, max_records))]


class Framebuffer:
    def __init__(self, width: int, height: int, num_layers: int = 2):
        L = load_library()
        h = C.c_void_p()
        _check(L.swr_framebuffer_create(width, height, num_layers, C.byref(h)))
        self.h = h
        self.width, self.height, self.num_layers = width, height, num_layers

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_framebuffer_destroy(self.h)
            self.h = None

    def clear(self, color: int, depth: float) -> None:
        _check(_lib.swr_framebuffer_clear(self.h, C.c_uint32(color), C.c_float(depth)))

    def clear_layer(self, layer: int, value: int) -> None:
        _check(_lib.swr_framebuffer_clear_layer(self.h, layer, C.c_uint32(value)))

    def get_pixels(self, layer: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width), dtype=np.uint32)
        _check(_lib.swr_framebuffer_get_pixels(self.h, layer, out.ctypes.data, out.shape[1]))
        return out

    def get_pixels_device(self, layer: int, dest_device) -> None:
        _check(_lib.swr_framebuffer_get_pixels_device(self.h, layer, _ptr(dest_device)))

    def layer_data(self, layer: int) -> int:
        p = C.c_void_p()
        _check(_lib.swr_framebuffer_layer_data(self.h, layer, C.byref(p)))
        return p.value

    def invalidate(self) -> None:
        _check(_lib.swr_framebuffer_invalidate(self.h))


def create_framebuffer(width: int, height: int, num_layers: int = 2) -> Framebuffer:
    return Framebuffer(width, height, num_layers)


class Texture2D:
    def __init__(self, fmt: int, width: int, height: int, max_levels: int = 1, num_layers: int = 1):
        L = load_library()
        h = C.c_void_p()
        _check(L.swr_texture_create(fmt, width, height, max_levels, num_layers, C.byref(h)))
        self.h = h
        self.fmt, self.width, self.height, self.num_layers = fmt, width, height, num_layers
        levels, stride = C.c_uint32(), C.c_uint32()
        offs = (C.c_uint32 * 16)()
        _check(L.swr_texture_info(self.h, C.byref(levels), C.byref(stride), offs))
        self.mip_levels, self.layer_stride, self.mip_offsets = levels.value, stride.value, list(offs)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_texture_destroy(self.h)
            self.h = None

    @property
    def words(self) -> int:
        return self.layer_stride * self.num_layers + 64

    def set_pixels(self, pixels: np.ndarray, layer: int = 0) -> None:
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        _check(_lib.swr_texture_set_pixels(self.h, pixels.ctypes.data, pixels.shape[1], layer))

    def set_pixels_device(self, pixels, layer: int = 0) -> None:
        """Row-major texels already on the device (e.g. a torch int32 tensor of shape (h, w))."""
        _check(_lib.swr_texture_set_pixels_device(self.h, _ptr(pixels), self.width, layer))

    def generate_mips(self) -> None:
        _check(_lib.swr_texture_generate_mips(self.h))

    def get_data(self) -> np.ndarray:
        out = np.empty(self.words, dtype=np.uint32)
        _check(_lib.swr_texture_get_data(self.h, out.ctypes.data, out.size))
        return out

    def set_data(self, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data, dtype=np.uint32)
        _check(_lib.swr_texture_set_data(self.h, data.ctypes.data, data.size))


def create_texture2d(fmt: int, width: int, height: int, max_levels: int = 1, num_layers: int = 1) -> Texture2D:
    return Texture2D(fmt, width, height, max_levels, num_layers)


class Scene:
    """Device-resident Meshlet and Material pools (Scene.h:117-128)."""

    def __init__(self):
        L = load_library()
        h = C.c_void_p()
        _check(L.swr_scene_create(C.byref(h)))
        self.h = h
        self.textures = []

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_scene_destroy(self.h)
            self.h = None

    def upload_meshlets(self, meshlets: np.ndarray, first: int = 0) -> None:
        assert meshlets.dtype.itemsize == 1728 and meshlets.flags.c_contiguous
        _check(_lib.swr_scene_upload_meshlets(self.h, meshlets.ctypes.data, first, len(meshlets)))

    def set_materials(self, materials: np.ndarray, textures: list | None = None) -> None:
        self.textures = list(textures or [])
        arr = (SwrMaterial * max(1, len(materials)))()
        for i, m in enumerate(materials):
            t = int(m["texture"])
            arr[i].texture = self.textures[t].h.value if self.textures and t < len(self.textures) else None
            arr[i].is_double_sided = int(m["is_double_sided"])
            arr[i].alpha_cutoff = int(m["alpha_cutoff"])
        _check(_lib.swr_scene_set_materials(self.h, arr, len(materials)))


class ShadingContext:
    """ShadingContext (Shading.h:12-50) bound to a device Scene."""

    VisBufferShader = VisBufferShader
    DeferredShader = DeferredShader
    OverdrawShader = OverdrawShader

    def __init__(self, scene: Scene, object_to_clip, world_to_clip=None, object_to_world=None,
                 meshlet_offset: int = 0, cull_bitmap=None, skybox: Texture2D | None = None, view_pos=(0, 0, 0),
                 exposure: float = 1.0, lights: list | None = None):
        s = SwrShadingContext()
        s.scene = scene.h.value
        s.meshlet_offset = meshlet_offset
        s.cull_bitmap = _ptr(cull_bitmap)
        s.object_to_clip = _f16(object_to_clip)
        s.world_to_clip = _f16(world_to_clip if world_to_clip is not None else object_to_clip)
        ow = np.ascontiguousarray(object_to_world if object_to_world is not None else np.eye(3), dtype=np.float32)
        s.object_to_world = (C.c_float * 9)(*ow.reshape(9).tolist())
        s.skybox = skybox.h.value if skybox is not None else None
        s.view_pos = (C.c_float * 3)(*[float(v) for v in view_pos])
        s.exposure = exposure
        self._lights = (SwrLight * max(1, len(lights or [])))(*(lights or []))
        s.lights = C.cast(self._lights, C.c_void_p) if lights else None
        s.num_lights = len(lights or [])
        self.s = s
        self.scene = scene
        self._keep = (cull_bitmap, skybox)

    def resolve(self, rast: "Rasterizer", fb: Framebuffer) -> None:
        _check(_lib.swr_resolve(rast.h, fb.h, C.byref(self.s)))

    def resolve_debug(self, rast: "Rasterizer", fb: Framebuffer, layer: int) -> None:
        """ShadingContext::ResolveDebug (Shading.cpp:734-773); layer is a DEBUG_* value."""
        _check(_lib.swr_resolve_debug(rast.h, fb.h, C.byref(self.s), layer))

    def resolve_neural(self, rast: "Rasterizer", fb: Framebuffer, model: "NeuralMaterials",
                       want_stats: bool = False):
        """resolve() with the texture levels the model covers decoded by its network; returns
        (texels decoded, 128-texel tiles) when want_stats (synchronises)."""
        st = SwrNeuralStats()
        _check(_lib.swr_resolve_neural(rast.h, fb.h, C.byref(self.s), model.h, C.byref(st) if want_stats else None))
        return (st.requests, st.tiles, list(st.level_texels)) if want_stats else None


CULL_FRUSTUM = 1
CULL_BACKFACE_CONE = 2


def cull_meshlets(scene: Scene, first: int, count: int, bitmap_device, proj, view, model, prev_view,
                  frame_w: float, frame_h: float, depth_map: Texture2D | None = None, want_count: bool = False,
                  cone: bool = False):
    """ShadingContext::CullMeshlets (Shading.cpp:775-869) into a device bitmap (uint16 per 16); with
    cone, meshlets facing away from the camera as a whole are dropped too (swr_cull_meshlets_ex)."""
    cnt = C.c_uint32(0)
    _check(_lib.swr_cull_meshlets_ex(scene.h, first, count, _ptr(bitmap_device), _f16(proj), _f16(view), _f16(model),
                                     _f16(prev_view), float(frame_w), float(frame_h),
                                     depth_map.h if depth_map is not None else None,
                                     C.byref(cnt) if want_count else None, CULL_BACKFACE_CONE if cone else 0))
    return cnt.value if want_count else None


def downsample_depth(fb: Framebuffer, dest: Texture2D) -> None:
    _check(_lib.swr_downsample_depth(fb.h, dest.h))


def hiz_texture_size(width: int, height: int) -> tuple[int, int]:
    """Hi-Z texture size the reference frame driver allocates for a frame (Main.cpp:54-56): each
    dimension is the power of two at or above half the frame's."""
    def half(v):
        return 1 << ((v - 1) // 2).bit_length()
    return half(width), half(height)


class Batch:
    """Batched multi-view rendering (swr_batch_*): many framebuffers, one CUDA graph per frame.

    views: list of (Framebuffer, proj, view, model, depth_only)."""

    def __init__(self, rast: "Rasterizer", scene: Scene, views, first: int = 0, count: int | None = None,
                 frustum_cull: bool = True, cone: bool = False):
        L = load_library()
        if count is None:
            c = C.c_uint32()
            _check(L.swr_scene_meshlet_count(scene.h, C.byref(c)))
            count = c.value - first
        self._views = list(views)
        arr = self._descs(self._views)
        h = C.c_void_p()
        flags = (CULL_FRUSTUM if frustum_cull else 0) | (CULL_BACKFACE_CONE if cone else 0)
        _check(L.swr_batch_create(rast.h, scene.h, first, count, arr, len(self._views), flags, C.byref(h)))
        self.h = h
        self.count, self.rast, self.scene = count, rast, scene

    @staticmethod
    def _descs(views):
        arr = (SwrViewDesc * len(views))()
        for i, (fb, proj, view, model, depth_only) in enumerate(views):
            arr[i].fb = fb.h.value
            arr[i].proj, arr[i].view, arr[i].model = _f16(proj), _f16(view), _f16(model)
            arr[i].depth_only = int(depth_only)
        return arr

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_batch_destroy(self.h)
            self.h = None

    def set_views(self, views) -> None:
        self._views = list(views)
        _check(_lib.swr_batch_set_views(self.h, self._descs(self._views), len(self._views)))

    def set_tuning(self, chunk_tiles: int = 0, warps_per_block: int = 0) -> None:
        _check(_lib.swr_batch_set_tuning(self.h, chunk_tiles, warps_per_block))

    def set_chunk_shape(self, width_tiles: int, height_tiles: int) -> None:
        """Rectangular chunks of width_tiles x height_tiles 4x4 tiles (after set_tuning)."""
        _check(_lib.swr_batch_set_chunk_shape(self.h, width_tiles, height_tiles))

    def render(self) -> None:
        _check(_lib.swr_batch_render(self.h))

    def counters(self) -> np.ndarray:
        out = np.zeros(4, dtype=np.uint64)
        _check(_lib.swr_batch_get_counters(self.h, out.ctypes.data))
        return out

    def reset_counters(self) -> None:
        _check(_lib.swr_batch_reset_counters(self.h))


class Rasterizer:
    def __init__(self, num_threads: int = 0):
        L = load_library()
        h = C.c_void_p()
        _check(L.swr_rasterizer_create(num_threads, C.byref(h)))
        self.h = h
        self._flags = [True, True, True]
        self._apply()

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_rasterizer_destroy(self.h)
            self.h = None

    def _apply(self):
        _check(_lib.swr_rasterizer_set_flags(self.h, *[int(f) for f in self._flags]))

    @property
    def EnableBinning(self):
        return self._flags[0]

    @EnableBinning.setter
    def EnableBinning(self, v):
        self._flags[0] = bool(v)
        self._apply()

    @property
    def EnableClipping(self):
        return self._flags[1]

    @EnableClipping.setter
    def EnableClipping(self, v):
        self._flags[1] = bool(v)
        self._apply()

    @property
    def EnableGuardband(self):
        return self._flags[2]

    @EnableGuardband.setter
    def EnableGuardband(self, v):
        self._flags[2] = bool(v)
        self._apply()

    def draw_meshlets(self, fb: Framebuffer, count: int, ctx: ShadingContext, shader: int = VisBufferShader) -> None:
        _check(_lib.swr_draw_meshlets(self.h, fb.h, count, shader, C.byref(ctx.s)))

    def set_queue_capacity(self, triangles: int) -> None:
        _check(_lib.swr_rasterizer_set_queue_capacity(self.h, triangles))

    def counters(self) -> np.ndarray:
        out = np.zeros(4, dtype=np.uint64)
        _check(_lib.swr_rasterizer_get_counters(self.h, out.ctypes.data))
        return out

    def reset_counters(self) -> None:
        _check(_lib.swr_rasterizer_reset_counters(self.h))


# ---------------------------------------------------------------- learned texture decoder
NEURAL_PARAMS = 5704


class SwrNeuralInfo(C.Structure):
    _fields_ = [("num_materials", C.c_uint32), ("latent_levels", C.c_uint32), ("texels_per_material", C.c_uint32),
                ("level_offset", C.c_uint32 * 4), ("level_width", C.c_uint32 * 4), ("level_height", C.c_uint32 * 4),
                ("latent_bytes", C.c_uint64), ("weight_bytes", C.c_uint64), ("fallback_bytes", C.c_uint64),
                ("plain_bytes", C.c_uint64)]


class SwrNeuralStats(C.Structure):
    _fields_ = [("requests", C.c_uint32), ("tiles", C.c_uint32), ("level_texels", C.c_uint32 * 6)]


def pack_texel(level, x, y):
    """Packed texel address used by the decoder entry points: level<<28 | y<<14 | x."""
    return (np.asarray(level, dtype=np.uint32) << 28) | (np.asarray(y, dtype=np.uint32) << 14) | np.asarray(x, dtype=np.uint32)


class NeuralMaterials:
    """Learned texture decoder over a set of material textures (no counterpart in the reference):
    per material an FP16 latent pyramid (8 channels; latent level k has texture level k+2's size)
    and an 11->64->64->8 GELU MLP (latents, bias, level-0/1 flags) decoding texture levels
    0..latent_levels+1, trained on the device by tensor-core kernels."""

    def __init__(self, textures: list, latent_levels: int = 4, seed: int = 1):
        L = load_library()
        arr = (C.c_void_p * len(textures))(*[t.h.value if t is not None else None for t in textures])
        h = C.c_void_p()
        _check(L.swr_neural_create(arr, len(textures), latent_levels, C.c_uint64(seed), C.byref(h)))
        self.h = h
        self._textures = list(textures)
        info = SwrNeuralInfo()
        _check(L.swr_neural_get_info(h, C.byref(info)))
        self.info = info
        self.num_materials = info.num_materials
        self.latent_levels = info.latent_levels
        self.texels_per_material = info.texels_per_material
        self.level_offset = list(info.level_offset)[:latent_levels]
        self.level_size = [(info.level_width[l], info.level_height[l]) for l in range(latent_levels)]

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.swr_neural_destroy(self.h)
            self.h = None

    def memory(self) -> dict:
        i = self.info
        return {"latent_bytes": i.latent_bytes, "weight_bytes": i.weight_bytes, "fallback_bytes": i.fallback_bytes,
                "plain_bytes": i.plain_bytes}

    def save(self) -> bytes:
        """The training checkpoint (swr_neural_save)."""
        size = C.c_size_t()
        _check(_lib.swr_neural_save(self.h, None, 0, C.byref(size)))
        buf = (C.c_uint8 * size.value)()
        _check(_lib.swr_neural_save(self.h, buf, size.value, C.byref(size)))
        return bytes(buf)

    def load(self, blob: bytes) -> None:
        """Restores a training checkpoint of a model of the same shape (swr_neural_load)."""
        buf = (C.c_uint8 * len(blob)).from_buffer_copy(blob)
        _check(_lib.swr_neural_load(self.h, buf, len(blob)))

    def set_wait_limit(self, limit_ns: int) -> None:
        """Time limit of each bounded device-side wait of the model's kernels (default 1 s)."""
        _check(_lib.swr_neural_set_wait_limit(self.h, C.c_uint64(limit_ns)))

    def train(self, steps: int, batch: int = 65536, materials_per_step: int = 8, lr: float = 1e-3,
              want_loss: bool = False, level_weighting: int = 1):
        """level_weighting w: texture level l drawn with weight 2^(w * (latent_levels+1-l)); 2 = by
        texel count, 1 = by edge length, 0 = uniform."""
        loss = C.c_float(0.0)
        _check(_lib.swr_neural_train(self.h, steps, batch, materials_per_step, level_weighting, C.c_float(lr),
                                     C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def gradients(self, material: int, samples_device, count: int, want_latent: bool = True):
        """(param_grad[5704], latent_grad[texels, 8] or None, summed squared error) for explicit samples."""
        pg = np.zeros(NEURAL_PARAMS, dtype=np.float32)
        lg = np.zeros((self.texels_per_material, 8), dtype=np.float32) if want_latent else None
        loss = C.c_float(0.0)
        _check(_lib.swr_neural_gradients(self.h, material, _ptr(samples_device), count, pg.ctypes.data,
                                         lg.ctypes.data if lg is not None else None, C.byref(loss)))
        return pg, lg, loss.value

    def get_params(self, material: int) -> np.ndarray:
        p = np.zeros(NEURAL_PARAMS, dtype=np.float32)
        _check(_lib.swr_neural_get_params(self.h, material, p.ctypes.data))
        return p

    def set_params(self, material: int, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == NEURAL_PARAMS
        _check(_lib.swr_neural_set_params(self.h, material, p.ctypes.data))

    def get_latents(self, material: int) -> np.ndarray:
        p = np.zeros((self.texels_per_material, 8), dtype=np.float32)
        _check(_lib.swr_neural_get_latents(self.h, material, p.ctypes.data))
        return p

    def set_latents(self, material: int, latents: np.ndarray) -> None:
        p = np.ascontiguousarray(latents, dtype=np.float32)
        assert p.size == self.texels_per_material * 8
        _check(_lib.swr_neural_set_latents(self.h, material, p.ctypes.data))

    def decode(self, material: int, texels_device, count: int, out_device) -> None:
        _check(_lib.swr_neural_decode(self.h, material, _ptr(texels_device), count, _ptr(out_device)))
