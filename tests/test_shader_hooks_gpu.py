"""The shader hooks (include/swr/shader.cuh) and the DeferredShader built on them, against the oracle.

* A user fragment shader (tests/user_shader/hook_shaders.cu, compiled with nvcc into its own library
  as a user would) writes the surface id and the bits of the perspective-correct interpolated
  texcoords; the oracle's DrawTriangle computes the same per fragment in draw order
  (Rasterizer.h:287-323, rcp14 + Newton step, clip remap). Layers 0-3 must be bit-identical: on the
  small plain-path construction, and from a camera inside a volume, where triangles are clipped
  (their barycentrics go through TriangleClipData).
* A user mesh shader (its own transform, culling by PrimCount 0, per-meshlet cull mode and
  FragmentShaderId selecting between two fragment entry points) against the oracle given the
  equivalent inputs (a cull bitmap, double-sided materials).
* SWR_SHADER_DEFERRED (FS_EncodeGBuffer, Shading.cpp:344-414): depth, base colour and packed
  normal / metal / roughness bit-identical to the oracle, with alpha-tested and opaque two-layer
  materials, from outside and inside the volume.
"""
import ctypes as C

import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import TexturePair, render_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hooks():
    from glimpsw_gb300 import api
    from tests.user_shader import build
    api.load_library()
    lib = C.CDLL(build.build())
    for name in ("hook_draw_texcoords", "hook_draw_custom_mesh"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        getattr(lib, name).restype = C.c_int
    return lib


def _layers(fb, n):
    return [fb.get_pixels(k) for k in range(n)]


def _assert_layers_equal(got, exp, names):
    for g, e, name in zip(got, exp, names):
        bad = np.argwhere(g != e)
        if len(bad):
            y, x = bad[0]
            raise AssertionError(f"{name}: {len(bad)} pixels differ; first at (x={x}, y={y}): gpu {g[y, x]:#010x} "
                                 f"oracle {e[y, x]:#010x}")


def _gpu_hook_draw(fn, scene, rast, view, w, h, count, binning=False):
    from glimpsw_gb300 import api
    fb = api.Framebuffer(w, h, 4)
    fb.clear(0xFF000000, 0.0)
    fb.clear_layer(2, 0)
    fb.clear_layer(3, 0)
    rast.EnableBinning = binning
    ctx = api.ShadingContext(scene, view.world_to_clip)
    st = fn(rast.h, fb.h, count, C.byref(ctx.s))
    assert st == api.SWR_OK, api._lib.swr_last_error().decode()
    return fb


def _oracle_texcoords(meshlets, mats, view, w, h, binning=False, cull_bitmap=None):
    from oracle import oracle as O
    ofb = O.Framebuffer(w, h, 4)
    ofb.clear(0xFF000000, 0.0)
    ofb.clear_layer(2, 0)
    ofb.clear_layer(3, 0)
    render_oracle(meshlets, mats, view.world_to_clip, w, h, binning=binning, fb=ofb, shader=O.SHADER_TEXCOORD,
                  cull_bitmap=cull_bitmap)
    return ofb


@pytest.mark.parametrize("which", ["grid", "inside"])
def test_user_fragment_shader_barycentrics_bit_exact(hooks, which):
    from glimpsw_gb300 import api
    if which == "grid":
        sc = scenes.grid_scene(n_side=32, width=640, height=360)
        view, mats = sc.views[0], sc.materials
    else:
        sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=8, env_size=8)
        view = scenes.make_view(480, 272, eye=np.zeros(3), target=(0.3, 0.1, 1.0))
        mats = sc.materials.copy()
        mats["is_double_sided"][::2] = 1
    w, h, n = view.width, view.height, len(sc.meshlets)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(mats)
    rast = api.Rasterizer()
    rast.reset_counters()
    fb = _gpu_hook_draw(hooks.hook_draw_texcoords, scene, rast, view, w, h, n)
    ofb = _oracle_texcoords(sc.meshlets, mats, view, w, h)
    got, exp = _layers(fb, 4), _layers(ofb, 4)
    _assert_layers_equal(got, exp, ["surface id", "depth", "u bits", "v bits"])
    covered = exp[1] != 0
    assert covered.sum() > 5000 and len(np.unique(exp[2][covered])) > 1000
    if which == "inside":
        assert rast.counters()[2] > 0  # clipped triangles were drawn and shaded


def test_user_mesh_shader_bit_exact(hooks):
    """CustomMesh: its own transform (here the view's), PrimCount 0 for meshlets 4 mod 5, double-sided
    for 0 mod 3, FragmentShaderId idx & 1 (entry point 1 sets bit 30 of the surface id)."""
    from glimpsw_gb300 import api
    sc = scenes.grid_scene(n_side=32, width=640, height=360)
    view = sc.views[0]
    w, h, n = view.width, view.height, len(sc.meshlets)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials)
    rast = api.Rasterizer()
    fb = _gpu_hook_draw(hooks.hook_draw_custom_mesh, scene, rast, view, w, h, n)
    # the oracle with equivalent inputs: material 0 single-sided, 1 double-sided; a cull bitmap
    om = sc.meshlets.copy()
    idx = np.arange(n)
    om["MaterialId"] = np.where(idx % 3 == 0, 1, 0)
    omats = np.zeros(2, dtype=scenes.MATERIAL_DTYPE)
    omats["alpha_cutoff"] = 255
    omats["is_double_sided"] = [0, 1]
    keep = (idx % 5 != 4).astype(np.uint8)
    bm = np.packbits(np.concatenate([keep, np.zeros((-n) % 16, np.uint8)]), bitorder="little").view(np.uint16)
    ofb = _oracle_texcoords(om, omats, view, w, h, cull_bitmap=bm)
    exp = _layers(ofb, 4)
    ids = exp[0]
    shown = exp[1] != 0
    meshlet = np.where(shown, ids // 128, 0)
    exp[0] = np.where(shown & (meshlet % 2 == 1), ids | 0x40000000, ids)
    _assert_layers_equal(_layers(fb, 4), exp, ["surface id", "depth", "u bits", "v bits"])
    assert shown.sum() > 5000 and len(np.unique(meshlet[shown])) > 300
    assert np.any(shown & (meshlet % 3 == 0)) and not np.any(shown & (meshlet % 5 == 4))


@pytest.fixture(scope="module")
def deferred_scene():
    from glimpsw_gb300 import api
    api.load_library()
    sc = scenes.volume_scene(n=6000, width=640, height=360, n_materials=4, extent=40.0, texture_size=256, env_size=8,
                             alpha_every=2, alpha_cutoff=128)
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], 256) for i in range(4)]
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials, [t.g for t in texs])
    return sc, texs, scene


@pytest.mark.parametrize("camera", ["outside", "inside"])
def test_deferred_shader_gbuffer_bit_exact(deferred_scene, camera):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, scene = deferred_scene
    if camera == "outside":
        view = sc.views[0]
    else:
        view = scenes.make_view(640, 360, eye=(2.0, 1.0, -3.0), target=(0.0, 0.0, 20.0))
    w, h, n = view.width, view.height, len(sc.meshlets)
    rot = np.array([0.8, 0.6, 0.0, -0.6, 0.8, 0.0, 0.0, 0.0, 1.0], np.float32)  # ObjectToWorldMat
    rast = api.Rasterizer()
    rast.EnableBinning = False
    rast.reset_counters()
    fb = api.Framebuffer(w, h, 3)
    fb.clear(0xFF000000, 0.0)
    fb.clear_layer(2, 0)
    ctx = api.ShadingContext(scene, view.world_to_clip, object_to_world=rot.reshape(3, 3))
    rast.draw_meshlets(fb, n, ctx, api.SHADER_DEFERRED)
    ofb = O.Framebuffer(w, h, 3)
    ofb.clear(0xFF000000, 0.0)
    ofb.clear_layer(2, 0)
    octx = O.Context(sc.meshlets, sc.materials, view.world_to_clip, textures=[t.o for t in texs],
                     object_to_world=rot.reshape(3, 3))
    O.draw_meshlets(ofb, octx, n, shader=O.SHADER_DEFERRED)
    got, exp = _layers(fb, 3), _layers(ofb, 3)
    _assert_layers_equal(got, exp, ["base colour", "depth", "normal/metal/rough"])
    shown = exp[1] != 0
    assert shown.sum() > 20000 and np.count_nonzero(exp[2][shown]) > 0.9 * shown.sum()
    # alpha-tested materials cut holes: some pixels show the surface behind an alpha-tested one
    mats_shown = np.unique(exp[0][shown] >> 24)
    assert len(mats_shown) > 1
    if camera == "inside":
        assert rast.counters()[2] > 0
