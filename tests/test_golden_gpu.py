"""The CUDA path against the committed golden fixtures (tests/golden/): vis-buffers bit-exact in
every mode, resolved colour within 1/255, Hi-Z texels and cull bitmaps bit-exact."""
import os

import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.golden import make_golden as G
from tests.helpers import GpuRenderer, TexturePair, default_lights, gpu_lights

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
W, H = G.W, G.H


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def check_hash(gold, *arrays):
    assert G.scene_hash(*arrays) == str(gold["scene_hash"]), "scene generator differs on this platform"


def test_grid_matches_golden():
    gold = load("raster_grid")
    sc = G.grid_scene()
    v = sc.views[0]
    check_hash(gold, sc.meshlets, sc.materials, v.world_to_clip)
    g = GpuRenderer(sc.meshlets, sc.materials)
    for name, binning in (("binned", True), ("unbinned", False)):
        fb, counters = g.render(v.world_to_clip, W, H, binning=binning)
        assert np.array_equal(fb.get_pixels(0), gold[f"{name}_ids"]), name
        assert np.array_equal(fb.get_pixels(1), gold[f"{name}_depth"]), name
        assert list(counters[:3]) == list(gold[f"{name}_counters"]), name


def test_inside_matches_golden():
    gold = load("raster_inside")
    sc, mats, view = G.inside_scene()
    check_hash(gold, sc.meshlets, mats, view.world_to_clip)
    g = GpuRenderer(sc.meshlets, mats)
    for name, (binning, clipping, guardband) in (("clip", (False, True, True)), ("noguard", (False, True, False)),
                                                 ("binned", (True, True, True))):
        fb, counters = g.render(view.world_to_clip, W, H, binning=binning, clipping=clipping, guardband=guardband)
        assert np.array_equal(fb.get_pixels(0), gold[f"{name}_ids"]), name
        assert np.array_equal(fb.get_pixels(1), gold[f"{name}_depth"]), name
        assert list(counters[:3]) == list(gold[f"{name}_counters"]), name


def test_resolve_hiz_cull_match_golden():
    import torch
    from glimpsw_gb300 import api
    gold = load("resolve_volume")
    sc = G.resolve_scene()
    v0, v1 = sc.views
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], sc.texture_size) for i in range(4)]
    env = TexturePair([scenes.env_map_r11g11b10(32, 5)], 32, fmt=1)
    check_hash(gold, sc.meshlets, sc.materials, v0.world_to_clip, v1.world_to_clip, *[t.o.data for t in texs], env.o.data)
    g = GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])
    fb, _ = g.render(v0.world_to_clip, W, H)
    hw, hh = api.hiz_texture_size(W, H)
    hiz = api.Texture2D(api.FORMAT_R32F, hw, hh, 16, 1)
    hiz.set_data(np.full(hiz.words, 0x7F7FFFFE, np.uint32))
    api.downsample_depth(fb, hiz)
    assert np.array_equal(hiz.get_data()[: gold["hiz"].size], gold["hiz"])
    n = len(sc.meshlets)
    bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
    visible = api.cull_meshlets(g.scene, 0, n, bm, v1.proj, v1.view, scenes.IDENTITY, v0.view, W, H, hiz, want_count=True)
    assert np.array_equal(bm.cpu().numpy().view(np.uint16), gold["cull_bitmap"])
    assert visible == int(gold["cull_visible"])
    ctx = api.ShadingContext(g.scene, v0.world_to_clip, world_to_clip=v0.world_to_clip, skybox=env.g, view_pos=v0.eye,
                             lights=gpu_lights(default_lights()))
    ctx.resolve(g.rast, fb)
    a = fb.get_pixels(0).view(np.uint8).astype(np.int32)
    b = gold["color"].view(np.uint8).astype(np.int32)
    assert np.abs(a - b).max() <= 1


def test_alpha_overdraw_debug_match_golden():
    from glimpsw_gb300 import api
    gold = load("alpha_debug")
    sc, view = G.alpha_scene()
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], sc.texture_size) for i in range(4)]
    check_hash(gold, sc.meshlets, sc.materials, view.world_to_clip, *[t.o.data for t in texs])
    g = GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])
    fb, counters = g.render(view.world_to_clip, W, H)
    assert np.array_equal(fb.get_pixels(0), gold["alpha_ids"])
    assert np.array_equal(fb.get_pixels(1), gold["alpha_depth"])
    assert list(counters[:3]) == list(gold["alpha_counters"])
    ctx = api.ShadingContext(g.scene, view.world_to_clip)
    for layer in (1, 4):
        fb, _ = g.render(view.world_to_clip, W, H)
        ctx.resolve_debug(g.rast, fb, layer)
        assert np.array_equal(fb.get_pixels(0), gold[f"debug{layer}"]), layer
    fb, _ = g.render(view.world_to_clip, W, H, clear=(0, 0.0), shader=api.OverdrawShader)
    assert np.array_equal(fb.get_pixels(0), gold["overdraw_counts"])
    assert np.array_equal(fb.get_pixels(1), gold["overdraw_depth"])
    ctx.resolve_debug(g.rast, fb, 7)
    assert np.array_equal(fb.get_pixels(0), gold["debug7"])
