"""Full-size checks on the benchmark's large scene (100k meshlets, 12.4M triangles):

* the 1920x1080 vis-buffer is bit-exact against the oracle (unbinned semantics, all meshlets);
* the same frame resolved with small textures stays within 1/255 of the oracle's resolve;
* properties that hold at any size: drawing the same meshlets again changes nothing (equal keys),
  and the tile depth bounds change nothing (a draw through the entry point that keeps no bounds,
  swr_draw_meshlets_noalloc, gives the same vis-buffer at 1280x720);
* a batched draw of two views equals the two single-view draws.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import GpuRenderer, TexturePair, assert_visbuffer_equal, default_lights, gpu_lights, render_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    sc = scenes.volume_scene(n=100_000, width=1920, height=1080, texture_size=64, env_size=64)
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], 64) for i in range(len(sc.materials))]
    g = GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])
    return sc, texs, g


def test_fullsize_visbuffer_and_resolve_match_oracle(big):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, g = big
    v = sc.views[0]
    gfb, gc = g.render(v.world_to_clip, v.width, v.height)
    ofb, oc = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height)
    assert_visbuffer_equal(gfb, ofb)
    assert list(gc[:3]) == list(oc[:3]) and gc[0] == 12_400_000
    env = TexturePair([scenes.env_map_r11g11b10(64, 5)], 64, fmt=1)
    octx = O.Context(sc.meshlets, sc.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                     textures=[t.o for t in texs], lights=default_lights(), skybox=env.o, view_pos=v.eye)
    O.resolve(ofb, octx, threads=8)
    gctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, skybox=env.g, view_pos=v.eye,
                              lights=gpu_lights(default_lights()))
    gctx.resolve(g.rast, gfb)
    a = gfb.get_pixels(0).view(np.uint8).astype(np.int32)
    b = ofb.get_pixels(0).view(np.uint8).astype(np.int32)
    assert np.abs(a - b).max() <= 1


def test_redraw_is_idempotent(big):
    sc, _, g = big
    v = sc.views[0]
    fb, _ = g.render(v.world_to_clip, v.width, v.height)
    ids, depth = fb.get_pixels(0).copy(), fb.get_pixels(1).copy()
    g.render(v.world_to_clip, v.width, v.height, fb=fb)  # same meshlets again into the finished frame
    assert np.array_equal(fb.get_pixels(0), ids) and np.array_equal(fb.get_pixels(1), depth)


def test_tile_depth_bounds_change_nothing(big):
    """swr_draw_meshlets keeps per-tile depth bounds and skips hidden tiles; the allocation-free
    entry point keeps none and shades every tile: both must give the same vis-buffer."""
    import ctypes as C
    import torch
    from glimpsw_gb300 import api
    from tests.test_zz_no_alloc import detile
    sc, _, g = big
    W, H = 1280, 720
    v = scenes.make_view(W, H, eye=sc.views[0].eye, target=(0.0, 0.0, 0.0))
    fb, _ = g.render(v.world_to_clip, W, H)
    n = len(sc.meshlets)
    meshlets = torch.from_numpy(sc.meshlets.view(np.uint8).copy()).cuda()
    flags = torch.from_numpy(sc.materials["is_double_sided"].astype(np.uint8)).cuda()
    ids = torch.full((W * H,), -16777216, dtype=torch.int32, device="cuda")  # 0xFF000000
    depth = torch.zeros(W * H, dtype=torch.float32, device="cuda")
    m = (C.c_float * 16)(*np.asarray(v.world_to_clip, dtype=np.float32).tolist())
    lib = api.load_library()
    api.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        st = lib.swr_draw_meshlets_noalloc(meshlets.data_ptr(), 0, n, flags.data_ptr(), len(sc.materials), None, m,
                                           ids.data_ptr(), depth.data_ptr(), W, H, 0, 1, 1)
        assert st == api.SWR_OK, lib.swr_last_error().decode()
        torch.cuda.synchronize()
    finally:
        api.set_stream(None)
    assert np.array_equal(detile(depth.cpu().numpy().view(np.uint32), W, H), fb.get_pixels(1))
    assert np.array_equal(detile(ids.cpu().numpy().view(np.uint32), W, H), fb.get_pixels(0))


def test_batched_two_views_equal_single_view_draws(big):
    import torch
    from glimpsw_gb300 import api
    sc, _, g = big
    vs = [scenes.make_view(1280, 720, eye=sc.views[0].eye, target=(0.0, 0.0, 0.0)),
          scenes.make_view(640, 360, eye=(3.0, 2.0, -20.0), target=(0.0, 0.0, 40.0))]
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fbs = [api.Framebuffer(v.width, v.height) for v in vs]
    batch = api.Batch(rast, g.scene, [(fb, v.proj, v.view, scenes.IDENTITY, False) for fb, v in zip(fbs, vs)])
    batch.render()
    n = len(sc.meshlets)
    for fb, v in zip(fbs, vs):
        ref = api.Framebuffer(v.width, v.height)
        ref.clear(0xFF000000, 0.0)
        bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
        api.cull_meshlets(g.scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None)
        rast.draw_meshlets(ref, n, api.ShadingContext(g.scene, v.world_to_clip, cull_bitmap=bm))
        assert np.array_equal(fb.get_pixels(0), ref.get_pixels(0))
        assert np.array_equal(fb.get_pixels(1), ref.get_pixels(1))


def test_combined_million_meshlets_view_bit_exact():
    """One view of the combined stress scene (1M meshlets, 124M triangles) against the oracle."""
    import os
    sc = scenes.combined_scene(copies=10, texture_size=8, env_size=8)
    v = min(sc.views, key=lambda q: q.width * q.height)
    g = GpuRenderer(sc.meshlets, sc.materials)
    gfb, gc = g.render(v.world_to_clip, v.width, v.height)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, threads=os.cpu_count() or 1)
    assert_visbuffer_equal(gfb, ofb)
    assert gc[0] == 124_000_000 and gc[1] > 100_000
