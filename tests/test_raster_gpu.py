"""GPU parity of the vis-buffer rasterizer against the CPU oracle: bit-exact depth and surface ids.

Cases: the small grid scene (the 1024-meshlet plain-path construction, at 640x360 and at its own
1280x720), a volume scene with the
camera inside it (near-plane clipping, guard band), both binned (Mode A) and unbinned (Mode B)
semantics, guard band off, equal-depth ties, meshlet offsets with cull bitmaps, multi-draw frames.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import (CLIP_FROM_OBJECT, GpuRenderer, assert_visbuffer_equal, meshlet_from_clip_triangles,
                           render_oracle)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid():
    sc = scenes.grid_scene(n_side=32, width=640, height=360)
    return sc, GpuRenderer(sc.meshlets, sc.materials)


@pytest.fixture(scope="module")
def inside():
    # camera inside a dense volume: triangles cross the near plane and the guard band
    sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=8)
    mats = sc.materials.copy()
    mats["is_double_sided"][::2] = 1
    return sc, mats, GpuRenderer(sc.meshlets, mats)


@pytest.mark.parametrize("binning", [True, False])
def test_grid_bit_exact(grid, binning):
    sc, g = grid
    v = sc.views[0]
    gfb, gc = g.render(v.world_to_clip, v.width, v.height, binning=binning)
    ofb, oc = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, binning=binning)
    assert_visbuffer_equal(gfb, ofb)
    assert list(gc[:3]) == list(oc[:3])


@pytest.mark.parametrize("binning", [True, False])
def test_config1_size_bit_exact(binning):
    """The small plain-path configuration at its own size: 1024 grid meshlets at 1280x720."""
    sc = scenes.grid_scene(n_side=32, width=1280, height=720)
    v = sc.views[0]
    assert len(sc.meshlets) == 1024 and (v.width, v.height) == (1280, 720)
    gfb, gc = GpuRenderer(sc.meshlets, sc.materials).render(v.world_to_clip, v.width, v.height, binning=binning)
    ofb, oc = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, binning=binning)
    assert_visbuffer_equal(gfb, ofb)
    assert list(gc[:3]) == list(oc[:3])


@pytest.mark.parametrize("binning,clipping,guardband", [(True, True, True), (False, True, True), (False, False, True),
                                                        (False, True, False)])
def test_inside_volume_bit_exact(inside, binning, clipping, guardband):
    sc, mats, g = inside
    for v in sc.views:
        eye = np.array([0.0, 0.0, 0.0])
        view = scenes.make_view(v.width, v.height, eye=eye, target=(0.3, 0.1, 1.0))
        gfb, gc = g.render(view.world_to_clip, v.width, v.height, binning=binning, clipping=clipping,
                           guardband=guardband)
        ofb, oc = render_oracle(sc.meshlets, mats, view.world_to_clip, v.width, v.height, binning=binning,
                                clipping=clipping, guardband=guardband)
        assert_visbuffer_equal(gfb, ofb)
        assert list(gc[:3]) == list(oc[:3])
        if binning or clipping:  # TrianglesClipped counts only then (Rasterizer.cpp:209-210, 567-568)
            assert oc[2] > 0  # the case really exercises non-trivial triangles


def test_crafted_triangles_bit_exact():
    rng = np.random.default_rng(11)
    mats = np.zeros(1, dtype=scenes.MATERIAL_DTYPE)
    mats["alpha_cutoff"] = 255
    mats["is_double_sided"] = 1
    parts = []
    for _ in range(40):
        tris = []
        for _ in range(20):
            c = rng.uniform(-1.5, 1.5, 2)
            s = 10 ** rng.uniform(-3, 0.5)
            w = rng.uniform(-0.3, 3.0, 3)
            t = [[c[0] + s * rng.normal(), c[1] + s * rng.normal(), w[k]] for k in range(3)]
            tris.append(t)
        parts.append(meshlet_from_clip_triangles(tris))
    m = scenes.concat_meshlets(parts)
    g = GpuRenderer(m, mats)
    for (w, h) in [(64, 64), (200, 120), (2896, 2896)]:
        for binning in (True, False):
            gfb, gc = g.render(CLIP_FROM_OBJECT, w, h, binning=binning)
            ofb, oc = render_oracle(m, mats, CLIP_FROM_OBJECT, w, h, binning=binning)
            assert_visbuffer_equal(gfb, ofb)
            assert list(gc[:3]) == list(oc[:3])


def test_equal_depth_ties_resolve_to_first_submitted(grid):
    sc, _ = grid
    v = sc.views[0]
    m = scenes.concat_meshlets([sc.meshlets[:64], sc.meshlets[:64], sc.meshlets[:64]])
    g = GpuRenderer(m, sc.materials)
    gfb, _ = g.render(v.world_to_clip, v.width, v.height)
    ofb, _ = render_oracle(m, sc.materials, v.world_to_clip, v.width, v.height)
    assert_visbuffer_equal(gfb, ofb)
    ids = gfb.get_pixels(0)[gfb.get_pixels(1) != 0]
    assert ids.max() < 64 * 128  # every duplicate lost its tie


def test_offsets_bitmaps_and_multi_draw(grid):
    """Two draw calls (MeshletOffset 0 and 512) with cull bitmaps, as the frame driver batches them
    (Main.cpp:222-243)."""
    sc, g = grid
    v = sc.views[0]
    rng = np.random.default_rng(3)
    bm0 = rng.integers(0, 1 << 16, 32).astype(np.uint16)
    bm1 = rng.integers(0, 1 << 16, 32).astype(np.uint16)
    import torch
    d0, d1 = torch.from_numpy(bm0.view(np.int16)).cuda(), torch.from_numpy(bm1.view(np.int16)).cuda()
    from glimpsw_gb300 import api
    fb = api.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    g.render(v.world_to_clip, v.width, v.height, count=512, meshlet_offset=0, cull_bitmap=d0, fb=fb)
    g.render(v.world_to_clip, v.width, v.height, count=512, meshlet_offset=512, cull_bitmap=d1, fb=fb)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, count=512,
                           meshlet_offset=0, cull_bitmap=bm0)
    render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, count=512, meshlet_offset=512,
                  cull_bitmap=bm1, fb=ofb)
    assert_visbuffer_equal(fb, ofb)


def test_clear_values_and_layers(grid):
    sc, g = grid
    v = sc.views[0]
    for clear in [(0x12345678, 0.0), (0xFF000000, 0.02)]:
        gfb, _ = g.render(v.world_to_clip, v.width, v.height, clear=clear)
        ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, clear=clear)
        assert_visbuffer_equal(gfb, ofb)


def test_two_rasterizers_on_two_streams(inside):
    """Batches drawn in turn by two rasterizers on two streams into one framebuffer (one batch's
    chunk stage overlaps the next batch's mesh stage, as the end-to-end frame does): the keys are
    order-independent, so the vis-buffer equals one draw's, and the oracle's."""
    import torch

    from glimpsw_gb300 import api
    sc, mats, g = inside
    v = sc.views[0]
    view = scenes.make_view(v.width, v.height, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))
    n = len(sc.meshlets)
    other = api.Rasterizer()
    other.EnableBinning = False
    main, side = torch.cuda.Stream(), torch.cuda.Stream()
    cleared, joined = torch.cuda.Event(), torch.cuda.Event()
    g.rast.EnableBinning, g.rast.EnableClipping, g.rast.EnableGuardband = False, True, True
    bounds = [0, 400, 1100, 2000, n]
    try:
        api.set_stream(main)
        fb = api.Framebuffer(v.width, v.height)
        fb.clear(0xFF000000, 0.0)
        cleared.record(main)
        side.wait_event(cleared)
        for k in range(4):
            rast, s = (g.rast, main) if k % 2 == 0 else (other, side)
            api.set_stream(s)
            ctx = api.ShadingContext(g.scene, view.world_to_clip, meshlet_offset=bounds[k])
            rast.draw_meshlets(fb, bounds[k + 1] - bounds[k], ctx)
        api.set_stream(main)
        joined.record(side)
        main.wait_event(joined)
        ofb, _ = render_oracle(sc.meshlets, mats, view.world_to_clip, v.width, v.height, binning=False)
        assert_visbuffer_equal(fb, ofb)
    finally:
        api.set_stream(0)  # the per-thread default stream again


def test_get_pixels_into_pinned_memory(grid):
    """GetPixels into page-locked memory (written by the de-tiling kernel over the host link) with a
    row stride wider than the frame: the same words as the staged copy into pageable memory, and
    the padding words between rows untouched."""
    import ctypes as C

    import torch

    from glimpsw_gb300 import api
    sc, g = grid
    v = sc.views[0]
    gfb, _ = g.render(v.world_to_clip, v.width, v.height)
    stride = v.width + 12
    for layer in (0, 1):
        ref = gfb.get_pixels(layer)
        pinned = torch.full((v.height, stride), -1, dtype=torch.int32).pin_memory()
        api._check(api._lib.swr_framebuffer_get_pixels(gfb.h, layer, C.c_void_p(pinned.data_ptr()), stride))
        got = pinned.numpy().view(np.uint32)
        assert np.array_equal(got[:, :v.width], ref)
        assert np.all(got[:, v.width:] == 0xFFFFFFFF)


@pytest.mark.parametrize("capacity", [1, 64])
def test_full_queue_gives_the_same_image(inside, capacity):
    """With a tiny large-triangle queue the mesh stage rasterizes the overflow itself (and clipped
    triangles fall back to per-lane rasterization); the image must not change."""
    sc, mats, g = inside
    v = sc.views[0]
    view = scenes.make_view(v.width, v.height, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))
    g.rast.set_queue_capacity(capacity)
    try:
        gfb, gc = g.render(view.world_to_clip, v.width, v.height, binning=False)
    finally:
        g.rast.set_queue_capacity(0)
    ofb, oc = render_oracle(sc.meshlets, mats, view.world_to_clip, v.width, v.height, binning=False)
    assert_visbuffer_equal(gfb, ofb)
    assert list(gc[:3]) == list(oc[:3])
