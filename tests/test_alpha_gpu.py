"""Alpha-tested vis-buffer (FS_EncodeSurfaceId<true>, Shading.cpp:309-331) on the GPU, bit-exact
against the oracle: perspective-correct texcoords, the tile's implicit LOD (magnified and minified
textures, so both filters), clipped triangles (camera inside the scene), several cutoffs, a full
queue (the mesh stage's serial fallback), batched views, and opaque and alpha-tested materials in
one draw."""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import GpuRenderer, TexturePair, assert_visbuffer_equal, render_oracle

pytestmark = pytest.mark.gpu

EMPTY = 0xFF000000


def _pairs(sc, size):
    return [TexturePair([sc.texture_pixels(i, 0)], size) for i in range(len(sc.materials))]


@pytest.fixture(scope="module")
def inside():
    # camera inside a dense volume: triangles cross the near plane and the guard band
    sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=64, alpha_every=2)
    texs = _pairs(sc, 64)
    return sc, texs, GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])


@pytest.fixture(scope="module")
def far():
    # many small triangles seen from outside: minified textures (nearest filter) and magnified ones
    sc = scenes.volume_scene(n=20_000, width=1280, height=720, n_materials=8, texture_size=256, alpha_every=2)
    texs = _pairs(sc, 256)
    return sc, texs, GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])


def _inside_view(sc):
    v = sc.views[0]
    return scenes.make_view(v.width, v.height, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))


def _check(sc, texs, g, view, mats=None, **kw):
    mats = sc.materials if mats is None else mats
    gfb, gc = g.render(view.world_to_clip, view.width, view.height, **kw)
    ofb, oc = render_oracle(sc.meshlets, mats, view.world_to_clip, view.width, view.height,
                            textures=[t.o for t in texs], threads=1 if "binning" in kw else 8, **kw)
    assert_visbuffer_equal(gfb, ofb)
    if "binning" in kw:
        assert list(gc[:3]) == list(oc[:3])
    return gfb


@pytest.mark.parametrize("binning", [True, False])
def test_inside_bit_exact(inside, binning):
    sc, texs, g = inside
    fb = _check(sc, texs, g, _inside_view(sc), binning=binning)
    ids = fb.get_pixels(0)
    mat = sc.meshlets["MaterialId"].astype(np.int64)[np.minimum(ids, len(sc.meshlets) * 128 - 1) // 128]
    assert ((ids != EMPTY) & (sc.materials["alpha_cutoff"][mat] < 255)).sum() > 1000  # alpha-tested pixels shown


@pytest.mark.parametrize("cutoff", [1, 64, 200, 254])
def test_cutoffs_bit_exact(inside, cutoff):
    sc, texs, g = inside
    mats = sc.materials.copy()
    mats["alpha_cutoff"][::2] = cutoff
    g.scene.set_materials(mats, [t.g for t in texs])
    try:
        _check(sc, texs, g, _inside_view(sc), mats=mats)
    finally:
        g.scene.set_materials(sc.materials, [t.g for t in texs])


def test_alpha_removes_fragments(inside):
    """The same draw with every material opaque differs (the test is not vacuous)."""
    sc, texs, g = inside
    view = _inside_view(sc)
    a, _ = g.render(view.world_to_clip, view.width, view.height)
    mats = sc.materials.copy()
    mats["alpha_cutoff"] = 255
    g.scene.set_materials(mats, [t.g for t in texs])
    try:
        b, _ = g.render(view.world_to_clip, view.width, view.height)
    finally:
        g.scene.set_materials(sc.materials, [t.g for t in texs])
    assert (a.get_pixels(0) != b.get_pixels(0)).sum() > 1000


@pytest.mark.parametrize("capacity", [1, 2, 3, 64])
def test_full_queue_gives_the_same_image(inside, capacity):
    """Alpha-tested triangles take two queue slots; with a tiny queue the mesh stage rasterizes
    them itself (one lane per triangle) and an odd capacity leaves a single empty slot."""
    sc, texs, g = inside
    g.rast.set_queue_capacity(capacity)
    try:
        _check(sc, texs, g, _inside_view(sc), binning=False)
    finally:
        g.rast.set_queue_capacity(0)


def test_far_view_bit_exact(far):
    sc, texs, g = far
    _check(sc, texs, g, sc.views[0])
    _check(sc, texs, g, sc.views[1])


def test_batched_views_equal_single_draws(far):
    import torch
    from glimpsw_gb300 import api
    sc, texs, g = far
    vs = [sc.views[0], scenes.make_view(640, 360, eye=(5.0, 3.0, -60.0), target=(0.0, 0.0, 20.0))]
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


def test_batch_follows_material_changes(inside):
    """A batch records its draw once; changing the scene's materials afterwards (here: alpha testing
    switched off, then on again) must be seen by the next render."""
    import torch
    from glimpsw_gb300 import api
    sc, texs, g = inside
    v = _inside_view(sc)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fb = api.Framebuffer(v.width, v.height)
    batch = api.Batch(rast, g.scene, [(fb, v.proj, v.view, scenes.IDENTITY, False)])
    opaque = sc.materials.copy()
    opaque["alpha_cutoff"] = 255
    n = len(sc.meshlets)
    try:
        for mats in (sc.materials, opaque, sc.materials):
            g.scene.set_materials(mats, [t.g for t in texs])
            batch.render()
            ref = api.Framebuffer(v.width, v.height)
            ref.clear(0xFF000000, 0.0)
            bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
            api.cull_meshlets(g.scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None)
            rast.draw_meshlets(ref, n, api.ShadingContext(g.scene, v.world_to_clip, cull_bitmap=bm))
            assert np.array_equal(fb.get_pixels(0), ref.get_pixels(0))
            assert np.array_equal(fb.get_pixels(1), ref.get_pixels(1))
    finally:
        g.scene.set_materials(sc.materials, [t.g for t in texs])
