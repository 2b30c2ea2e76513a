"""Edge cases of the raster against the oracle:

* ragged meshlets: every NumVertices from 1 to 64 (ShadeMeshlet transforms 16-vertex chunks up to
  it, Shading.cpp:295-298) and NumTriangles from 0 to 128, with degenerate triangles (a repeated
  index, three collinear vertices, three equal vertices) among random ones, single- and
  double-sided, at a small size and near the largest framebuffer, binned and unbinned;
* a draw of no meshlets and a meshlet range past the scene's end;
* a frame of degenerate triangles only.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import GpuRenderer, assert_visbuffer_equal, render_oracle

pytestmark = pytest.mark.gpu


def ragged_meshlets(n=320, seed=5):
    rng = np.random.default_rng(seed)
    m = np.zeros(n, dtype=scenes.MESHLET_DTYPE)
    for i in range(n):
        nv = 1 + i % 64 if i < 128 else int(rng.integers(1, 65))
        nt = int(rng.integers(0, 129)) if i % 7 else 0
        centre = rng.uniform(-6, 6, 3) + np.array([0.0, 0.0, 14.0])
        pos = centre + rng.normal(0, 0.6, (nv, 3))
        if nv >= 6:  # collinear and coincident vertex groups for degenerate triangles
            pos[3] = pos[1] + 0.5 * (pos[2] - pos[1])
            pos[5] = pos[4]
        m["Positions"][i, :, :nv] = pos.T.astype(np.float32)
        idx = rng.integers(0, nv, (3, 128)).astype(np.uint8)
        for t in range(0, nt, 9):
            kind = (t // 9) % 3
            if kind == 0:
                idx[1, t] = idx[0, t]                       # repeated index
            elif nv >= 6:
                idx[:, t] = [1, 2, 3] if kind == 1 else [4, 5, 5]  # collinear / coincident
        m["Indices"][i] = idx
        m["NumVertices"][i] = nv
        m["NumTriangles"][i] = nt
        m["AlphaCutoff"][i] = 255
        m["MaterialId"][i] = i % 2
        m["BoundCenter"][i] = pos.mean(axis=0)
        m["BoundRadius"][i] = float(np.linalg.norm(pos - pos.mean(axis=0), axis=1).max())
    mats = np.zeros(2, dtype=scenes.MATERIAL_DTYPE)
    mats["alpha_cutoff"] = 255
    mats["is_double_sided"] = [0, 1]
    return m, mats


@pytest.fixture(scope="module")
def ragged():
    m, mats = ragged_meshlets()
    return m, mats, GpuRenderer(m, mats)


@pytest.mark.parametrize("size", [(320, 180), (2880, 1620)])
@pytest.mark.parametrize("binning", [True, False])
def test_ragged_meshlets_bit_exact(ragged, size, binning):
    m, mats, g = ragged
    w, h = size
    view = scenes.make_view(w, h, eye=(0.0, 0.0, 0.0), target=(0.0, 0.0, 1.0))
    gfb, gc = g.render(view.world_to_clip, w, h, binning=binning)
    ofb, oc = render_oracle(m, mats, view.world_to_clip, w, h, binning=binning)
    assert_visbuffer_equal(gfb, ofb)
    assert list(gc[:3]) == list(oc[:3])
    ids = ofb.get_pixels(0)
    depth = ofb.get_pixels(1)
    covered = depth != 0
    assert covered.sum() > 0.2 * w * h
    meshlets_shown = np.unique(ids[covered] >> 7)
    assert len(meshlets_shown) > 100 and np.any(m["NumVertices"][meshlets_shown] < 16)


def test_empty_draw_and_range_past_the_end(ragged):
    from glimpsw_gb300 import api
    m, mats, g = ragged
    view = scenes.make_view(320, 180, eye=(0.0, 0.0, 0.0), target=(0.0, 0.0, 1.0))
    fb = api.Framebuffer(320, 180)
    fb.clear(0x12345678, 0.25)
    g.rast.reset_counters()
    g.rast.draw_meshlets(fb, 0, api.ShadingContext(g.scene, view.world_to_clip))
    assert np.all(fb.get_pixels(0) == 0x12345678)
    assert np.all(fb.get_pixels(1) == np.float32(0.25).view(np.uint32))
    assert list(g.rast.counters()[:3]) == [0, 0, 0]
    with pytest.raises(api.SwrError):
        g.rast.draw_meshlets(fb, 2, api.ShadingContext(g.scene, view.world_to_clip, meshlet_offset=len(m) - 1))


def test_degenerate_triangles_only_draw_nothing():
    m, mats = ragged_meshlets(n=64, seed=9)
    for i in range(len(m)):  # every triangle reads one vertex three times
        m["Indices"][i][1] = m["Indices"][i][0]
        m["Indices"][i][2] = m["Indices"][i][0]
        m["NumTriangles"][i] = 128
    view = scenes.make_view(640, 360, eye=(0.0, 0.0, 0.0), target=(0.0, 0.0, 1.0))
    g = GpuRenderer(m, mats)
    for binning in (True, False):
        gfb, gc = g.render(view.world_to_clip, 640, 360, binning=binning)
        ofb, oc = render_oracle(m, mats, view.world_to_clip, 640, 360, binning=binning)
        assert_visbuffer_equal(gfb, ofb)
        assert list(gc[:3]) == list(oc[:3])
        assert np.all(ofb.get_pixels(1) == 0)
