"""The debug views on the GPU against the oracle, bit for bit: the OverdrawShader (counters and the
maximum-depth layer; both draw semantics, clipping, a full queue, alpha-tested materials drawn
like any other) and ShadingContext::ResolveDebug for all eight DebugLayer values."""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import GpuRenderer, TexturePair, render_oracle

pytestmark = pytest.mark.gpu


def _pairs(sc, size):
    return [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], size) for i in range(len(sc.materials))]


@pytest.fixture(scope="module")
def inside():
    sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=64, alpha_every=2)
    texs = _pairs(sc, 64)
    return sc, texs, GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])


def _inside_view(sc):
    v = sc.views[0]
    return scenes.make_view(v.width, v.height, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))


def _overdraw_pair(sc, texs, g, view, **kw):
    from glimpsw_gb300 import api
    gfb, gc = g.render(view.world_to_clip, view.width, view.height, clear=(0, 0.0), shader=api.OverdrawShader, **kw)
    ofb, oc = render_oracle(sc.meshlets, sc.materials, view.world_to_clip, view.width, view.height, clear=(0, 0.0),
                            textures=[t.o for t in texs], shader=2, **kw)
    return gfb, gc, ofb, oc


@pytest.mark.parametrize("binning", [True, False])
def test_overdraw_bit_exact(inside, binning):
    sc, texs, g = inside
    gfb, gc, ofb, oc = _overdraw_pair(sc, texs, g, _inside_view(sc), binning=binning)
    assert np.array_equal(gfb.get_pixels(0), ofb.get_pixels(0))
    assert np.array_equal(gfb.get_pixels(1), ofb.get_pixels(1))
    assert list(gc[:3]) == list(oc[:3])
    assert (gfb.get_pixels(0) >> 16).max() > 3


@pytest.mark.parametrize("capacity", [1, 64])
def test_overdraw_full_queue(inside, capacity):
    sc, texs, g = inside
    g.rast.set_queue_capacity(capacity)
    try:
        gfb, _, ofb, _ = _overdraw_pair(sc, texs, g, _inside_view(sc))
    finally:
        g.rast.set_queue_capacity(0)
    assert np.array_equal(gfb.get_pixels(0), ofb.get_pixels(0))
    assert np.array_equal(gfb.get_pixels(1), ofb.get_pixels(1))


def test_overdraw_then_visbuffer_draw(inside):
    """A vis-buffer draw after an overdraw draw into the same framebuffer starts from its depth layer."""
    from glimpsw_gb300 import api
    sc, texs, g = inside
    v = _inside_view(sc)
    gfb, _ = g.render(v.world_to_clip, v.width, v.height, clear=(0, 0.0), shader=api.OverdrawShader)
    g.render(v.world_to_clip, v.width, v.height, fb=gfb)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, clear=(0, 0.0), shader=2,
                           textures=[t.o for t in texs])
    render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, fb=ofb, textures=[t.o for t in texs])
    assert np.array_equal(gfb.get_pixels(0), ofb.get_pixels(0))
    assert np.array_equal(gfb.get_pixels(1), ofb.get_pixels(1))


@pytest.mark.parametrize("layer", range(8))
def test_resolve_debug_bit_exact(inside, layer):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, g = inside
    v = scenes.make_view(480, 272, eye=(0.0, 2.0, -30.0), target=(0.0, 0.0, 0.0))
    shader, clear = (api.OverdrawShader, (0, 0.0)) if layer >= 6 else (api.VisBufferShader, (0xFF000000, 0.0))
    gfb, _ = g.render(v.world_to_clip, v.width, v.height, clear=clear, shader=shader)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, clear=clear,
                           textures=[t.o for t in texs], shader=2 if layer >= 6 else 0)
    api.ShadingContext(g.scene, v.world_to_clip).resolve_debug(g.rast, gfb, layer)
    O.resolve_debug(ofb, O.Context(sc.meshlets, sc.materials, v.world_to_clip, textures=[t.o for t in texs]), layer,
                    threads=8)
    a, b = gfb.get_pixels(0), ofb.get_pixels(0)
    bad = np.argwhere(a != b)
    assert len(bad) == 0, f"{len(bad)} mismatches, first {bad[0]}: {a[tuple(bad[0])]:#x} vs {b[tuple(bad[0])]:#x}"
    assert len(np.unique(a)) >= (3 if layer == 0 else 4)  # layer 0: black surfaces and the checkerboard
