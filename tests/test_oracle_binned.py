"""The oracle's threaded binned draw (Rasterizer(N)::DrawMeshlets with binning, restated in the
reference's work split: meshlets strided over workers, 128x128 bins rasterized by their elected
worker) against its single-threaded binned draw. It is the timed CPU baseline, so it must do the
same work: on scenes without equal-depth ties the vis-buffer and the triangle counters are the same
for every worker count (ties resolve in bin-list order when several workers bin them, as in the
reference)."""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import render_oracle


@pytest.mark.parametrize("which", ["grid", "inside"])
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_binned_threaded_draw_equals_single_threaded(which, threads):
    from oracle import oracle as O
    if which == "grid":
        sc = scenes.grid_scene(n_side=32, width=640, height=360)
        v = sc.views[0]
    else:
        sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=8, env_size=8)
        v = scenes.make_view(480, 272, eye=np.zeros(3), target=(0.3, 0.1, 1.0))
    ref, rc = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height, binning=True)
    fb = O.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    c = O.draw_meshlets_binned(fb, O.Context(sc.meshlets, sc.materials, v.world_to_clip), len(sc.meshlets), threads)
    assert np.array_equal(fb.get_pixels(0), ref.get_pixels(0))
    assert np.array_equal(fb.get_pixels(1), ref.get_pixels(1))
    assert list(c[:3]) == list(rc[:3])
    assert c[3] > 0  # bins were flushed
    if which == "inside":
        assert rc[2] > 0  # non-trivial triangles were met (and dropped, as the binned path does)
