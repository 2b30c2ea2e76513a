"""Batched multi-view rendering: every view of one batched graph launch must equal, bit for bit,
the per-view sequence clear + frustum cull + draw through the regular entry points (and so the
oracle), for any tuning, after view updates, and for depth-only views."""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import assert_visbuffer_equal, render_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    from glimpsw_gb300 import api
    api.load_library()
    api.set_stream(torch.cuda.current_stream().cuda_stream)
    sc = scenes.multiview_scene(n=4096, n_cameras=6, cube_size=96, min_res=(64, 64), max_res=(640, 360))
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fbs = [api.Framebuffer(v.width, v.height) for v in sc.views]
    views = [(fb, v.proj, v.view, scenes.IDENTITY, v.depth_only) for fb, v in zip(fbs, sc.views)]
    batch = api.Batch(rast, scene, views)
    return sc, scene, rast, fbs, views, batch


def per_view(api, sc, scene, rast, v):
    import torch
    n = len(sc.meshlets)
    fb = api.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
    api.cull_meshlets(scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None)
    rast.draw_meshlets(fb, n, api.ShadingContext(scene, v.world_to_clip, cull_bitmap=bm))
    return fb


def check_all(api, sc, scene, rast, fbs):
    for fb, v in zip(fbs, sc.views):
        ref = per_view(api, sc, scene, rast, v)
        assert np.array_equal(fb.get_pixels(1), ref.get_pixels(1)), "depth differs"
        if not v.depth_only:
            assert np.array_equal(fb.get_pixels(0), ref.get_pixels(0)), "surface ids differ"


@pytest.mark.parametrize("tuning", [(0, 0), (2, 4), (16, 16), (4, 8), (16, 8, 2), (2, 16, 8), (8, 4, 16)])
def test_batch_equals_per_view_draws(setup, tuning):
    """Any chunk size, chunk shape (width x height tiles) and warps per block gives the same views."""
    from glimpsw_gb300 import api
    sc, scene, rast, fbs, views, batch = setup
    batch.set_tuning(*tuning[:2])
    if len(tuning) == 3:
        batch.set_chunk_shape(tuning[0], tuning[2])
    batch.render()
    check_all(api, sc, scene, rast, fbs)


def test_batch_matches_oracle_and_updates_views(setup):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, scene, rast, fbs, views, batch = setup
    moved = []
    for (fb, proj, view, model, d), v in zip(views, sc.views):
        nv = scenes.look_at(v.eye + np.array([0.5, 0.25, -0.5], dtype=np.float32), v.eye + np.array([1.0, -0.3, 0.7]))
        moved.append((fb, proj, nv, model, d))
    batch.set_views(moved)
    batch.render()
    for (fb, proj, view, model, d), v in zip(moved, sc.views):
        wtc = scenes.mat_mul(proj, view)
        bm, _ = O.cull_meshlets(sc.meshlets, len(sc.meshlets), proj, view, model, view, v.width, v.height, None)
        ofb, _ = render_oracle(sc.meshlets, sc.materials, wtc, v.width, v.height, cull_bitmap=bm)
        if d:
            assert np.array_equal(fb.get_pixels(1), ofb.get_pixels(1))
        else:
            assert_visbuffer_equal(fb, ofb)
    batch.set_views(views)


def test_batch_counts_kernels_and_autotunes(setup, tmp_path, monkeypatch):
    from glimpsw_gb300 import api, autotune
    sc, scene, rast, fbs, views, batch = setup
    monkeypatch.setenv("SWR_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    best, timings = autotune.tune(batch, key="test", repeats=1)
    squares = [(c, w, c) for c, w in autotune.CANDIDATES]
    assert all(s in timings for s in squares) and best in timings
    c0, w0, _ = min(squares, key=timings.get)
    assert len(timings) == len(squares) + len(autotune.shape_candidates(c0))
    assert any(cw != ch for cw, _, ch in timings)  # rectangular chunks were timed
    best2, _ = autotune.tune(batch, key="test")  # cached
    assert best2 == best
    n0 = api.launch_count()
    batch.render()
    assert api.launch_count() - n0 >= 4  # clear, cull, mesh stage, chunk stage
    check_all(api, sc, scene, rast, fbs)


def test_depth_only_views_keep_layer0(setup):
    """Depth-only views write only the depth layer when their layers are next read; layer 0 keeps
    the clear colour while the depth layer matches a full per-view draw."""
    from glimpsw_gb300 import api
    sc, scene, rast, fbs, views, batch = setup
    batch.render()
    for fb, v in zip(fbs, sc.views):
        if v.depth_only:
            assert np.all(fb.get_pixels(0) == 0xFF000000)
            assert np.array_equal(fb.get_pixels(1), per_view(api, sc, scene, rast, v).get_pixels(1))
