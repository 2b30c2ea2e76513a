"""Backface-cone culling on the GPU (swr_cull_meshlets_ex with SWR_CULL_BACKFACE_CONE, and batches
created with it): it removes meshlets, and the vis-buffer stays bit-identical to the one drawn
with frustum culling alone, which itself equals the oracle's.

Cases: the open patch scene (meshlets with real cones; a quarter of its materials double-sided,
which must never be culled) from cameras outside and inside the volume; the closed meshlets of the
small and large plain-path constructions (degenerate cones: nothing is culled); a mirrored model
matrix (the test turns itself off); a batch of views with and without the cone test.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import GpuRenderer, assert_visbuffer_equal, render_oracle
from tests.test_cone_cull import cone_culled

pytestmark = pytest.mark.gpu

CAMERAS = [((0.0, 0.0, -130.0), (0.0, 0.0, 0.0)), ((60.0, 40.0, -20.0), (0.0, 5.0, 0.0)),
           ((5.0, -3.0, 2.0), (1.0, 0.0, 9.0))]


@pytest.fixture(scope="module")
def patches():
    sc = scenes.patch_scene(n=6000, width=640, height=360, n_materials=4, extent=100.0, texture_size=8, env_size=8)
    mats = sc.materials.copy()
    mats["is_double_sided"][::4] = 1
    return sc.meshlets, mats, GpuRenderer(sc.meshlets, mats)


def _bitmaps(g, n, view, model=None, cone=False):
    import torch

    from glimpsw_gb300 import api
    model = scenes.IDENTITY if model is None else model
    bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
    cnt = api.cull_meshlets(g.scene, 0, n, bm, view.proj, view.view, model, view.view, view.width, view.height,
                            want_count=True, cone=cone)
    return bm, cnt


def _bits(bm, n):
    return np.unpackbits(bm.cpu().numpy().view(np.uint8), bitorder="little")[:n].astype(bool)


@pytest.mark.parametrize("eye,target", CAMERAS)
def test_cone_culled_visbuffer_identical(patches, eye, target):
    from oracle import oracle as O
    m, mats, g = patches
    n = len(m)
    v = scenes.make_view(640, 360, eye=eye, target=target)
    bf, nf = _bitmaps(g, n, v)
    bc, nc = _bitmaps(g, n, v, cone=True)
    frustum, cone = _bits(bf, n), _bits(bc, n)
    assert not (cone & ~frustum).any()
    removed = frustum & ~cone
    print(f"cone cull: {nf} meshlets in the frustum, {nf - nc} of them culled by their cones")
    assert nc < 0.9 * nf
    assert not (removed & mats["is_double_sided"][m["MaterialId"]].astype(bool)).any()
    # the kernels' decisions are the float32 test restated on the CPU
    ds = mats["is_double_sided"][m["MaterialId"]].astype(bool)
    expect = frustum & cone_culled(m, v.eye, ds)
    assert (removed != expect).sum() <= max(2, n // 1000)

    gf, _ = g.render(v.world_to_clip, v.width, v.height, cull_bitmap=bf)
    gc, _ = g.render(v.world_to_clip, v.width, v.height, cull_bitmap=bc)
    assert_visbuffer_equal(gc, gf)
    obm, ocount = O.cull_meshlets(m, n, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height)
    assert ocount == nf
    ofb, _ = render_oracle(m, mats, v.world_to_clip, v.width, v.height, cull_bitmap=obm)
    assert_visbuffer_equal(gf, ofb)
    assert np.any(gc.get_pixels(1))


@pytest.mark.parametrize("which", ["grid", "volume"])
def test_closed_meshlets_are_never_cone_culled(which):
    if which == "grid":
        sc = scenes.grid_scene(n_side=32, width=640, height=360)
    else:
        sc = scenes.volume_scene(n=6000, width=640, height=360, n_materials=4, extent=40.0, texture_size=8, env_size=8)
    g = GpuRenderer(sc.meshlets, sc.materials)
    v = sc.views[0]
    n = len(sc.meshlets)
    bf, nf = _bitmaps(g, n, v)
    bc, nc = _bitmaps(g, n, v, cone=True)
    assert nf == nc and np.array_equal(_bits(bf, n), _bits(bc, n))


def test_mirrored_model_turns_the_cone_test_off(patches):
    """Under a mirroring model matrix FrontCCW keeps the triangles that face away; the cone test
    must not cull then (it would remove the visible ones)."""
    m, mats, g = patches
    n = len(m)
    v = scenes.make_view(640, 360, eye=CAMERAS[0][0], target=CAMERAS[0][1])
    mirror = np.diag([-1.0, 1.0, 1.0, 1.0]).astype(np.float32).reshape(16)
    bf, nf = _bitmaps(g, n, v, model=mirror)
    bc, nc = _bitmaps(g, n, v, model=mirror, cone=True)
    assert nf == nc and nf > 0
    # and without the mirror the same camera does cull
    _, nf2 = _bitmaps(g, n, v)
    _, nc2 = _bitmaps(g, n, v, cone=True)
    assert nc2 < nf2


def test_batched_cone_cull_identical(patches):
    from glimpsw_gb300 import api
    m, mats, g = patches
    views = [scenes.make_view(w, h, eye=e, target=t) for (e, t), (w, h) in zip(CAMERAS, [(640, 360), (320, 320), (480, 272)])]
    out = {}
    for cone in (False, True):
        fbs = [api.Framebuffer(v.width, v.height) for v in views]
        b = api.Batch(g.rast, g.scene, [(fb, v.proj, v.view, scenes.IDENTITY, False) for fb, v in zip(fbs, views)],
                      cone=cone)
        b.render()
        out[cone] = [(fb.get_pixels(0), fb.get_pixels(1)) for fb in fbs]
        processed = b.counters()[0]
        out[(cone, "tris")] = processed
    for (i0, d0), (i1, d1) in zip(out[False], out[True]):
        assert np.array_equal(i0, i1) and np.array_equal(d0, d1)
    assert out[(True, "tris")] < out[(False, "tris")]
