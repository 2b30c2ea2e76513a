"""CPU tests of the oracle itself: layout, hand-derived known answers, rasterization rules.

The reference ships no tests or golden vectors and cannot be built here, so the oracle is pinned
by values derived by hand from the reference's formulas (Rasterizer.cpp:257-351) and by
properties its rules imply (top-left fill convention, order independence of the depth test).
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from oracle import oracle as O
from tests.helpers import CLIP_FROM_OBJECT, meshlet_from_clip_triangles, render_oracle

MATS = np.zeros(1, dtype=scenes.MATERIAL_DTYPE)
MATS["alpha_cutoff"] = 255


def test_meshlet_layout_matches_reference():
    assert O.lib().orc_meshlet_size() == 1728 == scenes.MESHLET_DTYPE.itemsize
    assert scenes.MESHLET_DTYPE.fields["Positions"][1] == 64
    assert scenes.MESHLET_DTYPE.fields["Indices"][1] == 1344


def test_template_is_closed_64_vertex_patch():
    p, t = scenes.meshlet_template()
    assert p.shape == (64, 3) and t.shape == (124, 3)
    # every edge of a closed 2-manifold is shared by exactly two triangles with opposite direction
    edges = {}
    for a, b, c in t:
        for e in ((a, b), (b, c), (c, a)):
            edges[e] = edges.get(e, 0) + 1
    assert all(v == 1 for v in edges.values())
    assert all((b, a) in edges for (a, b) in edges)


def test_known_answer_right_triangle_top_left_rule():
    """NDC (-.5,-.5), (-.5,.5), (.5,-.5) on a 16x16 target snap to subpixels (-64,-64), (-64,64),
    (64,-64): int det = 16384, A12 = B12 = -128 so the hypotenuse is not a top-left edge and its
    samples (px + py == 15) are excluded. Covered: px, py >= 4 and px + py <= 14 (28 pixels);
    clip z = 0.1 with w = 1 gives a constant depth of 0.1."""
    tri = [[-0.5, -0.5, 1.0], [-0.5, 0.5, 1.0], [0.5, -0.5, 1.0]]
    fb, counters = render_oracle(meshlet_from_clip_triangles(tri), MATS, CLIP_FROM_OBJECT, 16, 16)
    depth = fb.get_pixels(1).view(np.float32)
    ids = fb.get_pixels(0)
    py, px = np.nonzero(depth > 0)
    expected = {(x, y) for x in range(16) for y in range(16) if x >= 4 and y >= 4 and x + y <= 14}
    assert set(zip(px.tolist(), py.tolist())) == expected
    assert np.all(depth[depth > 0] == np.float32(0.1))
    assert np.all(ids[depth > 0] == 0)
    assert list(counters[:3]) == [1, 1, 0]


def test_known_answer_backface_culled():
    tri = [[-0.5, -0.5, 1.0], [0.5, -0.5, 1.0], [-0.5, 0.5, 1.0]]  # clockwise: det < 0
    fb, counters = render_oracle(meshlet_from_clip_triangles(tri), MATS, CLIP_FROM_OBJECT, 16, 16)
    assert not np.any(fb.get_pixels(1))
    assert list(counters[:3]) == [1, 0, 0]
    mats = MATS.copy()
    mats["is_double_sided"] = 1  # FaceCullMode::None keeps it (Shading.cpp:304)
    fb, _ = render_oracle(meshlet_from_clip_triangles(tri), mats, CLIP_FROM_OBJECT, 16, 16)
    # the int-det flip (Rasterizer.cpp:306-312) restores the orientation, so the hypotenuse keeps
    # A12 = -128 and stays excluded: the same 28 pixels
    assert (fb.get_pixels(1) != 0).sum() == 28


def test_shared_edge_covered_exactly_once():
    """Two triangles sharing a diagonal (a quad) cover every pixel of the quad exactly once."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        # four points on an ellipse in increasing angle: a convex, counter-clockwise quad
        ang = np.sort(rng.uniform(0, 2 * np.pi, 4))
        c, r = rng.uniform(-0.2, 0.2, 2), rng.uniform(0.3, 0.7, 2)
        q = np.stack([c[0] + r[0] * np.cos(ang), c[1] + r[1] * np.sin(ang)], axis=1)
        t0 = [[*q[0], 1], [*q[1], 1], [*q[2], 1]]
        t1 = [[*q[0], 1], [*q[2], 1], [*q[3], 1]]
        mats = MATS.copy()
        mats["is_double_sided"] = 1
        cover = np.zeros((64, 64), dtype=np.int32)
        for t in (t0, t1):
            fb, _ = render_oracle(meshlet_from_clip_triangles([t]), mats, CLIP_FROM_OBJECT, 64, 64)
            cover += (fb.get_pixels(1) != 0)
        both, _ = render_oracle(meshlet_from_clip_triangles([t0, t1]), mats, CLIP_FROM_OBJECT, 64, 64)
        assert cover.max() <= 1
        assert np.array_equal(cover == 1, both.get_pixels(1) != 0)


def test_equal_depth_first_submitted_wins():
    """Identical triangles in two meshlets: the depth test is strict (Shading.cpp:313), so the
    first meshlet keeps every pixel."""
    tri = [[-0.5, -0.5, 2.0], [-0.5, 0.5, 2.0], [0.5, -0.5, 2.0]]
    m = scenes.concat_meshlets([meshlet_from_clip_triangles(tri), meshlet_from_clip_triangles(tri)])
    fb, _ = render_oracle(m, MATS, CLIP_FROM_OBJECT, 32, 32)
    ids = fb.get_pixels(0)[fb.get_pixels(1) != 0]
    assert len(ids) > 0 and np.all(ids == 0)


def test_binned_mode_drops_nontrivial_unbinned_clips():
    """A triangle crossing the near plane is non-trivial: binned semantics count and drop it
    (Rasterizer.cpp:567-569), unbinned semantics clip and draw it (209-249)."""
    tri = [[-0.5, -0.5, 1.0], [-0.5, 0.5, 1.0], [0.5, -0.5, -0.5]]
    m = meshlet_from_clip_triangles(tri)
    fa, ca = render_oracle(m, MATS, CLIP_FROM_OBJECT, 64, 64, binning=True)
    fbb, cb = render_oracle(m, MATS, CLIP_FROM_OBJECT, 64, 64, binning=False)
    assert ca[2] == 1 and cb[2] == 1
    assert not np.any(fa.get_pixels(1))
    assert np.any(fbb.get_pixels(1))


def test_grid_scene_frontfaces_only():
    """Back-face culling keeps the visible hemispheres: drawing the back faces too (double-sided)
    draws a superset, so its reversed-Z depth is never smaller, and it differs only at the few
    silhouette pixels where the displaced (slightly non-convex) surface lets a back face win."""
    sc = scenes.grid_scene(n_side=8, width=320, height=180)
    v = sc.views[0]
    f1, c1 = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height)
    mats = sc.materials.copy()
    mats["is_double_sided"] = 1
    f2, c2 = render_oracle(sc.meshlets, mats, v.world_to_clip, v.width, v.height)
    d1, d2 = f1.get_pixels(1).view(np.float32), f2.get_pixels(1).view(np.float32)
    assert np.all(d2 >= d1)
    assert (d1 != d2).mean() < 0.005
    assert c1[0] == c2[0] == 64 * 124 and c1[1] < c2[1]


@pytest.mark.parametrize("threads", [2, 3])
def test_threaded_strips_equal_single_thread(threads):
    sc = scenes.grid_scene(n_side=8, width=320, height=180)
    v = sc.views[0]
    f1, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height)
    fb = O.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    O.draw_meshlets(fb, O.Context(sc.meshlets, sc.materials, v.world_to_clip), len(sc.meshlets), threads=threads)
    assert np.array_equal(f1.data, fb.data)


def _resolve_scene(mode):
    from tests.helpers import TexturePair, default_lights
    sc = scenes.volume_scene(n=3000, width=320, height=180, n_materials=2, extent=30.0, texture_size=128, env_size=64)
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], 128, gpu=False) for i in range(2)]
    env = TexturePair([scenes.env_map_r11g11b10(64, 5)], 64, fmt=1, gpu=False)
    v = sc.views[0]
    fb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, v.width, v.height)
    ctx = O.Context(sc.meshlets, sc.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                    textures=[t.o for t in texs], lights=default_lights(), skybox=env.o, view_pos=v.eye)
    assert O.set_approx_mode(mode)
    try:
        O.resolve(fb, ctx)
    finally:
        O.set_approx_mode(0)
    return fb.get_pixels(0).view(np.uint8).reshape(v.height, v.width, 4).astype(np.int32)


@pytest.mark.skipif(not O.lib().orc_approx_mode_available(1), reason="needs an AVX-512 host")
def test_resolve_with_rcp14_tables_equals_instructions():
    """The resolve with the table restatement of rcp14/rsqrt14 (mode 0, what the GPU runs) is
    identical to the resolve with the AVX-512 instructions the reference runs (mode 1), while
    correctly rounded IEEE reciprocals (mode 2) change some pixels of this scene."""
    a, b, c = _resolve_scene(0), _resolve_scene(1), _resolve_scene(2)
    assert np.array_equal(a, b)
    d = np.abs(c - b).max(axis=2)
    assert 0 < (d > 0).sum() and d.max() <= 8


def test_resolve_is_deterministic_and_lit():
    a = _resolve_scene(0)
    assert np.array_equal(a, _resolve_scene(0))
    assert a[..., :3].std() > 10 and np.all(a[..., 3] == 255)
