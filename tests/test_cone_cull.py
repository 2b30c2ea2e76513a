"""Backface-cone culling on the CPU: the normal cones the scene builder and the meshlet builder
write (meshoptimizer's convention, as the reference's records carry them: Scene.h:18-19,
Scene.cpp:240-244), and the conservative cull test of swr_cull_meshlets_ex restated in numpy.

Every meshlet the test culls must have all its triangles facing away from the camera by a clear
margin: TrianglePacket::Setup's determinant (Rasterizer.cpp:262-266) of the projected vertices,
evaluated in float64, is negative by more than 1e-4 of its terms, so float32 rounding cannot flip
it. The test must also cull a good share of the open patch scene, and nothing of the closed
meshlets (whose cones are degenerate).
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes

MARGIN = np.float32(1.0 / 32.0)


def cone_culled(m, eye, double_sided=None):
    """The kernels' cone_culled (float32) for every record of m, camera at eye (object space)."""
    f32 = np.float32
    apex, axis = m["ConeApex"].astype(f32), m["ConeAxis"].astype(f32)
    cen, rad, cut = m["BoundCenter"].astype(f32), m["BoundRadius"].astype(f32), m["ConeCutoff"].astype(f32)
    d = apex - np.asarray(eye, f32)
    l2 = (d * d).sum(1, dtype=f32)
    proj = (d * axis).sum(1, dtype=f32)
    a2 = (axis * axis).sum(1, dtype=f32)
    reach = np.sqrt(((cen - apex) ** 2).sum(1, dtype=f32)) + rad
    cm = cut + MARGIN
    out = (cm < 1) & (proj > 0) & (a2 > 0.5) & (proj * proj >= cm * cm * l2 * a2) & (l2 >= 16 * reach * reach)
    if double_sided is not None:
        out &= ~double_sided
    return out


def face_dets(m, object_to_clip):
    """TrianglePacket::Setup's determinant of every live triangle (float64), its largest term, the
    live mask and the least clip w of its vertices (the determinant decides the face only where all
    three are in front of the camera; a triangle across the camera plane is clipped, and its pieces
    lie in its plane, facing the same way)."""
    M = np.asarray(object_to_clip, np.float64).reshape(4, 4)  # column-major: M[c, r]
    P = m["Positions"].astype(np.float64)                    # (n, 3, 64)
    clip = np.einsum("nkv,kr->nvr", P, M[:3]) + M[3][None, None, :]
    ndc = clip[..., :2] / clip[..., 3:4]
    idx = m["Indices"].astype(np.int64)                      # (n, 3, 128)
    nt = m["NumTriangles"].astype(np.int64)
    g = lambda k: np.take_along_axis(ndc, np.where(idx[:, k, :] < 32, idx[:, k, :], 32 + (idx[:, k, :] & 31))[..., None],
                                     axis=1)
    p0, p1, p2 = g(0), g(1), g(2)
    wv = clip[..., 3]
    w = np.minimum(np.minimum(np.take_along_axis(wv, idx[:, 0, :], axis=1), np.take_along_axis(wv, idx[:, 1, :], axis=1)),
                   np.take_along_axis(wv, idx[:, 2, :], axis=1))
    t1 = (p2[..., 0] - p0[..., 0]) * (p1[..., 1] - p0[..., 1])
    t2 = (p0[..., 0] - p1[..., 0]) * (p0[..., 1] - p2[..., 1])
    live = np.arange(128)[None, :] < nt[:, None]
    return t1 - t2, np.maximum(np.abs(t1), np.abs(t2)), live, w


@pytest.mark.parametrize("eye,target", [((0.0, 0.0, -130.0), (0.0, 0.0, 0.0)), ((60.0, 40.0, -20.0), (0.0, 5.0, 0.0)),
                                        ((5.0, -3.0, 2.0), (1.0, 0.0, 9.0))])
def test_culled_meshlets_face_away_by_a_margin(eye, target):
    sc = scenes.patch_scene(n=6000, width=640, height=360, extent=100.0, texture_size=8, env_size=8)
    m = sc.meshlets
    v = scenes.make_view(640, 360, eye=eye, target=target)
    culled = cone_culled(m, v.eye)
    assert culled.mean() > 0.10, f"only {culled.mean():.3f} of the patches culled"
    det, term, live, w = face_dets(m[culled], v.world_to_clip)
    front = w > 0
    sel = live & front
    rel = det[sel] / np.maximum(term[sel], 1e-300)
    assert rel.max() < -1e-4, f"a culled triangle faces the camera or is nearly edge-on: {rel.max():.3g}"


def test_closed_meshlets_have_degenerate_cones():
    sc = scenes.volume_scene(n=2000, width=640, height=360, n_materials=4, extent=40.0, texture_size=8, env_size=8)
    assert np.all(sc.meshlets["ConeCutoff"] == 1.0)
    assert not cone_culled(sc.meshlets, sc.views[0].eye).any()


def test_patch_cones_bound_their_normals():
    """The builder's cones: all triangle normals lie within the cone's half-angle of the axis, and
    the apex is behind every triangle's plane."""
    rng = np.random.default_rng(7)
    n = 500
    m = scenes.build_patch_meshlets(rng.uniform(-20, 20, (n, 3)), np.exp(rng.uniform(-2, 2, n)), np.zeros(n, int), rng)
    _, tris = scenes.patch_template()
    P = np.transpose(m["Positions"].astype(np.float64), (0, 2, 1))
    a, b, c = P[:, tris[:, 0]], P[:, tris[:, 1]], P[:, tris[:, 2]]
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    ok = m["ConeCutoff"] < 1
    assert ok.mean() > 0.99
    axis = m["ConeAxis"].astype(np.float64)
    cos_min = np.sqrt(1.0 - m["ConeCutoff"].astype(np.float64) ** 2)
    dots = np.einsum("ntk,nk->nt", nrm, axis)
    assert np.all(dots[ok] >= cos_min[ok, None] - 1e-5)
    behind = np.einsum("ntk,ntk->nt", m["ConeApex"].astype(np.float64)[:, None, :] - a, nrm)
    assert np.all(behind[ok] <= 1e-4 * np.exp(2))


def test_meshlet_builder_cones():
    """swr_build_meshlets on a flat grid (one cone of zero width) and a closed box (degenerate cones)."""
    import ctypes as C

    from glimpsw_gb300 import api

    lib = api.load_library()

    def build(pos, idx):
        pos = np.ascontiguousarray(pos, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        desc = api.SwrMeshDesc()
        desc.positions = pos.ctypes.data
        desc.num_vertices = len(pos)
        desc.indices = idx.ctypes.data
        desc.num_triangles = len(idx) // 3
        desc.material_id = 0xFFFFFFFF
        desc.alpha_cutoff = 255
        cap = lib.swr_meshlet_bound(desc.num_triangles)
        out = np.zeros(cap, dtype=scenes.MESHLET_DTYPE)
        cnt = C.c_uint32()
        assert lib.swr_build_meshlets(C.byref(desc), out.ctypes.data, cap, C.byref(cnt)) == 0
        return out[: cnt.value]

    g = np.arange(9, dtype=np.float32)
    gx, gz = np.meshgrid(g, g)
    pos = np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], 1)
    quads = [(r * 9 + c, (r + 1) * 9 + c, r * 9 + c + 1) for r in range(8) for c in range(8)]
    quads += [(r * 9 + c + 1, (r + 1) * 9 + c, (r + 1) * 9 + c + 1) for r in range(8) for c in range(8)]
    m = build(pos, np.array(quads).ravel())
    n = np.cross(pos[quads[0][1]] - pos[quads[0][0]], pos[quads[0][2]] - pos[quads[0][0]])
    n /= np.linalg.norm(n)
    assert np.all(m["ConeCutoff"] < 1e-3)
    assert np.allclose(m["ConeAxis"], n[None], atol=1e-5)
    # a camera on the side the normals point to keeps the grid, one behind it culls it
    assert not cone_culled(m, n * 50 + [4, 0, 4]).any()
    assert cone_culled(m, -n * 50 + [4, 0, 4]).all()
    # a closed cube: the cone of a meshlet holding several faces is degenerate
    box = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    faces = [(0, 1, 3), (0, 3, 2), (4, 6, 7), (4, 7, 5), (0, 4, 5), (0, 5, 1), (2, 3, 7), (2, 7, 6), (0, 2, 6),
             (0, 6, 4), (1, 5, 7), (1, 7, 3)]
    mb = build(box, np.array(faces).ravel())
    assert np.all(mb["ConeCutoff"] == 1.0)
