"""glTF import (Scene::ImportGltf, Scene.cpp:156-347) on the CPU: the PNG decoder, .gltf and .glb
giving the same model, the meshlet builder's invariants (every triangle exactly once, at most 64
vertices / 128 triangles, bounds containing their vertices), node transforms and lights, the
material rules (alpha cutoff, layer combination), an oracle render of the imported model, and the
reference's own Sponza_LowPoly asset where the reference tree is present."""
import os

import numpy as np
import pytest

from glimpsw_gb300 import gltf, scenes
from tests import gltf_fixtures

# The reference's own Sponza_LowPoly asset (assets/models/Sponza/Sponza_LowPoly.gltf in the reference
# tree), named by the SWR_SPONZA_GLTF environment variable; the tests that read it skip without it.
SPONZA = os.environ.get("SWR_SPONZA_GLTF", "")


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = tmp_path_factory.mktemp("gltf")
    return gltf_fixtures.build(str(d))


def _meshlet_triangles(m):
    """Triangles of the meshlets as sorted tuples of vertex positions."""
    out = []
    for r in m:
        P = r["Positions"]
        for i in range(int(r["NumTriangles"])):
            tri = []
            for k in range(3):
                v = int(r["Indices"][k][i])
                assert v < int(r["NumVertices"])
                tri.append((float(P[0][v]), float(P[1][v]), float(P[2][v])))
            out.append(tuple(sorted(tri)))
    return sorted(out)


def _check_meshlets(meshlets, positions, indices):
    assert np.all(meshlets["NumVertices"] <= 64) and np.all(meshlets["NumTriangles"] <= 128)
    assert np.all(meshlets["NumTriangles"] > 0)
    want = sorted(tuple(sorted(tuple(float(c) for c in positions[v]) for v in t)) for t in indices.reshape(-1, 3))
    assert _meshlet_triangles(meshlets) == want
    for r in meshlets:
        n = int(r["NumVertices"])
        p = np.stack([r["Positions"][a][:n] for a in range(3)], axis=1).astype(np.float64)
        d = np.linalg.norm(p - r["BoundCenter"].astype(np.float64), axis=1)
        assert np.all(d <= float(r["BoundRadius"]))
    # all but the last meshlet of a primitive are closed by the limits: >= 62 vertices or 128 triangles
    full = (meshlets["NumVertices"] >= 62) | (meshlets["NumTriangles"] == 128)
    assert full[:-1].all()


@pytest.mark.parametrize("color_type", [2, 6])
def test_png_decoder_every_filter(color_type):
    px = scenes.value_noise_rgba(37, 5, cells=1, layer=0, cutout=True)[:29]  # 29x37, odd sizes
    if color_type == 2:
        px = px | np.uint32(0xFF000000)
    assert np.array_equal(gltf.decode_png(gltf_fixtures.encode_png(px, color_type)), px)


def test_gltf_and_glb_import_the_same_model(files):
    a, b = gltf.load(files[0]), gltf.load(files[1])
    assert not a.warnings and not b.warnings
    assert np.array_equal(a.meshlets.view(np.uint8), b.meshlets.view(np.uint8))
    assert np.array_equal(a.materials, b.materials)
    assert len(a.textures) == len(b.textures) == 2
    for la, lb in zip(a.textures, b.textures):
        assert len(la) == len(lb) and all(np.array_equal(x, y) for x, y in zip(la, lb))
    assert [(i.meshlet_offset, i.meshlet_count) for i in a.instances] == [(i.meshlet_offset, i.meshlet_count) for i in b.instances]


def test_meshlets_cover_every_triangle_once(files):
    m = gltf.load(files[0])
    sp, st, *_ = gltf_fixtures._sphere()
    pp, pt, _ = gltf_fixtures._plane()
    sphere = m.meshlets[: m.instances[0].meshlet_count]
    plane = m.meshlets[m.instances[1].meshlet_offset: m.instances[1].meshlet_offset + m.instances[1].meshlet_count]
    _check_meshlets(sphere, sp, st)
    _check_meshlets(plane, pp, pt)
    assert np.all(sphere["MaterialId"] == 0) and np.all(sphere["AlphaCutoff"] == 255)
    assert np.all(plane["MaterialId"] == 1) and np.all(plane["AlphaCutoff"] == int(np.float32(0.45) * 255 + 0.5))
    # per-vertex words: texcoords of the sphere's vertices, handedness from the tangents' w
    assert np.any(sphere["TexCoords"] != 0) and np.any(sphere["TangentHandedness"] != 0)


def test_nodes_materials_and_lights(files):
    m = gltf.load(files[0])
    assert [i.node for i in m.instances] == [0, 1, 3]
    t0 = m.instances[0].transform.reshape(4, 4).T  # back to column vectors
    assert np.allclose(t0[:3, 3], [0, 1, 0]) and np.allclose(np.linalg.norm(t0[:3, 0]), 1.5)
    t3 = m.instances[2].transform.reshape(4, 4).T
    assert np.allclose(t3[:3, 3], [2.5, 0.5, 1.0]) and np.allclose(np.diag(t3)[:3], 0.5)
    t1 = m.instances[1].transform.reshape(4, 4).T
    assert np.allclose(t1[:3, 3], [0, -0.2, 0]) and np.allclose(np.diag(t1)[:3], 4.0)
    assert list(m.materials["is_double_sided"]) == [0, 1]
    assert len(m.textures[0]) == 2 and len(m.textures[1]) == 1  # normal + metal/rough combined into layer 1
    (light,) = m.lights
    assert light["type"] == 1 and np.allclose(light["position"], [0, 4, 0]) and light["radius"] == 12.0
    assert np.isclose(light["inv_radius_sq"], 1 / 144)


def test_combine_normal_mr_and_emissive_mask():
    n = np.array([[0xFF7F7FFF, 0x80FF7F7F]], dtype=np.uint32)   # (255,127,127) and (127,127,255)
    mr = np.array([[0x00336699, 0x00336699]], dtype=np.uint32)
    out = gltf.combine_normal_mr(n, mr)
    ch = np.stack([(out >> (8 * k)) & 255 for k in range(4)], axis=-1)
    assert ch[0, 0, 0] == 254 and ch[0, 1, 1] == 127 and np.all(ch[0, :, 2] == 0x33) and np.all(ch[0, :, 3] == 0x66)
    base = np.array([[0xFFFFFFFF, 0x80FFFFFF]], dtype=np.uint32)
    em = np.array([[0x00000009, 0x00000000]], dtype=np.uint32)
    masked = gltf.insert_emissive_mask(base, em)
    assert masked[0, 0] >> 24 == 255 and masked[0, 1] >> 24 == 0x80


def test_oracle_renders_the_imported_model(files):
    from oracle import oracle as O
    from tests.helpers import TexturePair
    m = gltf.load(files[0])
    texs = [TexturePair(layers, layers[0].shape[0], gpu=False) for layers in m.textures]
    v = scenes.make_view(320, 192, eye=(0.0, 3.0, -6.0), target=(0.5, 0.5, 0.0))
    fb = O.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    for inst in m.instances:
        bm, _ = O.cull_meshlets(m.meshlets[inst.meshlet_offset:], inst.meshlet_count, v.proj, v.view, inst.transform,
                                v.view, v.width, v.height)
        ctx = O.Context(m.meshlets, m.materials, scenes.mat_mul(v.world_to_clip, inst.transform),
                        meshlet_offset=inst.meshlet_offset, cull_bitmap=bm, textures=[t.o for t in texs])
        O.draw_meshlets(fb, ctx, inst.meshlet_count)
    ids = fb.get_pixels(0)
    drawn = ids[ids != 0xFF000000] // 128
    assert len(drawn) > 5000
    assert set(np.unique(drawn)) & set(range(m.instances[1].meshlet_offset, len(m.meshlets)))  # the plane shows


@pytest.mark.skipif(not os.path.exists(SPONZA), reason="the reference's Sponza_LowPoly asset is not present")
def test_reference_sponza_lowpoly():
    import json
    m = gltf.load(SPONZA)
    assert not m.warnings and len(m.instances) == 2 and len(m.materials) == 0
    assert int(m.meshlets["NumTriangles"].sum()) == (175905 + 13347) // 3
    doc = json.load(open(SPONZA))
    bufs = gltf._buffers(doc, os.path.dirname(SPONZA), None)
    for inst, (pa, ia) in zip(m.instances, ((0, 1), (2, 3))):
        pos = gltf.read_accessor(doc, bufs, pa)
        idx = gltf.read_accessor(doc, bufs, ia).reshape(-1)
        sub = m.meshlets[inst.meshlet_offset: inst.meshlet_offset + inst.meshlet_count]
        _check_meshlets(sub, pos, idx)
        assert np.all(sub["MaterialId"] == 0xFFFFFFFF)
