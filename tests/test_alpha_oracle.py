"""The oracle's alpha-tested vis-buffer shader (FS_EncodeSurfaceId<true>, Shading.cpp:309-331) on
the CPU: properties that pin its meaning without a GPU.

* A texture that is opaque everywhere, a cutoff of 0 and a material without a texture all draw
  exactly what the opaque shader draws.
* A texture that is transparent everywhere draws nothing of that material.
* A known answer: a screen-aligned quad whose texture is opaque on its left half and transparent on
  its right half keeps the left half of its pixels (bilinear magnification puts the edge at u = 1/2).
* Noise alpha removes a real share of the material's fragments, and only fragments of alpha-tested
  materials change.
"""
import numpy as np

from glimpsw_gb300 import scenes
from tests.helpers import CLIP_FROM_OBJECT, TexturePair, render_oracle

EMPTY = 0xFF000000


def _scene():
    sc = scenes.grid_scene(n_side=16, width=320, height=192, texture_size=64)
    m = sc.meshlets.copy()
    m["MaterialId"] = np.arange(len(m)) % 2
    return sc, m


def _mats(cutoffs, textures=(0, 1)):
    mats = np.zeros(len(cutoffs), dtype=scenes.MATERIAL_DTYPE)
    mats["texture"] = textures
    mats["alpha_cutoff"] = cutoffs
    return mats


def _render(m, mats, v, textures):
    fb, counters = render_oracle(m, mats, v.world_to_clip, v.width, v.height, textures=[t.o for t in textures])
    return fb.get_pixels(0), fb.get_pixels(1), counters


def _textures(cutout, alpha=None):
    out = []
    for seed in (3, 4):
        px = scenes.value_noise_rgba(64, seed, layer=0, cutout=cutout)
        if alpha is not None:
            px = (px & 0x00FFFFFF) | np.uint32(alpha << 24)
        out.append(TexturePair([px], 64, gpu=False))
    return out


def test_opaque_texture_zero_cutoff_and_untextured_draw_as_opaque():
    sc, m = _scene()
    v = sc.views[0]
    noise = _textures(True)
    ids0, d0, c0 = _render(m, _mats([255, 255]), v, noise)
    for mats, texs in [(_mats([255, 128]), _textures(False)),          # alpha 255 everywhere
                       (_mats([255, 0]), noise),                       # cutoff 0 passes every texel
                       (_mats([255, 128], textures=(0, 0xFFFFFFFF)), noise)]:  # no texture
        ids, d, c = _render(m, mats, v, texs)
        assert np.array_equal(ids, ids0) and np.array_equal(d, d0)
        assert list(c[:3]) == list(c0[:3])


def test_transparent_texture_draws_nothing_of_its_material():
    sc, m = _scene()
    v = sc.views[0]
    ids, _, _ = _render(m, _mats([255, 128]), v, _textures(False, alpha=0))
    drawn = ids[ids != EMPTY]
    assert len(drawn) > 0
    assert np.all(m["MaterialId"][drawn // 128] == 0)


def test_noise_alpha_removes_only_alpha_tested_fragments():
    sc, m = _scene()
    v = sc.views[0]
    noise = _textures(True)
    ids0, _, _ = _render(m, _mats([255, 255]), v, noise)
    ids, _, _ = _render(m, _mats([255, 128]), v, noise)
    mat_of = m["MaterialId"].astype(np.int64)[np.minimum(ids0, len(m) * 128 - 1) // 128]
    mat0 = np.where(ids0 != EMPTY, mat_of, -1)
    lost = (ids != ids0) & (mat0 == 1)
    assert lost.sum() > 0.1 * (mat0 == 1).sum()   # noise alpha around 128 cuts a real share
    # where a pixel changed, the opaque frame showed the alpha-tested material there
    assert np.all(mat0[ids != ids0] == 1)


def test_half_transparent_quad_keeps_its_left_half():
    """Quad over pixels [16, 48)^2 of a 64x64 frame, w = 1, u from 0 (left) to 1 (right); its 8x8
    texture is opaque in texel columns 0-3 and transparent in 4-7."""
    W = H = 64
    q = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [-0.5, 0.5]], dtype=np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float16)
    m = np.zeros(1, dtype=scenes.MESHLET_DTYPE)
    m["Positions"][0, 0, :4] = q[:, 0]
    m["Positions"][0, 1, :4] = q[:, 1]
    m["Positions"][0, 2, :4] = 1.0
    tc = uv.view(np.uint16).astype(np.uint32)
    m["TexCoords"][0, :4] = tc[:, 0] | (tc[:, 1] << 16)
    m["NumVertices"] = 4
    m["NumTriangles"] = 2
    m["AlphaCutoff"] = 255
    idx = np.zeros((3, 128), dtype=np.uint8)
    idx[:, 0] = [0, 1, 2]
    idx[:, 1] = [0, 2, 3]
    m["Indices"] = idx[None]
    mats = np.zeros(1, dtype=scenes.MATERIAL_DTYPE)
    mats["alpha_cutoff"] = 128
    mats["is_double_sided"] = 1
    px = np.full((8, 8), 0x00808080, dtype=np.uint32)
    px[:, :4] |= np.uint32(0xFF000000)
    tex = TexturePair([px], 8, gpu=False)
    fb, _ = render_oracle(m, mats, CLIP_FROM_OBJECT, W, H, textures=[tex.o])
    ids = fb.get_pixels(0)
    drawn = ids != EMPTY
    assert drawn[16:48, 16:31].all()        # u < 1/2 - 1/64: opaque side
    assert not drawn[:, 33:].any()          # u > 1/2 + 1/64: cut away
    assert not drawn[:, :16].any() and not drawn[:16].any() and not drawn[48:].any()
