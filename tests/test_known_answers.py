"""Known answers for the resolve's and the sampler's building blocks in the oracle, derived by hand
from the reference's formulas (the reference ships no tests or golden vectors, so these pin the
restatement on values worked out independently of it):

* simd::lerp16 (SIMD.h:450): a + mulhrs(b - a, t) per 16-bit half, mulhrs(x, t) = (x t + 2^14) >> 15;
* RGBA8u::UnpackSrgb (Texture.h:37-54): c = (256 v + 255)^2 >> 16 (mulhi squaring) scaled by 1/65535,
  alpha (256 a + 255) / 65535 unsquared;
* R11G11B10f unpack (Texture.h:170-182): exponent rebias only, no denormals (code 0 reads 2^-15);
* texutil::CalcMipLevel (Texture.h:276-280): ilog2(max(|d/dx|^2 sx^2, |d/dy|^2 sy^2)) >> 1, with the
  x86 default NaN for NaN gradients;
* texutil::MapOctahedron / UnmapOctahedron (Texture.h:282-296) at the poles, the equator and the
  seams (every corner of the square is the -z pole);
* SampleLevel<SurfaceSampler> (Texture.h:412-459, 506-556) on an 8x8 ramp at texel centres, across
  the right edge (the right neighbour is masked, not wrapped), at u = 1 (Repeat wraps to texel 0),
  between texels (the 1.15 fixed-point weight), and with a minified lane (nearest for the whole
  tile, from the box-filtered mip).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O


def _f(v):
    return np.float32(v)


def test_lerp16():
    L = O.lib()
    assert L.orc_debug_lerp16(0x00000000, 0x00FF00FF, 0x40004000) == 0x00800080  # (255 * 2^14 + 2^14) >> 15 = 128
    assert L.orc_debug_lerp16(0x00FF00FF, 0x00000000, 0x40004000) == 0x00800080  # 255 + (-4161536 >> 15) = 255 - 127
    assert L.orc_debug_lerp16(0x00120034, 0x00560078, 0) == 0x00120034          # t = 0: a
    assert L.orc_debug_lerp16(0x0000000A, 0x00FF0014, 0x7FFF7FFF) == 0x00FF0014  # t = 1 - 2^-15 still reaches b


def test_unpack_srgb():
    out = (C.c_float * 4)()
    O.lib().orc_debug_unpack_srgb(0xFF8000FF, out)  # R 255, G 0, B 128, A 255
    s = _f(1.0) / _f(65535)
    assert out[0] == _f(65534) * s          # 65535^2 >> 16 = 65534
    assert out[1] == 0.0                     # 255^2 >> 16 = 0
    assert out[2] == _f(16639) * s          # 33023^2 = 1090518529, >> 16 = 16639
    assert out[3] == _f(65535) * s          # alpha: (256 * 255 + 255) / 65535, not squared


def test_unpack_r11g11b10():
    out = (C.c_float * 3)()
    L = O.lib()
    L.orc_debug_unpack_r11g11b10((0x3C0 << 21) | (0x3C1 << 10) | 0x1E0, out)
    assert list(out) == [1.0, 1.015625, 1.0]  # exponent 15 = 2^0; mantissa 1/64 on G
    L.orc_debug_unpack_r11g11b10((0x7FF << 21) | (0 << 10) | 0x3FF, out)
    assert list(out) == [130048.0, 2.0 ** -15, 129024.0]  # the largest codes; code 0 is 2^-15


@pytest.mark.parametrize("grad,expected", [
    ((1 / 64, 0, 0, 1 / 64), 0),        # one texel per pixel
    ((4 / 64, 0, 0, 0), 2),             # 16 -> ilog2 4 -> 2
    ((3 / 64, 0, 0, 0), 1),             # 9 -> ilog2 3 -> 1
    ((0.5 / 64, 0, 0, 0), -1),          # magnified: 1/4 -> ilog2 -2 -> -1
    ((0, 0, 0, 0), -64),                # 0.0: (0 - 127 << 23) >> 23 = -127, >> 1 = -64
    ((float("nan"), 0, 0, 0), -64),     # x86 NaN 0xFFC00000: -1069547520 >> 23 = -128, >> 1 = -64
])
def test_calc_mip_level(grad, expected):
    assert O.lib().orc_debug_calc_mip_level(*[C.c_float(g) for g in grad], C.c_float(64), C.c_float(64)) == expected


def _map(n):
    uv = (C.c_float * 2)()
    O.lib().orc_debug_map_oct((C.c_float * 3)(*n), uv)
    return list(uv)


def _unmap(uv):
    n = (C.c_float * 3)()
    O.lib().orc_debug_unmap_oct((C.c_float * 2)(*uv), n)
    return list(n)


def test_octahedral_poles_equator_and_seams():
    assert _map((0.0, 0.0, 1.0)) == [0.5, 0.5]     # +z: the centre
    assert _map((1.0, 0.0, 0.0)) == [1.0, 0.5]     # equator: the edge midpoint
    assert _map((0.0, 0.0, -1.0)) == [1.0, 1.0]    # -z folds to a corner (the sign of +0 picks which)
    assert _map((-0.0, -0.0, -1.0)) == [0.0, 0.0]
    assert _unmap((0.5, 0.5)) == [0.0, 0.0, 1.0]
    assert _unmap((1.0, 0.5)) == [1.0, 0.0, 0.0]
    for corner in ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0)):
        assert _unmap(corner) == [0.0, 0.0, -1.0]  # every corner is the -z pole


@pytest.fixture(scope="module")
def ramp():
    """8x8 RGBA8 texture, texel (x, y) = (16 x, 16 y, 0, 255), full mips."""
    t = O.Texture(8, 8, 16, 1)
    y, x = np.mgrid[0:8, 0:8]
    t.set_pixels(((16 * x) | ((16 * y) << 8) | (255 << 24)).astype(np.uint32), 0)
    t.generate_mips()
    return t


def _sample(t, us, vs, mips):
    u = (C.c_float * 16)(*[_f(a) for a in us])
    v = (C.c_float * 16)(*[_f(b) for b in vs])
    m = (C.c_int32 * 16)(*mips)
    out = (C.c_uint32 * 16)()
    O.lib().orc_debug_sample_rgba8(C.byref(t.s), u, v, 0, m, out)
    return [(o & 255, (o >> 8) & 255) for o in out]


def test_sampler_texel_centres_and_edges(ramp):
    # texel centres: the weight is 1 / 256 of the right neighbour, rounded away by mulhrs: exact texels
    xs = list(range(8)) * 2
    got = _sample(ramp, [(x + 0.5) / 8 for x in xs], [(3 + 0.5) / 8] * 16, [0] * 16)
    assert got == [(16 * x, 48) for x in xs]
    # u = 0.99: texel 7, weight 109 / 256 towards a right neighbour outside the texture: masked, not
    # wrapped to texel 0; u = 1: su = 2048 wraps (Repeat) to texel 0; u = 0: texel 0 (no left blend);
    # u = 3/8: texel 2 blended with texel 3 at 129/256: 32 + ((16 * 16512 + 16384) >> 15) = 40
    got = _sample(ramp, [0.99, 1.0, 0.0, 0.375] * 4, [0.5 / 8] * 16, [0] * 16)
    assert [g[0] for g in got[:4]] == [112, 0, 0, 40]


def test_sampler_minified_lane_picks_nearest_for_the_tile(ramp):
    # one lane at mip 1 makes the whole tile nearest (no -127 half-texel shift): at u = 3/8, v = 1/16
    # su = 768, sv = 128. That lane reads the 4x4 level's texel (768 >> 1 >> 8, 128 >> 1 >> 8) = (1, 0),
    # the box filter of level-0 texels 2..3 x 0..1: R = (32 + 48) / 2 = 40, G = (0 + 16) / 2 = 8; the
    # others read level-0 texel (3, 0) directly: R = 48, G = 0. Bilinear at mip 0 would give R = 40.
    got = _sample(ramp, [0.375] * 16, [0.5 / 8] * 16, [1] + [0] * 15)
    assert got[0] == (40, 8)
    assert all(g == (48, 0) for g in got[1:])
    assert all(g == (40, 0) for g in _sample(ramp, [0.375] * 16, [0.5 / 8] * 16, [0] * 16))
