"""Image-based lighting precompute on the GPU (swr_ibl_*) against the oracle, bit for bit: the
64x64 irradiance map (1024 of its texels), every mip level of the 256x256 radiance map (texels of each
level), and the whole 128x128 environment-BRDF table, from the same 8-bit-quantised R11G11B10
octahedral environment map with mips."""
import numpy as np
import pytest

from glimpsw_gb300 import scenes

pytestmark = pytest.mark.gpu


def _tiled(x, y, row_shift):
    return (y & 7) | (x << 3) | ((y & ~7) << row_shift)


@pytest.fixture(scope="module")
def env():
    from glimpsw_gb300 import api
    from tests.helpers import TexturePair
    api.load_library()
    return TexturePair([scenes.env_map_r11g11b10(128, 5)], 128, fmt=1)


def test_irradiance_map_bit_exact(env):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    out = api.Texture2D(api.FORMAT_R11G11B10F, 64, 64, 1, 1)
    api._check(api._lib.swr_ibl_irradiance_map(env.g.h, out.h))
    data = out.get_data()
    rs = int(np.log2(64))
    rng = np.random.default_rng(2)
    pts = rng.integers(0, 64, (1024, 2))
    got = np.array([data[_tiled(x, y, rs)] for x, y in pts], np.uint32)
    exp = np.array([O.ibl_irradiance_texel(env.o, int(x), int(y), 64, 64) for x, y in pts], np.uint32)
    assert np.array_equal(got, exp), f"{(got != exp).sum()} of {len(pts)} texels differ"
    assert len(np.unique(exp)) > 100


@pytest.mark.parametrize("w,h", [(8, 4), (16, 8)])
def test_small_irradiance_maps_bit_exact(env, w, h):
    """The smallest map (8x4: one block of 32 texels) and a non-square one, every texel."""
    from glimpsw_gb300 import api
    from oracle import oracle as O
    out = api.Texture2D(api.FORMAT_R11G11B10F, w, h, 1, 1)
    api._check(api._lib.swr_ibl_irradiance_map(env.g.h, out.h))
    data = out.get_data()
    rs = int(np.log2(w))
    got = np.array([[data[_tiled(x, y, rs)] for x in range(w)] for y in range(h)], np.uint32)
    exp = np.array([[O.ibl_irradiance_texel(env.o, x, y, w, h) for x in range(w)] for y in range(h)], np.uint32)
    assert np.array_equal(got, exp), f"{(got != exp).sum()} of {w * h} texels differ"


def test_radiance_map_bit_exact(env):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    out = api.Texture2D(api.FORMAT_R11G11B10F, 256, 256, 8, 1)
    api._check(api._lib.swr_ibl_radiance_map(env.g.h, out.h))
    data = out.get_data()
    rng = np.random.default_rng(3)
    levels = out.mip_levels
    for level in range(levels):
        w = 256 >> level
        pts = rng.integers(0, w, (96, 2))
        got = np.array([data[out.mip_offsets[level] + _tiled(x, y, 8 - level)] for x, y in pts], np.uint32)
        exp = np.array([O.ibl_radiance_texel(env.o, level, levels, int(x), int(y), 256, 256) for x, y in pts], np.uint32)
        assert np.array_equal(got, exp), f"level {level}: {(got != exp).sum()} texels differ"


def test_env_brdf_lut_bit_exact():
    from glimpsw_gb300 import api
    from oracle import oracle as O
    out = api.Texture2D(api.FORMAT_RG16F, 128, 128, 1, 1)
    api._check(api._lib.swr_ibl_env_brdf_lut(out.h))
    data = out.get_data()
    got = np.array([[data[_tiled(x, y, 7)] for x in range(128)] for y in range(128)], np.uint32)
    exp = np.array([[O.ibl_env_brdf_texel(x, y, 128, 128) for x in range(128)] for y in range(128)], np.uint32)
    assert np.array_equal(got, exp), f"{(got != exp).sum()} texels differ"
