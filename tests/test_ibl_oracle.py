"""The oracle's image-based lighting precompute (Shading.cpp:35-219) on known inputs: a constant
environment map has that constant as its irradiance and as its prefiltered radiance at every
roughness (the integrals' weights are normalised), and the split-sum BRDF table has the known shape
(scale + bias <= 1, the scale rising towards 1 and the bias falling towards 0 for smooth surfaces
seen head-on)."""
import numpy as np

from oracle import oracle as O


def _pack_r11g11b10(v):
    f = np.float32(v).view(np.uint32)
    return ((int(f) >> 17 & 0x3FFF) - 0x1C00) << 21 | ((int(f) >> 17 & 0x3FFF) - 0x1C00) << 10 | ((int(f) >> 18 & 0x1FFF) - 0x0E00)


def _unpack(p):
    def f11(x):
        return np.uint32(((x << 17) & 0x0FFE0000) + 0x38000000).view(np.float32)

    def f10(x):
        return np.uint32(((x << 18) & 0x0FFC0000) + 0x38000000).view(np.float32)
    return float(f11(p >> 21)), float(f11((p >> 10) & 0x7FF)), float(f10(p & 0x3FF))


def _constant_env(value=2.0, size=64):
    env = O.Texture(size, size, 16, 1, fmt=1)
    env.set_pixels(np.full((size, size), _pack_r11g11b10(value), np.uint32), 0)
    env.generate_mips()
    return env


def test_constant_environment_irradiance_and_radiance():
    env = _constant_env(2.0)
    rng = np.random.default_rng(1)
    for x, y in rng.integers(0, 64, (8, 2)):
        r = _unpack(O.ibl_irradiance_texel(env, int(x), int(y), 64, 64))
        assert np.allclose(r, 2.0, rtol=0.02), r
    for level in range(7):
        w = 256 >> level
        x, y = rng.integers(0, w, 2)
        r = _unpack(O.ibl_radiance_texel(env, level, 7, int(x), int(y), 256, 256))
        assert np.allclose(r, 2.0, rtol=0.02), (level, r)


def test_env_brdf_table_shape():
    def h2f(h):
        return float(np.array([h], np.uint16).view(np.float16)[0])
    tab = np.array([[O.ibl_env_brdf_texel(x, y, 32, 32) for x in range(32)] for y in range(32)], np.uint32)
    scale = np.vectorize(h2f)(tab & 0xFFFF)
    bias = np.vectorize(h2f)(tab >> 16)
    assert np.all(scale >= 0) and np.all(bias >= 0) and np.all(scale + bias <= 1.001)
    assert scale[0, -1] > 0.95 and bias[0, -1] < 0.02      # smooth, head-on
    assert np.all(np.diff(scale[0]) >= -1e-3)              # smooth: the scale rises with NoV
    assert bias[0, 0] > bias[0, -1]
