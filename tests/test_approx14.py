"""The integer restatement of VRCP14PS / VRSQRT14PS (include/swr/approx14.h) against the
instructions themselves (on an AVX-512 host), and its numpy and importer users.

The reference calls the instructions through simd::approx_rcp / approx_rsqrt / approx_sqrt
(src/SwRast/SIMD.h:294-296) in culling (ProjectSphere, Shading.cpp:264-279), the alpha test's
perspective correction (Rasterizer.h:306-307), lighting (Shading.cpp:17-33, 581-645), normal
reconstruction (Shading.cpp:563) and octahedral mapping (Texture.h:282-288). The oracle and the
kernels share the tables; these tests pin the tables to the hardware.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

from glimpsw_gb300 import approx14 as A
from oracle import oracle as O

needs_avx512 = pytest.mark.skipif(not O.lib().orc_approx_mode_available(1), reason="needs an AVX-512 host")

SPECIALS = np.array([0, 0x80000000, 1, 0x00400000, 0x007FFFFF, 0x00800000, 0x00800001, 0x3F800000, 0x40000000,
                     0x40800000, 0xBF800000, 0xBFC00000, 0x7E800000, 0x7E800001, 0x7EFFFFFF, 0x7F000000, 0x7F000001,
                     0x7F7FFFFF, 0x7F800000, 0xFF800000, 0x7FC00000, 0x7F800001, 0xFFC00001, 0x00200000, 0x80400000],
                    dtype=np.uint32)


@needs_avx512
@pytest.mark.parametrize("which", [0, 1], ids=["rcp14", "rsqrt14"])
def test_tables_equal_instruction_on_whole_binades(which):
    """Every mantissa of 13 exponents (denormals, the normal range's ends, both parities, inf/NaN)
    of both signs: 218M inputs per instruction."""
    for e in (0, 1, 2, 100, 125, 126, 127, 128, 129, 200, 253, 254, 255):
        for sign in (0, 1):
            first = (sign << 31) | (e << 23)
            assert O.approx14_mismatches(which, first, 1 << 23) == 0, f"exponent {e} sign {sign}"


@needs_avx512
def test_tables_equal_instruction_on_random_and_special_inputs():
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.integers(0, 2**32, 2_000_000, dtype=np.uint64).astype(np.uint32), SPECIALS]).view(np.float32)
    for which in (0, 1):
        assert O.set_approx_mode(1)
        try:
            hw = O.approx_eval(which, x).view(np.uint32)
        finally:
            O.set_approx_mode(0)
        assert np.array_equal(O.approx_eval(which, x).view(np.uint32), hw)


def test_numpy_rcp14_equals_tables():
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32), SPECIALS]).view(np.float32)
    O.set_approx_mode(0)
    assert np.array_equal(A.rcp14(x).view(np.uint32), O.approx_eval(0, x).view(np.uint32))


def test_tables_known_answers():
    """Hand-checkable points: exact powers give exact results; rcp14(3) and rsqrt14(2) carry the
    instruction's 17-bit significands; the bound |rcp14(x) x - 1| < 2^-14 holds."""
    O.set_approx_mode(0)
    x = np.array([1.0, 2.0, 0.25, 4.0, 3.0], dtype=np.float32)
    assert O.approx_eval(0, x[:3]).tolist() == [1.0, 0.5, 4.0]
    assert O.approx_eval(1, x[[0, 2, 3]]).tolist() == [1.0, 2.0, 0.5]
    assert O.approx_eval(0, x[4:]).view(np.uint32)[0] == 0x3EAAAA80
    assert O.approx_eval(1, np.float32([2.0])).view(np.uint32)[0] == 0x3F350280
    rng = np.random.default_rng(13)
    y = rng.uniform(1e-30, 1e30, 100_000).astype(np.float32)
    r = O.approx_eval(0, y).astype(np.float64)
    assert np.abs(r * y - 1).max() < 2.0 ** -14
    q = O.approx_eval(1, y).astype(np.float64)
    assert np.abs(q * q * y - 1).max() < 2.0 ** -13


def test_fma32_is_one_rounding():
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.fmaf.restype = ctypes.c_float
    libm.fmaf.argtypes = [ctypes.c_float] * 3
    rng = np.random.default_rng(14)
    n = 20_000
    a = rng.integers(-4096, 4096, n).astype(np.float32)
    b = (rng.integers(-4096, 4096, n) * 2.0 ** -12).astype(np.float32)
    c = (rng.integers(-(2 ** 20), 2 ** 20, n) * 2.0 ** -24).astype(np.float32)
    a = np.concatenate([a, rng.standard_normal(n).astype(np.float32)])
    b = np.concatenate([b, rng.standard_normal(n).astype(np.float32)])
    c = np.concatenate([c, (rng.standard_normal(n) * 1e-3).astype(np.float32)])
    want = np.array([libm.fmaf(float(p), float(q), float(r)) for p, q, r in zip(a, b, c)], dtype=np.float32)
    assert np.array_equal(A.fma32(a, b, c).view(np.uint32), want.view(np.uint32))


def test_map_octahedron_follows_reference_ops():
    """gltf.map_octahedron against a scalar restatement of Texture.h:282-288 with the oracle's
    rcp14 and libm's fmaf."""
    from glimpsw_gb300 import gltf
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.fmaf.restype = ctypes.c_float
    libm.fmaf.argtypes = [ctypes.c_float] * 3
    rng = np.random.default_rng(15)
    n = rng.standard_normal((5000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True).astype(np.float32)
    got = gltf.map_octahedron(n)
    O.set_approx_mode(0)
    w = O.approx_eval(0, (np.abs(n[:, 0]) + np.abs(n[:, 1]) + np.abs(n[:, 2])).astype(np.float32))
    for i in range(len(n)):
        x, y, z = (np.float32(c) for c in n[i])
        t = max(np.float32(-z * w[i]), np.float32(0.0))
        u = np.float32(libm.fmaf(float(x), float(w[i]), float(np.copysign(t, x))))
        v = np.float32(libm.fmaf(float(y), float(w[i]), float(np.copysign(t, y))))
        assert got[i, 0] == np.float32(u * np.float32(0.5) + np.float32(0.5))
        assert got[i, 1] == np.float32(v * np.float32(0.5) + np.float32(0.5))
