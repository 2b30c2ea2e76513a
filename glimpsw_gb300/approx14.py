"""VRCP14PS (simd::approx_rcp, SIMD.h:295) for numpy arrays, bit for bit.

Host-side data preparation (the glTF importer's octahedral normal packing, Scene.cpp:270-272 ->
texutil::MapOctahedron, Texture.h:282-288) runs the reference's approx_rcp. This restates the
integer segment tables of include/swr/approx14.h, the same ones the kernels use, reading them
from that header so there is one copy of the data.
"""
from __future__ import annotations

import os
import re

import numpy as np

_HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "swr", "approx14.h")
_segments = None


def segments() -> np.ndarray:
    """(128, 2) int64 array of (A, B): rows 0-63 rcp14, 64-95 / 96-127 rsqrt14 (even / odd exponent)."""
    global _segments
    if _segments is None:
        text = open(_HEADER).read()
        body = text[text.index("#define SWR_A14_SEGMENTS"):]
        body = body[:body.index("\n    }") + 1]
        pairs = re.findall(r"\{(\d+)u, (\d+)u\}", body)
        if len(pairs) != 128:
            raise RuntimeError(f"{_HEADER}: expected 128 segments, found {len(pairs)}")
        _segments = np.array(pairs, dtype=np.int64)
    return _segments


def rcp14(x: np.ndarray) -> np.ndarray:
    """Element-wise VRCP14PS of a float32 array (same rules as swr_rcp14 in approx14.h)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.int64)
    sign = u & 0x80000000
    e = (u >> 23) & 0xFF
    m = u & 0x7FFFFF
    # denormal inputs: normalise the mantissa, exponent 1 - shift
    den = (e == 0) & (m != 0)
    sh = np.where(den, 23 - np.floor(np.log2(np.maximum(m, 1))).astype(np.int64), 0)
    m = np.where(den, (m << sh) & 0x7FFFFF, m)
    E = np.where(den, 1 - sh, e)
    seg = segments()[:64]
    i = m >> 17
    sig = ((seg[i, 0] - seg[i, 1] * ((m >> 7) & 1023)) >> 9) << 7
    re_ = 253 - E
    exact = m == 0
    sig = np.where(exact, 0x800000, sig)
    re_ = np.where(exact, re_ + 1, re_)
    normal = sign | (np.clip(re_, 0, 255) << 23) | (sig & 0x7FFFFF)
    sub = sign | (sig >> np.clip(1 - re_, 0, 31))
    out = np.where(re_ >= 1, normal, sub)
    out = np.where(re_ >= 255, sign | 0x7F800000, out)
    out = np.where((e == 0) & (m == 0) & ~den, sign | 0x7F800000, out)          # +-0 -> +-inf
    out = np.where(e == 0xFF, np.where((u & 0x7FFFFF) != 0, u | 0x400000, sign), out)  # NaN, inf
    return out.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def fma32(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Correctly rounded float32 a*b + c (one rounding), for normal-range results.

    The float32 product is exact in float64; TwoSum gives s + e == a*b + c exactly. Rounding s to
    float32 is then correct unless s lies exactly on a float32 rounding midpoint, where the sign of
    e decides: s moves one float64 step towards e first."""
    a64, b64, c64 = (np.asarray(v, dtype=np.float32).astype(np.float64) for v in (a, b, c))
    p = a64 * b64
    s = p + c64
    bv = s - p
    e = (p - (s - bv)) + (c64 - bv)
    low = s.view(np.uint64) & np.uint64((1 << 29) - 1)
    midpoint = (low == np.uint64(1 << 28)) & (e != 0)
    s = np.where(midpoint, np.nextafter(s, s + e), s)
    return s.astype(np.float32)
