"""Generate include/swr/approx14.h: exact integer tables of the AVX-512 reciprocal approximations.

The reference's shading and culling code calls `simd::approx_rcp` and `simd::approx_rsqrt`
(src/SwRast/SIMD.h:294-296), i.e. the x86 instructions VRCP14PS and VRSQRT14PS. Their results are
not specified beyond a 2^-14 relative error bound, so this script measures them on an AVX-512 host
and fits the measurement with piecewise-linear integer segments:

- rcp14, input 1.m x 2^e: index i = m[22:17] (64 segments), t = m[16:7]; the 17-bit result
  significand q (value q x 2^-17 in (0.5, 1)) is (A[i] - B[i] * t) >> 9. Bits m[6:0] are ignored.
- rsqrt14: index i = m[22:18] (32 segments per exponent parity), t = m[17:8];
  q = (A[i] - B[i] * t) >> 9 with value q x 2^-17 in [0.5, 1). Bits m[7:0] are ignored.
- inputs with m == 0 (exact powers of two for rcp14, of four for rsqrt14) give the exact result.

Every segment is solved exactly: for each candidate slope B the feasible A interval is the
intersection over all t of [q*512 + B*t, (q+1)*512 + B*t - 1]; the script requires it to be
non-empty and takes its lower end. The emitted header is checked against the instructions over
all 2^32 inputs by `orc_approx14_mismatches` (oracle) in the CPU tests.

Run on an x86-64 host with AVX-512F:  python -m glimpsw_gb300.gen_approx14
"""
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "include", "swr", "approx14.h")

PROBE_C = r"""
#include <immintrin.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
/* argv: which (0 rcp14, 1 rsqrt14), biased exponent, index bits. Writes one result word per index
   for inputs (exponent, mantissa = index << (23 - bits) | 1). */
__attribute__((target("avx512f"))) int main(int argc, char** argv) {
    int which = atoi(argv[1]), e = atoi(argv[2]), bits = atoi(argv[3]);
    uint32_t n = 1u << bits;
    for (uint32_t i = 0; i < n; i += 16) {
        uint32_t in[16], out[16];
        for (int j = 0; j < 16; j++) in[j] = ((uint32_t)e << 23) | ((i + j) << (23 - bits)) | 1u;
        __m512 v; memcpy(&v, in, 64);
        __m512 r = which ? _mm512_rsqrt14_ps(v) : _mm512_rcp14_ps(v);
        memcpy(out, &r, 64);
        fwrite(out, 4, 16, stdout);
    }
    return 0;
}
"""


def _probe(which: int, exponent: int, bits: int, exe: str) -> np.ndarray:
    raw = subprocess.run([exe, str(which), str(exponent), str(bits)], check=True, capture_output=True).stdout
    return np.frombuffer(raw, dtype=np.uint32)


def _significand17(words: np.ndarray, top_exponent: int) -> np.ndarray:
    """Result significand in units of 2^-17 of a value in [0.5, 1): results with the top exponent
    (exactly 1.0 and above) do not occur for the sampled inputs."""
    e = (words >> 23) & 0xFF
    assert np.all(e == top_exponent), "unexpected result exponent"
    y = (words & 0x7FFFFF).astype(np.int64) | (1 << 23)
    assert np.all(y & 0x7F == 0), "result has more than 17 significant bits"
    return y >> 7


def _fit(q: np.ndarray, index_bits: int):
    n = len(q) >> index_bits
    t = np.arange(n, dtype=np.int64)
    table = []
    for seg in q.reshape(1 << index_bits, n):
        slope = -np.polyfit(t, seg.astype(np.float64), 1)[0] * 512
        for b in sorted(range(int(slope) - 8, int(slope) + 9), key=lambda v: abs(v - slope)):
            lo = int((seg * 512 + b * t).max())
            hi = int(((seg + 1) * 512 + b * t).min()) - 1
            if lo <= hi:
                table.append((lo, b))
                break
        else:
            raise RuntimeError("segment has no exact (A, B) at shift 9")
    return table


def generate() -> str:
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "probe.c"), os.path.join(d, "probe")
        with open(src, "w") as f:
            f.write(PROBE_C)
        subprocess.run(["gcc", "-O1", "-o", exe, src], check=True)
        rcp = _fit(_significand17(_probe(0, 127, 16, exe), 126), 6)
        rsq_even = _fit(_significand17(_probe(1, 127, 15, exe), 126), 5)
        rsq_odd = _fit(_significand17(_probe(1, 128, 15, exe), 126), 5)
    return _emit(rcp, rsq_even, rsq_odd)


HEADER = r"""// Exact restatement of the AVX-512 instructions VRCP14PS and VRSQRT14PS that the reference's
// simd::approx_rcp / simd::approx_rsqrt / simd::approx_sqrt run (src/SwRast/SIMD.h:294-296).
// Generated by glimpsw_gb300/gen_approx14.py from measurements of the instructions; do not edit.
// The functions reproduce the instructions' results bit for bit for every 32-bit input (checked
// over all 2^32 inputs on an AVX-512 host), with the default MXCSR state (no DAZ/FTZ):
//  - normal and denormal inputs: a 17-bit significand from a piecewise-linear integer segment,
//    (A - B * t) >> 9, indexed by the leading mantissa bits; exact powers of two (rcp14) and of
//    four (rsqrt14) give the exact result; results below the normal range are denormalised;
//  - zeros give infinities of the same sign, +inf gives +0 (rcp14 of -inf: -0), NaNs are
//    quietened; rsqrt14 of a negative number or of -inf is the default NaN 0xFFC00000.
// Used by host code (the library's oracle) and device code (culling, the alpha test, the resolve).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SWR_A14_FN static __host__ __device__ __forceinline__
#else
#define SWR_A14_FN static inline
#endif

// Segments: [0, 64) rcp14 by m[22:17]; [64, 96) rsqrt14 of even exponents by m[22:18];
// [96, 128) rsqrt14 of odd exponents by m[22:18]. Each entry is (A, B).
#define SWR_A14_SEGMENTS { \
    @ROWS@
    }

static const uint32_t swr_a14_host_segments[128][2] = SWR_A14_SEGMENTS;
#if defined(__CUDACC__)
static __device__ const uint2 swr_a14_device_segments[128] = SWR_A14_SEGMENTS;
#endif

// 17-bit significand, in bits 23..7 of the returned word, of segment s at interpolation t.
SWR_A14_FN uint32_t swr_a14_significand(uint32_t s, uint32_t t) {
#if defined(__CUDA_ARCH__)
    const uint2 ab = __ldg(&swr_a14_device_segments[s]);
    return ((ab.x - ab.y * t) >> 9) << 7;
#else
    return ((swr_a14_host_segments[s][0] - swr_a14_host_segments[s][1] * t) >> 9) << 7;
#endif
}

SWR_A14_FN uint32_t swr_a14_clz(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__clz((int)v);
#else
    return (uint32_t)__builtin_clz(v);
#endif
}

SWR_A14_FN float swr_a14_from_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

// VRCP14PS on one lane.
SWR_A14_FN float swr_rcp14(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFF;
    uint32_t m = u & 0x7FFFFFu;
    if (e == 0xFF) return swr_a14_from_bits(m ? (u | 0x400000u) : sign);
    int E = (int)e;
    if (e == 0) {
        if (m == 0) return swr_a14_from_bits(sign | 0x7F800000u);
        const uint32_t sh = swr_a14_clz(m) - 8;
        m = (m << sh) & 0x7FFFFFu;
        E = 1 - (int)sh;
    }
    int re = 253 - E;
    uint32_t sig;
    if (m == 0) sig = 0x800000u, re += 1;
    else sig = swr_a14_significand(m >> 17, (m >> 7) & 1023);
    if (re >= 255) return swr_a14_from_bits(sign | 0x7F800000u);
    if (re >= 1) return swr_a14_from_bits(sign | ((uint32_t)re << 23) | (sig & 0x7FFFFFu));
    return swr_a14_from_bits(sign | (sig >> (1 - re)));
}

// VRSQRT14PS on one lane.
SWR_A14_FN float swr_rsqrt14(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFF;
    uint32_t m = u & 0x7FFFFFu;
    if (e == 0xFF) return swr_a14_from_bits(m ? (u | 0x400000u) : (sign ? 0xFFC00000u : 0u));
    if (e == 0 && m == 0) return swr_a14_from_bits(sign | 0x7F800000u);
    if (sign) return swr_a14_from_bits(0xFFC00000u);
    int E = (int)e - 127;
    if (e == 0) {
        const uint32_t sh = swr_a14_clz(m) - 8;
        m = (m << sh) & 0x7FFFFFu;
        E = -126 - (int)sh;
    }
    const int odd = E & 1;
    const int half = (E - odd) / 2;
    if (!odd && m == 0) return swr_a14_from_bits((uint32_t)(127 - half) << 23);
    const uint32_t sig = swr_a14_significand(64 + 32 * odd + (m >> 18), (m >> 8) & 1023);
    return swr_a14_from_bits(((uint32_t)(126 - half) << 23) | (sig & 0x7FFFFFu));
}

// simd::approx_sqrt (SIMD.h:296).
SWR_A14_FN float swr_sqrt14(float x) { return swr_rsqrt14(x) * x; }
"""


def _emit(rcp, rsq_even, rsq_odd) -> str:
    rows = rcp + rsq_even + rsq_odd
    assert len(rows) == 128 and all(0 <= a < 2**31 and 0 < b < 2**12 for a, b in rows)
    lines = []
    for i in range(0, 128, 4):
        lines.append("    " + ", ".join("{%du, %du}" % r for r in rows[i:i + 4]) + ", \\")
    return HEADER.replace("@ROWS@", "\n".join(lines).lstrip())


if __name__ == "__main__":
    text = generate()
    with open(OUT, "w") as f:
        f.write(text)
    print("wrote", OUT)
