// Exact restatement of the AVX-512 instructions VRCP14PS and VRSQRT14PS that the reference's
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
    {67107072u, 1009u}, {66074112u, 977u}, {65073664u, 949u}, {64102400u, 921u}, \
    {63159040u, 893u}, {62244608u, 869u}, {61354752u, 843u}, {60491264u, 821u}, \
    {59650560u, 797u}, {58833920u, 777u}, {58038272u, 755u}, {57264640u, 735u}, \
    {56511488u, 717u}, {55778048u, 699u}, {55062784u, 681u}, {54365184u, 663u}, \
    {53686016u, 647u}, {53022976u, 631u}, {52377088u, 617u}, {51745536u, 601u}, \
    {51129600u, 587u}, {50528000u, 573u}, {49940992u, 561u}, {49366272u, 547u}, \
    {48805376u, 535u}, {48257024u, 523u}, {47721728u, 513u}, {47196672u, 501u}, \
    {46683904u, 491u}, {46181632u, 479u}, {45690368u, 469u}, {45209344u, 459u}, \
    {44739072u, 451u}, {44277504u, 441u}, {43826176u, 433u}, {43382784u, 423u}, \
    {42949120u, 415u}, {42523904u, 407u}, {42106880u, 399u}, {41698048u, 391u}, \
    {41297920u, 385u}, {40903936u, 377u}, {40517888u, 369u}, {40139520u, 363u}, \
    {39768320u, 357u}, {39402752u, 349u}, {39044608u, 343u}, {38692864u, 337u}, \
    {38347520u, 331u}, {38008064u, 325u}, {37674496u, 319u}, {37347840u, 315u}, \
    {37025280u, 309u}, {36708608u, 303u}, {36398080u, 299u}, {36091648u, 293u}, \
    {35791360u, 289u}, {35495680u, 285u}, {35204352u, 279u}, {34919168u, 275u}, \
    {34638080u, 271u}, {34361088u, 267u}, {34088192u, 263u}, {33819392u, 259u}, \
    {67105920u, 1001u}, {66080896u, 955u}, {65102464u, 915u}, {64166144u, 877u}, \
    {63268608u, 841u}, {62407552u, 807u}, {61580928u, 775u}, {60786816u, 747u}, \
    {60022016u, 719u}, {59285632u, 693u}, {58575744u, 669u}, {57891328u, 647u}, \
    {57229568u, 625u}, {56589568u, 603u}, {55971712u, 585u}, {55373184u, 567u}, \
    {54793088u, 549u}, {54231424u, 533u}, {53686144u, 517u}, {53156864u, 501u}, \
    {52643456u, 487u}, {52144512u, 473u}, {51659776u, 461u}, {51188096u, 449u}, \
    {50728832u, 437u}, {50281856u, 425u}, {49847040u, 415u}, {49422080u, 403u}, \
    {49008512u, 393u}, {48605952u, 385u}, {48211840u, 375u}, {47828224u, 367u}, \
    {47450752u, 707u}, {46726272u, 675u}, {46034432u, 647u}, {45371904u, 619u}, \
    {44738048u, 595u}, {44129152u, 571u}, {43544704u, 549u}, {42982528u, 527u}, \
    {42442368u, 509u}, {41921920u, 491u}, {41419392u, 473u}, {40935040u, 457u}, \
    {40467072u, 441u}, {40015104u, 427u}, {39577728u, 413u}, {39155072u, 401u}, \
    {38744960u, 389u}, {38347136u, 377u}, {37961600u, 365u}, {37588096u, 355u}, \
    {37224832u, 345u}, {36871936u, 335u}, {36528640u, 325u}, {36195328u, 317u}, \
    {35870976u, 309u}, {35554944u, 301u}, {35246976u, 293u}, {34946816u, 285u}, \
    {34654848u, 279u}, {34369152u, 271u}, {34091008u, 265u}, {33819392u, 259u}, \
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
