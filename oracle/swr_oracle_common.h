// Oracle internals shared by its translation units (test infrastructure only).
#pragma once
#include "swr_oracle.h"

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace orc {

// Meshlet, Scene.h:15-30 (1728 bytes, positions 64-byte aligned).
struct Meshlet {
    float BoundCenter[3];
    float BoundRadius;
    float ConeApex[3], ConeAxis[3];
    float ConeCutoff;
    uint8_t NumVertices, NumTriangles;
    uint8_t AlphaCutoff;
    uint32_t MaterialId;
    uint64_t TangentHandedness;
    alignas(64) float Positions[3][64];
    uint32_t TexCoords[64];
    uint32_t NormalTangents[64];
    uint8_t Indices[3][128];
};
static_assert(sizeof(Meshlet) == 1728, "Meshlet layout");
static_assert(offsetof(Meshlet, NumVertices) == 44 && offsetof(Meshlet, MaterialId) == 48, "Meshlet header");
static_assert(offsetof(Meshlet, Positions) == 64 && offsetof(Meshlet, TexCoords) == 832, "Meshlet SoA");
static_assert(offsetof(Meshlet, NormalTangents) == 1088 && offsetof(Meshlet, Indices) == 1344, "Meshlet SoA");

enum { CULL_NONE = 0, CULL_FRONT_CCW = 1, CULL_FRONT_CW = 2 };  // FaceCullMode, Rasterizer.h:80

// simd::round2i (SIMD.h:304): cvtps2dq with the default round-to-nearest-even mode;
// NaN and out-of-range inputs give the x86 "integer indefinite" 0x80000000.
static inline int32_t round2i(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}
// simd::conv<int> (truncation, cvttps2dq) with the same indefinite value.
static inline int32_t trunc2i(float x) {
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)x;
}
// simd::max_abs (SIMD.h:335): vrangeps imm 0b1011, |larger magnitude| (NaN inputs are
// outside the oracle's contract).
static inline float max_abs(float a, float b) {
    float fa = std::fabs(a), fb = std::fabs(b);
    return fa > fb ? fa : fb;
}
// simd::min/max on floats (SIMD.h:308-328) compile to vminps/vmaxps under -ffast-math:
// the second operand is returned when the compare is false (including NaN).
static inline float vmin(float a, float b) { return a < b ? a : b; }
static inline float vmax(float a, float b) { return a > b ? a : b; }

// simd::ilog2, SIMD.h:426.
static inline int32_t ilog2(float x) {
    int32_t b;
    memcpy(&b, &x, 4);
    return (int32_t)((uint32_t)b - (127u << 23)) >> 23;
}

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

// simd::ilog2 where a NaN reads as the x86 default NaN 0xFFC00000: every NaN on these paths comes
// from an invalid operation, which the reference's x86 host answers with that pattern.
static inline int32_t ilog2_x86(float x) {
    if (x != x) x = u2f(0xFFC00000u);
    return ilog2(x);
}

// AVX-512 rcp14/rsqrt14 (SIMD.h:294-296): exact tables, the instructions or IEEE (approx mode).
float approx_rcp(float x);
float approx_rsqrt(float x);
static inline float approx_sqrt(float x) { return approx_rsqrt(x) * x; }

// simd::gather_preload64 (SIMD.h:219-227): permutex2var over two 32-entry halves, so an
// index selects entry idx for idx < 32 and 32 + (idx & 31) otherwise.
static inline uint32_t preload64_index(uint32_t idx) { return idx < 32 ? idx : 32 + (idx & 31); }

struct V4 { float x, y, z, w; };

// simd::mul(mat4, v_float4) with w = 1 (SIMD.h:457-464), m column-major.
static inline V4 transform_point(const float* m, float x, float y, float z) {
    V4 r;
    r.x = std::fma(x, m[0], std::fma(y, m[4], std::fma(z, m[8], 1.0f * m[12])));
    r.y = std::fma(x, m[1], std::fma(y, m[5], std::fma(z, m[9], 1.0f * m[13])));
    r.z = std::fma(x, m[2], std::fma(y, m[6], std::fma(z, m[10], 1.0f * m[14])));
    r.w = std::fma(x, m[3], std::fma(y, m[7], std::fma(z, m[11], 1.0f * m[15])));
    return r;
}

// One half of a packed half2 (vcvtph2ps, exact).
static inline float half_to_float(uint32_t h) {
    uint32_t s = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
    float v;
    if (e == 0) v = std::ldexp((float)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 1024), (int)e - 25);
    return s ? -v : v;
}

// Texture2D::SampleLevel<SurfaceSampler> on an RGBA8 texture for the 16 lanes of a 4x4 tile
// (u, v, mip levels per lane; the filter is chosen over all 16), swr_oracle_resolve.cpp.
void sample_rgba8(const orc_texture& t, const float* u, const float* v, int layer, const int32_t* mipIn, uint32_t* out);
// FS_EncodeGBuffer's shading after its depth test for the 16 lanes of a tile, swr_oracle_resolve.cpp.
uint32_t gbuffer_tile(const orc_shading_context* sc, const void* meshletRecord, const uint32_t vid[3], const float* bu,
                      const float* bv, uint32_t mask, uint32_t* baseColor, uint32_t* ch2);

}  // namespace orc
