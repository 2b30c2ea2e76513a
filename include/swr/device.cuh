// Device-side helpers shared by the kernels of libswr_gb300 and by user shaders compiled against
// include/swr/shader.cuh.
//
// Exactness: the vis-buffer must equal the reference's single-threaded CPU result bit for bit,
// so every float operation on that path is an explicit round-to-nearest intrinsic (the result
// does not depend on whether the including translation unit lets nvcc contract a*b+c). Only the
// reference's explicit simd::fma calls (SIMD.h:288-291) become __fmaf_rn.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace swr {

// Meshlet record layout (Scene.h:15-30).
constexpr uint32_t kMeshletSize = 1728;
constexpr uint32_t kOffNumVertices = 44;   // u8 NumVertices, u8 NumTriangles, u8 AlphaCutoff
constexpr uint32_t kOffMaterialId = 48;
constexpr uint32_t kOffHandedness = 56;
constexpr uint32_t kOffPositions = 64;     // float[3][64]
constexpr uint32_t kOffTexCoords = 832;    // half2[64]
constexpr uint32_t kOffNormalTangents = 1088;
constexpr uint32_t kOffIndices = 1344;     // u8[3][128]

enum : int { kCullNone = 0, kCullFrontCCW = 1, kCullFrontCW = 2 };  // FaceCullMode, Rasterizer.h:80

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// simd::round2i (SIMD.h:304): RNE conversion; NaN/out of range give x86's 0x80000000.
__device__ __forceinline__ int32_t round2i(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return __float2int_rn(x);
}
// simd::conv<int> (cvttps2dq truncation) with the same out-of-range value.
__device__ __forceinline__ int32_t trunc2i(float x) {
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return INT32_MIN;
    return __float2int_rz(x);
}
// vminps / vmaxps operand semantics (second operand when the compare fails, e.g. on NaN).
__device__ __forceinline__ float vmin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float vmax(float a, float b) { return a > b ? a : b; }

// simd::gather_preload64 index mapping (SIMD.h:219-227).
__device__ __forceinline__ uint32_t preload64_index(uint32_t idx) { return idx < 32 ? idx : 32 + (idx & 31); }

// Framebuffer::GetPixelOffset (Rasterizer.h:50-56): 4x4 tiles.
__device__ __forceinline__ uint32_t pixel_offset(uint32_t x, uint32_t y, uint32_t width) {
    return ((x & ~3u) << 2) + (y & ~3u) * width + (x & 3) + (y & 3) * 4;
}

// Packed (x, y) int16 pairs as the reference keeps them in one int32 lane (Rasterizer.cpp:277-351).
__device__ __forceinline__ int32_t lo16(uint32_t v) { return (int32_t)(int16_t)(v & 0xFFFF); }
__device__ __forceinline__ int32_t hi16(uint32_t v) { return (int32_t)(int16_t)(v >> 16); }
__device__ __forceinline__ uint32_t srai16_4(uint32_t v) {
    return ((uint32_t)(lo16(v) >> 4) & 0xFFFF) | ((uint32_t)(hi16(v) >> 4) << 16);
}

// Total order on floats as unsigned integers (monotone for all non-NaN values, -0 == +0).
__device__ __forceinline__ uint32_t float_order(float f) {
    uint32_t b = __float_as_uint(f);
    b = (b == 0x80000000u) ? 0u : b;                      // -0 orders like +0
    return b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u);  // positive: set sign; negative: invert
}
__device__ __forceinline__ float float_unorder(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// Vis-buffer key: (ordered depth << 32) | (0xFFFFFFFE - rank). A larger key is a deeper-in-
// reversed-Z (nearer) fragment, ties broken towards the lower rank, i.e. the fragment a
// single-threaded draw submits first. A key whose low word is 0xFFFFFFFF holds a depth that
// was not written by a fragment of the current draw sequence.
constexpr uint32_t kKeyEmptyLow = 0xFFFFFFFFu;
__device__ __forceinline__ unsigned long long make_key(float depth, uint32_t rank) {
    return ((unsigned long long)float_order(depth) << 32) | (unsigned long long)(0xFFFFFFFEu - rank);
}

// Rank = single-threaded submission order of a triangle within the frame:
// meshlet (21 bits) | packet (3) | clipped (1) | lane in packet (4) | clip fan index (3).
__device__ __forceinline__ uint32_t make_rank(uint32_t globalMeshlet, uint32_t prim, uint32_t clipped, uint32_t fan) {
    return (globalMeshlet << 11) | ((prim >> 4) << 8) | (clipped << 7) | ((prim & 15) << 3) | fan;
}
__device__ __forceinline__ uint32_t rank_surface_id(uint32_t rank) {
    return (rank >> 11) * 128u + ((rank >> 8) & 7) * 16u + ((rank >> 3) & 15);
}

}  // namespace swr
