// RGBA8 surface sampling shared by the rasterizer's alpha test and the resolve:
// Texture2D<RGBA8u, TiledY8>::SampleLevel<SurfaceSampler> (Texture.h:412-459, 506-556) with the
// sampler of Shading.cpp:6-10 (Repeat wrap, bilinear magnification, nearest minification, the
// filter chosen once for the whole 4x4 tile by the caller).
#pragma once
#include <cuda_fp16.h>

#include "swr_device.cuh"
#include "swr_internal.h"

namespace swr {

// Texture2D::GetTexelOffset for TiledY8 (Texture.h:493-501).
__device__ __forceinline__ uint32_t texel_offset(int32_t x, int32_t y, int32_t stride) {
    return (uint32_t)((y & 7) | (x << 3) | ((y & ~7) << stride));
}

// simd::lerp16 (SIMD.h:450) on both 16-bit halves: a + mulhrs(b - a, t).
__device__ __forceinline__ uint32_t lerp16(uint32_t a, uint32_t b, uint32_t t) {
    uint32_t r = 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        int32_t ah = (int16_t)(a >> (16 * h)), bh = (int16_t)(b >> (16 * h)), th = (int16_t)(t >> (16 * h));
        int32_t d = (int16_t)(bh - ah);
        int32_t mm = (int16_t)((d * th + 0x4000) >> 15);
        r |= (uint32_t)(uint16_t)(ah + mm) << (16 * h);
    }
    return r;
}

// vcvtph2ps of one half (exact).
__device__ __forceinline__ float h2f(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)h)); }

// simd::ilog2 (SIMD.h:426) where a NaN reads as the x86 default NaN 0xFFC00000 (every NaN on the
// paths that take it comes from an invalid operation, which x86 answers with that pattern).
__device__ __forceinline__ int32_t ilog2_x86(float x) {
    uint32_t b = (x != x) ? 0xFFC00000u : __float_as_uint(x);
    return (int32_t)(b - (127u << 23)) >> 23;
}

// Bilinear blend of four RGBA8 texels with 1.15 fixed-point weights (the 16-bit lane lerps of
// SampleLevel<SurfaceSampler>, Texture.h:540-556).
__device__ __forceinline__ uint32_t filter_rgba8(uint32_t d00, uint32_t d10, uint32_t d01, uint32_t d11, uint32_t fx, uint32_t fy) {
    uint32_t rb1 = lerp16(d00 & 0x00FF00FF, d10 & 0x00FF00FF, fx), ga1 = lerp16((d00 >> 8) & 0x00FF00FF, (d10 >> 8) & 0x00FF00FF, fx);
    uint32_t rb2 = lerp16(d01 & 0x00FF00FF, d11 & 0x00FF00FF, fx), ga2 = lerp16((d01 >> 8) & 0x00FF00FF, (d11 >> 8) & 0x00FF00FF, fx);
    return lerp16(rb1, rb2, fy) | (lerp16(ga1, ga2, fy) << 8);
}

// The texel coordinates one lane's SampleLevel<SurfaceSampler> reads (Texture.h:412-459): level m,
// the nearest texel (tx, ty), or for bilinear the top-left texel, whether its right / lower
// neighbours are inside the level, and the packed 1.15 weights.
struct TexelQuad {
    int32_t m, stride, tx, ty;
    bool inX, inY;
    uint32_t fx, fy;
};
__device__ __forceinline__ TexelQuad texel_quad(const DevTexture& t, float u, float v, int32_t mipIn, bool nearest) {
    TexelQuad q;
    int32_t ix = round2i(__fmul_rn(u, t.scale_lerp_u)) & t.mask_lerp_u;
    int32_t iy = round2i(__fmul_rn(v, t.scale_lerp_v)) & t.mask_lerp_v;
    q.m = min(max(mipIn, 0), (int32_t)t.mip_levels - 1);
    q.stride = (int32_t)t.row_shift - q.m;
    ix >>= q.m, iy >>= q.m;
    if (nearest) {
        q.tx = ix >> 8, q.ty = iy >> 8, q.inX = q.inY = false, q.fx = q.fy = 0;
        return q;
    }
    int32_t xf = max(ix - 127, 0), yf = max(iy - 127, 0);
    q.tx = xf >> 8, q.ty = yf >> 8;
    q.inX = ((q.tx + 1) << q.m) < (int32_t)t.width, q.inY = ((q.ty + 1) << q.m) < (int32_t)t.height;
    uint32_t fx = (uint32_t)(xf & 255) << 7, fy = (uint32_t)(yf & 255) << 7;
    q.fx = q.inX ? ((fx << 16) | fx) : 0u, q.fy = (fy << 16) | fy;
    return q;
}

// SampleLevel<SurfaceSampler> for one lane once the tile's filter is known (Texture.h:412-459).
__device__ __forceinline__ uint32_t sample_rgba8(const DevTexture& t, float u, float v, int layer, int32_t mipIn, bool nearest) {
    const TexelQuad q = texel_quad(t, u, v, mipIn, nearest);
    const uint32_t* base = t.data + (size_t)layer * t.layer_stride + t.mip_offsets[q.m & 15];
    if (nearest) return base[texel_offset(q.tx, q.ty, q.stride)];
    uint32_t i00 = texel_offset(q.tx, q.ty, q.stride), i01 = texel_offset(q.tx, q.ty + (q.inY ? 1 : 0), q.stride);
    return filter_rgba8(base[i00], base[i00 + 8], base[i01], base[i01 + 8], q.fx, q.fy);
}

}  // namespace swr
