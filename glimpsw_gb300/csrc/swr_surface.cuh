// Surface math of the shading stages (ResolveSurface / EvalLighting, Shading.cpp:417-645, and
// FS_EncodeGBuffer, Shading.cpp:344-414): simd::dot / normalize / lerp / mul (SIMD.h:427-464) and the
// octahedral unmapping (Texture.h:290-296), with the reference's explicit fmas and rcp14/rsqrt14
// from the exact tables. Translation units including this are compiled with -fmad=false, so the
// plain products and sums round as the reference's separate vector operations do.
#pragma once
#include "../../include/swr/approx14.h"
#include "swr_device.cuh"

namespace swr {

struct F3 { float x, y, z; };

__device__ __forceinline__ float approx_rcp(float x) { return swr_rcp14(x); }
__device__ __forceinline__ float approx_rsqrt(float x) { return swr_rsqrt14(x); }
__device__ __forceinline__ float approx_sqrt(float x) { return swr_sqrt14(x); }
__device__ __forceinline__ float mulsign(float x, float y) {
    return __uint_as_float(__float_as_uint(x) ^ (__float_as_uint(y) & 0x80000000u));
}
__device__ __forceinline__ float dot3(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ F3 normalize3(F3 a) {
    float r = approx_rsqrt(dot3(a, a));
    return { a.x * r, a.y * r, a.z * r };
}
__device__ __forceinline__ float lerpf(float a, float b, float t) { return fmaf(t, b, fmaf(-t, a, a)); }
__device__ __forceinline__ F3 xform4(const float* m, F3 p, float& w) {  // simd::mul(mat4, (p, 1))
    F3 r = { fmaf(p.x, m[0], fmaf(p.y, m[4], fmaf(p.z, m[8], 1.0f * m[12]))),
             fmaf(p.x, m[1], fmaf(p.y, m[5], fmaf(p.z, m[9], 1.0f * m[13]))),
             fmaf(p.x, m[2], fmaf(p.y, m[6], fmaf(p.z, m[10], 1.0f * m[14]))) };
    w = fmaf(p.x, m[3], fmaf(p.y, m[7], fmaf(p.z, m[11], 1.0f * m[15])));
    return r;
}
// simd::mul(glm::mat3, v_float3) (SIMD.h:466-472), column-major m.
__device__ __forceinline__ F3 mul3(const float* M, F3 n) {
    return F3{ fmaf(n.x, M[0], fmaf(n.y, M[3], n.z * M[6])), fmaf(n.x, M[1], fmaf(n.y, M[4], n.z * M[7])),
               fmaf(n.x, M[2], fmaf(n.y, M[5], n.z * M[8])) };
}
// simd::cross (SIMD.h:431-437).
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
    return F3{ fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x) };
}
// texutil::UnmapOctahedron (Texture.h:290-296).
__device__ __forceinline__ F3 unmap_oct(float u, float v) {
    u = u * 2.0f - 1.0f, v = v * 2.0f - 1.0f;
    F3 n = { u, v, 1.0f - fabsf(u) - fabsf(v) };
    float t = vmax(-n.z, 0.0f);
    n.x -= mulsign(t, n.x);
    n.y -= mulsign(t, n.y);
    return normalize3(n);
}
// texutil::MapOctahedron (Texture.h:282-288).
__device__ __forceinline__ void map_oct(F3 n, float& u, float& v) {
    const float w = approx_rcp(fabsf(n.x) + fabsf(n.y) + fabsf(n.z));
    const float t = vmax(-n.z * w, 0.0f);
    u = fmaf(n.x, w, mulsign(t, n.x)) * 0.5f + 0.5f;
    v = fmaf(n.y, w, mulsign(t, n.y)) * 0.5f + 0.5f;
}
// UnpackNormalTangent (Shading.cpp:232-236): RGBA8u::Unpack then two octahedral unmaps.
__device__ __forceinline__ void unpack_normal_tangent(uint32_t p, F3& n, F3& t) {
    const float s = 1.0f / 255;
    n = unmap_oct((float)(p & 255) * s, (float)((p >> 8) & 255) * s);
    t = unmap_oct((float)((p >> 16) & 255) * s, (float)(p >> 24) * s);
}

}  // namespace swr
