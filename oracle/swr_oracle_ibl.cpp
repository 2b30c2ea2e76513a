// Oracle (test infrastructure, see swr_oracle.h): the image-based lighting precompute of GLimpSW
// (Shading.cpp:35-219), one output texel at a time: GenerateIrradianceMap with
// PrefilterDiffuseIrradiance, GenerateRadianceMap with PrefilterEnvMap, GenerateEnvBRDFLut with
// IntegrateBRDF, and the EnvSampler path of SampleOctLevel (Texture.h:412-480, 506-575) they read.
//
// The reference evaluates 16 texels of a tile as one vector; its two tile-wide decisions
// (`any(NoL > 0)` in PrefilterEnvMap / IntegrateBRDF, `any(mipFrac > 0)` in SampleOctLevel) only
// add exact zeros for the lanes they do not concern, so one texel is restated alone. The
// reference's scalar per-step terms come from the same formulas: cosf / sinf of the irradiance
// angles, Hammersley points, and simd::sincos_2pi (SIMD.h:390-413) of the sample azimuths.
#include "swr_oracle_common.h"

#include <vector>

namespace orc {
namespace {

constexpr float kPi = 3.141592653589793f, kTau = 6.283185307179586f, kInvPi = 0.3183098861837907f;
struct F3 { float x, y, z; };

inline float mulsign(float x, float y) { return u2f(f2u(x) ^ (f2u(y) & 0x80000000u)); }
inline float dot3(F3 a, F3 b) { return std::fma(a.x, b.x, std::fma(a.y, b.y, a.z * b.z)); }
inline F3 normalize3(F3 a) {
    const float r = approx_rsqrt(dot3(a, a));
    return { a.x * r, a.y * r, a.z * r };
}
inline F3 cross3(F3 a, F3 b) {
    return { std::fma(a.y, b.z, -a.z * b.y), std::fma(a.z, b.x, -a.x * b.z), std::fma(a.x, b.y, -a.y * b.x) };
}
inline void map_oct(F3 n, float& u, float& v) {  // Texture.h:282-288
    const float w = approx_rcp(std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    const float t = vmax(-n.z * w, 0.0f);
    u = std::fma(n.x, w, mulsign(t, n.x)) * 0.5f + 0.5f;
    v = std::fma(n.y, w, mulsign(t, n.y)) * 0.5f + 0.5f;
}
inline F3 unmap_oct(float u, float v) {  // Texture.h:290-296
    u = u * 2.0f - 1.0f, v = v * 2.0f - 1.0f;
    F3 n = { u, v, 1.0f - std::fabs(u) - std::fabs(v) };
    const float t = vmax(-n.z, 0.0f);
    n.x -= mulsign(t, n.x);
    n.y -= mulsign(t, n.y);
    return normalize3(n);
}
inline float unpack_f11(uint32_t x) { x <<= 17; return u2f((x & 0x0FFE0000u) + 0x38000000u); }
inline float unpack_f10(uint32_t x) { x <<= 18; return u2f((x & 0x0FFC0000u) + 0x38000000u); }
inline F3 unpack_r11g11b10(uint32_t p) { return { unpack_f11(p >> 21), unpack_f11(p >> 10), unpack_f10(p) }; }
inline uint32_t pack_r11g11b10(F3 c) {  // R11G11B10f::Pack, Texture.h:146-167
    auto f11 = [](float x) {
        x = vmin(vmax(x, 1.0f / (1 << 15)), 130048.0f);
        return ((f2u(x) >> 17) & 0x3FFF) - 0x1C00;
    };
    auto f10 = [](float x) {
        x = vmin(vmax(x, 1.0f / (1 << 15)), 129024.0f);
        return ((f2u(x) >> 18) & 0x1FFF) - 0x0E00;
    };
    return f11(c.x) << 21 | f11(c.y) << 10 | f10(c.z);
}
// vcvtps2ph with round-to-nearest-even (RG16f::Pack, Texture.h:127-131).
inline uint32_t float_to_half(float f) {
    const uint32_t b = f2u(f), s = (b >> 16) & 0x8000u;
    const uint32_t a = b & 0x7FFFFFFFu;
    if (a >= 0x7F800000u) return s | (a > 0x7F800000u ? 0x7E00u : 0x7C00u);  // NaN (quiet) / inf
    if (a >= 0x477FF000u) return s | 0x7C00u;                                  // rounds to >= 65536: inf
    if (a < 0x38800000u) {                                                     // half subnormal or zero
        const float r = std::fabs(f) * 16777216.0f;                            // units of 2^-24, exact scaling
        return s | (uint32_t)std::nearbyint(r);
    }
    uint32_t m = a - 0x38000000u;                  // rebias exponent 127 -> 15 (in the float's bit positions)
    const uint32_t low = m & 0x1FFFu;
    m >>= 13;
    if (low > 0x1000u || (low == 0x1000u && (m & 1))) m++;
    return s | m;
}

inline int32_t texel_offset(int32_t x, int32_t y, int32_t stride) { return (y & 7) | (x << 3) | ((y & ~7) << stride); }

// SampleLevel<EnvSampler>: ClampToEdge, linear, float SampleLinear.
F3 sample_env_level(const orc_texture& t, float u, float v, int32_t mipIn) {
    int32_t ix = std::min(std::max(round2i(u * t.scale_lerp_u), 0), t.mask_lerp_u);
    int32_t iy = std::min(std::max(round2i(v * t.scale_lerp_v), 0), t.mask_lerp_v);
    const int32_t m = std::min(std::max(mipIn, 0), (int32_t)t.mip_levels - 1);
    const int32_t stride = (int32_t)t.row_shift - m;
    ix >>= m, iy >>= m;
    const uint32_t* base = t.data + t.mip_offsets[m & 15];
    const int32_t xf = std::max(ix - 127, 0), yf = std::max(iy - 127, 0);
    const int32_t tx = xf >> 8, ty = yf >> 8;
    const bool inX = ((tx + 1) << m) < (int32_t)t.width, inY = ((ty + 1) << m) < (int32_t)t.height;
    const int32_t i00 = texel_offset(tx, ty, stride), i01 = texel_offset(tx, ty + (inY ? 1 : 0), stride);
    const F3 c00 = unpack_r11g11b10(base[i00]), c10 = unpack_r11g11b10(base[i00 + 8]);
    const F3 c01 = unpack_r11g11b10(base[i01]), c11 = unpack_r11g11b10(base[i01 + 8]);
    const float fracScale = 1.0f / 256;
    float fx = (float)(xf & 255) * fracScale;
    const float fy = (float)(yf & 255) * fracScale;
    if (!inX) fx = 0;
    const F3 ra = { c00.x + (c10.x - c00.x) * fx, c00.y + (c10.y - c00.y) * fx, c00.z + (c10.z - c00.z) * fx };
    const F3 rb = { c01.x + (c11.x - c01.x) * fx, c01.y + (c11.y - c01.y) * fx, c01.z + (c11.z - c01.z) * fx };
    return { ra.x + (rb.x - ra.x) * fy, ra.y + (rb.y - ra.y) * fy, ra.z + (rb.z - ra.z) * fy };
}
F3 sample_oct_level(const orc_texture& t, F3 dir, float level) {
    float u, v;
    map_oct(dir, u, v);
    const int32_t baseMip = trunc2i(level);
    const F3 b = sample_env_level(t, u, v, baseMip);
    const float frac = level - (float)baseMip;
    if (frac > 0.0f && baseMip < (int32_t)t.mip_levels - 1) {
        const F3 l = sample_env_level(t, u, v, baseMip + 1);
        return { b.x + (l.x - b.x) * frac, b.y + (l.y - b.y) * frac, b.z + (l.z - b.z) * frac };
    }
    return b;
}
F3 tonemap_sample(F3 c, bool inverse) {  // TonemapSample / TonemapSampleInv, Shading.cpp:36-44
    const float luma = dot3(c, { 0.299f, 0.587f, 0.114f });
    const float r = approx_rcp(inverse ? 1.0f - luma : 1.0f + luma);
    return { c.x * r, c.y * r, c.z * r };
}
void tangent_frame(F3 N, F3& tx, F3& ty) {
    const bool nz = std::fabs(N.z) < 0.999f;
    const F3 up = { nz ? 0.0f : 1.0f, 0.0f, nz ? 1.0f : 0.0f };
    tx = normalize3(cross3(up, N));
    ty = cross3(N, tx);
}
F3 importance_sample_ggx(float xiY, float cphi, float sphi, float roughness, F3 N, F3 tx, F3 ty) {  // Shading.cpp:56-70
    const float a = roughness * roughness;
    const float cosTheta = std::sqrt((1.0f - xiY) / (1.0f + (a * a - 1.0f) * xiY));
    const float sinTheta = std::sqrt(1.0f - cosTheta * cosTheta);
    const F3 H = { cphi * sinTheta, sphi * sinTheta, cosTheta };
    return { tx.x * H.x + ty.x * H.y + N.x * H.z, tx.y * H.x + ty.y * H.y + N.y * H.z, tx.z * H.x + ty.z * H.y + N.z * H.z };
}
float approx_log2(float x) { return std::fma((float)f2u(x), 1.1920928955078125e-7f, -126.94269504f); }  // SIMD.h:416-419

void sincos_2pi(float x, float& s, float& c) {  // SIMD.h:390-409
    x = x + 0.25f;
    x = x - std::nearbyint(x);
    const float x1 = std::fabs(x) - 0.25f;
    const float x2 = x1 * x1;
    s = std::fma(x2, std::fma(x2, std::fma(x2, -70.993433272f, 81.340768887f), -41.337142371f), 6.283164044f) * x1;
    c = mulsign(std::fma(x2, std::fma(x2, std::fma(x2, -78.216131988f, 64.660541218f), -19.735752060f), 0.999993295f), x);
}
// Hammersley(i, n) (Shading.cpp:46-54) and simd::cos / sin of phi = 2 pi Xi.x (Shading.cpp:59).
void hammersley(uint32_t i, uint32_t n, float& xiY, float& c, float& s) {
    uint32_t bits = i;
    bits = (bits << 16) | (bits >> 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    const float xiX = (float)i / (float)n;
    xiY = (float)(bits * (1.0 / 4294967295.0));
    const float phi = (float)(2.0 * (double)kPi * (double)xiX);
    sincos_2pi(phi * 0.15915494309189535f, s, c);
}

}  // namespace
}  // namespace orc

using namespace orc;

extern "C" {

// PrefilterDiffuseIrradiance (Shading.cpp:72-102) of texel (x, y) of a w x h irradiance map.
uint32_t orc_ibl_irradiance_texel(const orc_texture* env, uint32_t x, uint32_t y, uint32_t w, uint32_t h) {
    const float u = ((float)x + 0.5f) * (1.0f / (float)w), v = ((float)y + 0.5f) * (1.0f / (float)h);
    const F3 N = unmap_oct(u, v);
    F3 right, up;
    tangent_frame(N, right, up);
    F3 color = { 0.0f, 0.0f, 0.0f };
    uint32_t sampleCount = 0;
    const float halfPi = (float)((double)kPi * 0.5);
    const float deltaPhi = (float)((double)kTau / 360.0), deltaTheta = (float)((double)halfPi / 90.0);
    for (float phi = 0.0f; phi < kTau; phi += deltaPhi) {
        const float cp = cosf(phi), sp = sinf(phi);
        const F3 tmp = { cp * right.x + sp * up.x, cp * right.y + sp * up.y, cp * right.z + sp * up.z };
        for (float theta = 0.0f; theta < halfPi; theta += deltaTheta) {
            const float ct = cosf(theta), st = sinf(theta);
            const F3 dir = { ct * N.x + st * tmp.x, ct * N.y + st * tmp.y, ct * N.z + st * tmp.z };
            const F3 s = tonemap_sample(sample_oct_level(*env, dir, 2.0f), false);
            color = { color.x + s.x * ct * st, color.y + s.y * ct * st, color.z + s.z * ct * st };
            sampleCount++;
        }
    }
    const float k = kPi * 1.0f / (float)sampleCount;
    return pack_r11g11b10(tonemap_sample({ color.x * k, color.y * k, color.z * k }, true));
}

// PrefilterEnvMap (Shading.cpp:105-147) of texel (x, y) of level `level` of a radiance map of
// `levels` mips whose level 0 is w0 x h0.
uint32_t orc_ibl_radiance_texel(const orc_texture* env, uint32_t level, uint32_t levels, uint32_t x, uint32_t y, uint32_t w0,
                                uint32_t h0) {
    const uint32_t w = w0 >> level, h = h0 >> level;
    const float u = ((float)x + 0.5f) * (1.0f / (float)w), v = ((float)y + 0.5f) * (1.0f / (float)h);
    const F3 R = unmap_oct(u, v);
    const float roughness = std::max((float)level / ((float)levels - 1.0f), 0.01f);
    F3 tx, ty;
    tangent_frame(R, tx, ty);
    const uint32_t numSamples = 128;
    const float omegaP = 4.0f * kPi / (float)(6u * env->width * env->width);
    F3 pre = { 0.0f, 0.0f, 0.0f };
    float total = 0.0f;
    for (uint32_t i = 0; i < numSamples; i++) {
        float xiY, c, s;
        hammersley(i, numSamples, xiY, c, s);
        const F3 H = importance_sample_ggx(xiY, c, s, roughness, R, tx, ty);
        const float VoH = dot3(R, H);
        const float NoH = vmax(VoH, 0.0f);
        const F3 L = { 2.0f * VoH * H.x - R.x, 2.0f * VoH * H.y - R.y, 2.0f * VoH * H.z - R.z };
        const float NoL = vmax(dot3(R, L), 0.0f);
        if (NoL > 0.0f) {
            const float a = NoH * roughness;  // D_GGX, Shading.cpp:19-23
            const float kk = roughness * approx_rcp(1.0f - NoH * NoH + a * a);
            const float pdf = kk * kk * kInvPi / 4.0f + 0.001f;
            const float omegaS = 1.0f / ((float)numSamples * pdf);
            const float mip = vmax(0.5f * approx_log2(omegaS / omegaP), 0.0f);
            const F3 col = tonemap_sample(sample_oct_level(*env, L, mip), false);
            pre = { pre.x + col.x * NoL, pre.y + col.y * NoL, pre.z + col.z * NoL };
            total += NoL;
        }
    }
    return pack_r11g11b10(tonemap_sample({ pre.x / total, pre.y / total, pre.z / total }, true));
}

// IntegrateBRDF (Shading.cpp:149-175) of texel (x, y) of a w x h table, packed as RG16f.
uint32_t orc_ibl_env_brdf_texel(uint32_t x, uint32_t y, uint32_t w, uint32_t h) {
    const float NoV = ((float)x + 0.5f) * (1.0f / (float)w), roughness = ((float)y + 0.5f) * (1.0f / (float)h);
    const F3 N = { 0.0f, 0.0f, 1.0f };
    const F3 V = { std::sqrt(1.0f - NoV * NoV), 0.0f, NoV };
    F3 tx, ty;
    tangent_frame(N, tx, ty);
    float rx = 0.0f, ry = 0.0f;
    const uint32_t sampleCount = 1024;
    for (uint32_t i = 0; i < sampleCount; i++) {
        float xiY, c, s;
        hammersley(i, sampleCount, xiY, c, s);
        const F3 H = importance_sample_ggx(xiY, c, s, roughness, N, tx, ty);
        const float VdH = dot3(V, H);
        const F3 L = { 2.0f * VdH * H.x - V.x, 2.0f * VdH * H.y - V.y, 2.0f * VdH * H.z - V.z };
        const float VoH = vmax(0.0f, VdH), NoL = vmax(0.0f, L.z), NoH = vmax(0.0f, H.z);
        if (NoL > 0.0f) {
            const float r2 = roughness * roughness;  // V_SmithGGXCorrelatedFast, Shading.cpp:24-28
            const float a = 2.0f * NoL * NoV, b = NoL + NoV;
            const float G = 0.5f / std::fma(r2, b, std::fma(-r2, a, a));
            const float Gv = G * 4.0f * VoH * NoL / NoH;
            const float om = 1.0f - VoH;
            const float Fc = (om * om) * (om * om) * om;
            rx += Gv * (1.0f - Fc);
            ry += Gv * Fc;
        }
    }
    return float_to_half(rx * (1.0f / sampleCount)) | (float_to_half(ry * (1.0f / sampleCount)) << 16);
}

}  // extern "C"
