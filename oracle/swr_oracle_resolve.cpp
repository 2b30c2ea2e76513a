// Oracle (test infrastructure, see swr_oracle.h): the vis-buffer resolve of GLimpSW
// (ShadingContext::Resolve, Shading.cpp:658-690) with its sampler (Texture.h:412-575).
//
// The reference shades a 4x4 tile as one 16-lane vector and takes several decisions for the
// whole tile: the texture filter (`any(mipLevel > 0)`, Texture.h:432), normal mapping
// (`any((NMR & 0xFFFF) != 0)`, Shading.cpp:555), light skipping (`all(NoL < 1e-4)`, 624-627) and
// the surface/sky branches (672, 676). This restatement therefore evaluates every quantity for
// all 16 lanes. Lanes the reference leaves uninitialised (sky lanes of ResolveSurface,
// Shading.cpp:473-477) are zero here, and where the reference inspects float bits of a NaN
// (ilog2 in CalcMipLevel) the NaN is the x86 default NaN 0xFFC00000.
#include "swr_oracle_common.h"
#include "../include/swr/hostmath.h"

#include <algorithm>
#include <thread>
#include <vector>

namespace orc {
namespace {

constexpr int L = 16;
struct F3 { float x, y, z; };

inline float mulsign(float x, float y) { return u2f(f2u(x) ^ (f2u(y) & 0x80000000u)); }  // SIMD.h:341-344
inline float dot3(F3 a, F3 b) { return std::fma(a.x, b.x, std::fma(a.y, b.y, a.z * b.z)); }  // SIMD.h:429
inline F3 normalize3(F3 a) {  // SIMD.h:439
    float r = approx_rsqrt(dot3(a, a));
    return { a.x * r, a.y * r, a.z * r };
}
inline float lerpf(float a, float b, float t) { return std::fma(t, b, std::fma(-t, a, a)); }  // SIMD.h:446

// simd::lerp16 (SIMD.h:450) on both 16-bit halves: a + mulhrs(b - a, t).
inline uint32_t lerp16(uint32_t a, uint32_t b, uint32_t t) {
    uint32_t r = 0;
    for (int h = 0; h < 2; h++) {
        int32_t ah = (int16_t)(a >> (16 * h)), bh = (int16_t)(b >> (16 * h)), th = (int16_t)(t >> (16 * h));
        int32_t d = (int16_t)(bh - ah);
        int32_t m = (int16_t)((d * th + 0x4000) >> 15);
        r |= (uint32_t)(uint16_t)(ah + m) << (16 * h);
    }
    return r;
}

// pixfmt (Texture.h:28-200)
struct F4 { float x, y, z, w; };
inline F4 unpack_rgba8(uint32_t p) {
    const float s = 1.0f / 255;
    return { (float)(p & 255) * s, (float)((p >> 8) & 255) * s, (float)((p >> 16) & 255) * s, (float)(p >> 24) * s };
}
inline F4 unpack_srgb(uint32_t p) {  // Texture.h:37-54 (mulhi_epu16 squaring)
    uint32_t rb1 = ((p << 8) & 0xFF00FF00u) + 0x00FF00FFu;
    uint32_t ag1 = ((p << 0) & 0xFF00FF00u) + 0x00FF00FFu;
    auto mulhi = [](uint32_t v) {
        uint32_t lo = v & 0xFFFF, hi = v >> 16;
        return ((lo * lo) >> 16) | (((hi * hi) >> 16) << 16);
    };
    uint32_t rb2 = mulhi(rb1), ag2 = mulhi(ag1);
    const float s = 1.0f / 65535;
    return { (float)(rb2 & 65535) * s, (float)(ag2 & 65535) * s, (float)(rb2 >> 16) * s, (float)(ag1 >> 16) * s };
}
inline uint32_t sat_u8(int32_t v) {
    int32_t s = std::min(std::max(v, -32768), 32767);
    return (uint32_t)std::min(std::max(s, 0), 255);
}
inline uint32_t pack_rgba8(F4 v) {
    return sat_u8(round2i(v.x * 255.0f)) | (sat_u8(round2i(v.y * 255.0f)) << 8) | (sat_u8(round2i(v.z * 255.0f)) << 16) |
           (sat_u8(round2i(v.w * 255.0f)) << 24);
}
inline float unpack_f11(uint32_t x) { x <<= 17; return u2f((x & 0x0FFE0000u) + 0x38000000u); }
inline float unpack_f10(uint32_t x) { x <<= 18; return u2f((x & 0x0FFC0000u) + 0x38000000u); }
inline F3 unpack_r11g11b10(uint32_t p) { return { unpack_f11(p >> 21), unpack_f11(p >> 10), unpack_f10(p) }; }

inline uint32_t texel_offset(int32_t x, int32_t y, int32_t stride) {
    return (uint32_t)((y & 7) | (x << 3) | ((y & ~7) << stride));
}

// texutil::CalcMipLevel(grad, scale) (Texture.h:276-280) with the squared scales.
inline int32_t calc_mip_level(float gx, float gy, float gz, float gw, float ssu, float ssv) {
    const float dx = std::fma(gx, gx, gy * gy) * ssu;
    const float dy = std::fma(gz, gz, gw * gw) * ssv;
    return ilog2_x86(vmax(dx, dy)) >> 1;
}

// texutil::MapOctahedron / UnmapOctahedron (Texture.h:282-296)
inline void map_oct(F3 n, float& u, float& v) {
    float w = approx_rcp(std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    float t = vmax(-n.z * w, 0.0f);
    u = std::fma(n.x, w, mulsign(t, n.x)) * 0.5f + 0.5f;
    v = std::fma(n.y, w, mulsign(t, n.y)) * 0.5f + 0.5f;
}
inline F3 unmap_oct(float u, float v) {
    u = u * 2.0f - 1.0f, v = v * 2.0f - 1.0f;
    F3 n = { u, v, 1.0f - std::fabs(u) - std::fabs(v) };
    float t = vmax(-n.z, 0.0f);
    n.x -= mulsign(t, n.x);
    n.y -= mulsign(t, n.y);
    return normalize3(n);
}

}  // namespace

// ---------------------------------------------------------------------------- sampler
// Texture2D::SampleLevel<SurfaceSampler> (Texture.h:412-459, Shading.cpp:6-10) for RGBA8 textures,
// 16 lanes: Repeat wrap, bilinear magnification, nearest minification, filter chosen per tile.
void sample_rgba8(const orc_texture& t, const float* u, const float* v, int layer, const int32_t* mipIn, uint32_t* out) {
    int32_t ix[L], iy[L], mip[L];
    bool anyMin = false;
    for (int l = 0; l < L; l++) {
        ix[l] = round2i(u[l] * t.scale_lerp_u) & t.mask_lerp_u;
        iy[l] = round2i(v[l] * t.scale_lerp_v) & t.mask_lerp_v;
        if (mipIn[l] > 0) anyMin = true;
        mip[l] = std::min(std::max(mipIn[l], 0), (int32_t)t.mip_levels - 1);
    }
    for (int l = 0; l < L; l++) {
        int32_t m = mip[l], stride = (int32_t)t.row_shift - m;
        int32_t x = ix[l] >> m, y = iy[l] >> m;
        const uint32_t* base = t.data + (size_t)layer * t.layer_stride + t.mip_offsets[m & 15];
        if (anyMin) {  // nearest (Texture.h:449-457)
            out[l] = base[texel_offset(x >> 8, y >> 8, stride)];
            continue;
        }
        // SampleLinear, RGBA8 fixed point (Texture.h:506-556)
        int32_t xf = std::max(x - 127, 0), yf = std::max(y - 127, 0);
        int32_t tx = xf >> 8, ty = yf >> 8;
        bool inX = ((tx + 1) << m) < (int32_t)t.width, inY = ((ty + 1) << m) < (int32_t)t.height;
        uint32_t i00 = texel_offset(tx, ty, stride), i01 = texel_offset(tx, ty + (inY ? 1 : 0), stride);
        uint32_t d00 = base[i00], d10 = base[i00 + 8], d01 = base[i01], d11 = base[i01 + 8];
        uint32_t fx = (uint32_t)(xf & 255) << 7, fy = (uint32_t)(yf & 255) << 7;
        fx = (fx << 16) | fx, fy = (fy << 16) | fy;
        if (!inX) fx = 0;
        uint32_t rb1 = lerp16(d00 & 0x00FF00FF, d10 & 0x00FF00FF, fx), ga1 = lerp16((d00 >> 8) & 0x00FF00FF, (d10 >> 8) & 0x00FF00FF, fx);
        uint32_t rb2 = lerp16(d01 & 0x00FF00FF, d11 & 0x00FF00FF, fx), ga2 = lerp16((d01 >> 8) & 0x00FF00FF, (d11 >> 8) & 0x00FF00FF, fx);
        out[l] = lerp16(rb1, rb2, fy) | (lerp16(ga1, ga2, fy) << 8);
    }
}

namespace {

// Texture2D::SampleOctLevel<EnvSampler> (Texture.h:467-480, Shading.cpp:11-15) on an R11G11B10 map:
// ClampToEdge, bilinear in float, blend of two mips when the level has a fraction.
void sample_env(const orc_texture& t, const F3* dir, float mipLevel, F3* out) {
    float u[L], v[L];
    for (int l = 0; l < L; l++) map_oct(dir[l], u[l], v[l]);
    int32_t baseMip = trunc2i(mipLevel);
    auto level = [&](int32_t mipReq, F3* res) {
        int32_t m = std::min(std::max(mipReq, 0), (int32_t)t.mip_levels - 1);
        for (int l = 0; l < L; l++) {
            int32_t x = std::min(std::max(round2i(u[l] * t.scale_lerp_u), 0), t.mask_lerp_u);
            int32_t y = std::min(std::max(round2i(v[l] * t.scale_lerp_v), 0), t.mask_lerp_v);
            int32_t stride = (int32_t)t.row_shift - m;
            x >>= m, y >>= m;
            const uint32_t* base = t.data + t.mip_offsets[m & 15];
            int32_t xf = std::max(x - 127, 0), yf = std::max(y - 127, 0);
            int32_t tx = xf >> 8, ty = yf >> 8;
            bool inX = ((tx + 1) << m) < (int32_t)t.width, inY = ((ty + 1) << m) < (int32_t)t.height;
            uint32_t i00 = texel_offset(tx, ty, stride), i01 = texel_offset(tx, ty + (inY ? 1 : 0), stride);
            F3 c00 = unpack_r11g11b10(base[i00]), c10 = unpack_r11g11b10(base[i00 + 8]);
            F3 c01 = unpack_r11g11b10(base[i01]), c11 = unpack_r11g11b10(base[i01 + 8]);
            const float fs = 1.0f / 256;
            float fx = (float)(xf & 255) * fs, fy = (float)(yf & 255) * fs;
            if (!inX) fx = 0;
            F3 a = { c00.x + (c10.x - c00.x) * fx, c00.y + (c10.y - c00.y) * fx, c00.z + (c10.z - c00.z) * fx };
            F3 b = { c01.x + (c11.x - c01.x) * fx, c01.y + (c11.y - c01.y) * fx, c01.z + (c11.z - c01.z) * fx };
            res[l] = { a.x + (b.x - a.x) * fy, a.y + (b.y - a.y) * fy, a.z + (b.z - a.z) * fy };
        }
    };
    level(baseMip, out);
    float frac = mipLevel - (float)baseMip;
    if (frac > 0.0f && baseMip < (int32_t)t.mip_levels - 1) {
        F3 lower[L];
        level(baseMip + 1, lower);
        for (int l = 0; l < L; l++)
            out[l] = { out[l].x + (lower[l].x - out[l].x) * frac, out[l].y + (lower[l].y - out[l].y) * frac,
                       out[l].z + (lower[l].z - out[l].z) * frac };
    }
}

// ---------------------------------------------------------------------------- surface
struct Surface { uint32_t albedo; F3 normal; float metallic, roughness; };

// simd::mul(mat4, (p, 1)) and mul(mat3, n), SIMD.h:457-471.
inline F4 mul4(const float* m, F3 p) {
    V4 r = transform_point(m, p.x, p.y, p.z);
    return { r.x, r.y, r.z, r.w };
}
inline F3 mul3(const float* m, F3 n) {
    return { std::fma(n.x, m[0], std::fma(n.y, m[3], n.z * m[6])), std::fma(n.x, m[1], std::fma(n.y, m[4], n.z * m[7])),
             std::fma(n.x, m[2], std::fma(n.y, m[5], n.z * m[8])) };
}
inline F3 bary_lerp(const float* b, F3 a0, F3 a1, F3 a2) {  // BaryLerp, Rasterizer.h:101-104
    return { std::fma(a0.x, b[0], std::fma(a1.x, b[1], a2.x * b[2])), std::fma(a0.y, b[0], std::fma(a1.y, b[1], a2.y * b[2])),
             std::fma(a0.z, b[0], std::fma(a1.z, b[1], a2.z * b[2])) };
}

}  // namespace

// FS_EncodeGBuffer (Shading.cpp:344-414) after its depth test, for the 16 lanes of a tile: the
// caller gives the perspective-correct barycentrics of every lane (bu, bv) and the lanes that passed
// the depth test (mask); returns the lanes that also pass the alpha test, with their base colour
// and packed layer-2 word. A material without a texture (the reference dereferences it) passes
// every lane with base colour 0xFFFFFFFF and layer 2 = 0.
uint32_t gbuffer_tile(const orc_shading_context* sc, const void* meshletRecord, const uint32_t vid[3], const float* bu,
                      const float* bv, uint32_t mask, uint32_t* baseColor, uint32_t* ch2) {
    const Meshlet& mesh = *(const Meshlet*)meshletRecord;
    const orc_material& mat = sc->materials[mesh.MaterialId];
    const orc_texture* tex = (mat.texture != UINT32_MAX && sc->textures && sc->textures[mat.texture].data)
                                 ? &sc->textures[mat.texture] : nullptr;
    for (int l = 0; l < L; l++) baseColor[l] = 0xFFFFFFFFu, ch2[l] = 0;
    if (!tex) return mask;
    // Mesh::TexCoords / NormalTangents [VertexId]: index bytes past the arrays read the record's
    // following words (0 past the record)
    const uint8_t* rec = (const uint8_t*)meshletRecord;
    auto word = [&](uint32_t offset, uint32_t idx) -> uint32_t {
        uint32_t w = 0;
        if (offset + 4 * idx < sizeof(Meshlet)) memcpy(&w, rec + offset + 4 * idx, 4);
        return w;
    };
    const uint32_t offTC = (uint32_t)offsetof(Meshlet, TexCoords), offNT = (uint32_t)offsetof(Meshlet, NormalTangents);
    float b[L][3], u[L], v[L], su[L], sv[L];
    float tc[3][2];
    for (int k = 0; k < 3; k++) {  // UnpackHalf2x16 (Shading.cpp:228-231)
        const uint32_t w = word(offTC, vid[k]);
        tc[k][0] = half_to_float(w & 0xFFFF), tc[k][1] = half_to_float(w >> 16);
    }
    for (int l = 0; l < L; l++) {
        b[l][0] = 1 - bu[l] - bv[l], b[l][1] = bu[l], b[l][2] = bv[l];
        u[l] = std::fma(tc[0][0], b[l][0], std::fma(tc[1][0], b[l][1], tc[2][0] * b[l][2]));
        v[l] = std::fma(tc[0][1], b[l][0], std::fma(tc[1][1], b[l][1], tc[2][1] * b[l][2]));
        su[l] = u[l] * tex->scale_lerp_u, sv[l] = v[l] * tex->scale_lerp_v;
    }
    // SampleImplicitLod (Texture.h:403-410): CalcMipLevel(grad) - LerpFracBits
    int32_t mip[L];
    for (int l = 0; l < L; l++) {
        float gx = su[l | 1] - su[l & ~1], gy = sv[l | 1] - sv[l & ~1];
        float gz = su[l | 4] - su[l & ~4], gw = sv[l | 4] - sv[l & ~4];
        mip[l] = (ilog2_x86(vmax(std::fma(gx, gx, gy * gy), std::fma(gz, gz, gw * gw))) >> 1) - 8;
    }
    sample_rgba8(*tex, u, v, 0, mip, baseColor);
    for (int l = 0; l < L; l++)
        if (baseColor[l] < ((uint32_t)mat.alpha_cutoff << 24)) mask &= ~(1u << l);  // Shading.cpp:357-358
    if (!mask || tex->num_layers < 2) return mask;
    uint32_t nmr[L];
    sample_rgba8(*tex, u, v, 1, mip, nmr);
    F3 n[3], t[3];
    for (int k = 0; k < 3; k++) {  // UnpackNormalTangent (Shading.cpp:232-236)
        const F4 o = unpack_rgba8(word(offNT, vid[k]));
        n[k] = unmap_oct(o.x, o.y);
        t[k] = unmap_oct(o.z, o.w);
    }
    const uint32_t hand = (uint32_t)((mesh.TangentHandedness >> (vid[0] & 63)) & 1) << 31;
    for (int l = 0; l < L; l++) {
        const float tx = (float)(nmr[l] & 255) * (1.0f / 127.5f) - 1.0f;
        const float ty = (float)((nmr[l] >> 8) & 255) * (1.0f / 127.5f) - 1.0f;
        const float tz = approx_sqrt(1.0f - (tx * tx + ty * ty));
        const F3 N = normalize3(mul3(sc->object_to_world, bary_lerp(b[l], n[0], n[1], n[2])));
        const F3 T = normalize3(mul3(sc->object_to_world, bary_lerp(b[l], t[0], t[1], t[2])));
        F3 B = { std::fma(N.y, T.z, -N.z * T.y), std::fma(N.z, T.x, -N.x * T.z), std::fma(N.x, T.y, -N.y * T.x) };
        B = { u2f(f2u(B.x) ^ hand), u2f(f2u(B.y) ^ hand), u2f(f2u(B.z) ^ hand) };
        const F3 R = normalize3({ tx * T.x + ty * B.x + tz * N.x, tx * T.y + ty * B.y + tz * N.y, tx * T.z + ty * B.z + tz * N.z });
        float ou, ov;
        map_oct(R, ou, ov);
        uint32_t c = (uint32_t)(ou * 1023.0f + 0.5f);  // conv<uint32_t>: truncation
        c |= (uint32_t)(ov * 1023.0f + 0.5f) << 10;
        c |= ((nmr[l] >> 18) & 0x3F) << 20;
        c |= ((nmr[l] >> 26) & 0x3F) << 26;
        ch2[l] = c;
    }
    return mask;
}

namespace {

// ResolveSurface (Shading.cpp:471-579) + IntersectTriangle (417-464), 16 lanes.
void resolve_surface(const orc_shading_context* sc, const uint32_t* ids, uint16_t active, const float* su, const float* sv,
                     float W, float H, Surface* out) {
    const Meshlet* meshlets = (const Meshlet*)sc->meshlets;
    F3 pos[3][L] = {};
    uint32_t tc[3][L] = {}, nt[3][L] = {}, hand[L] = {}, matId[L] = {};
    for (uint16_t pending = active; pending;) {
        uint32_t sid = ids[__builtin_ctz(pending)];
        uint32_t mId = sid / 128, tri = sid % 128;
        uint16_t iter = 0;
        for (int l = 0; l < L; l++) if (ids[l] == sid) iter |= (uint16_t)(1u << l);
        pending &= (uint16_t)~iter;
        if (mId >= sc->num_meshlets) continue;  // not a surface id of this scene (undefined in the reference)
        const Meshlet& m = meshlets[mId];
        for (int vi = 0; vi < 3; vi++) {
            uint32_t idx = m.Indices[vi][tri] & 63;
            for (int l = 0; l < L; l++) {
                if (!((iter >> l) & 1)) continue;
                pos[vi][l] = { m.Positions[0][idx], m.Positions[1][idx], m.Positions[2][idx] };
                tc[vi][l] = m.TexCoords[idx];
                nt[vi][l] = m.NormalTangents[idx];
                if (vi == 0 && ((m.TangentHandedness >> idx) & 1)) hand[l] = 1u << 31;
            }
        }
        for (int l = 0; l < L; l++) if ((iter >> l) & 1) matId[l] = m.MaterialId;
    }

    float texU[L], texV[L], grad[4][L], bary[3][L];
    for (int l = 0; l < L; l++) {
        F4 v0 = mul4(sc->object_to_clip, pos[0][l]), v1 = mul4(sc->object_to_clip, pos[1][l]), v2 = mul4(sc->object_to_clip, pos[2][l]);
        float iw0 = 1.0f / v0.w, iw1 = 1.0f / v1.w, iw2 = 1.0f / v2.w;
        float p0x = v0.x * iw0, p0y = v0.y * iw0, p1x = v1.x * iw1, p1y = v1.y * iw1, p2x = v2.x * iw2, p2y = v2.y * iw2;
        float m0x = p2x - p1x, m0y = p2y - p1y, m1x = p0x - p1x, m1y = p0y - p1y;
        float invDet = 1.0f / (m0x * m1y - m1x * m0y);
        float s0 = invDet * iw0, s1 = invDet * iw1, s2 = invDet * iw2;
        float dx[3] = { (p1y - p2y) * s0, (p2y - p0y) * s1, (p0y - p1y) * s2 };
        float dy[3] = { (p2x - p1x) * s0, (p0x - p2x) * s1, (p1x - p0x) * s2 };
        float dxs = dx[0] + dx[1] + dx[2], dys = dy[0] + dy[1] + dy[2];
        float r0x = su[l] - p0x, r0y = sv[l] - p0y;
        float interpInvW = iw0 + r0x * dxs + r0y * dys;
        float interpW = 1.0f / interpInvW;
        float b[3];
        b[1] = interpW * (r0x * dx[1] + r0y * dy[1]);
        b[2] = interpW * (r0x * dx[2] + r0y * dy[2]);
        b[0] = 1 - b[1] - b[2];
        float kx = 2.0f / W, ky = -(2.0f / H);
        for (int k = 0; k < 3; k++) dx[k] *= kx, dy[k] *= ky;
        dxs *= kx, dys *= ky;
        float wdx = 1.0f / (interpInvW + dxs), wdy = 1.0f / (interpInvW + dys);
        for (int k = 0; k < 3; k++) {
            dx[k] = wdx * (b[k] * interpInvW + dx[k]) - b[k];
            dy[k] = wdy * (b[k] * interpInvW + dy[k]) - b[k];
        }
        for (int k = 0; k < 3; k++) bary[k][l] = b[k];
        float t0x = half_to_float(tc[0][l] & 0xFFFF), t0y = half_to_float(tc[0][l] >> 16);
        float t10x = half_to_float(tc[1][l] & 0xFFFF) - t0x, t10y = half_to_float(tc[1][l] >> 16) - t0y;
        float t20x = half_to_float(tc[2][l] & 0xFFFF) - t0x, t20y = half_to_float(tc[2][l] >> 16) - t0y;
        texU[l] = t0x + t10x * b[1] + t20x * b[2];
        texV[l] = t0y + t10y * b[1] + t20y * b[2];
        grad[0][l] = t10x * dx[1] + t20x * dx[2];
        grad[1][l] = t10y * dx[1] + t20y * dx[2];
        grad[2][l] = t10x * dy[1] + t20x * dy[2];
        grad[3][l] = t10y * dy[1] + t20y * dy[2];
    }

    uint32_t albedo[L] = {}, nmr[L] = {};
    uint16_t pendingMat = 0;
    for (int l = 0; l < L; l++) if (((active >> l) & 1) && matId[l] != UINT32_MAX) pendingMat |= (uint16_t)(1u << l);
    while (pendingMat) {
        uint32_t id = matId[__builtin_ctz(pendingMat)];
        uint16_t iter = 0;
        for (int l = 0; l < L; l++) if (matId[l] == id) iter |= (uint16_t)(1u << l);
        pendingMat &= (uint16_t)~iter;
        const orc_material& mat = sc->materials[id];
        if (mat.texture == UINT32_MAX) continue;
        const orc_texture& tex = sc->textures[mat.texture];
        int32_t mip[L];
        float ssu = tex.scale_u * tex.scale_u, ssv = tex.scale_v * tex.scale_v;
        for (int l = 0; l < L; l++) mip[l] = calc_mip_level(grad[0][l], grad[1][l], grad[2][l], grad[3][l], ssu, ssv);
        uint32_t s[L];
        sample_rgba8(tex, texU, texV, 0, mip, s);
        for (int l = 0; l < L; l++) if ((iter >> l) & 1) albedo[l] = s[l];
        if (tex.num_layers >= 2) {
            sample_rgba8(tex, texU, texV, 1, mip, s);
            for (int l = 0; l < L; l++) if ((iter >> l) & 1) nmr[l] = s[l];
        }
    }

    F3 nrm[3][L], tan[3][L];
    bool anyNormalMap = false;
    for (int l = 0; l < L; l++) {
        for (int k = 0; k < 3; k++) {  // UnpackNormalTangent, Shading.cpp:232-236
            F4 o = unpack_rgba8(nt[k][l]);
            nrm[k][l] = unmap_oct(o.x, o.y);
            tan[k][l] = unmap_oct(o.z, o.w);
        }
        if ((nmr[l] & 0xFFFF) != 0) anyNormalMap = true;
    }
    for (int l = 0; l < L; l++) {
        const float b[3] = { bary[0][l], bary[1][l], bary[2][l] };
        F3 nws = normalize3(mul3(sc->object_to_world, bary_lerp(b, nrm[0][l], nrm[1][l], nrm[2][l])));
        F3 n = nws;
        if (anyNormalMap) {
            F3 tws = normalize3(mul3(sc->object_to_world, bary_lerp(b, tan[0][l], tan[1][l], tan[2][l])));
            F3 bws = { std::fma(nws.y, tws.z, -nws.z * tws.y), std::fma(nws.z, tws.x, -nws.x * tws.z),
                       std::fma(nws.x, tws.y, -nws.y * tws.x) };  // simd::cross, SIMD.h:431-437
            bws = { u2f(f2u(bws.x) ^ hand[l]), u2f(f2u(bws.y) ^ hand[l]), u2f(f2u(bws.z) ^ hand[l]) };
            float tx = (float)(nmr[l] & 255) * (1.0f / 127.5f) - 1.0f;
            float ty = (float)((nmr[l] >> 8) & 255) * (1.0f / 127.5f) - 1.0f;
            float tz = approx_sqrt(1.0f - (tx * tx + ty * ty));
            n = normalize3({ tx * tws.x + ty * bws.x + tz * nws.x, tx * tws.y + ty * bws.y + tz * nws.y,
                             tx * tws.z + ty * bws.z + tz * nws.z });
        }
        out[l].albedo = albedo[l];
        out[l].normal = n;
        out[l].metallic = (float)((nmr[l] >> 16) & 255) * (1.0f / 255);
        out[l].roughness = (float)((nmr[l] >> 24) & 255) * (1.0f / 255);
    }
}

// EvalLighting (Shading.cpp:602-645) with D_GGX / V_SmithGGXCorrelatedFast / F_Schlick (19-33)
// and GetLightAttenuation (581-600), 16 lanes.
void eval_lighting(const Surface* s, const orc_light* lights, uint32_t numLights, float exposure, const F3* worldPos,
                   F3 viewPos, F3* out) {
    const float invPi = 0.3183098861837907f;
    F3 base[L], f0[L], diffuse[L], viewDir[L];
    float alphaR[L], NoV[L];
    const float refl = 0.5f, f0d = 0.16f * refl * refl;
    for (int l = 0; l < L; l++) {
        F4 c = unpack_srgb(s[l].albedo);
        base[l] = { c.x, c.y, c.z };
        alphaR[l] = vmax(s[l].roughness * s[l].roughness, 1e-4f);
        f0[l] = { lerpf(f0d, c.x, s[l].metallic), lerpf(f0d, c.y, s[l].metallic), lerpf(f0d, c.z, s[l].metallic) };
        float dm = 1.0f - s[l].metallic;
        diffuse[l] = { c.x * dm, c.y * dm, c.z * dm };
        viewDir[l] = normalize3({ viewPos.x - worldPos[l].x, viewPos.y - worldPos[l].y, viewPos.z - worldPos[l].z });
        NoV[l] = std::fabs(dot3(s[l].normal, viewDir[l])) + 1e-5f;
        out[l] = { 0, 0, 0 };
    }
    for (uint32_t i = 0; i < numLights; i++) {
        const orc_light& li = lights[i];
        F3 ld[L];
        float NoL[L], att[L];
        bool allLow = true;
        for (int l = 0; l < L; l++) {
            if (li.type == 0) ld[l] = { -li.direction[0], -li.direction[1], -li.direction[2] };
            else ld[l] = normalize3({ li.position[0] - worldPos[l].x, li.position[1] - worldPos[l].y, li.position[2] - worldPos[l].z });
            NoL[l] = dot3(s[l].normal, ld[l]);
            if (!(NoL[l] < 1e-4f)) allLow = false;
        }
        if (allLow) continue;
        bool allWeak = true;
        for (int l = 0; l < L; l++) {
            float a = 1.0f;
            if (li.type != 0) {
                F3 p2l = { li.position[0] - worldPos[l].x, li.position[1] - worldPos[l].y, li.position[2] - worldPos[l].z };
                float d2 = dot3(p2l, p2l);
                float f = d2 * li.inv_radius_sq;
                float sm = vmax(1.0f - f * f, 0.0f);
                a = (sm * sm) * approx_rcp(vmax(d2, 1e-4f));
                if (li.type == 2) {
                    F3 nd = normalize3(p2l);
                    float cd = dot3({ -li.direction[0], -li.direction[1], -li.direction[2] }, nd);
                    float sa = vmin(vmax(cd * li.spot_scale + li.spot_offset, 0.0f), 1.0f);
                    a *= sa * sa;
                }
            }
            att[l] = a * li.intensity * exposure;
            if (!(NoL[l] * att[l] < 1e-4f)) allWeak = false;
        }
        if (allWeak) continue;
        for (int l = 0; l < L; l++) {
            F3 h = normalize3({ viewDir[l].x + ld[l].x, viewDir[l].y + ld[l].y, viewDir[l].z + ld[l].z });
            float NoH = vmin(vmax(dot3(s[l].normal, h), 0.0f), 1.0f);
            float LoH = vmin(vmax(dot3(ld[l], h), 0.0f), 1.0f);
            float r = alphaR[l];
            float a = NoH * r;
            float k = r * approx_rcp(1.0f - NoH * NoH + a * a);
            float D = k * k * invPi;
            float va = 2.0f * NoL[l] * NoV[l], vb = NoL[l] + NoV[l];
            float V = 0.5f / lerpf(va, vb, r);
            float x = 1.0f - LoH;
            float f = (x * x) * (x * x) * x;
            F3 F = { f + f0[l].x * (1.0f - f), f + f0[l].y * (1.0f - f), f + f0[l].z * (1.0f - f) };
            float DV = D * V;
            float w = vmax(NoL[l] * att[l], 0.0f);
            out[l].x += (diffuse[l].x * invPi + DV * F.x) * li.color[0] * w;
            out[l].y += (diffuse[l].y * invPi + DV * F.y) * li.color[1] * w;
            out[l].z += (diffuse[l].z * invPi + DV * F.z) * li.color[2] * w;
        }
    }
    for (int l = 0; l < L; l++) {
        out[l].x += base[l].x * 0.05f;
        out[l].y += base[l].y * 0.05f;
        out[l].z += base[l].z * 0.05f;
    }
}

}  // namespace
}  // namespace orc

using namespace orc;

// ShadingContext::Resolve (Shading.cpp:658-690). The light-sprite overlay (691-731) is not part
// of the restatement. The number of meshlets of the scene bounds the surface ids it accepts.
extern "C" void orc_resolve_rows(orc_framebuffer* fb, const orc_shading_context* sc, uint32_t row_begin, uint32_t row_end) {
    float invProj[16] = {};
    if (!swr_hostmath::inverse_screen_proj(sc->world_to_clip, fb->width, fb->height, invProj)) {
        fprintf(stderr, "orc_resolve: singular world-to-clip matrix\n");
        return;
    }
    const float W = (float)fb->width, H = (float)fb->height;
    const float scaleU = 2.0f / W, scaleV = 2.0f / H;
    const float centerU = 0.5f * scaleU - 1.0f, centerV = 0.5f * scaleV - 1.0f;
    uint32_t* colorLayer = fb->data;
    const float* depthLayer = (const float*)(fb->data + fb->layer_stride);
    const F3 viewPos = { sc->view_pos[0], sc->view_pos[1], sc->view_pos[2] };

    for (uint32_t y0 = row_begin & ~3u; y0 < std::min(row_end, fb->height); y0 += 4) {
        for (uint32_t x0 = 0; x0 < fb->width; x0 += 4) {
            uint32_t tileOffset = ((x0 & ~3u) << 2) + (y0 & ~3u) * fb->width;
            uint32_t ids[L];
            float su[L], sv[L];
            F3 world[L];
            uint16_t sky = 0;
            for (int l = 0; l < L; l++) {
                ids[l] = colorLayer[tileOffset + l];
                float d = depthLayer[tileOffset + l];
                bool isSky = d <= 0.0f;
                if (isSky) sky |= (uint16_t)(1u << l);
                float px = (float)(int32_t)(x0 + (l & 3)), py = (float)(int32_t)(y0 + (l >> 2));
                su[l] = px * scaleU + centerU;
                sv[l] = py * scaleV + centerV;
                V4 q = transform_point(invProj, px, py, isSky ? 1.0f : d);  // mul(invProj, (x, y, z, 1))
                float rw = 1.0f / q.w;
                world[l] = { q.x * rw, q.y * rw, q.z * rw };
            }
            F3 color[L] = {};
            if (sky != 0xFFFF) {
                Surface surf[L];
                resolve_surface(sc, ids, (uint16_t)~sky, su, sv, W, H, surf);
                eval_lighting(surf, sc->lights, sc->num_lights, sc->exposure * 0.001f, world, viewPos, color);
            }
            if (sky != 0 && sc->skybox != nullptr) {
                F3 dir[L], env[L];
                for (int l = 0; l < L; l++) dir[l] = { world[l].x - viewPos.x, world[l].y - viewPos.y, world[l].z - viewPos.z };
                sample_env(*sc->skybox, dir, 1.0f, env);
                for (int l = 0; l < L; l++) if ((sky >> l) & 1) color[l] = env[l];
            }
            for (int l = 0; l < L; l++) {  // Tonemap_Unreal (Shading.cpp:221-226) and RGBA8u::Pack
                float e = sc->exposure;
                F3 c = { color[l].x * e, color[l].y * e, color[l].z * e };
                F4 t = { c.x / (c.x + 0.155f) * 1.019f, c.y / (c.y + 0.155f) * 1.019f, c.z / (c.z + 0.155f) * 1.019f, 1.0f };
                colorLayer[tileOffset + l] = pack_rgba8(t);
            }
        }
    }
}

extern "C" void orc_resolve(orc_framebuffer* fb, const orc_shading_context* sc) { orc_resolve_rows(fb, sc, 0, fb->height); }

// Tiles are independent, so rows of 4x4 tiles split over threads give the same image.
extern "C" void orc_resolve_mt(orc_framebuffer* fb, const orc_shading_context* sc, uint32_t num_threads) {
    if (num_threads <= 1) { orc_resolve(fb, sc); return; }
    std::vector<std::thread> threads;
    uint32_t rows = ((fb->height + num_threads - 1) / num_threads + 3) & ~3u;
    for (uint32_t t = 0; t < num_threads; t++) {
        uint32_t r0 = t * rows, r1 = std::min(fb->height, r0 + rows);
        if (r0 >= r1) break;
        threads.emplace_back([=]() { orc_resolve_rows(fb, sc, r0, r1); });
    }
    for (auto& th : threads) th.join();
}

// ------------------------------------------------------------------------- debug layers
namespace orc {
namespace {

// Turbo colormap (Google Research 2019, polynomial fit; Shading.cpp:249-260), evaluated in Horner
// form in the reference's operation order.
F3 colormap_turbo(float x) {
    static const float c[18] = {
        0.13572138f, 4.61539260f,  -42.66032258f, 132.13108234f, -152.94239396f, 59.28637943f,
        0.09140261f, 2.19418839f,  4.84296658f,   -14.18503333f, 4.27729857f,    2.82956604f,
        0.10667330f, 12.64194608f, -60.58204836f, 110.36276771f, -89.90310912f,  27.34824973f,
    };
    auto poly = [&](const float* k) { return x * (x * (x * (x * (x * k[5] + k[4]) + k[3]) + k[2]) + k[1]) + k[0]; };
    return { poly(c), poly(c + 6), poly(c + 12) };
}

}  // namespace
}  // namespace orc

// ShadingContext::ResolveDebug (Shading.cpp:734-773): the selected layer as RGBA8 over the
// vis-buffer (or, for the overdraw layers, the OverdrawShader's counters); sky pixels (depth <= 0)
// get a checkerboard of 4x4 tiles.
extern "C" void orc_resolve_debug_rows(orc_framebuffer* fb, const orc_shading_context* sc, uint32_t layer,
                                       uint32_t row_begin, uint32_t row_end) {
    const float W = (float)fb->width, H = (float)fb->height;
    const float scaleU = 2.0f / W, scaleV = 2.0f / H;
    const float centerU = 0.5f * scaleU - 1.0f, centerV = 0.5f * scaleV - 1.0f;
    uint32_t* colorLayer = fb->data;
    const float* depthLayer = (const float*)(fb->data + fb->layer_stride);
    for (uint32_t y0 = row_begin & ~3u; y0 < std::min(row_end, fb->height); y0 += 4) {
        for (uint32_t x0 = 0; x0 < fb->width; x0 += 4) {
            uint32_t tileOffset = ((x0 & ~3u) << 2) + (y0 & ~3u) * fb->width;
            uint32_t data[L];
            float su[L], sv[L];
            uint16_t sky = 0;
            for (int l = 0; l < L; l++) {
                data[l] = colorLayer[tileOffset + l];
                if (depthLayer[tileOffset + l] <= 0.0f) sky |= (uint16_t)(1u << l);
                su[l] = (float)(int32_t)(x0 + (l & 3)) * scaleU + centerU;
                sv[l] = (float)(int32_t)(y0 + (l >> 2)) * scaleV + centerV;
            }
            Surface surf[L] = {};
            if (layer >= 1 && layer <= 3) resolve_surface(sc, data, (uint16_t)~sky, su, sv, W, H, surf);
            const uint32_t background = ((x0 ^ y0) & 4) ? 0xFFA0A0A0u : 0xFFFFFFFFu;
            for (int l = 0; l < L; l++) {
                F3 c = { 0.0f, 0.0f, 0.0f };
                if (layer == 1) {
                    F4 a = unpack_rgba8(surf[l].albedo);
                    c = { a.x, a.y, a.z };
                } else if (layer == 2) {
                    c = { surf[l].normal.x * 0.5f + 0.5f, surf[l].normal.y * 0.5f + 0.5f, surf[l].normal.z * 0.5f + 0.5f };
                } else if (layer == 3) {
                    c = { surf[l].metallic, surf[l].roughness, 0.0f };
                } else if (layer == 4 || layer == 5) {
                    F4 a = unpack_rgba8((layer == 4 ? data[l] / 128u : data[l]) * 123456789u);
                    c = { a.x, a.y, a.z };
                } else if (layer == 6) {
                    c = colormap_turbo((float)(data[l] >> 16) / 30.0f);
                } else if (layer == 7) {
                    float countPix = (float)(data[l] >> 16), countFrag = (float)(data[l] & 0xFFFF);
                    c = colormap_turbo((countPix + countFrag * 0.5f) / 30.0f);
                }
                colorLayer[tileOffset + l] = ((sky >> l) & 1) ? background : pack_rgba8({ c.x, c.y, c.z, 1.0f });
            }
        }
    }
}

extern "C" void orc_resolve_debug_mt(orc_framebuffer* fb, const orc_shading_context* sc, uint32_t layer,
                                     uint32_t num_threads) {
    num_threads = std::max(num_threads, 1u);
    std::vector<std::thread> threads;
    uint32_t rows = ((fb->height + num_threads - 1) / num_threads + 3) & ~3u;
    for (uint32_t t = 0; t < num_threads; t++) {
        uint32_t r0 = t * rows, r1 = std::min(fb->height, r0 + rows);
        if (r0 >= r1) break;
        threads.emplace_back([=]() { orc_resolve_debug_rows(fb, sc, layer, r0, r1); });
    }
    for (auto& th : threads) th.join();
}

// The pieces of the resolve and its sampler on their own, for the known-answer tests of tests/.
extern "C" {
uint32_t orc_debug_lerp16(uint32_t a, uint32_t b, uint32_t t) { return lerp16(a, b, t); }
void orc_debug_unpack_srgb(uint32_t p, float* out) {
    const F4 v = unpack_srgb(p);
    out[0] = v.x, out[1] = v.y, out[2] = v.z, out[3] = v.w;
}
void orc_debug_unpack_r11g11b10(uint32_t p, float* out) {
    const F3 v = unpack_r11g11b10(p);
    out[0] = v.x, out[1] = v.y, out[2] = v.z;
}
int32_t orc_debug_calc_mip_level(float gx, float gy, float gz, float gw, float scaleU, float scaleV) {
    return calc_mip_level(gx, gy, gz, gw, scaleU * scaleU, scaleV * scaleV);
}
void orc_debug_map_oct(const float* n, float* uv) { map_oct({ n[0], n[1], n[2] }, uv[0], uv[1]); }
void orc_debug_unmap_oct(const float* uv, float* n) {
    const F3 r = unmap_oct(uv[0], uv[1]);
    n[0] = r.x, n[1] = r.y, n[2] = r.z;
}
void orc_debug_sample_rgba8(const orc_texture* t, const float* u, const float* v, int layer, const int32_t* mip,
                            uint32_t* out) {
    sample_rgba8(*t, u, v, layer, mip, out);
}
}
