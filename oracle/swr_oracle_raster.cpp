// Oracle (test infrastructure, see swr_oracle.h): framebuffer, mesh shader, clipper,
// triangle setup and the vis-buffer fragment shader of GLimpSW's meshlet rasterizer,
// restated lane by lane in the reference's operation order.
#include "swr_oracle_common.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- framebuffer
// CreateFramebuffer, Rasterizer.h:66-78: layer stride rounded to 64 words.
uint32_t fb_layer_stride(uint32_t w, uint32_t h) { return (w * h + 63) & ~63u; }

// Framebuffer::GetPixelOffset, Rasterizer.h:50-56 (4x4 tiles).
static inline uint32_t pixel_offset(const orc_framebuffer* fb, uint32_t x, uint32_t y) {
    uint32_t tileOffset = ((x & ~3u) << 2) + (y & ~3u) * fb->width;
    uint32_t pixelOffset = (x & 3) + (y & 3) * 4;
    return pixelOffset + tileOffset;
}

// ----------------------------------------------------------- packed int16 ops
// The reference keeps (x, y) viewport positions as two int16 halves of one int32
// lane and mixes per-16-bit ops (_mm512_*_epi16) with 32-bit adds/ands.
static inline int32_t lo16(uint32_t v) { return (int16_t)(v & 0xFFFF); }
static inline int32_t hi16(uint32_t v) { return (int16_t)(v >> 16); }
static inline uint32_t pack16(int32_t lo, int32_t hi) { return (uint32_t)(uint16_t)lo | ((uint32_t)(uint16_t)hi << 16); }
static inline uint32_t min16(uint32_t a, uint32_t b) { return pack16(std::min(lo16(a), lo16(b)), std::min(hi16(a), hi16(b))); }
static inline uint32_t max16(uint32_t a, uint32_t b) { return pack16(std::max(lo16(a), lo16(b)), std::max(hi16(a), hi16(b))); }
static inline uint32_t add16(uint32_t a, uint32_t b) { return pack16(lo16(a) + lo16(b), hi16(a) + hi16(b)); }
static inline uint32_t srai16(uint32_t a, int s) { return pack16(lo16(a) >> s, hi16(a) >> s); }

// ------------------------------------------------------------ triangle packet
using Vtx = V4;

struct TriSetup {   // one lane of TrianglePacket (Rasterizer.h:145-161)
    uint32_t Pos0, Pos1, Pos2;
    float Z0, Z1, Z2, W0, W1, W2;
};
struct EdgeVars {   // one lane of TriangleEdgeVars (Rasterizer.h:162-176)
    int32_t Edge0, Edge1, Edge2, A01, A12, A20, B01, B12, B20;
    float Z0, Z10, Z20, W0, W0S, W1S, W2S;
};

// simd::perspective_div, SIMD.h:473-476.
static inline Vtx perspective_div(Vtx v) {
    float rw = 1.0f / v.w;
    return { v.x * rw, v.y * rw, v.z * rw, rw };
}

// TrianglePacket::GetBoundingBox / GetRenderBoundingBox, Rasterizer.cpp:331-351.
static inline void render_bbox(const TriSetup& t, int halfW, int halfH, uint32_t& bbMin, uint32_t& bbMax) {
    uint32_t minPos = min16(min16(t.Pos0, t.Pos1), t.Pos2);
    uint32_t maxPos = max16(max16(t.Pos0, t.Pos1), t.Pos2);
    minPos = srai16(minPos + 0x00070007u, 4);  // 32-bit add: a carry out of x reaches y
    maxPos = srai16(maxPos + 0x00070007u, 4);

    uint32_t vpSize = (uint32_t)halfW | ((uint32_t)halfH << 16);
    uint32_t x = min16(max16(add16(minPos, vpSize), 0), vpSize * 2);
    uint32_t y = min16(max16(add16(maxPos, vpSize), 0), vpSize * 2);
    bbMin = (x + 0x00000000u) & ~0x00030003u;
    bbMax = (y + 0x00030003u) & ~0x00030003u;
}

// TrianglePacket::Setup, Rasterizer.cpp:257-289. Returns the lane's keep bit.
static bool tri_setup(Vtx v0, Vtx v1, Vtx v2, int halfW, int halfH, int cullMode, TriSetup& t) {
    v0 = perspective_div(v0);
    v1 = perspective_div(v1);
    v2 = perspective_div(v2);

    float det = (v2.x - v0.x) * (v1.y - v0.y) - (v0.x - v1.x) * (v0.y - v2.y);
    if (cullMode != CULL_FRONT_CCW) {
        bool flip = (cullMode == CULL_FRONT_CW) ? true : (det < 0);
        det = flip ? -det : det;
    }
    bool keep = det > 0;

    float fsx = (float)(halfW * 16), fsy = (float)(halfH * 16);
    int32_t x0 = round2i(v0.x * fsx), y0 = round2i(v0.y * fsy);
    int32_t x1 = round2i(v1.x * fsx), y1 = round2i(v1.y * fsy);
    int32_t x2 = round2i(v2.x * fsx), y2 = round2i(v2.y * fsy);
    t.Pos0 = ((uint32_t)x0 & 0xFFFF) | ((uint32_t)y0 << 16);
    t.Pos1 = ((uint32_t)x1 & 0xFFFF) | ((uint32_t)y1 << 16);
    t.Pos2 = ((uint32_t)x2 & 0xFFFF) | ((uint32_t)y2 << 16);

    uint32_t bbMin, bbMax;
    render_bbox(t, halfW, halfH, bbMin, bbMax);
    // cmpge_epi16 on both halves, kept only if neither half has min >= max.
    if (lo16(bbMin) >= lo16(bbMax) || hi16(bbMin) >= hi16(bbMax)) keep = false;

    t.Z0 = v0.z, t.Z1 = v1.z, t.Z2 = v2.z;
    t.W0 = v0.w, t.W1 = v1.w, t.W2 = v2.w;
    return keep;
}

// ComputeEdge, Rasterizer.cpp:291-295 (wrapping int32 arithmetic).
static inline int32_t compute_edge(int32_t a, int32_t x, int32_t b, int32_t y) {
    int32_t w = (int32_t)((uint32_t)a * (uint32_t)x + (uint32_t)b * (uint32_t)y);
    w = (int32_t)((uint32_t)w + ((a > 0 || (a == 0 && b > 0)) ? 0u : 0xFFFFFFFFu));
    return w >> 4;
}

// TriangleEdgeVars::Setup, Rasterizer.cpp:296-329.
static void edge_setup(const TriSetup& t, int halfW, int halfH, EdgeVars& e) {
    int32_t x0 = (int32_t)(t.Pos0 << 16) >> 16, y0 = (int32_t)t.Pos0 >> 16;
    int32_t x1 = (int32_t)(t.Pos1 << 16) >> 16, y1 = (int32_t)t.Pos1 >> 16;
    int32_t x2 = (int32_t)(t.Pos2 << 16) >> 16, y2 = (int32_t)t.Pos2 >> 16;

    int32_t A01 = y1 - y0, B01 = x0 - x1;
    int32_t A12 = y2 - y1, B12 = x1 - x2;
    int32_t A20 = y0 - y2, B20 = x2 - x0;
    int32_t det = (int32_t)((uint32_t)B20 * (uint32_t)A01 - (uint32_t)B01 * (uint32_t)A20);
    if (det < 0) {  // per-lane flip of the `any(det < 0)` block
        A01 = -A01, B01 = -B01, A12 = -A12, B12 = -B12, A20 = -A20, B20 = -B20;
        det = -det;
    }
    int32_t sampleX = (int32_t)((uint32_t)(-halfW) << 4) + 8, sampleY = (int32_t)((uint32_t)(-halfH) << 4) + 8;
    e.Edge0 = compute_edge(A12, sampleX - x1, B12, sampleY - y1);
    e.Edge1 = compute_edge(A20, sampleX - x2, B20, sampleY - y2);
    e.Edge2 = compute_edge(A01, sampleX - x0, B01, sampleY - y0);
    e.A01 = A01, e.A12 = A12, e.A20 = A20, e.B01 = B01, e.B12 = B12, e.B20 = B20;

    float rcpArea = 16.0f / (float)det;
    e.Z0 = t.Z0;
    e.Z10 = (t.Z1 - t.Z0) * rcpArea;
    e.Z20 = (t.Z2 - t.Z0) * rcpArea;
    e.W0 = t.W0;
    e.W0S = t.W0 * rcpArea;
    e.W1S = t.W1 * rcpArea;
    e.W2S = t.W2 * rcpArea;
}

// ----------------------------------------------------------------- clip codes
enum { PLANE_LEFT = 0, PLANE_RIGHT, PLANE_TOP, PLANE_BOTTOM, PLANE_NEAR, PLANE_FAR };

struct ClipCodes { uint16_t AcceptMask, NonTrivialMask; uint8_t OutCodes[16]; };

// Clipper::ComputeClipCodes, Rasterizer.cpp:353-397.
static ClipCodes compute_clip_codes(const Vtx v[3][16], float bx, float by) {
    ClipCodes cc = {};
    bool allInside = true;
    for (int l = 0; l < 16; l++) {
        for (int i = 0; i < 3; i++) {
            const Vtx& p = v[i][l];
            float m = max_abs(max_abs(p.x, p.y), p.z);
            if (!(m < p.w)) allInside = false;
        }
    }
    if (allInside) { cc.AcceptMask = 0xFFFF; return cc; }

    for (int l = 0; l < 16; l++) {
        uint8_t partial = 0, combined = 255;
        bool trivial = true;
        for (int i = 0; i < 3; i++) {
            const Vtx& p = v[i][l];
            uint8_t oc = 0;
            oc |= (p.x < -p.w) ? (1 << PLANE_LEFT) : 0;
            oc |= (p.x > +p.w) ? (1 << PLANE_RIGHT) : 0;
            oc |= (p.y < -p.w) ? (1 << PLANE_TOP) : 0;
            oc |= (p.y > +p.w) ? (1 << PLANE_BOTTOM) : 0;
            oc |= (p.z < -p.w) ? (1 << PLANE_NEAR) : 0;
            oc |= (p.z > +p.w) ? (1 << PLANE_FAR) : 0;
            partial |= oc;
            combined &= oc;
            trivial = trivial && (std::fabs(p.x) < p.w * bx && std::fabs(p.y) < p.w * by);
        }
        if (partial & ((1 << PLANE_NEAR) | (1 << PLANE_FAR))) trivial = false;
        bool accept = combined == 0;
        if (accept && trivial) cc.AcceptMask |= 1u << l;
        if (accept && !trivial) cc.NonTrivialMask |= 1u << l;
        cc.OutCodes[l] = partial;
    }
    return cc;
}

// ---------------------------------------------------------------- draw state
struct DrawCtx {
    orc_framebuffer* fb;
    const orc_shading_context* sc;
    int halfW, halfH;
    uint32_t rowBegin, rowEnd;  // rows this call may write
    uint64_t* counters;
};

// Rasterizer::DrawTriangle<FS_EncodeSurfaceId<false>, IsClipped> (Rasterizer.h:250-328 with
// Shading.cpp:309-331). The opaque vis-buffer shader uses only Depth and the ids, so the
// perspective-correct barycentrics (rcp14 + Newton) do not affect its output.
static void draw_triangle(DrawCtx& dc, const EdgeVars& e, uint32_t bbMin, uint32_t bbMax,
                          uint32_t meshletId, uint32_t primId) {
    orc_framebuffer* fb = dc.fb;
    uint32_t minX = bbMin & 0xFFFF, minY = bbMin >> 16;
    uint32_t maxX = bbMax & 0xFFFF, maxY = bbMax >> 16;
    uint32_t y0 = std::max(minY, dc.rowBegin), y1 = std::min(maxY, dc.rowEnd);
    float* depthBuf = (float*)&fb->data[1 * fb->layer_stride];
    uint32_t* colorBuf = &fb->data[0];
    uint32_t surfaceId = (dc.sc->meshlet_offset + meshletId) * 128u + primId;

    for (uint32_t y = y0; y < y1; y++) {
        for (uint32_t x = minX; x < maxX; x++) {
            int32_t e0 = (int32_t)((uint32_t)e.Edge0 + (uint32_t)e.A12 * x + (uint32_t)e.B12 * y);
            int32_t e1 = (int32_t)((uint32_t)e.Edge1 + (uint32_t)e.A20 * x + (uint32_t)e.B20 * y);
            int32_t e2 = (int32_t)((uint32_t)e.Edge2 + (uint32_t)e.A01 * x + (uint32_t)e.B01 * y);
            if ((e0 | e1 | e2) < 0) continue;

            float u = (float)e1, v = (float)e2;
            float depth = std::fma(u, e.Z10, std::fma(v, e.Z20, e.Z0));
            uint32_t off = pixel_offset(fb, x, y);
            if (!(depth > depthBuf[off])) continue;  // FS_EncodeSurfaceId depth test, Shading.cpp:312-313
            depthBuf[off] = depth;
            colorBuf[off] = surfaceId;
        }
    }
}

// Inputs of FS_EncodeSurfaceId<true> (Shading.cpp:309-331) for one triangle: the material's
// texture (layer 0) and cutoff, the texcoords of the triangle's three vertices and, for a clipped
// triangle, its TriangleClipData rows (Rasterizer.cpp:455-458).
struct AlphaTri {
    const orc_texture* tex;
    uint32_t cutoff;        // AlphaCutoff << 24
    float uv[3][2];
    bool clipped;
    float ru[3], rv[3];
};

// Mesh::TexCoords[VertexId] (Shading.cpp:320-322). The index byte is not bounded by the
// reference: an index past the 64 texcoords reads the words that follow them in the record
// (NormalTangents, Indices). That is restated for indices below 224; indices from 224 on would
// read the next record and read 0 here.
static uint32_t texcoord_word(const Meshlet& mesh, uint32_t idx) {
    if (idx >= 224) return 0;
    uint32_t w;
    memcpy(&w, (const uint8_t*)&mesh + offsetof(Meshlet, TexCoords) + 4 * idx, 4);
    return w;
}

// DrawTriangle<FS_EncodeSurfaceId<true>, IsClipped> (Rasterizer.h:250-328, Shading.cpp:309-331)
// tile by tile, as the reference's 16 lanes: every lane of a visited tile computes its
// perspective-correct barycentrics, texcoord and scaled sample position, whether or not it is
// covered; the implicit LOD takes 2x2 finite differences across the tile (texutil::dFdx/dFdy,
// Texture.h:258-275) and the filter is chosen over all 16 lanes (Texture.h:432).
static void draw_triangle_alpha(DrawCtx& dc, const EdgeVars& e, uint32_t bbMin, uint32_t bbMax, uint32_t meshletId,
                                uint32_t primId, const AlphaTri& at) {
    orc_framebuffer* fb = dc.fb;
    uint32_t minX = bbMin & 0xFFFF, minY = bbMin >> 16;
    uint32_t maxX = bbMax & 0xFFFF, maxY = bbMax >> 16;
    float* depthBuf = (float*)&fb->data[1 * fb->layer_stride];
    uint32_t* colorBuf = &fb->data[0];
    uint32_t surfaceId = (dc.sc->meshlet_offset + meshletId) * 128u + primId;
    const orc_texture& tex = *at.tex;

    for (uint32_t ty = std::max(minY, dc.rowBegin & ~3u); ty < maxY && ty < dc.rowEnd; ty += 4) {
        for (uint32_t tx = minX; tx < maxX; tx += 4) {
            float u[16], v[16], depth[16];
            uint32_t mask = 0;
            for (uint32_t l = 0; l < 16; l++) {
                uint32_t x = tx + (l & 3), y = ty + (l >> 2);
                int32_t e0 = (int32_t)((uint32_t)e.Edge0 + (uint32_t)e.A12 * x + (uint32_t)e.B12 * y);
                int32_t e1 = (int32_t)((uint32_t)e.Edge1 + (uint32_t)e.A20 * x + (uint32_t)e.B20 * y);
                int32_t e2 = (int32_t)((uint32_t)e.Edge2 + (uint32_t)e.A01 * x + (uint32_t)e.B01 * y);
                if ((e0 | e1 | e2) >= 0) mask |= 1u << l;
                u[l] = (float)e1, v[l] = (float)e2;
                depth[l] = std::fma(u[l], e.Z10, std::fma(v[l], e.Z20, e.Z0));
            }
            if (mask == 0) continue;  // DrawTriangle visits only tiles with a covered sample
            // depth test (Shading.cpp:312-313); rows this call does not own are never written
            for (uint32_t l = 0; l < 16; l++) {
                uint32_t y = ty + (l >> 2);
                if (!((mask >> l) & 1)) continue;
                if (y < dc.rowBegin || y >= dc.rowEnd || !(depth[l] > depthBuf[pixel_offset(fb, tx + (l & 3), y)]))
                    mask &= ~(1u << l);
            }
            if (mask == 0) continue;

            float uvx[16], uvy[16], su[16], sv[16];
            for (uint32_t l = 0; l < 16; l++) {
                // perspective correction (Rasterizer.h:300-317)
                float pw0 = std::fma(u[l] + v[l], -e.W0S, e.W0);
                float w = std::fma(u[l], e.W1S, std::fma(v[l], e.W2S, pw0));
                float rcpW = approx_rcp(w);
                rcpW *= std::fma(-w, rcpW, 2.0f);
                float bu = u[l] * (e.W1S * rcpW);
                float bv = v[l] * (e.W2S * rcpW);
                if (at.clipped) {
                    float cu = std::fma(bu, at.ru[1], std::fma(bv, at.ru[2], at.ru[0]));
                    float cv = std::fma(bu, at.rv[1], std::fma(bv, at.rv[2], at.rv[0]));
                    bu = cu, bv = cv;
                }
                float b0 = 1 - bu - bv;
                // FragmentVars::Interpolate = BaryLerp (Rasterizer.h:101-104)
                uvx[l] = std::fma(at.uv[0][0], b0, std::fma(at.uv[1][0], bu, at.uv[2][0] * bv));
                uvy[l] = std::fma(at.uv[0][1], b0, std::fma(at.uv[1][1], bu, at.uv[2][1] * bv));
                su[l] = uvx[l] * tex.scale_lerp_u;
                sv[l] = uvy[l] * tex.scale_lerp_v;
            }
            // SampleImplicitLod (Texture.h:403-410): CalcMipLevel(grad) - LerpFracBits
            int32_t mip[16];
            for (uint32_t l = 0; l < 16; l++) {
                float gx = su[l | 1] - su[l & ~1u], gy = sv[l | 1] - sv[l & ~1u];
                float gz = su[l | 4] - su[l & ~4u], gw = sv[l | 4] - sv[l & ~4u];
                float dx = std::fma(gx, gx, gy * gy);
                float dy = std::fma(gz, gz, gw * gw);
                mip[l] = (ilog2_x86(vmax(dx, dy)) >> 1) - 8;
            }
            uint32_t color[16];
            sample_rgba8(tex, uvx, uvy, 0, mip, color);
            for (uint32_t l = 0; l < 16; l++) {
                if (!((mask >> l) & 1) || color[l] < at.cutoff) continue;  // Shading.cpp:326
                uint32_t off = pixel_offset(fb, tx + (l & 3), ty + (l >> 2));
                depthBuf[off] = depth[l];
                colorBuf[off] = surfaceId;
            }
        }
    }
}

// DrawTriangle<FragFn> (Rasterizer.h:250-328) for the fragment shaders that need the full
// FragmentVars: FS_EncodeGBuffer (kind ORC_SHADER_DEFERRED, Shading.cpp:344-414) and the texcoord
// shader of the shader-hook tests (ORC_SHADER_TEXCOORD: depth test, depth, surface id in layer 0 and
// the bits of the interpolated texcoords, FragmentVars::Interpolate of Mesh::TexCoords[VertexId],
// in layers 2 and 3). Per 4x4 tile with a covered sample: depth test, then the perspective-correct
// barycentrics of all 16 lanes (rcp14 + Newton step, clip remap, Rasterizer.h:300-317).
static void draw_triangle_frag(DrawCtx& dc, const EdgeVars& e, uint32_t bbMin, uint32_t bbMax, uint32_t meshletId,
                               uint32_t primId, const uint8_t vid8[3], const float* ru, const float* rv, int kind) {
    orc_framebuffer* fb = dc.fb;
    const uint32_t minX = bbMin & 0xFFFF, minY = bbMin >> 16, maxX = bbMax & 0xFFFF, maxY = bbMax >> 16;
    float* depthBuf = (float*)&fb->data[1 * fb->layer_stride];
    uint32_t* colorBuf = &fb->data[0];
    const uint32_t g = dc.sc->meshlet_offset + meshletId;
    const Meshlet& mesh = ((const Meshlet*)dc.sc->meshlets)[g];
    const uint32_t vid[3] = { vid8[0], vid8[1], vid8[2] };
    for (uint32_t ty = std::max(minY, dc.rowBegin & ~3u); ty < maxY && ty < dc.rowEnd; ty += 4) {
        for (uint32_t tx = minX; tx < maxX; tx += 4) {
            float u[16], v[16], depth[16];
            uint32_t mask = 0;
            for (uint32_t l = 0; l < 16; l++) {
                const uint32_t x = tx + (l & 3), y = ty + (l >> 2);
                const int32_t e0 = (int32_t)((uint32_t)e.Edge0 + (uint32_t)e.A12 * x + (uint32_t)e.B12 * y);
                const int32_t e1 = (int32_t)((uint32_t)e.Edge1 + (uint32_t)e.A20 * x + (uint32_t)e.B20 * y);
                const int32_t e2 = (int32_t)((uint32_t)e.Edge2 + (uint32_t)e.A01 * x + (uint32_t)e.B01 * y);
                if ((e0 | e1 | e2) >= 0) mask |= 1u << l;
                u[l] = (float)e1, v[l] = (float)e2;
                depth[l] = std::fma(u[l], e.Z10, std::fma(v[l], e.Z20, e.Z0));
            }
            if (mask == 0) continue;
            for (uint32_t l = 0; l < 16; l++) {  // depth test; rows this call does not own are never written
                const uint32_t y = ty + (l >> 2);
                if (!((mask >> l) & 1)) continue;
                if (y < dc.rowBegin || y >= dc.rowEnd || !(depth[l] > depthBuf[pixel_offset(fb, tx + (l & 3), y)]))
                    mask &= ~(1u << l);
            }
            if (mask == 0) continue;
            float bu[16], bv[16];
            for (uint32_t l = 0; l < 16; l++) {
                const float pw0 = std::fma(u[l] + v[l], -e.W0S, e.W0);
                const float w = std::fma(u[l], e.W1S, std::fma(v[l], e.W2S, pw0));
                float rcpW = approx_rcp(w);
                rcpW *= std::fma(-w, rcpW, 2.0f);
                bu[l] = u[l] * (e.W1S * rcpW);
                bv[l] = v[l] * (e.W2S * rcpW);
                if (ru) {
                    const float cu = std::fma(bu[l], ru[1], std::fma(bv[l], ru[2], ru[0]));
                    const float cv = std::fma(bu[l], rv[1], std::fma(bv[l], rv[2], rv[0]));
                    bu[l] = cu, bv[l] = cv;
                }
            }
            uint32_t out0[16], out2[16], out3[16];
            bool writeColor = true;
            if (kind == ORC_SHADER_DEFERRED) {
                if (mesh.MaterialId == UINT32_MAX) {
                    writeColor = false;  // Shading.cpp:350-353: depth only
                } else {
                    mask = gbuffer_tile(dc.sc, &mesh, vid, bu, bv, mask, out0, out2);
                }
            } else {
                float tc[3][2];
                for (int k = 0; k < 3; k++) {
                    uint32_t w = 0;
                    if (832u + 4u * vid[k] < sizeof(Meshlet)) memcpy(&w, (const uint8_t*)&mesh + 832 + 4 * vid[k], 4);
                    tc[k][0] = half_to_float(w & 0xFFFF), tc[k][1] = half_to_float(w >> 16);
                }
                for (uint32_t l = 0; l < 16; l++) {
                    const float b0 = 1 - bu[l] - bv[l];
                    const float su = std::fma(tc[0][0], b0, std::fma(tc[1][0], bu[l], tc[2][0] * bv[l]));
                    const float sv = std::fma(tc[0][1], b0, std::fma(tc[1][1], bu[l], tc[2][1] * bv[l]));
                    out0[l] = g * 128u + primId;
                    memcpy(&out2[l], &su, 4);
                    memcpy(&out3[l], &sv, 4);
                }
            }
            for (uint32_t l = 0; l < 16; l++) {
                if (!((mask >> l) & 1)) continue;
                const uint32_t off = pixel_offset(fb, tx + (l & 3), ty + (l >> 2));
                depthBuf[off] = depth[l];
                if (!writeColor) continue;
                colorBuf[off] = out0[l];
                if (fb->num_layers > 2) fb->data[2 * fb->layer_stride + off] = out2[l];
                if (kind == ORC_SHADER_TEXCOORD && fb->num_layers > 3) fb->data[3 * fb->layer_stride + off] = out3[l];
            }
        }
    }
}

// DrawTriangle<FS_Overdraw> (Rasterizer.h:250-328, Shading.cpp:333-342): no depth test; every tile
// of the box with a covered sample adds 1 to the high 16 bits of its covered pixels' colour words
// and 1 to the low 16 bits of the others (saturating, _mm512_adds_epu16), and stores
// max(Depth, old) on all 16 samples.
static inline uint32_t adds_epu16(uint32_t a, uint32_t b) {
    uint32_t lo = std::min((a & 0xFFFF) + (b & 0xFFFF), 0xFFFFu), hi = std::min((a >> 16) + (b >> 16), 0xFFFFu);
    return lo | (hi << 16);
}
static void draw_triangle_overdraw(DrawCtx& dc, const EdgeVars& e, uint32_t bbMin, uint32_t bbMax) {
    orc_framebuffer* fb = dc.fb;
    uint32_t minX = bbMin & 0xFFFF, minY = bbMin >> 16;
    uint32_t maxX = bbMax & 0xFFFF, maxY = bbMax >> 16;
    float* depthBuf = (float*)&fb->data[1 * fb->layer_stride];
    uint32_t* colorBuf = &fb->data[0];
    for (uint32_t ty = std::max(minY, dc.rowBegin & ~3u); ty < maxY && ty < dc.rowEnd; ty += 4) {
        for (uint32_t tx = minX; tx < maxX; tx += 4) {
            float depth[16];
            uint32_t mask = 0;
            for (uint32_t l = 0; l < 16; l++) {
                uint32_t x = tx + (l & 3), y = ty + (l >> 2);
                int32_t e0 = (int32_t)((uint32_t)e.Edge0 + (uint32_t)e.A12 * x + (uint32_t)e.B12 * y);
                int32_t e1 = (int32_t)((uint32_t)e.Edge1 + (uint32_t)e.A20 * x + (uint32_t)e.B20 * y);
                int32_t e2 = (int32_t)((uint32_t)e.Edge2 + (uint32_t)e.A01 * x + (uint32_t)e.B01 * y);
                if ((e0 | e1 | e2) >= 0) mask |= 1u << l;
                depth[l] = std::fma((float)e1, e.Z10, std::fma((float)e2, e.Z20, e.Z0));
            }
            if (mask == 0) continue;
            for (uint32_t l = 0; l < 16; l++) {
                uint32_t y = ty + (l >> 2);
                if (y < dc.rowBegin || y >= dc.rowEnd) continue;
                uint32_t off = pixel_offset(fb, tx + (l & 3), y);
                colorBuf[off] = adds_epu16(colorBuf[off], ((mask >> l) & 1) ? 0x00010000u : 0x00000001u);
                depthBuf[off] = vmax(depth[l], depthBuf[off]);
            }
        }
    }
}

// ShadeMeshlet, Shading.cpp:281-307. ShadedMeshlet (Rasterizer.h:82-99) with vertices past the
// transformed 16-vertex chunks zero-initialised (uninitialised stack memory in the reference).
struct Shaded {
    uint32_t PrimCount;
    int CullMode;
    uint32_t FragmentShaderId;
    uint32_t MaterialId;
    uint8_t Indices[3][128];
    Vtx Pos[64];
};

static void shade_meshlet(const orc_shading_context* sc, uint32_t index, Shaded& out) {
    out.PrimCount = 0;
    out.CullMode = CULL_FRONT_CCW;
    out.FragmentShaderId = 0;
    out.MaterialId = UINT32_MAX;
    if (sc->cull_bitmap != nullptr) {
        uint16_t mask = sc->cull_bitmap[index / 16];
        if (((mask >> (index % 16)) & 1) == 0) return;
    }
    const Meshlet& mesh = ((const Meshlet*)sc->meshlets)[sc->meshlet_offset + index];
    const float* m = sc->object_to_clip;
    for (uint32_t i = 0; i < 64; i++) out.Pos[i] = { 0, 0, 0, 0 };
    for (uint32_t i0 = 0; i0 < mesh.NumVertices; i0 += 16) {
        for (uint32_t i = i0; i < i0 + 16; i++) {
            float x = mesh.Positions[0][i], y = mesh.Positions[1][i], z = mesh.Positions[2][i];
            out.Pos[i] = transform_point(m, x, y, z);
        }
    }
    out.PrimCount = mesh.NumTriangles;
    memcpy(out.Indices, mesh.Indices, sizeof(mesh.Indices));
    out.MaterialId = mesh.MaterialId;
    if (mesh.MaterialId != UINT32_MAX) {
        const orc_material& mat = sc->materials[mesh.MaterialId];
        out.CullMode = mat.is_double_sided ? CULL_NONE : CULL_FRONT_CCW;
        out.FragmentShaderId = mat.alpha_cutoff < 255 ? 1 : 0;
    }
}

// Clipper::ClipTriangles + FlushPacket, Rasterizer.cpp:398-491, for one packet. Emits the
// clipped triangles in output order (prim id, then fan index); a callback draws each one.
struct ClipOut { TriSetup t; bool keep; uint32_t primId; float ru[3], rv[3]; };

static void clip_packet(const Vtx v[3][16], const ClipCodes& cc, uint16_t nonTrivialMask, float bx, float by,
                        int halfW, int halfH, int cullMode, std::vector<ClipOut>& outs) {
    float V[6][16 * 3 + 16];
    for (uint32_t i = 0; i < 3; i++) {
        for (uint32_t l = 0; l < 16; l++) {
            uint32_t j = i * 16 + l;
            V[0][j] = v[i][l].x, V[1][j] = v[i][l].y, V[2][j] = v[i][l].z, V[3][j] = v[i][l].w;
            V[4][j] = (i == 1) ? 1.0f : 0.0f;
            V[5][j] = (i == 2) ? 1.0f : 0.0f;
        }
    }
    const float guard[2] = { bx, by };
    uint32_t outIdx = 0;
    for (uint32_t primId = 0; primId < 16; primId++) {
        if (!((nonTrivialMask >> primId) & 1)) continue;
        uint8_t indices[32] = { (uint8_t)(primId), (uint8_t)(primId + 16), (uint8_t)(primId + 32) };
        uint32_t vertCount = 3, nextIdx = 48;

        for (uint32_t planeId = 0; planeId < 8; planeId++) {
            if (!((cc.OutCodes[primId] >> planeId) & 1)) continue;
            uint8_t outIndices[32];
            uint32_t outCount = 0;
            float planeScale = planeId < 4 ? guard[planeId / 2] : 1.0f;

            for (uint32_t vi = 0; vi < vertCount; vi++) {
                uint8_t ia = indices[vi], ib = indices[(vi + 1) % vertCount];
                // Clipper::GetIntersectDist, Rasterizer.cpp:76-81
                float aa = V[planeId / 2][ia], ab = V[planeId / 2][ib];
                if (planeId % 2) aa = -aa, ab = -ab;
                float da = aa + V[3][ia] * planeScale;
                float db = ab + V[3][ib] * planeScale;

                if (da >= 0) outIndices[outCount++] = ia;
                if ((da >= 0) != (db >= 0)) {
                    float t = da / (da - db);
                    for (uint32_t k = 0; k < 6; k++) {
                        V[k][nextIdx] = std::fma(V[k][ib], t, std::fma(-t, V[k][ia], V[k][ia]));
                    }
                    outIndices[outCount++] = (uint8_t)nextIdx++;
                }
            }
            if (vertCount < 3) break;  // stale count check, Rasterizer.cpp:443
            vertCount = outCount;
            memcpy(indices, outIndices, sizeof(indices));
        }
        if (vertCount < 2) continue;

        for (uint32_t vi = 0; vi + 2 < vertCount; vi++) {
            uint32_t i0 = indices[0], i1 = indices[vi + 1], i2 = indices[vi + 2];
            Vtx a = { V[0][i0], V[1][i0], V[2][i0], V[3][i0] };
            Vtx b = { V[0][i1], V[1][i1], V[2][i1], V[3][i1] };
            Vtx c = { V[0][i2], V[1][i2], V[2][i2], V[3][i2] };
            ClipOut co;
            co.keep = tri_setup(a, b, c, halfW, halfH, cullMode, co.t);
            co.primId = primId;
            float u0 = V[4][i0], v0 = V[5][i0];  // TriangleClipData, Rasterizer.cpp:455-458
            co.ru[0] = u0, co.ru[1] = V[4][i1] - u0, co.ru[2] = V[4][i2] - u0;
            co.rv[0] = v0, co.rv[1] = V[5][i1] - v0, co.rv[2] = V[5][i2] - v0;
            outs.push_back(co);
            if (++outIdx >= 8 * 16) return;  // output truncation, Rasterizer.cpp:470-472
        }
    }
}

static void draw_meshlets(DrawCtx& dc, uint32_t count, const orc_raster_flags* flags) {
    const orc_shading_context* sc = dc.sc;
    orc_framebuffer* fb = dc.fb;
    int halfW = (int)fb->width / 2, halfH = (int)fb->height / 2;
    dc.halfW = halfW, dc.halfH = halfH;
    // DrawMeshletsST (Rasterizer.cpp:154-156) honours EnableGuardband; the binned path does not (509).
    float bx = 2896.0f / (float)fb->width, by = 2896.0f / (float)fb->height;
    bool binned = flags->enable_binning != 0;
    if (!binned && !flags->enable_guardband) bx = 1.0f, by = 1.0f;
    bool clip = !binned && flags->enable_clipping;

    Shaded mesh;
    std::vector<ClipOut> clipOuts;
    clipOuts.reserve(128);

    for (uint32_t meshIdx = 0; meshIdx < count; meshIdx++) {
        shade_meshlet(sc, meshIdx, mesh);
        if (mesh.PrimCount == 0) continue;
        if (dc.counters) dc.counters[ORC_TRIS_PROCESSED] += mesh.PrimCount;
        // FS_EncodeSurfaceId<true> for alpha-tested materials. The reference dereferences the
        // material's texture unconditionally; a material without one passes every fragment here.
        const orc_texture* alphaTex = nullptr;
        uint32_t cutoff = 0;
        const bool overdraw = flags->shader == ORC_SHADER_OVERDRAW;  // one entry point for every FS id (Rasterizer.h:356-360)
        const int fragKind = (flags->shader == ORC_SHADER_DEFERRED || flags->shader == ORC_SHADER_TEXCOORD) ? flags->shader : 0;
        if (mesh.FragmentShaderId != 0 && !overdraw && !fragKind) {
            const orc_material& mat = sc->materials[mesh.MaterialId];
            if (mat.texture != UINT32_MAX && sc->textures && sc->textures[mat.texture].data) alphaTex = &sc->textures[mat.texture];
            cutoff = (uint32_t)mat.alpha_cutoff << 24;
        }
        const Meshlet& rec = ((const Meshlet*)sc->meshlets)[sc->meshlet_offset + meshIdx];
        auto alpha_tri = [&](uint32_t prim, const ClipOut* co) {
            AlphaTri at = {};
            at.tex = alphaTex;
            at.cutoff = cutoff;
            for (int k = 0; k < 3; k++) {
                uint32_t w = texcoord_word(rec, mesh.Indices[k][prim]);  // UnpackHalf2x16, Shading.cpp:228-231
                at.uv[k][0] = half_to_float(w & 0xFFFF), at.uv[k][1] = half_to_float(w >> 16);
            }
            at.clipped = co != nullptr;
            if (co) memcpy(at.ru, co->ru, sizeof(at.ru)), memcpy(at.rv, co->rv, sizeof(at.rv));
            return at;
        };

        for (uint32_t primOffset = 0; primOffset < mesh.PrimCount; primOffset += 16) {
            Vtx v[3][16];
            for (uint32_t l = 0; l < 16; l++) {
                for (uint32_t k = 0; k < 3; k++) v[k][l] = mesh.Pos[preload64_index(mesh.Indices[k][primOffset + l])];
            }
            ClipCodes cc = compute_clip_codes(v, bx, by);
            if (primOffset + 16 > mesh.PrimCount) {
                uint16_t trail = (uint16_t)((1u << (mesh.PrimCount % 16)) - 1);
                cc.AcceptMask &= trail;
                cc.NonTrivialMask &= trail;
            }
            if (cc.NonTrivialMask && dc.counters && (binned || clip))
                dc.counters[ORC_TRIS_CLIPPED] += (uint64_t)__builtin_popcount(cc.NonTrivialMask);

            if (cc.AcceptMask != 0) {
                for (uint32_t l = 0; l < 16; l++) {
                    if (!((cc.AcceptMask >> l) & 1)) continue;
                    TriSetup t;
                    if (!tri_setup(v[0][l], v[1][l], v[2][l], halfW, halfH, mesh.CullMode, t)) continue;
                    uint32_t bbMin, bbMax;
                    render_bbox(t, halfW, halfH, bbMin, bbMax);
                    EdgeVars e;
                    edge_setup(t, halfW, halfH, e);
                    const uint32_t p = primOffset + l;
                    if (overdraw) draw_triangle_overdraw(dc, e, bbMin, bbMax);
                    else if (fragKind) {
                        const uint8_t vid[3] = { mesh.Indices[0][p], mesh.Indices[1][p], mesh.Indices[2][p] };
                        draw_triangle_frag(dc, e, bbMin, bbMax, meshIdx, p, vid, nullptr, nullptr, fragKind);
                    } else if (alphaTex) draw_triangle_alpha(dc, e, bbMin, bbMax, meshIdx, p, alpha_tri(p, nullptr));
                    else draw_triangle(dc, e, bbMin, bbMax, meshIdx, p);
                    if (dc.counters) dc.counters[ORC_TRIS_RASTERIZED]++;
                }
            }
            if (cc.NonTrivialMask != 0 && clip) {
                clipOuts.clear();
                clip_packet(v, cc, cc.NonTrivialMask, bx, by, halfW, halfH, mesh.CullMode, clipOuts);
                for (const ClipOut& co : clipOuts) {
                    if (!co.keep) continue;
                    uint32_t bbMin, bbMax;
                    render_bbox(co.t, halfW, halfH, bbMin, bbMax);
                    EdgeVars e;
                    edge_setup(co.t, halfW, halfH, e);
                    uint32_t prim = primOffset + co.primId;
                    if (overdraw) draw_triangle_overdraw(dc, e, bbMin, bbMax);
                    else if (fragKind) {
                        const uint8_t vid[3] = { mesh.Indices[0][prim], mesh.Indices[1][prim], mesh.Indices[2][prim] };
                        draw_triangle_frag(dc, e, bbMin, bbMax, meshIdx, prim, vid, co.ru, co.rv, fragKind);
                    } else if (alphaTex) draw_triangle_alpha(dc, e, bbMin, bbMax, meshIdx, prim, alpha_tri(prim, &co));
                    else draw_triangle(dc, e, bbMin, bbMax, meshIdx, prim);
                    if (dc.counters) dc.counters[ORC_TRIS_RASTERIZED]++;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- binned, threaded draw
// Rasterizer::DrawMeshlets with binning on (Rasterizer.cpp:493-644) and N worker threads, in the
// reference's work split: worker w shades meshlets w, w+N, w+2N, ... and sets up their packets into
// its own batch of at most MaxWorkerBatch packets, inserting each packet's accepted lanes into
// per-(bin, worker) lists of at most MaxBinSize entries over 128x128-pixel bins
// (DistributeToBins/InsertBin, Rasterizer.cpp:663-700, 759-768). When a worker's batch or one of its
// bins is full, or it has nothing left, the workers meet at a barrier, worker 0 commits the batches
// (BinQueue::Commit, 770-790), and each worker rasterizes the bins elected to it, bin b going to
// worker (b % 64) % N (the elect mask of 505-508), every bin's lists in worker order with each
// triangle clamped to the bin (RasterizeBin, 701-740). Non-trivial triangles are dropped. This is
// the timed CPU baseline in the reference's own shape; with several workers, equal-depth ties
// resolve in bin-list order, as in the reference.
namespace {

constexpr uint32_t kMaxWorkerBatch = 256, kMaxBinSize = 63, kBinShift = 7, kBinSize = 1u << kBinShift;

struct Packet {  // TrianglePacket as committed to the rasterizer
    TriSetup lane[16];
    uint32_t meshletId, basePrim, fsId;
};
struct Bin {
    uint32_t count;
    uint32_t ids[kMaxBinSize];  // packetIdx << 16 | lane mask
};

class SpinBarrier {  // a generation barrier (the reference's Barrier, SYNC_SPIN_ONLY)
public:
    explicit SpinBarrier(uint32_t n) : n_(n) {}
    void wait() {
        const uint32_t gen = gen_.load(std::memory_order_acquire);
        if (count_.fetch_add(1, std::memory_order_acq_rel) + 1 == n_) {
            count_.store(0, std::memory_order_relaxed);
            gen_.fetch_add(1, std::memory_order_acq_rel);
        } else {
            while (gen_.load(std::memory_order_acquire) == gen) std::this_thread::yield();
        }
    }
private:
    uint32_t n_;
    std::atomic<uint32_t> count_{ 0 }, gen_{ 0 };
};

}  // namespace

static void draw_meshlets_binned(orc_framebuffer* fb, uint32_t meshCount, const orc_shading_context* sc,
                                 uint32_t numWorkers, uint64_t counters[4]) {
    const int halfW = (int)fb->width / 2, halfH = (int)fb->height / 2;
    const float bx = 2896.0f / (float)fb->width, by = 2896.0f / (float)fb->height;  // guard band always on (509)
    const uint32_t binsPerRow = (fb->width + kBinSize - 1) >> kBinShift;
    const uint32_t binsPerFrame = ((fb->height + kBinSize - 1) >> kBinShift) * binsPerRow;
    const uint32_t bitmapWords = (binsPerFrame + 63) / 64;
    std::vector<Packet> batch((size_t)kMaxWorkerBatch * numWorkers), committedBatch(batch.size());
    std::vector<Bin> bins((size_t)binsPerFrame * numWorkers), committedBins(bins.size());
    for (Bin& b : bins) b.count = 0;
    for (Bin& b : committedBins) b.count = 0;
    std::vector<uint64_t> workerBitmap((size_t)bitmapWords * numWorkers, 0), frameBitmap(bitmapWords, 0);
    uint64_t electMask = 0;
    for (uint32_t i = 0; i < 64; i += numWorkers) electMask |= 1ull << i;
    SpinBarrier ready(numWorkers);
    std::atomic<uint32_t> doneMeshCount{ 0 };
    std::vector<std::array<uint64_t, 4>> perWorker(numWorkers, std::array<uint64_t, 4>{ 0, 0, 0, 0 });

    auto insert_bin = [&](uint32_t w, uint32_t binId, uint32_t packetIdx, uint32_t mask) {
        Bin& b = bins[(size_t)binId * numWorkers + w];
        b.ids[b.count++] = (packetIdx << 16) | mask;
        workerBitmap[(size_t)w * bitmapWords + binId / 64] |= 1ull << (binId & 63);
        return b.count < kMaxBinSize;
    };
    auto rasterize_bin = [&](uint32_t binId, uint32_t w) {
        DrawCtx dc = {};
        dc.fb = fb;
        dc.sc = sc;
        dc.halfW = halfW, dc.halfH = halfH;
        dc.rowBegin = 0, dc.rowEnd = fb->height;
        dc.counters = nullptr;
        const uint32_t binX = (binId % binsPerRow) * kBinSize, binY = (binId / binsPerRow) * kBinSize;
        const uint32_t binMin = binX | (binY << 16), binMax = binMin + kBinSize * 0x00010001u;
        for (uint32_t wk = 0; wk < numWorkers; wk++) {
            Bin& b = committedBins[(size_t)binId * numWorkers + wk];
            for (uint32_t i = 0; i < b.count; i++) {
                const Packet& pk = committedBatch[b.ids[i] >> 16];
                const uint32_t mask = b.ids[i] & 0xFFFF;
                const Meshlet& rec = ((const Meshlet*)sc->meshlets)[sc->meshlet_offset + pk.meshletId];
                for (uint32_t l = 0; l < 16; l++) {
                    if (!((mask >> l) & 1)) continue;
                    uint32_t bbMin, bbMax;
                    render_bbox(pk.lane[l], halfW, halfH, bbMin, bbMax);
                    bbMin = max16(bbMin, binMin);
                    bbMax = min16(bbMax, binMax);
                    EdgeVars e;
                    edge_setup(pk.lane[l], halfW, halfH, e);
                    const uint32_t prim = pk.basePrim + l;
                    if (pk.fsId != 0) {
                        const orc_material& mat = sc->materials[rec.MaterialId];
                        AlphaTri at = {};
                        if (mat.texture != UINT32_MAX && sc->textures && sc->textures[mat.texture].data)
                            at.tex = &sc->textures[mat.texture];
                        at.cutoff = (uint32_t)mat.alpha_cutoff << 24;
                        for (int k = 0; k < 3; k++) {
                            const uint32_t tw = texcoord_word(rec, rec.Indices[k][prim]);
                            at.uv[k][0] = half_to_float(tw & 0xFFFF), at.uv[k][1] = half_to_float(tw >> 16);
                        }
                        if (at.tex) {
                            draw_triangle_alpha(dc, e, bbMin, bbMax, pk.meshletId, prim, at);
                            continue;
                        }
                    }
                    draw_triangle(dc, e, bbMin, bbMax, pk.meshletId, prim);
                }
            }
            b.count = 0;
        }
    };

    auto worker = [&](uint32_t w) {
        Shaded mesh;
        mesh.PrimCount = 0;
        uint32_t meshJobs = 0, nextMeshIdx = w, meshIdx = w, primOffset = 0;
        uint32_t nextPacketIdx = w * kMaxWorkerBatch;
        const uint32_t maxPacketIdx = nextPacketIdx + kMaxWorkerBatch;
        std::array<uint64_t, 4>& cnt = perWorker[w];
        while (true) {
            bool batchFull = false, isIdle = true;
            if (nextMeshIdx < meshCount && primOffset >= mesh.PrimCount) {
                isIdle = false;
                meshIdx = nextMeshIdx;
                nextMeshIdx += numWorkers;
                meshJobs++;
                shade_meshlet(sc, meshIdx, mesh);
                if (mesh.PrimCount == 0) continue;
                cnt[ORC_TRIS_PROCESSED] += mesh.PrimCount;
                primOffset = 0;
            }
            for (; primOffset < mesh.PrimCount && !batchFull; primOffset += 16) {
                isIdle = false;
                Vtx v[3][16];
                for (uint32_t l = 0; l < 16; l++)
                    for (uint32_t k = 0; k < 3; k++) v[k][l] = mesh.Pos[preload64_index(mesh.Indices[k][primOffset + l])];
                ClipCodes cc = compute_clip_codes(v, bx, by);
                if (primOffset + 16 > mesh.PrimCount) {
                    const uint16_t trail = (uint16_t)((1u << (mesh.PrimCount % 16)) - 1);
                    cc.AcceptMask &= trail;
                    cc.NonTrivialMask &= trail;
                }
                if (cc.NonTrivialMask) cnt[ORC_TRIS_CLIPPED] += (uint64_t)__builtin_popcount(cc.NonTrivialMask);
                if (cc.AcceptMask == 0) continue;
                Packet& pk = batch[nextPacketIdx];
                uint32_t accept = 0;
                for (uint32_t l = 0; l < 16; l++)
                    if (tri_setup(v[0][l], v[1][l], v[2][l], halfW, halfH, mesh.CullMode, pk.lane[l])) accept |= 1u << l;
                accept &= cc.AcceptMask;
                if (accept == 0) continue;
                cnt[ORC_TRIS_RASTERIZED] += (uint64_t)__builtin_popcount(accept);
                pk.meshletId = meshIdx, pk.basePrim = primOffset, pk.fsId = mesh.FragmentShaderId;
                // DistributeToBins: every bin a lane's render box touches
                uint32_t bMin[16], bMax[16];
                uint32_t x0 = UINT32_MAX, y0 = UINT32_MAX, x1 = 0, y1 = 0;
                for (uint32_t l = 0; l < 16; l++) {
                    if (!((accept >> l) & 1)) continue;
                    uint32_t lo, hi;
                    render_bbox(pk.lane[l], halfW, halfH, lo, hi);
                    bMin[l] = ((lo & 0xFFFF) >> kBinShift) | (((lo >> 16) >> kBinShift) << 16);
                    const uint32_t hm = hi - 0x00010001u;
                    bMax[l] = ((hm & 0xFFFF) >> kBinShift) | (((hm >> 16) >> kBinShift) << 16);
                    x0 = std::min(x0, bMin[l] & 0xFFFF), y0 = std::min(y0, bMin[l] >> 16);
                    x1 = std::max(x1, bMax[l] & 0xFFFF), y1 = std::max(y1, bMax[l] >> 16);
                }
                bool underCap = true;
                for (uint32_t y = y0; y <= y1; y++)
                    for (uint32_t x = x0; x <= x1; x++) {
                        uint32_t m = 0;
                        for (uint32_t l = 0; l < 16; l++)
                            if (((accept >> l) & 1) && x >= (bMin[l] & 0xFFFF) && x <= (bMax[l] & 0xFFFF) &&
                                y >= (bMin[l] >> 16) && y <= (bMax[l] >> 16))
                                m |= 1u << l;
                        if (m) underCap &= insert_bin(w, x + y * binsPerRow, nextPacketIdx, m);
                    }
                batchFull |= !underCap;
                batchFull |= nextPacketIdx + 1 >= maxPacketIdx;
                nextPacketIdx++;
            }
            if (batchFull || isIdle) {
                ready.wait();
                if (doneMeshCount.load(std::memory_order_acquire) >= meshCount) break;
                if (w == 0) {
                    std::swap(committedBatch, batch);
                    std::swap(committedBins, bins);
                    std::fill(frameBitmap.begin(), frameBitmap.end(), 0ull);
                    for (uint32_t i = 0; i < numWorkers; i++)
                        for (uint32_t j = 0; j < bitmapWords; j++) {
                            frameBitmap[j] |= workerBitmap[(size_t)i * bitmapWords + j];
                            workerBitmap[(size_t)i * bitmapWords + j] = 0;
                        }
                }
                ready.wait();
                for (uint32_t i = 0; i < bitmapWords; i++) {
                    const uint64_t m = frameBitmap[i] & (electMask << (w % 64));
                    for (uint64_t bits = m; bits; bits &= bits - 1) rasterize_bin(i * 64 + (uint32_t)__builtin_ctzll(bits), w);
                    cnt[ORC_BIN_FLUSHES] += (uint64_t)__builtin_popcountll(m);
                }
                if (nextMeshIdx >= meshCount && primOffset >= mesh.PrimCount) {
                    doneMeshCount.fetch_add(meshJobs, std::memory_order_acq_rel);
                    meshJobs = 0;
                }
                nextPacketIdx = w * kMaxWorkerBatch;
            }
        }
    };
    std::vector<std::thread> threads;
    for (uint32_t w = 1; w < numWorkers; w++) threads.emplace_back(worker, w);
    worker(0);
    for (auto& t : threads) t.join();
    if (counters)
        for (const auto& c : perWorker)
            for (int k = 0; k < 4; k++) counters[k] += c[k];
}

}  // namespace orc

using namespace orc;

extern "C" {

void orc_draw_meshlets_binned(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx, uint32_t num_threads,
                              uint64_t counters[4]) {
    draw_meshlets_binned(fb, count, ctx, std::max(1u, std::min(num_threads, 64u)), counters);
}


uint32_t orc_meshlet_size(void) { return (uint32_t)sizeof(Meshlet); }

uint32_t orc_fb_layer_stride(uint32_t width, uint32_t height) { return fb_layer_stride(width, height); }

void orc_fb_init(orc_framebuffer* fb, uint32_t width, uint32_t height, uint32_t num_layers, uint32_t* storage) {
    fb->width = width;
    fb->height = height;
    fb->tile_stride = width / 4;
    fb->layer_stride = fb_layer_stride(width, height);
    fb->num_layers = num_layers;
    fb->data = storage;
}

// Framebuffer::ClearLayer, Rasterizer.h:39-48 (fills Width*Height words of the layer).
void orc_fb_clear_layer(orc_framebuffer* fb, uint32_t layer, uint32_t value) {
    uint32_t* p = &fb->data[(size_t)layer * fb->layer_stride];
    for (uint32_t i = 0; i < fb->width * fb->height; i++) p[i] = value;
}

// Framebuffer::Clear, Rasterizer.h:35-38.
void orc_fb_clear(orc_framebuffer* fb, uint32_t color, float depth) {
    orc_fb_clear_layer(fb, 0, color);
    uint32_t d;
    memcpy(&d, &depth, 4);
    orc_fb_clear_layer(fb, 1, d);
}

// Framebuffer::GetPixels, ImageHelpers.cpp:109-147 (de-tiles a layer to row-major).
void orc_fb_get_pixels(const orc_framebuffer* fb, uint32_t layer, uint32_t* dest, uint32_t stride) {
    const uint32_t* src = &fb->data[(size_t)layer * fb->layer_stride];
    for (uint32_t y = 0; y < fb->height; y++)
        for (uint32_t x = 0; x < fb->width; x++) dest[(size_t)y * stride + x] = src[pixel_offset(fb, x, y)];
}

void orc_draw_meshlets_rows(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                            const orc_raster_flags* flags, uint64_t counters[4], uint32_t row_begin, uint32_t row_end) {
    DrawCtx dc = {};
    dc.fb = fb;
    dc.sc = ctx;
    dc.rowBegin = row_begin;
    dc.rowEnd = std::min(row_end, fb->height);
    dc.counters = counters;
    draw_meshlets(dc, count, flags);
}

void orc_draw_meshlets(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                       const orc_raster_flags* flags, uint64_t counters[4]) {
    orc_draw_meshlets_rows(fb, count, ctx, flags, counters, 0, fb->height);
}

void orc_draw_meshlets_mt(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                          const orc_raster_flags* flags, uint32_t num_threads) {
    if (num_threads <= 1) { orc_draw_meshlets(fb, count, ctx, flags, nullptr); return; }
    std::vector<std::thread> threads;
    uint32_t rows = (fb->height + num_threads - 1) / num_threads;
    rows = (rows + 3) & ~3u;
    for (uint32_t t = 0; t < num_threads; t++) {
        uint32_t r0 = t * rows, r1 = std::min(fb->height, r0 + rows);
        if (r0 >= r1) break;
        threads.emplace_back([=]() { orc_draw_meshlets_rows(fb, count, ctx, flags, nullptr, r0, r1); });
    }
    for (auto& th : threads) th.join();
}

}  // extern "C"
