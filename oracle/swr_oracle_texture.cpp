// Oracle (test infrastructure, see swr_oracle.h): approximation model, textures and mips,
// the Hi-Z depth pyramid and meshlet culling.
#include "swr_oracle_common.h"
#include "../include/swr/approx14.h"
#include "../include/swr/hostmath.h"

#include <algorithm>

#if defined(__x86_64__)
#include <immintrin.h>
#define ORC_X86 1
#else
#define ORC_X86 0
#endif

namespace orc {

static int g_approxMode = 0;

#if ORC_X86
// The AVX-512 instructions the reference uses (SIMD.h:294-295), compiled for this function only
// and used only after a runtime CPU check.
__attribute__((target("avx512f"))) static float hw_rcp14(float x) {
    return _mm_cvtss_f32(_mm512_castps512_ps128(_mm512_rcp14_ps(_mm512_set1_ps(x))));
}
__attribute__((target("avx512f"))) static float hw_rsqrt14(float x) {
    return _mm_cvtss_f32(_mm512_castps512_ps128(_mm512_rsqrt14_ps(_mm512_set1_ps(x))));
}
// 16 inputs per instruction, for the exhaustive comparison with the tables.
__attribute__((target("avx512f"))) static void hw_approx16(int which, const uint32_t* in, uint32_t* out) {
    __m512 v;
    memcpy(&v, in, 64);
    __m512 r = which ? _mm512_rsqrt14_ps(v) : _mm512_rcp14_ps(v);
    memcpy(out, &r, 64);
}
static bool hw_available() { return __builtin_cpu_supports("avx512f"); }
#else
static float hw_rcp14(float x) { return swr_rcp14(x); }
static float hw_rsqrt14(float x) { return swr_rsqrt14(x); }
static void hw_approx16(int, const uint32_t*, uint32_t*) {}
static bool hw_available() { return false; }
#endif

// simd::approx_rcp / approx_rsqrt (SIMD.h:294-295). Mode 0: the exact integer restatement of
// VRCP14PS/VRSQRT14PS (include/swr/approx14.h, the same functions the GPU kernels run); mode 1:
// the instructions themselves on an AVX-512 host; mode 2: the correctly rounded IEEE 1/x and
// 1/sqrtf(x), kept to measure what the approximation changes.
float approx_rcp(float x) {
    return g_approxMode == 0 ? swr_rcp14(x) : g_approxMode == 1 ? hw_rcp14(x) : 1.0f / x;
}
float approx_rsqrt(float x) {
    return g_approxMode == 0 ? swr_rsqrt14(x) : g_approxMode == 1 ? hw_rsqrt14(x) : 1.0f / std::sqrt(x);
}

// Texture2D::GetTexelOffset for TiledY8, Texture.h:493-501.
static inline uint32_t texel_offset(uint32_t x, uint32_t y, uint32_t stride) {
    return (y & 7) | (x << 3) | ((y & ~7u) << stride);
}

// pixfmt::RGBA8u::Unpack / Pack, Texture.h:28-36, 55-67.
struct F4 { float x, y, z, w; };
static inline F4 unpack_rgba8(uint32_t p) {
    const float scale = 1.0f / 255;
    return { (float)((p >> 0) & 255) * scale, (float)((p >> 8) & 255) * scale,
             (float)((p >> 16) & 255) * scale, (float)((p >> 24) & 255) * scale };
}
static inline uint32_t sat_u8_from_i32(int32_t v) {
    // packs_epi32 (signed saturation to int16) then packus_epi16 (unsigned saturation to uint8)
    int32_t s = std::min(std::max(v, -32768), 32767);
    return (uint32_t)std::min(std::max(s, 0), 255);
}
static inline uint32_t pack_rgba8(F4 v) {
    uint32_t r = sat_u8_from_i32(round2i(v.x * 255.0f));
    uint32_t g = sat_u8_from_i32(round2i(v.y * 255.0f));
    uint32_t b = sat_u8_from_i32(round2i(v.z * 255.0f));
    uint32_t a = sat_u8_from_i32(round2i(v.w * 255.0f));
    return r | (g << 8) | (b << 16) | (a << 24);
}
// pixfmt::R11G11B10f, Texture.h:139-182 (clamp-only pack).
static inline float unpack_f11(uint32_t x) { x = x << 17; return u2f((x & 0x0FFE0000u) + 0x38000000u); }
static inline float unpack_f10(uint32_t x) { x = x << 18; return u2f((x & 0x0FFC0000u) + 0x38000000u); }
static inline uint32_t pack_f11(float x) {
    x = vmax(x, 1.0f / (1 << 15));
    x = vmin(x, 130048.0f);
    return ((f2u(x) >> 17) & 0x3FFF) - 0x1C00;
}
static inline uint32_t pack_f10(float x) {
    x = vmax(x, 1.0f / (1 << 15));
    x = vmin(x, 129024.0f);
    return ((f2u(x) >> 18) & 0x1FFF) - 0x0E00;
}

}  // namespace orc

using namespace orc;

extern "C" {

void orc_set_approx_mode(int mode) { g_approxMode = (mode == 2 || (mode == 1 && hw_available())) ? mode : 0; }
int orc_approx_mode_available(int mode) { return mode == 0 || mode == 2 || (mode == 1 && hw_available()); }

// approx_rcp (which = 0) or approx_rsqrt (which = 1) of n float bit patterns in the current mode.
void orc_approx_eval(int which, const uint32_t* in, uint32_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) out[i] = f2u(which ? approx_rsqrt(u2f(in[i])) : approx_rcp(u2f(in[i])));
}

// Number of inputs among `count` consecutive 32-bit patterns from `first` (a multiple of 16) for
// which the table restatement differs from the instruction (which: 0 rcp14, 1 rsqrt14); -1 when
// the host has no AVX-512.
int64_t orc_approx14_mismatches(int which, uint64_t first, uint64_t count) {
    if (!hw_available() || (first & 15)) return -1;
    int64_t bad = 0;
    for (uint64_t b = first; b < first + count; b += 16) {
        uint32_t in[16], hw[16];
        for (int j = 0; j < 16; j++) in[j] = (uint32_t)(b + j);
        hw_approx16(which, in, hw);
        for (int j = 0; j < 16 && b + j < first + count; j++) {
            const float f = u2f(in[j]);
            if (f2u(which ? swr_rsqrt14(f) : swr_rcp14(f)) != hw[j]) bad++;
        }
    }
    return bad;
}

// CreateTexture2D, Texture.h:599-636 (mips stop below 4 texels; levels 64-word aligned).
static void texture_layout(uint32_t width, uint32_t height, uint32_t maxLevels, uint32_t* mipOffsets,
                           uint32_t* mipLevels, uint32_t* layerStride) {
    uint32_t stride = 0, mip = 0;
    for (uint32_t i = 0; i < 16; i++) mipOffsets[i] = 0;
    for (; mip < maxLevels; mip++) {
        if ((width >> mip) < 4 || (height >> mip) < 4) break;
        mipOffsets[mip] = stride;
        stride += ((width >> mip) * (height >> mip) + 63) & ~63u;
    }
    *mipLevels = mip;
    *layerStride = stride;
}

uint64_t orc_texture_storage_words(uint32_t width, uint32_t height, uint32_t max_levels, uint32_t num_layers) {
    uint32_t offs[16], levels, stride;
    texture_layout(width, height, max_levels, offs, &levels, &stride);
    return (uint64_t)stride * num_layers + 64;
}

void orc_texture_init(orc_texture* tex, uint32_t width, uint32_t height, uint32_t max_levels,
                      uint32_t num_layers, uint32_t* storage) {
    uint32_t levels, stride;
    texture_layout(width, height, max_levels, tex->mip_offsets, &levels, &stride);
    tex->width = width;
    tex->height = height;
    tex->row_shift = (uint32_t)__builtin_ctz(std::max(width, 8u));
    tex->num_layers = num_layers;
    tex->layer_stride = stride;
    tex->mip_levels = levels;
    tex->scale_u = (float)width;
    tex->scale_v = (float)height;
    tex->mask_u = (int32_t)width - 1;
    tex->mask_v = (int32_t)height - 1;
    tex->mask_lerp_u = (int32_t)(width << 8) - 1;
    tex->mask_lerp_v = (int32_t)(height << 8) - 1;
    tex->scale_lerp_u = (float)(tex->mask_lerp_u + 1);
    tex->scale_lerp_v = (float)(tex->mask_lerp_v + 1);
    tex->data = storage;
}

// Texture2D::SetPixels (TiledY8), Texture.h:336-354.
void orc_texture_set_pixels(orc_texture* tex, const uint32_t* pixels, uint32_t stride, uint32_t layer, uint32_t mip) {
    uint32_t* dst = &tex->data[(size_t)layer * tex->layer_stride + tex->mip_offsets[mip]];
    for (uint32_t y = 0; y < tex->height; y++)
        for (uint32_t x = 0; x < tex->width; x++) dst[texel_offset(x, y, tex->row_shift)] = pixels[x + (size_t)y * stride];
}

// Texture2D::GenerateMips / GenerateMip, Texture.h:382-388, 577-596: 2x2 box filter in float
// on unpacked texels, ((c00 + c10) + c01 + c11) * 0.25, repacked per format.
void orc_texture_generate_mips(orc_texture* tex, uint32_t format) {
    for (uint32_t layer = 0; layer < tex->num_layers; layer++) {
        for (uint32_t level = 1; level < tex->mip_levels; level++) {
            uint32_t w = tex->width >> level, h = tex->height >> level;
            const uint32_t* src = &tex->data[(size_t)layer * tex->layer_stride + tex->mip_offsets[level - 1]];
            uint32_t* dst = &tex->data[(size_t)layer * tex->layer_stride + tex->mip_offsets[level]];
            uint32_t sstride = tex->row_shift - level + 1, dstride = tex->row_shift - level;
            for (uint32_t y = 0; y < h; y++) {
                for (uint32_t x = 0; x < w; x++) {
                    uint32_t p00 = src[texel_offset(2 * x + 0, 2 * y + 0, sstride)];
                    uint32_t p10 = src[texel_offset(2 * x + 1, 2 * y + 0, sstride)];
                    uint32_t p01 = src[texel_offset(2 * x + 0, 2 * y + 1, sstride)];
                    uint32_t p11 = src[texel_offset(2 * x + 1, 2 * y + 1, sstride)];
                    uint32_t out;
                    if (format == 0) {
                        F4 a = unpack_rgba8(p00), b = unpack_rgba8(p10), c = unpack_rgba8(p01), d = unpack_rgba8(p11);
                        F4 avg = { (a.x + b.x + c.x + d.x) * 0.25f, (a.y + b.y + c.y + d.y) * 0.25f,
                                   (a.z + b.z + c.z + d.z) * 0.25f, (a.w + b.w + c.w + d.w) * 0.25f };
                        out = pack_rgba8(avg);
                    } else if (format == 1) {
                        float r = (unpack_f11(p00 >> 21) + unpack_f11(p10 >> 21) + unpack_f11(p01 >> 21) + unpack_f11(p11 >> 21)) * 0.25f;
                        float g = (unpack_f11(p00 >> 10) + unpack_f11(p10 >> 10) + unpack_f11(p01 >> 10) + unpack_f11(p11 >> 10)) * 0.25f;
                        float b = (unpack_f10(p00) + unpack_f10(p10) + unpack_f10(p01) + unpack_f10(p11)) * 0.25f;
                        out = pack_f11(r) << 21 | pack_f11(g) << 10 | pack_f10(b);
                    } else {
                        out = f2u((u2f(p00) + u2f(p10) + u2f(p01) + u2f(p11)) * 0.25f);
                    }
                    dst[texel_offset(x, y, dstride)] = out;
                }
            }
        }
    }
}

// texutil::DownsampleDepth (ImageHelpers.cpp:150-247). The reference recursion writes mip m
// in 8x8-texel blocks for every 2^(m+4)-pixel region whose origin lies inside the frame, and
// the 4x4 root tile at mip rootLevel-3; a texel holds the min of the frame depths it covers,
// FLT_MAX where it covers none. Texels outside that set are left untouched.
struct Down {
    const orc_framebuffer* fb;
    orc_texture* dst;
    float depth(uint32_t x, uint32_t y) const {
        if (x >= fb->width || y >= fb->height) return FLT_MAX;
        uint32_t off = ((x & ~3u) << 2) + (y & ~3u) * fb->width + (x & 3) + (y & 3) * 4;
        return u2f(fb->data[fb->layer_stride * 1 + off]);
    }
    // min over a 2^(m+1) square of pixels, reduced in the reference's pairing order
    // (rows first, then columns, at every level).
    float texel(uint32_t m, uint32_t tx, uint32_t ty) const {
        if (m == 0) {
            uint32_t x = tx * 2, y = ty * 2;
            float r0 = vmin(depth(x, y), depth(x, y + 1));
            float r1 = vmin(depth(x + 1, y), depth(x + 1, y + 1));
            return vmin(r0, r1);
        }
        float r0 = vmin(texel(m - 1, 2 * tx, 2 * ty), texel(m - 1, 2 * tx, 2 * ty + 1));
        float r1 = vmin(texel(m - 1, 2 * tx + 1, 2 * ty), texel(m - 1, 2 * tx + 1, 2 * ty + 1));
        return vmin(r0, r1);
    }
    void store(uint32_t m, uint32_t tx, uint32_t ty, float v) {
        uint32_t stride = dst->row_shift - m;
        dst->data[dst->mip_offsets[m] + texel_offset(tx, ty, stride)] = f2u(v);
    }
};

void orc_downsample_depth(const orc_framebuffer* fb, orc_texture* dest) {
    uint32_t rootLevel = 32 - (uint32_t)__builtin_clz(std::max(fb->width, fb->height));
    Down d{ fb, dest };
    // Pyramid values depend only on the pixels covered (min is exact), so each written texel is
    // evaluated directly. Mip m (m <= rootLevel-4): 8x8 blocks at region origins inside the frame.
    for (uint32_t m = 0; m + 4 <= rootLevel; m++) {
        uint32_t region = 1u << (m + 4);
        for (uint32_t ry = 0; ry < fb->height; ry += region) {
            for (uint32_t rx = 0; rx < fb->width; rx += region) {
                uint32_t bx = rx >> (m + 1), by = ry >> (m + 1);
                for (uint32_t j = 0; j < 8; j++)
                    for (uint32_t i = 0; i < 8; i++) d.store(m, bx + i, by + j, d.texel(m, bx + i, by + j));
            }
        }
    }
    uint32_t m = rootLevel - 3;
    for (uint32_t j = 0; j < 4; j++)
        for (uint32_t i = 0; i < 4; i++) d.store(m, i, j, d.texel(m, i, j));
}

// ProjectSphere (Shading.cpp:264-279): Mara & McGuire 2013 bounds of a projected sphere.
static bool project_sphere(float cx, float cy, float cz, float r, const float proj[3], float bb[4]) {
    cz *= -1;
    bool mask = cz >= r + proj[0];
    float crx = cx * r, cry = cy * r, crz = cz * r;
    float vx = approx_sqrt(cx * cx + cz * cz - r * r);
    float vy = approx_sqrt(cy * cy + cz * cz - r * r);
    float sx = proj[1] * 0.5f, sy = proj[2] * 0.5f;
    bb[0] = (vx * cx - crz) * approx_rcp(vx * cz + crx) * sx + 0.5f;
    bb[1] = (vy * cy + crz) * approx_rcp(vy * cz - cry) * sy + 0.5f;
    bb[2] = (vx * cx + crz) * approx_rcp(vx * cz - crx) * sx + 0.5f;
    bb[3] = (vy * cy - crz) * approx_rcp(vy * cz + cry) * sy + 0.5f;
    return mask;
}

// ShadingContext::CullMeshlets, Shading.cpp:775-869, one lane at a time. Lanes of a 16-meshlet
// group never interact except through the loop bounds, which do not change the result.
uint32_t orc_cull_meshlets(uint16_t* bitmap, const void* meshlets, uint32_t count, const float proj[16],
                           const float view[16], const float model[16], const float prev_view[16],
                           float frame_w, float frame_h, const orc_texture* depth_map) {
    // Matrix products and planes come from the host-side helpers every consumer of a camera
    // shares (glm in the reference), so the oracle and the library derive identical values.
    float objectToPrevView[16], pv[16], objectToClip[16];
    swr_hostmath::mat4_mul(prev_view, model, objectToPrevView);
    swr_hostmath::mat4_mul(proj, view, pv);
    swr_hostmath::mat4_mul(pv, model, objectToClip);
    float planes[6][4];
    swr_hostmath::frustum_planes(objectToClip, planes);
    float objectToWorldScale = swr_hostmath::column0_length(model);
    float projFactors[3] = { proj[3 * 4 + 2], proj[0], proj[1 * 4 + 1] };
    uint32_t visibleCount = 0;
    const Meshlet* ms = (const Meshlet*)meshlets;

    for (uint32_t offset = 0; offset < count; offset += 16) {
        uint16_t mask = 0;
        for (uint32_t l = 0; l < 16; l++) {
            uint32_t idx = offset + l;
            if (idx >= count) continue;
            const Meshlet& m = ms[idx];
            float cx = m.BoundCenter[0], cy = m.BoundCenter[1], cz = m.BoundCenter[2], r = m.BoundRadius;
            bool visible = true;
            for (int i = 0; i < 5; i++) {
                // simd::dot(v_float3, float3) = fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)), SIMD.h:429
                float dist = std::fma(cx, planes[i][0], std::fma(cy, planes[i][1], cz * planes[i][2])) + planes[i][3];
                visible = visible && (dist > -r);
            }
            if (depth_map != nullptr && visible) {
                V4 vs = transform_point(objectToPrevView, cx, cy, cz);
                float rvs = r * objectToWorldScale;
                float bb[4];
                bool projMask = project_sphere(vs.x, vs.y, vs.z, rvs, projFactors, bb);
                if (projMask) {
                    float bw = (bb[2] - bb[0]) * frame_w, bh = (bb[3] - bb[1]) * frame_h;
                    int32_t mip = ilog2_x86(vmax(bw, bh));
                    mip = std::min(std::max(mip, 1), (int32_t)depth_map->mip_levels - 1);
                    int32_t x0 = std::max(trunc2i(bb[0] * frame_w), 0) >> mip;
                    int32_t y0 = std::max(trunc2i(bb[1] * frame_h), 0) >> mip;
                    int32_t x1 = std::min(trunc2i(bb[2] * frame_w), (int32_t)frame_w - 1) >> mip;
                    int32_t y1 = std::min(trunc2i(bb[3] * frame_h), (int32_t)frame_h - 1) >> mip;
                    float depthSphere = projFactors[0] / (-vs.z - rvs);
                    float depthVisible = FLT_MAX;
                    uint32_t level = (uint32_t)(mip - 1);
                    uint32_t stride = depth_map->row_shift - level;
                    const uint32_t* base = &depth_map->data[depth_map->mip_offsets[level & 15]];
                    for (int32_t y = y0; y <= y1; y++)
                        for (int32_t x = x0; x <= x1; x++)
                            depthVisible = vmin(depthVisible, u2f(base[texel_offset((uint32_t)x, (uint32_t)y, stride)]));
                    visible = depthSphere > depthVisible;
                }
            }
            if (visible) mask |= (uint16_t)(1u << l);
        }
        bitmap[offset / 16] = mask;
        visibleCount += (uint32_t)__builtin_popcount(mask);
    }
    return visibleCount;
}

}  // extern "C"
