// Meshlet rasterizer kernels: mesh shader (ShadeMeshlet), clip codes, triangle setup, clipping and
// vis-buffer rasterization (FS_EncodeSurfaceId<false> and, for alpha-tested materials,
// FS_EncodeSurfaceId<true>) for sm_103a.
//
// Work decomposition:
//   k_draw_meshlets  one warp per meshlet (dynamic fetch). Lanes transform the 64 vertices into
//                    shared memory, then own one triangle each: clip codes, setup and edge
//                    equations in registers. Triangles whose 4-aligned box covers at most
//                    kSmallTiles 4x4 tiles are rasterized by the whole warp, two tiles (32 pixels)
//                    per step; larger and clipped triangles, and every triangle of an
//                    alpha-tested material, go to a device queue.
//   k_raster_big     warps take 32x32-pixel chunks of queued triangles (flattened by a prefix of
//                    chunk counts kept in the queue), reject empty chunks by their corners and
//                    rasterize the rest two tiles per step.
//   k_finalize       converts per-pixel keys to the reference's depth and surfaceId layers.
// The depth test is a 64-bit atomicMax on (ordered depth, 0xFFFFFFFE - rank); the result is
// independent of execution order and equals the single-threaded reference. The alpha test is a
// function of the triangle and the fragment alone, so it only removes fragments and keeps that
// property.
//
// Tile depth culling: tileMin holds, per 4x4 tile, a lower bound of the depth words of its 16
// keys (keys only grow, and tileMin only takes minima of values its pixels had reached). Before a
// tile is shaded, an upper bound of the triangle's depth over the tile is compared with it; a tile
// the triangle cannot win anywhere is skipped. The vis-buffer is unchanged (only fragments that
// would fail the depth test are skipped), while the dense scenes' overdraw mostly disappears.
#include <cfloat>
#include <mutex>
#include <numeric>
#include <type_traits>

#include "../../include/swr/approx14.h"
#include "../../include/swr/raster_math.cuh"
#include "swr_device.cuh"
#include "swr_internal.h"
#include "swr_sample.cuh"

namespace swr {

constexpr int kWarpsPerBlock = 8;
constexpr int kSmallTiles = 16;
static_assert(kSmallTiles <= 16, "the small triangles' tile -> row multiply-shift is exact for at most 16 tiles");
constexpr int kPacketTiles = 128;  // in-warp tile budget of a 32-triangle step
constexpr int kSpreadTiles = 4;    // over budget, triangles above this many tiles are queued
constexpr int kChunkTiles = 8;  // chunk = 8x8 tiles = 32x32 pixels

// A record in a warp's shared memory padded to 80 bytes. TriRec and AlphaExt are 64 bytes; with a
// 64-byte stride the 16-byte loads of one field by lanes holding different triangles (the tile
// tests) fall into two of the eight 16-byte bank groups of a quarter warp, with an 80-byte stride
// into eight. The loads stay 16-byte vectors.
template <class T>
struct __align__(16) Padded {
    T v;
    uint4 pad;
};

// A draw's chunk shape as passed to the queue and chunk stage: width | height << 8, in tiles.
__host__ __device__ __forceinline__ uint32_t chunk_shape(const DrawArgs& a) {
    const uint32_t w = a.chunkTiles ? a.chunkTiles : (uint32_t)kChunkTiles;
    return w | ((a.chunkTilesY ? a.chunkTilesY : w) << 8);
}

// ShadeMeshlet's vertex transform (Shading.cpp:295-298): the clip position of a vertex slot; slots
// past the 16-vertex chunks up to NumVertices are zero.
__device__ __forceinline__ float4 clip_position(float x, float y, float z, bool live, const ViewParams& vp) {
    return live ? clip_transform(x, y, z, vp.m) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// TriangleEdgeVars::Setup (Rasterizer.cpp:296-329) into a TriRec with its rank (the opaque
// vis-buffer shader does not read the perspective-correct barycentrics; alpha_ext adds them from
// *rcpAreaOut). Returns the fixed-point determinant (> 0, or 0 for a triangle degenerate in fixed
// point).
__device__ __forceinline__ int32_t edge_setup(const Setup& t, int halfW, int halfH, uint32_t bbMin, uint32_t bbMax,
                                              uint32_t rank, TriRec& r, float* rcpAreaOut = nullptr) {
    const Edges e = edge_vars(t, halfW, halfH);
    r.E0 = e.E0, r.E1 = e.E1, r.E2 = e.E2;
    r.A12 = e.A12, r.B12 = e.B12, r.A20 = e.A20, r.B20 = e.B20, r.A01 = e.A01, r.B01 = e.B01;
    r.Z0 = e.Z0, r.Z10 = e.Z10, r.Z20 = e.Z20;
    r.bbMin = bbMin, r.bbMax = bbMax;
    r.lowword = 0xFFFFFFFEu - rank;
    r.pad = 0;
    if (rcpAreaOut) *rcpAreaOut = e.rcpArea;
    return e.det;
}


// ------------------------------------------------------------------ fragments
// DrawTriangle inner loop (Rasterizer.h:287-323) + FS_EncodeSurfaceId<false> (Shading.cpp:309-331)
// for one pixel inside the triangle's render box.
__device__ __forceinline__ void shade_fragment(const TriRec& r, uint32_t px, uint32_t py, unsigned long long* keys,
                                               uint32_t width) {
    int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    if ((e0 | e1 | e2) < 0) return;
    float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
    if (depth != depth) return;  // NaN never passes `Depth > old`
    unsigned long long key = ((unsigned long long)float_order(depth) << 32) | r.lowword;
    unsigned long long* p = keys + pixel_offset(px, py, width);
    if (key > *(volatile unsigned long long*)p) atomicMax(p, key);
}

// Tiny triangles, drawn by their own lane. A sample passes the edge tests only inside the closed
// fixed-point triangle (the tests are exact: floor(F / 16) >= 0 iff F >= 0, and the top-left
// biases only remove boundary samples), so its pixel p satisfies 16 (p - half) + 8 in
// [min, max] of the vertices, i.e. p in [(min + 7) >> 4, (max - 8) >> 4] + half, computed per
// 16-bit half (the render box's single 32-bit add can carry from x into y). The tile walk visits
// [bbMin, bbMax). The lane evaluates the pixels of both ranges' intersection: exactly the walk's
// covered pixels. A triangle degenerate in fixed point (det 0) can pass samples on its whole line
// and keeps the walk.
constexpr uint32_t kTinyPixels = 2;
// A meshlet is drawn in the single-view draw's first pass when its bounding sphere's radius exceeds
// this share of the clip w of its centre (about 94 pixels at 1920 pixels across and 60 degrees).
constexpr float kLargeMeshlet = 0.1f;
struct TinyBox { uint32_t x0, y0, x1, y1; };  // inclusive pixel range
__device__ __forceinline__ bool tiny_box(const Setup& t, int halfW, int halfH, uint32_t bbMin, uint32_t bbMax,
                                         TinyBox& b) {
    const uint32_t vp = (uint32_t)halfW | ((uint32_t)halfH << 16);
    const uint32_t lo = srai16_4(__vadd2(__vmins2(__vmins2(t.Pos0, t.Pos1), t.Pos2), 0x00070007u));
    const uint32_t hi = srai16_4(__vsub2(__vmaxs2(__vmaxs2(t.Pos0, t.Pos1), t.Pos2), 0x00080008u));
    const uint32_t x = __vmaxs2(__vadd2(lo, vp), bbMin);
    const uint32_t y = __vmins2(__vadd2(hi, vp), bbMax - 0x00010001u);
    b.x0 = x & 0xFFFF, b.y0 = x >> 16, b.x1 = y & 0xFFFF, b.y1 = y >> 16;
    const int w = (int)(int16_t)(y & 0xFFFF) - (int)(int16_t)(x & 0xFFFF) + 1;
    const int h = (int)(int16_t)(y >> 16) - (int)(int16_t)(x >> 16) + 1;
    return w <= 0 || h <= 0 || w * h <= (int)kTinyPixels;
}

__device__ __forceinline__ void shade_tiny(const TriRec& r, const TinyBox& b, unsigned long long* keys, uint32_t width) {
    for (int y = (int16_t)b.y0; y <= (int16_t)b.y1; y++)
        for (int x = (int16_t)b.x0; x <= (int16_t)b.x1; x++) {
            const uint32_t px = (uint32_t)x, py = (uint32_t)y;
            const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
            const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
            const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
            if ((e0 | e1 | e2) < 0) continue;
            const float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
            if (depth != depth) continue;
            atomicMax(keys + pixel_offset(px, py, width), ((unsigned long long)float_order(depth) << 32) | r.lowword);
        }
}

// ceil(256 / n) for n = 1..16, the multiplier of the small triangles' tile -> row multiply-shift:
// ceil(256 / n) - 1 packed 8 bits per entry in two words (an integer divide per triangle costs more
// than the rest of its tile bookkeeping).
__device__ __forceinline__ uint32_t row_magic(int n) {
    const unsigned long long t = n <= 8 ? 0x1f242a333f557fffull : 0xf1112131517191cull;
    return (uint32_t)((t >> (8 * ((n - 1) & 7))) & 0xFF) + 1u;
}

// Upper bound of the depth tile_pixel_key computes for any sample of the 4x4 tile at (px, py).
// The exact depth Z0 + Z10 e1 + Z20 e2 is affine in the pixel (the edge values are exact
// integers): it is the first sample's plus i Gx + j Gy at sample (i, j), with the per-pixel steps
// Gx = Z10 A20 + Z20 A01 and Gy = Z10 B20 + Z20 B01, so its maximum over the tile is the first
// sample's plus 3 max(Gx, 0) + 3 max(Gy, 0). A computed sample depth differs from the exact one by
// at most 4u S, u = 2^-24, S = |Z0| + |Z10| max|e1| + |Z20| max|e2| (two conversions, two fma
// roundings), and the bound's own evaluation by at most 10u S more; 2^-18 S covers both four times
// over. max|e| over the tile is at most |e(first)| + 3 (|A| + |B|). A NaN or infinite term gives +inf
// (never culled).
__device__ __forceinline__ float tile_depth_bound(const TriRec& r, uint32_t px, uint32_t py) {
    const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    const float f1 = __int2float_rn(e1), f2 = __int2float_rn(e2);
    const float d = ffma(f1, r.Z10, ffma(f2, r.Z20, r.Z0));
    const float gx = ffma(r.Z10, (float)r.A20, fmul(r.Z20, (float)r.A01));
    const float gy = ffma(r.Z10, (float)r.B20, fmul(r.Z20, (float)r.B01));
    const float dmax = fadd(d, fmul(3.0f, fadd(fmaxf(gx, 0.0f), fmaxf(gy, 0.0f))));
    const float a1 = fadd(fabsf(f1), fmul(3.0f, (float)(abs(r.A20) + abs(r.B20))));
    const float a2 = fadd(fabsf(f2), fmul(3.0f, (float)(abs(r.A01) + abs(r.B01))));
    const float s = fadd(fabsf(r.Z0), fadd(fmul(fabsf(r.Z10), a1), fmul(fabsf(r.Z20), a2)));
    const float b = fadd(dmax, fmul(s, 0x1p-18f));
    return b == b ? b : __int_as_float(0x7F800000);
}

// Raises the tile's depth bound to the minimum of the values its 16 pixels reported (the two
// halves of the warp shade one tile each: two whole-warp reductions, each over one half's values).
__device__ __forceinline__ void update_tile_min(uint32_t obs, uint32_t* tileMin, uint32_t tileIdx, uint32_t known,
                                                bool active, int lane) {
    const bool upper = lane & 16;
    const uint32_t lo = __reduce_min_sync(0xFFFFFFFFu, upper ? 0xFFFFFFFFu : obs);
    const uint32_t hi = __reduce_min_sync(0xFFFFFFFFu, upper ? obs : 0xFFFFFFFFu);
    obs = upper ? hi : lo;
    if (active && (lane & 15) == 0 && obs > known) atomicMax(&tileMin[tileIdx], obs);
}

// One lane rasterizes a whole triangle (fallback of the rare clipped triangle that finds the
// queue full; slow but exact).
__device__ __noinline__ void raster_serial(const TriRec& r, unsigned long long* keys, uint32_t width) {
    uint32_t minX = r.bbMin & 0xFFFF, minY = r.bbMin >> 16, maxX = r.bbMax & 0xFFFF, maxY = r.bbMax >> 16;
    for (uint32_t y = minY; y < maxY; y++)
        for (uint32_t x = minX; x < maxX; x++) shade_fragment(r, x, y, keys, width);
}

// Appends a triangle (its view index in r.pad) to the chunk queue; false when the queue is full
// (the caller rasterizes it).
__device__ __forceinline__ bool enqueue_big(const TriRec& r, const DrawArgs& a, uint32_t chunk) {
    int tilesX = ((r.bbMax & 0xFFFF) - (r.bbMin & 0xFFFF)) >> 2;
    int tilesY = ((r.bbMax >> 16) - (r.bbMin >> 16)) >> 2;
    const uint32_t cw = chunk & 0xFF, ch = chunk >> 8;
    unsigned long long chunks = (unsigned long long)((tilesX + cw - 1) / cw) * (unsigned long long)((tilesY + ch - 1) / ch);
    unsigned long long old = atomicAdd(&a.s.control[1], (1ull << 40) | chunks);
    unsigned long long slot = old >> 40;
    if (slot < a.s.bigCapacity) {
        a.s.big[slot] = r;
        a.s.bigBase[slot] = old & ((1ull << 40) - 1);
        return true;
    }
    atomicOr(&a.s.control[2], kStatusBigOverflow);
    return false;
}

// ------------------------------------------------------------------ alpha test
// FS_EncodeSurfaceId<true> (Shading.cpp:309-331): after the depth test, the fragment's
// perspective-correct barycentrics (Rasterizer.h:300-317, rcp14 reproduced exactly) interpolate the
// vertices' texcoords (FragmentVars::Interpolate = BaryLerp, Rasterizer.h:101-104), the material's
// texture is sampled at the implicit LOD of the 4x4 tile (SampleImplicitLod, Texture.h:403-410,
// with the 2x2 finite differences texutil::dFdx/dFdy, Texture.h:258-275) and the fragment survives
// if the texel is >= AlphaCutoff << 24. Every sample of a visited tile takes part in the
// differences and in the tile's filter choice, covered or not, as the reference's 16 lanes do.

// Mesh::TexCoords[VertexId]. The index byte is not bounded by the reference, whose record holds
// NormalTangents and Indices after the 64 texcoords: indices below 224 read that word of the
// record, larger ones (the next record in the reference) read 0.
__device__ __forceinline__ uint32_t texcoord_word(const uint8_t* mp, uint32_t idx) {
    return idx < 224 ? *(const uint32_t*)(mp + kOffTexCoords + 4 * idx) : 0u;
}

// Alpha-test terms of a triangle from its setup (TriangleEdgeVars W terms, Rasterizer.cpp:320-328).
__device__ __forceinline__ AlphaExt alpha_ext(const Setup& t, float rcpArea, uint32_t tc0, uint32_t tc1, uint32_t tc2,
                                              uint32_t material) {
    AlphaExt x;
    x.W0 = t.W0;
    x.W0S = fmul(t.W0, rcpArea), x.W1S = fmul(t.W1, rcpArea), x.W2S = fmul(t.W2, rcpArea);
#pragma unroll
    for (int k = 0; k < 3; k++) x.ru[k] = 0.0f, x.rv[k] = 0.0f;
    x.tc0 = tc0, x.tc1 = tc1, x.tc2 = tc2;
    x.zero0 = 0, x.zero1 = 0;
    x.material = material;
    return x;
}

struct TexCoord { float u, v; };

// Interpolated texcoord of the sample whose edge values are (u, v) (as floats).
__device__ __forceinline__ TexCoord alpha_texcoord(const AlphaExt& x, float u, float v) {
    float bu, bv;  // clipped (kTriAlpha): barycentrics of the source triangle
    perspective_bary(u, v, x.W0, x.W0S, x.W1S, x.W2S, (x.material & kTriAlpha) != 0, x.ru, x.rv, bu, bv);
    const float b0 = fsub(fsub(1.0f, bu), bv);
    TexCoord s;
    s.u = ffma(h2f(x.tc0 & 0xFFFF), b0, ffma(h2f(x.tc1 & 0xFFFF), bu, fmul(h2f(x.tc2 & 0xFFFF), bv)));
    s.v = ffma(h2f(x.tc0 >> 16), b0, ffma(h2f(x.tc1 >> 16), bu, fmul(h2f(x.tc2 >> 16), bv)));
    return s;
}

// CalcMipLevel(grad) - LerpFracBits (Texture.h:271-275, 408) from the differences of the scaled
// sample positions (d/dx su, d/dx sv, d/dy su, d/dy sv).
__device__ __forceinline__ int32_t alpha_mip(float gx, float gy, float gz, float gw) {
    const float dx = ffma(gx, gx, fmul(gy, gy)), dy = ffma(gz, gz, fmul(gw, gw));
    return (ilog2_x86(vmax(dx, dy)) >> 1) - 8;
}

// The opaque tile shading of shade_live_tiles with the alpha test, for pixel (tx + l % 4,
// ty + l / 4), l = lane % 16, called by all 32 lanes: each half-warp shades one tile of
// the same triangle (valid is false on a half without a tile). The x and y differences pair
// lanes l ^ 1 and l ^ 4 of a half.
__device__ __forceinline__ uint32_t shade_tile_pixel_alpha(const TriRec& r, const AlphaExt& x, const DevTexture& tex,
                                                           uint32_t cutoff, uint32_t tx, uint32_t ty, bool valid, int lane,
                                                           unsigned long long* keys, uint32_t width) {
    const uint32_t l = lane & 15;
    unsigned long long* p = keys + (tx << 2) + ty * width + l;
    const unsigned long long cur = valid ? *(volatile unsigned long long*)p : 0ull;
    const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
    const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    const float u = __int2float_rn(e1), v = __int2float_rn(e2);
    const float depth = ffma(u, r.Z10, ffma(v, r.Z20, r.Z0));
    const unsigned long long key = ((unsigned long long)float_order(depth) << 32) | r.lowword;
    bool pass = valid && (e0 | e1 | e2) >= 0 && depth == depth && key > cur;
    if (__any_sync(0xFFFFFFFFu, pass)) {
        const TexCoord s = alpha_texcoord(x, u, v);
        const float su = fmul(s.u, tex.scale_lerp_u), sv = fmul(s.v, tex.scale_lerp_v);
        const float sux = __shfl_xor_sync(0xFFFFFFFFu, su, 1), svx = __shfl_xor_sync(0xFFFFFFFFu, sv, 1);
        const float suy = __shfl_xor_sync(0xFFFFFFFFu, su, 4), svy = __shfl_xor_sync(0xFFFFFFFFu, sv, 4);
        const bool ox = l & 1, oy = l & 4;  // dFdx = p[l | 1] - p[l & ~1], dFdy = p[l | 4] - p[l & ~4]
        const int32_t mip = alpha_mip(ox ? fsub(su, sux) : fsub(sux, su), ox ? fsub(sv, svx) : fsub(svx, sv),
                                      oy ? fsub(su, suy) : fsub(suy, su), oy ? fsub(sv, svy) : fsub(svy, sv));
        const bool nearest = (__ballot_sync(0xFFFFFFFFu, mip > 0) & (0xFFFFu << (lane & 16))) != 0;
        if (pass) pass = sample_rgba8(tex, s.u, s.v, 0, mip, nearest) >= cutoff;
    }
    if (!pass) return (uint32_t)(cur >> 32);
    atomicMax(p, key);
    return (uint32_t)(key >> 32);
}

// One lane rasterizes a whole alpha-tested triangle, the 16 samples of each tile in turn
// (fallback of a triangle that finds the queue full; slow but exact).
__device__ __noinline__ void raster_serial_alpha(const TriRec& r, const AlphaExt& x, const DevMaterial* materials,
                                                 unsigned long long* keys, uint32_t width) {
    const DevMaterial& mt = materials[x.material & ~kTriAlpha];
    const uint32_t cutoff = mt.alpha_cutoff << 24;
    const uint32_t minX = r.bbMin & 0xFFFF, minY = r.bbMin >> 16, maxX = r.bbMax & 0xFFFF, maxY = r.bbMax >> 16;
    for (uint32_t ty = minY; ty < maxY; ty += 4) {
        for (uint32_t tx = minX; tx < maxX; tx += 4) {
            float su[16], sv[16], tu[16], tv[16];
            unsigned pass = 0;
            for (uint32_t l = 0; l < 16; l++) {
                const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
                const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
                const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
                const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
                const float u = __int2float_rn(e1), v = __int2float_rn(e2);
                const float depth = ffma(u, r.Z10, ffma(v, r.Z20, r.Z0));
                const unsigned long long key = ((unsigned long long)float_order(depth) << 32) | r.lowword;
                if ((e0 | e1 | e2) >= 0 && depth == depth && key > *(volatile unsigned long long*)(keys + (tx << 2) + ty * width + l))
                    pass |= 1u << l;
                const TexCoord s = alpha_texcoord(x, u, v);
                tu[l] = s.u, tv[l] = s.v;
                su[l] = fmul(s.u, mt.tex.scale_lerp_u), sv[l] = fmul(s.v, mt.tex.scale_lerp_v);
            }
            if (!pass) continue;
            int32_t mip[16];
            bool nearest = false;
            for (uint32_t l = 0; l < 16; l++) {
                const uint32_t lx = l & ~1u, hx = l | 1u, ly = l & ~4u, hy = l | 4u;
                mip[l] = alpha_mip(fsub(su[hx], su[lx]), fsub(sv[hx], sv[lx]), fsub(su[hy], su[ly]), fsub(sv[hy], sv[ly]));
                nearest |= mip[l] > 0;
            }
            for (uint32_t l = 0; l < 16; l++) {
                if (!((pass >> l) & 1) || sample_rgba8(mt.tex, tu[l], tv[l], 0, mip[l], nearest) < cutoff) continue;
                const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
                const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
                const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
                const float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
                atomicMax(keys + (tx << 2) + ty * width + l, ((unsigned long long)float_order(depth) << 32) | r.lowword);
            }
        }
    }
}

// Appends an alpha-tested triangle and its AlphaExt (in the next slot, which owns no chunks) to
// the chunk queue; false when the queue is full (the caller rasterizes it). A pair that finds
// one slot left leaves an empty record there, so every slot below the capacity is written.
__device__ __forceinline__ bool enqueue_alpha(const TriRec& r, const AlphaExt& x, const DrawArgs& a, uint32_t chunk) {
    const int tilesX = ((r.bbMax & 0xFFFF) - (r.bbMin & 0xFFFF)) >> 2;
    const int tilesY = ((r.bbMax >> 16) - (r.bbMin >> 16)) >> 2;
    const uint32_t cw = chunk & 0xFF, ch = chunk >> 8;
    const unsigned long long chunks = (unsigned long long)((tilesX + cw - 1) / cw) * (unsigned long long)((tilesY + ch - 1) / ch);
    const unsigned long long old = atomicAdd(&a.s.control[1], (2ull << 40) | chunks);
    const unsigned long long slot = old >> 40, base = old & ((1ull << 40) - 1);
    if (slot + 1 < a.s.bigCapacity) {
        a.s.big[slot] = r;
        a.s.big[slot + 1] = *(const TriRec*)&x;
        a.s.bigBase[slot] = base;
        a.s.bigBase[slot + 1] = base + chunks;
        return true;
    }
    if (slot < a.s.bigCapacity) {
        TriRec e = {};
        a.s.big[slot] = e;
        a.s.bigBase[slot] = base;
    }
    atomicOr(&a.s.control[2], kStatusBigOverflow);
    return false;
}

// A small triangle's record (the mesh stage's tile walk): pad = tilesX | row_magic << 8 | kPadReadKey.
constexpr uint32_t kPadReadKey = 1u << 24;
// The 4x4 tiles of a triangle's render box.
__device__ __forceinline__ uint32_t triangle_tiles(const TriRec& r) {
    return (((r.bbMax & 0xFFFF) - (r.bbMin & 0xFFFF)) >> 2) * (((r.bbMax >> 16) - (r.bbMin >> 16)) >> 2);
}

// Largest value over the tile [px, px+3] x [py, py+3] of the affine edge function e(px, py) + A*dx + B*dy.
__device__ __forceinline__ int32_t tile_max_edge(int32_t e, int32_t A, int32_t B) {
    return e + (A > 0 ? 3 * A : 0) + (B > 0 ? 3 * B : 0);
}
// True if no sample of the 4x4 tile at (px, py) can pass all three edges.
__device__ __forceinline__ bool tile_empty(const TriRec& r, uint32_t px, uint32_t py) {
    int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    return tile_max_edge(e0, r.A12, r.B12) < 0 || tile_max_edge(e1, r.A20, r.B20) < 0 ||
           tile_max_edge(e2, r.A01, r.B01) < 0;
}

// Upper bound of any fragment depth of a triangle from its vertex depths: a fragment's depth is its
// edge functions' interpolation of Z0, Z1, Z2 inside the triangle, so at most their maximum, plus the
// roundings of the plane terms and of the evaluation, within 16 ulp of the largest |Z| (2^-20);
// 2^-16 of it is kept. For a small triangle this is much tighter than the plane's value at the tile
// corners, which lie outside it. NaN vertex depths give a NaN, which never beats a fragment's.
__device__ __forceinline__ float triangle_depth_bound(const Setup& t) {
    const float m = fmaxf(fmaxf(fabsf(t.Z0), fabsf(t.Z1)), fabsf(t.Z2));
    const bool nan = t.Z0 != t.Z0 || t.Z1 != t.Z1 || t.Z2 != t.Z2;
    return nan ? __int_as_float(0x7F800000) : fadd(fmaxf(fmaxf(t.Z0, t.Z1), t.Z2), fmul(m, 0x1p-16f));
}

// True if the tile at (px, py) (4-aligned) can be shaded for r: some sample may pass the edges
// and, when a depth bound is kept, r may beat the tile's depth bound somewhere. *known receives
// the bound read (for the later update).
__device__ __forceinline__ bool tile_live(const TriRec& r, uint32_t px, uint32_t py, const uint32_t* tileMin,
                                          uint32_t tilesPerRow, uint32_t* known) {
    if (tile_empty(r, px, py)) return false;
    if (!tileMin) return true;
    *known = tileMin[(py >> 2) * tilesPerRow + (px >> 2)];
    return float_order(tile_depth_bound(r, px, py)) >= *known;
}
// tile_live with the triangle's own depth bound zmax (triangle_depth_bound) as a second bound.
__device__ __forceinline__ bool tile_live(const TriRec& r, uint32_t px, uint32_t py, const uint32_t* tileMin,
                                          uint32_t tilesPerRow, uint32_t* known, float zmax) {
    if (tile_empty(r, px, py)) return false;
    if (!tileMin) return true;
    *known = tileMin[(py >> 2) * tilesPerRow + (px >> 2)];
    return float_order(fminf(tile_depth_bound(r, px, py), zmax)) >= *known;
}

// Shades the live tiles of the warp-wide candidate set (the lanes in `mask` hold a tile origin
// tpx/tpy, its depth bound tmin and a triangle selector rsel for rec()), two tiles per step, and
// raises the tiles' depth bounds.
// The key DrawTriangle + FS_EncodeSurfaceId<false> (Rasterizer.h:287-323, Shading.cpp:309-331)
// offers for pixel (tx + l % 4, ty + l / 4) of the 4x4 tile at the 4-aligned (tx, ty), 0 if the
// sample is outside the triangle or its depth is NaN. The tiled key offset is the tile's base
// plus l, so a tile's 16 keys are one 128-byte line.
__device__ __forceinline__ unsigned long long tile_pixel_key(const TriRec& r, uint32_t tx, uint32_t ty, uint32_t l) {
    const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
    const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    if ((e0 | e1 | e2) < 0) return 0ull;
    const float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
    if (depth != depth) return 0ull;  // NaN never passes `Depth > old`
    return ((unsigned long long)float_order(depth) << 32) | r.lowword;
}

// Shades the live tiles of the warp-wide candidate set (the lanes in `mask` hold a tile origin
// tpx/tpy, its depth bound tmin and a triangle selector rsel for rec()) and raises the tiles' depth
// bounds (each pixel reports a lower bound of its depth word afterwards). Four tiles per step: each
// half-warp takes two, and a lane's two key loads are issued together (the walk is bound by their
// latency).
template <class Rec, class ReadKey>
__device__ __forceinline__ void shade_live_tiles(Rec&& rec, ReadKey&& readKey, uint32_t rsel, unsigned mask, uint32_t tpx,
                                                 uint32_t tpy, uint32_t tmin, unsigned long long* keys, uint32_t* tileMin,
                                                 uint32_t width, int lane) {
    const uint32_t half = lane >> 4, tw = width >> 2, l = lane & 15;
    const uint32_t txy = tpx | (tpy << 16);  // tile origins are below 2896
    while (mask) {
        int s[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            s[k] = mask ? __ffs(mask) - 1 : -1;
            if (s[k] >= 0) mask &= mask - 1;
        }
        const int srcA = half ? s[1] : s[0], srcB = half ? s[3] : s[2];
        const uint32_t pa_ = __shfl_sync(0xFFFFFFFFu, txy, srcA & 31), pb_ = __shfl_sync(0xFFFFFFFFu, txy, srcB & 31);
        const uint32_t ax = pa_ & 0xFFFF, ay = pa_ >> 16, bx = pb_ & 0xFFFF, by = pb_ >> 16;
        const uint32_t am = __shfl_sync(0xFFFFFFFFu, tmin, srcA & 31), ar = __shfl_sync(0xFFFFFFFFu, rsel, srcA & 31);
        const uint32_t bm = __shfl_sync(0xFFFFFFFFu, tmin, srcB & 31), br = __shfl_sync(0xFFFFFFFFu, rsel, srcB & 31);
        unsigned long long* pa = keys + (ax << 2) + ay * width + l;
        unsigned long long* pb = keys + (bx << 2) + by * width + l;
        // The key read filters losing atomics and gives the tile bound each pixel's new depth. For
        // triangles whose readKey(selector) is false (above the draw's keyReadTiles tiles) it is
        // skipped: the atomic is unconditional and a pixel's bound is max(new depth, old tile
        // bound), still a lower bound of its final key.
        const bool readA = srcA >= 0 && readKey(ar);
        const bool readB = srcB >= 0 && readKey(br);
        const unsigned long long curA = readA ? *(volatile unsigned long long*)pa : 0ull;
        const unsigned long long curB = readB ? *(volatile unsigned long long*)pb : 0ull;
        const unsigned long long keyA = srcA >= 0 ? tile_pixel_key(rec(ar), ax, ay, l) : 0ull;
        const unsigned long long keyB = srcB >= 0 ? tile_pixel_key(rec(br), bx, by, l) : 0ull;
        if (keyA > curA) atomicMax(pa, keyA);
        if (keyB > curB) atomicMax(pb, keyB);
        if (tileMin) {
            const uint32_t obsA = readA ? (uint32_t)((keyA > curA ? keyA : curA) >> 32) : max((uint32_t)(keyA >> 32), am);
            const uint32_t obsB = readB ? (uint32_t)((keyB > curB ? keyB : curB) >> 32) : max((uint32_t)(keyB >> 32), bm);
            update_tile_min(obsA, tileMin, (ay >> 2) * tw + (ax >> 2), am, srcA >= 0, lane);
            update_tile_min(obsB, tileMin, (by >> 2) * tw + (bx >> 2), bm, srcB >= 0, lane);
        }
    }
}

// shade_live_tiles for alpha-tested triangles of one material (texture tex, cutoff << 24): a
// candidate's triangle is rec(rsel), its alpha terms ext(rsel) (the two tiles of a step may belong
// to different triangles).
template <class Rec, class Ext>
__device__ __forceinline__ void shade_live_tiles_alpha(Rec&& rec, Ext&& ext, uint32_t rsel,
                                                       const DevTexture& tex, uint32_t cutoff, unsigned mask,
                                                       uint32_t tpx, uint32_t tpy, uint32_t tmin,
                                                       unsigned long long* keys, uint32_t* tileMin, uint32_t width,
                                                       int lane) {
    const uint32_t half = lane >> 4, tw = width >> 2;
    while (mask) {
        const int s0 = __ffs(mask) - 1;
        mask &= mask - 1;
        const int s1 = mask ? __ffs(mask) - 1 : -1;
        if (s1 >= 0) mask &= mask - 1;
        const int src = half ? s1 : s0;
        const uint32_t qx = __shfl_sync(0xFFFFFFFFu, tpx, src & 31);
        const uint32_t qy = __shfl_sync(0xFFFFFFFFu, tpy, src & 31);
        const uint32_t qm = __shfl_sync(0xFFFFFFFFu, tmin, src & 31);
        const uint32_t qr = __shfl_sync(0xFFFFFFFFu, rsel, src & 31);
        const uint32_t obs = shade_tile_pixel_alpha(rec(qr), ext(qr), tex, cutoff, qx, qy, src >= 0, lane, keys, width);
        if (tileMin) update_tile_min(obs, tileMin, (qy >> 2) * tw + (qx >> 2), qm, src >= 0, lane);
    }
}

// ceil(2^16 / n) for n = 1..16: t / n == (t * kDiv16[n]) >> 16 for every t < 256 (checked
// exhaustively), the tile index division of a chunk of at most 16 x 16 tiles.
__constant__ uint32_t kDiv16[17] = { 0, 65536, 32768, 21846, 16384, 13108, 10923, 9363, 8192,
                                     7282, 6554, 5958, 5462, 5042, 4682, 4370, 4096 };

// Rasterizes the tiles of [x0, x0 + 4*tilesX) x [y0, y0 + 4*tilesY) that are not provably empty
// or hidden: 32 tiles are tested at a time (one per lane), then shade(mask, tpx, tpy, tmin) shades
// the surviving ones. divMagic: kDiv16[tilesX] for a chunk (tilesX, tilesY <= 16), 0 otherwise.
template <class Shade>
__device__ __forceinline__ void raster_region_with(const TriRec& r, uint32_t x0, uint32_t y0, int tilesX, int tilesY,
                                                   const uint32_t* tileMin, uint32_t width, int lane, Shade&& shade,
                                                   uint32_t divMagic) {
    const int T = tilesX * tilesY;
    const uint32_t tw = width >> 2;
    for (int tb = 0; tb < T; tb += 32) {
        const int t = tb + lane;
        bool live = false;
        uint32_t tpx = 0, tpy = 0, tmin = 0;
        if (t < T) {
            int ty = divMagic ? (int)(((uint32_t)t * divMagic) >> 16) : t / tilesX, tx = t - ty * tilesX;
            tpx = x0 + tx * 4, tpy = y0 + ty * 4;
            live = tile_live(r, tpx, tpy, tileMin, tw, &tmin);
        }
        shade(__ballot_sync(0xFFFFFFFFu, live), tpx, tpy, tmin);
    }
}

// raster_region_with for an opaque triangle, two tiles per step.
__device__ __forceinline__ void raster_region(const TriRec& r, uint32_t x0, uint32_t y0, int tilesX, int tilesY,
                                              unsigned long long* keys, uint32_t* tileMin, uint32_t width, int lane, uint32_t readTiles,
                                              uint32_t divMagic = 0) {
    const bool readKey = readTiles == 0 || triangle_tiles(r) <= readTiles;
    raster_region_with(r, x0, y0, tilesX, tilesY, tileMin, width, lane,
                       [&](unsigned mask, uint32_t tpx, uint32_t tpy, uint32_t tmin) {
                           shade_live_tiles([&](uint32_t) -> const TriRec& { return r; }, [&](uint32_t) { return readKey; }, 0,
                                            mask, tpx, tpy, tmin, keys, tileMin, width, lane);
                       }, divMagic);
}

// The same for the alpha-tested triangle *rp with alpha terms *xp (material texture tex, cutoff << 24).
__device__ __forceinline__ void raster_region_alpha(const TriRec* rp, const AlphaExt* xp, const DevTexture& tex,
                                                    uint32_t cutoff, uint32_t x0, uint32_t y0, int tilesX, int tilesY,
                                                    unsigned long long* keys, uint32_t* tileMin, uint32_t width, int lane,
                                                    uint32_t divMagic = 0) {
    raster_region_with(*rp, x0, y0, tilesX, tilesY, tileMin, width, lane,
                       [&](unsigned mask, uint32_t tpx, uint32_t tpy, uint32_t tmin) {
                           shade_live_tiles_alpha([&](uint32_t) -> const TriRec& { return *rp; },
                                                  [&](uint32_t) -> const AlphaExt& { return *xp; }, 0, tex, cutoff, mask, tpx,
                                                  tpy, tmin, keys, tileMin, width, lane);
                       }, divMagic);
}

// ------------------------------------------------------------------ overdraw shader
// FS_Overdraw (Shading.cpp:333-342) for pixel l of the 4x4 tile at (tx, ty), called by all 32
// lanes (a half-warp per tile; valid is false on a half without one). DrawTriangle visits the tile
// only if a sample is covered; then every sample counts, covered ones in the high word of the
// pixel's counter and the others in the low word, and the tile's 16 depths feed a maximum kept in
// the key's high word (NaN never replaces: vmaxps keeps the old value).
__device__ __forceinline__ void shade_tile_pixel_overdraw(const TriRec& r, uint32_t tx, uint32_t ty, bool valid, int lane,
                                                          unsigned long long* keys, unsigned long long* counts,
                                                          uint32_t width) {
    const uint32_t l = lane & 15;
    const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
    const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
    const bool covered = valid && (e0 | e1 | e2) >= 0;
    if (!((__ballot_sync(0xFFFFFFFFu, covered) >> (lane & 16)) & 0xFFFFu) || !valid) return;
    const uint32_t off = (tx << 2) + ty * width + l;
    atomicAdd(&counts[off], covered ? (1ull << 32) : 1ull);
    const float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
    if (depth != depth) return;
    const unsigned long long key = (unsigned long long)float_order(depth) << 32;
    if (key > *(volatile unsigned long long*)&keys[off]) atomicMax(&keys[off], key);
}

// shade_live_tiles for the overdraw shader (no depth bounds: every tile a triangle covers counts).
template <class Rec>
__device__ __forceinline__ void shade_live_tiles_overdraw(Rec&& rec, uint32_t rsel, unsigned mask, uint32_t tpx, uint32_t tpy,
                                                          unsigned long long* keys, unsigned long long* counts,
                                                          uint32_t width, int lane) {
    const uint32_t half = lane >> 4;
    while (mask) {
        const int s0 = __ffs(mask) - 1;
        mask &= mask - 1;
        const int s1 = mask ? __ffs(mask) - 1 : -1;
        if (s1 >= 0) mask &= mask - 1;
        const int src = half ? s1 : s0;
        const uint32_t qx = __shfl_sync(0xFFFFFFFFu, tpx, src & 31);
        const uint32_t qy = __shfl_sync(0xFFFFFFFFu, tpy, src & 31);
        const uint32_t qr = __shfl_sync(0xFFFFFFFFu, rsel, src & 31);
        shade_tile_pixel_overdraw(rec(qr), qx, qy, src >= 0, lane, keys, counts, width);
    }
}

__device__ __forceinline__ void raster_region_overdraw(const TriRec& r, uint32_t x0, uint32_t y0, int tilesX, int tilesY,
                                                       unsigned long long* keys, unsigned long long* counts,
                                                       uint32_t width, int lane, uint32_t divMagic = 0) {
    raster_region_with(r, x0, y0, tilesX, tilesY, nullptr, width, lane,
                       [&](unsigned mask, uint32_t tpx, uint32_t tpy, uint32_t) {
                           shade_live_tiles_overdraw([&](uint32_t) -> const TriRec& { return r; }, 0, mask, tpx, tpy, keys,
                                                     counts, width, lane);
                       }, divMagic);
}

// One lane draws a whole triangle with the overdraw shader (the full-queue fallback of a clipped
// triangle).
__device__ __noinline__ void raster_serial_overdraw(const TriRec& r, unsigned long long* keys, unsigned long long* counts,
                                                    uint32_t width) {
    const uint32_t minX = r.bbMin & 0xFFFF, minY = r.bbMin >> 16, maxX = r.bbMax & 0xFFFF, maxY = r.bbMax >> 16;
    for (uint32_t ty = minY; ty < maxY; ty += 4) {
        for (uint32_t tx = minX; tx < maxX; tx += 4) {
            unsigned cov = 0;
            for (uint32_t l = 0; l < 16; l++) {
                const uint32_t px = tx + (l & 3), py = ty + (l >> 2);
                const int32_t e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
                const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
                const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
                if ((e0 | e1 | e2) >= 0) cov |= 1u << l;
            }
            if (!cov) continue;
            for (uint32_t l = 0; l < 16; l++) {
                const uint32_t px = tx + (l & 3), py = ty + (l >> 2), off = (tx << 2) + ty * width + l;
                atomicAdd(&counts[off], ((cov >> l) & 1) ? (1ull << 32) : 1ull);
                const int32_t e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
                const int32_t e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
                const float depth = ffma(__int2float_rn(e1), r.Z10, ffma(__int2float_rn(e2), r.Z20, r.Z0));
                if (depth == depth) atomicMax(&keys[off], (unsigned long long)float_order(depth) << 32);
            }
        }
    }
}

// Clipper::ClipTriangles + FlushPacket (Rasterizer.cpp:398-491) for this lane's triangle; the
// lanes of a packet are independent (each prim restarts its new-vertex slots). Fan outputs are
// set up with TrianglePacket::Setup and queued with rank (packet, clipped, lane, fan index).
// For an alpha-tested material (alphaMat != ~0u) the barycentric rows are clipped too and become
// the outputs' TriangleClipData; the texcoords are those of the source triangle (record mp, index
// bytes idxBytes).
__device__ __noinline__ void clip_and_queue(Vtx v0, Vtx v1, Vtx v2, uint32_t outcodes, const DrawArgs& a,
                                            const ViewParams& vp, uint32_t viewIndex, uint32_t chunk, int cullMode,
                                            uint32_t gMeshlet, uint32_t prim, uint32_t& nRaster,
                                            uint32_t alphaMat, const uint8_t* mp, const uint8_t* idxBytes) {
    const bool alpha = alphaMat != ~0u;
    ClipPoly P;
    if (!clip_polygon(v0, v1, v2, outcodes, vp.bx, vp.by, alpha ? 6 : 4, P)) {
        atomicOr(&a.s.control[2], kStatusClipOverflow);
        return;
    }
    const uint32_t vertCount = P.count;
    if (vertCount < 2) return;
    for (uint32_t vi = 0; vi + 2 < vertCount; vi++) {
        Vtx a0, a1, a2;
        float ru[3], rv[3];
        clip_fan(P, vi, a0, a1, a2, alpha ? ru : nullptr, rv);
        Setup t;
        uint32_t bbMin, bbMax;
        if (!tri_setup(a0, a1, a2, vp.halfW, vp.halfH, cullMode, t, bbMin, bbMax)) continue;
        TriRec r;
        float rcpArea;
        edge_setup(t, vp.halfW, vp.halfH, bbMin, bbMax, make_rank(gMeshlet, prim, 1, vi), r, &rcpArea);
        r.pad = viewIndex;
        nRaster++;
        if (alpha) {
            AlphaExt x = alpha_ext(t, rcpArea, texcoord_word(mp, idxBytes[prim]), texcoord_word(mp, idxBytes[128 + prim]),
                                   texcoord_word(mp, idxBytes[256 + prim]), alphaMat | kTriAlpha);
            for (int k = 0; k < 3; k++) x.ru[k] = ru[k], x.rv[k] = rv[k];  // TriangleClipData, Rasterizer.cpp:455-458
            r.pad = viewIndex | kTriAlpha;
            if (!enqueue_alpha(r, x, a, chunk)) raster_serial_alpha(r, x, a.materials, vp.keys, vp.width);
            continue;
        }
        if (enqueue_big(r, a, chunk)) continue;
        if (a.counts) raster_serial_overdraw(r, vp.keys, a.counts, vp.width);
        else raster_serial(r, vp.keys, vp.width);
    }
}

// Triangle p of a meshlet for one lane of a 32-triangle step: its projected vertices (gathered
// from the meshlet's per-vertex arrays as simd::gather_preload64 does) and its clip codes
// (Clipper::ComputeClipCodes, Rasterizer.cpp:353-397). The transform step computes each vertex's
// perspective division and codes once; a vertex is shared by about six triangles.
struct LaneTri {
    Ndc n0, n1, n2;     // projected vertices
    uint32_t partial;   // OR of the vertices' out codes
    bool acc, nontriv;  // trivially accepted / accepted but needs clipping
};

__device__ __forceinline__ LaneTri lane_triangle(const float4* ndc, const uint8_t* codes, const uint8_t* idxBytes,
                                                 uint32_t p, bool valid) {
    LaneTri lt;
    const uint32_t i0 = preload64_index(idxBytes[p & 127]);
    const uint32_t i1 = preload64_index(idxBytes[128 + (p & 127)]);
    const uint32_t i2 = preload64_index(idxBytes[256 + (p & 127)]);
    const float4 q0 = ndc[i0], q1 = ndc[i1], q2 = ndc[i2];
    lt.n0 = { q0.x, q0.y, q0.z, q0.w }, lt.n1 = { q1.x, q1.y, q1.z, q1.w }, lt.n2 = { q2.x, q2.y, q2.z, q2.w };
    const uint32_t c0 = codes[i0], c1 = codes[i1], c2 = codes[i2];
    const uint32_t partial = (c0 | c1 | c2) & 0x3Fu, combined = c0 & c1 & c2 & 0x3Fu;
    const bool trivial = (c0 & c1 & c2 & kCodeInBand) != 0 && !(partial & 0x30u);
    const bool accept = valid && combined == 0;
    lt.partial = partial;
    lt.acc = accept && trivial;
    lt.nontriv = accept && !trivial;
    return lt;
}

// ------------------------------------------------------------------ kernels
// Per-warp shared memory: transformed vertices, index bytes, triangle records, the view, and the
// owner lane of each tile in the concatenated tile list of the round's small triangles. The alpha
// pass also keeps each small triangle's alpha terms.
struct WarpSmem {
    float4 ndc[64];      // projected vertices: x/w, y/w, z/w, 1/w
    uint32_t idx[96];
    Padded<TriRec> tris[32];
    ViewParams view;
    uint8_t owner[32 * kSmallTiles];
    uint8_t code[64];    // vertex_code
    uint8_t live[128];   // the meshlet's triangles that survive the face test or need clipping
    float zmax[32];      // each small triangle's depth bound (triangle_depth_bound)
};
struct WarpSmemAlpha : WarpSmem {
    Padded<AlphaExt> exts[32];
};

// Mesh stage. A work item is one meshlet of one view: a single-view draw numbers its meshlets
// 0..count-1; a batched draw concatenates the meshlet ranges of its views (viewStart is their
// prefix), so one launch serves views of any size.
// Vis-buffer draws take two passes: the opaque pass draws every opaque meshlet and appends the
// work items of alpha-tested meshlets to alphaList; the alpha pass draws those with
// FS_EncodeSurfaceId<true>. The order of the passes does not change the keys. OverdrawShader draws
// take one pass over every meshlet.
// View of batched work position p: the largest v with viewStart[v] <= p.
__device__ __forceinline__ uint32_t view_of(const uint32_t* viewStart, uint32_t numViews, uint32_t p) {
    uint32_t lo = 0, hi = numViews - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (viewStart[mid] <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

enum : int { kPassOpaque = 0, kPassAlpha = 1, kPassOverdraw = 2 };
// kShaded: the meshlets come shaded by a user mesh shader (a.shaded, swr_shaded_meshlet records):
// clip positions, indices, PrimCount, CullMode and FragmentShaderId are read from the record
// instead of ShadeMeshlet's transform of the Meshlet (whose texcoords and material the alpha test
// still reads).
template <int kPass, bool kShaded = false>
__global__ void __launch_bounds__(512, 2) k_draw_meshlets(DrawArgs a) {
    constexpr bool kAlpha = kPass == kPassAlpha, kOver = kPass == kPassOverdraw;
    using Smem = typename std::conditional<kAlpha, WarpSmemAlpha, WarpSmem>::type;
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Smem& S = ((Smem*)smemRaw)[warp];
    const uint8_t* idxBytes = (const uint8_t*)S.idx;
    Padded<TriRec>* tris = S.tris;
    const ViewParams& vp = S.view;
    const uint32_t chunk = chunk_shape(a);
    const bool multi = a.views != nullptr;
    // Work positions. Position p of a view draws its meshlet draw_order(p) (order_stride); a batched
    // draw concatenates its views' positions, padded to multiples of kBatchGroup (viewStart); the
    // alpha pass walks its list of work items.
    const uint32_t totalItems = kAlpha ? (uint32_t)a.s.control[9] : (multi ? a.viewStart[a.numViews] : a.count);
    unsigned long long* const cursor = &a.s.control[kAlpha ? 10 : 0];
    unsigned long long* const idleWarps = &a.s.control[kAlpha ? 12 : 11];  // warps past their last item
    const uint32_t numWarps = gridDim.x * (blockDim.x >> 5);
    uint32_t curView = 0xFFFFFFFFu;
    if (!multi) {
        if (lane == 0) {
            ViewParams v = {};
            for (int k = 0; k < 16; k++) v.m[k] = a.m[k];
            v.halfW = a.halfW, v.halfH = a.halfH, v.width = a.width, v.height = a.height;
            v.bx = a.bx, v.by = a.by, v.meshletOffset = a.meshletOffset, v.count = a.count;
            v.keys = a.keys, v.tileMin = a.tileMin;
            S.view = v;
        }
        curView = 0;
        __syncwarp();
    }
    uint32_t nProcessed = 0, nRaster = 0, nClipped = 0;  // per warp, within 32 bits (< 2^21 meshlets x 128)
    if (!kAlpha && blockIdx.x == 0 && threadIdx.x == 0) a.s.control[8] = 0;  // the chunk stage's cursor (runs later)

    // Work items are fetched a group at a time: one contended atomic per group. A group's cull
    // bits are tested at once (one position per lane), then the warp walks the visible ones.
    // Batched draws, most of whose (view, meshlet) items are culled, fetch groups of 32. A work
    // item is viewStart[view] + m (m alone in single-view draws), as the alpha list records it.
    uint32_t fetchPos = 0, fetchLeft = 0;  // alpha pass: next position, positions left
    uint32_t laneMeshlet = 0;              // the meshlet of this lane's position in the group
    uint32_t fetchView = 0;                // batched draws: the view of the fetched group
    unsigned fetchMask = 0;                // lanes of the fetched group whose meshlet is visible
    uint32_t fetchGroup = kDrawGroup;      // single view: positions per fetch
    // Single-view draws walk their positions twice: meshlets large on screen first, then the rest
    // (a second cursor, control[7]), so the costliest work items start early and the last ones
    // are small: a cheaper tail, and near geometry raises the tile depth bounds before the far.
    const bool twoPass = !multi && !kAlpha && !kShaded;
    uint32_t pass = twoPass ? 0u : 1u;
    while (true) {
        uint32_t m, view = 0, item;
        if constexpr (kAlpha) {
            if (fetchLeft == 0) {
                uint32_t b = 0;
                if (lane == 0) b = (uint32_t)atomicAdd(cursor, (unsigned long long)kDrawGroup);
                fetchPos = __shfl_sync(0xFFFFFFFFu, b, 0);
                fetchLeft = kDrawGroup;
            }
            const uint32_t idx = fetchPos++;
            fetchLeft--;
            if (idx >= totalItems) break;
            item = a.s.alphaList[idx];
            m = item;
            if (multi) {
                view = view_of(a.viewStart, a.numViews, item);
                m = item - a.viewStart[view];
            }
        } else {
            if (multi) {
                if (fetchMask == 0) {
                    uint32_t b = 0;
                    if (lane == 0) b = (uint32_t)atomicAdd(cursor, (unsigned long long)kBatchGroup);
                    const uint32_t base = __shfl_sync(0xFFFFFFFFu, b, 0);
                    if (base >= totalItems) break;
                    // groups interleave the views: group G is group G / numViews of view G % numViews
                    const uint32_t G = base / kBatchGroup;
                    fetchView = G % a.numViews;
                    const ViewParams& fv = a.views[fetchView];
                    // the cull wrote the group's 32 results as one word, in draw order
                    const uint32_t g = G / a.numViews, q = g * kBatchGroup + lane;
                    const uint32_t n = fv.count - g * kBatchGroup;  // positions of the group in the view (> 0)
                    const unsigned inView = n >= 32 ? 0xFFFFFFFFu : (1u << n) - 1u;
                    fetchMask = (fv.groupMasks ? fv.groupMasks[g] : 0xFFFFFFFFu) & inView;
                    if (fetchMask == 0) continue;
                    laneMeshlet = q < fv.count ? draw_order(q, fv.count, fv.orderStride) : 0u;
                }
                view = fetchView;
                m = __shfl_sync(0xFFFFFFFFu, laneMeshlet, __ffs(fetchMask) - 1);
                fetchMask &= fetchMask - 1;
                item = a.viewStart[view] + m;
            } else {
                // Single view: groups of fetchGroup positions (2 to 32), their cull bits tested at
                // once (one position per lane). The group grows while groups come back empty (a
                // sparse view fetches 32 positions per atomic) and shrinks while they hold more than
                // one visible meshlet (a dense view fetches about one visible meshlet at a time, so
                // the last work items spread evenly over the warps).
                if (fetchMask == 0) {
                    uint32_t b = 0;
                    if (lane == 0) b = (uint32_t)atomicAdd(twoPass && pass == 1 ? &a.s.control[7] : cursor,
                                                           (unsigned long long)fetchGroup);
                    const uint32_t base = __shfl_sync(0xFFFFFFFFu, b, 0);
                    if (base >= totalItems) {
                        if (pass == 0) {  // the large meshlets are all taken: the rest from position 0
                            pass = 1, fetchGroup = kDrawGroup;
                            continue;
                        }
                        break;
                    }
                    const uint32_t q = base + lane;
                    bool vis = false;
                    if (lane < fetchGroup && q < totalItems) {
                        laneMeshlet = draw_order(q, a.count, a.orderStride);
                        vis = a.cullBitmap == nullptr || ((a.cullBitmap[laneMeshlet >> 4] >> (laneMeshlet & 15)) & 1);
                        if (vis && twoPass) {  // bounding sphere radius against the clip w of its centre
                            const float4 sp = *(const float4*)(a.meshlets + (size_t)(a.meshletOffset + laneMeshlet) * kMeshletSize);
                            const float w = fmaf(sp.x, a.m[3], fmaf(sp.y, a.m[7], fmaf(sp.z, a.m[11], a.m[15])));
                            vis = (sp.w > kLargeMeshlet * w) == (pass == 0);
                        }
                    }
                    fetchMask = __ballot_sync(0xFFFFFFFFu, vis);
                    const int got = __popc(fetchMask);
                    fetchGroup = got == 0 ? min(fetchGroup * 2, 32u) : (got > 1 ? max(fetchGroup / 2, 2u) : fetchGroup);
                    if (fetchMask == 0) continue;
                }
                m = __shfl_sync(0xFFFFFFFFu, laneMeshlet, __ffs(fetchMask) - 1);
                fetchMask &= fetchMask - 1;
                item = m;
            }
        }
        if (multi && view != curView) {
            __syncwarp();
            ((uint32_t*)&S.view)[lane] = ((const uint32_t*)&a.views[view])[lane];
            __syncwarp();
            curView = view;
        }
        // (the fetch skipped meshlets whose cull bit is clear, Shading.cpp:282-289; the alpha list
        // holds visible ones only)

        const uint32_t g = vp.meshletOffset + m;
        const uint8_t* mp = a.meshlets + (size_t)g * kMeshletSize;
        // The record's positions (all 64 slots) and index bytes are loaded together with its header,
        // not after it: one memory round trip per meshlet instead of two.
        const uint8_t* sp = kShaded ? a.shaded + (size_t)m * kShadedSize : nullptr;
        const float* P = (const float*)(kShaded ? sp + kShadedPositions : mp + kOffPositions);
        const float px0 = P[lane], py0 = P[64 + lane], pz0 = P[128 + lane];
        const float px1 = P[32 + lane], py1 = P[96 + lane], pz1 = P[160 + lane];
        float pw0 = 1.0f, pw1 = 1.0f;
        if constexpr (kShaded) pw0 = P[192 + lane], pw1 = P[224 + lane];
        const uint32_t* I = (const uint32_t*)(kShaded ? sp + kShadedIndices : mp + kOffIndices);
        const uint32_t ix0 = I[lane], ix1 = I[32 + lane], ix2 = I[64 + lane];
        const uint32_t hdr = *(const uint32_t*)(kShaded ? sp : mp + kOffNumVertices);
        const uint32_t matId = *(const uint32_t*)(mp + kOffMaterialId);
        // record arrays hold 64 / 128; a shaded meshlet defines all 64 vertex slots
        const uint32_t nv = kShaded ? 64u : hdr & 0xFF, nt = min((kShaded ? hdr : hdr >> 8) & 0xFF, 128u);
        int cullMode = kCullFrontCCW;
        bool alphaTested = false;  // FragmentShaderId 1
        if (matId != 0xFFFFFFFFu && matId < a.numMaterials) {  // Shading.cpp:302-306
            const DevMaterial& mt = a.materials[matId];
            cullMode = mt.is_double_sided ? kCullNone : kCullFrontCCW;
            alphaTested = a.alphaAll ? material_alpha_tested_all(mt) : material_alpha_tested(mt);
            if constexpr (kShaded) alphaTested = alphaTested && ((hdr >> 16) & 0xFF) == 1;
        }
        if constexpr (kShaded) cullMode = (int)((hdr >> 8) & 0xFF);
        if (kPass == kPassOpaque && alphaTested) {  // drawn by the alpha pass
            if (lane == 0) a.s.alphaList[atomicAdd(&a.s.control[9], 1ull)] = item;
            continue;
        }
        if (nt == 0) continue;
        nProcessed += nt;

        // ShadeMeshlet vertex loop (Shading.cpp:295-298): 16-vertex chunks up to NumVertices; the
        // slots past them are zero.
        const uint32_t nvr = min((nv + 15) & ~15u, 64u);
        auto xform = [&](uint32_t v, float x, float y, float z, float w) {
            const float4 c = kShaded ? make_float4(x, y, z, w) : clip_position(x, y, z, v < nvr, vp);
            const Ndc n = project(c.x, c.y, c.z, c.w);
            S.ndc[v] = make_float4(n.x, n.y, n.z, n.rw);
            S.code[v] = (uint8_t)vertex_code(c, vp.bx, vp.by);
        };
        xform(lane, px0, py0, pz0, pw0);
        xform(32 + lane, px1, py1, pz1, pw1);
        S.idx[lane] = ix0, S.idx[32 + lane] = ix1, S.idx[64 + lane] = ix2;
        __syncwarp();

        // About half of a closed meshlet's triangles face away. The face test runs first for all of
        // them and compacts the rest into S.live (index p, and bit 7 for a triangle that needs
        // clipping), so the setup and binning below run on full 32-triangle steps. Each triangle
        // keeps its index p (its rank), so the keys do not change.
        uint32_t nLive = 0;
        for (uint32_t base = 0; base < nt; base += 32) {
            const uint32_t p = base + lane;
            const LaneTri lt = lane_triangle(S.ndc, S.code, idxBytes, p, p < nt);
            if (a.countClipped) nClipped += __popc(__ballot_sync(0xFFFFFFFFu, lt.nontriv)) * (lane == 0);
            const bool clip = lt.nontriv && a.clipMode;
            const bool live = clip || (lt.acc && front_facing(lt.n0, lt.n1, lt.n2, cullMode));
            const unsigned liveMask = __ballot_sync(0xFFFFFFFFu, live);
            if (live) S.live[nLive + __popc(liveMask & ((1u << lane) - 1u))] = (uint8_t)(p | (clip ? 0x80u : 0u));
            nLive += __popc(liveMask);
        }
        __syncwarp();

        for (uint32_t base = 0; base < nLive; base += 32) {
            const bool valid = base + lane < nLive;
            const uint32_t e = valid ? S.live[base + lane] : 0u;
            const uint32_t p = e & 127u;
            const bool accepted = valid && !(e & 0x80u), clipped = valid && (e & 0x80u);

            int myTiles = 0;     // tiles of this lane's small triangle (0 if none)
            bool overflow = false;
            if (accepted) {  // trivially accepted and front-facing (the first pass's face test)
                Setup t;
                uint32_t bbMin, bbMax;
                const uint32_t i0 = preload64_index(idxBytes[p]), i1 = preload64_index(idxBytes[128 + p]),
                               i2 = preload64_index(idxBytes[256 + p]);
                const float4 q0 = S.ndc[i0], q1 = S.ndc[i1], q2 = S.ndc[i2];
                if (tri_setup_ndc_facing({ q0.x, q0.y, q0.z, q0.w }, { q1.x, q1.y, q1.z, q1.w }, { q2.x, q2.y, q2.z, q2.w },
                                         vp.halfW, vp.halfH, t, bbMin, bbMax)) {
                    TriRec r;
                    float rcpArea;
                    const int32_t det = edge_setup(t, vp.halfW, vp.halfH, bbMin, bbMax, make_rank(g, p, 0, 0), r, &rcpArea);
                    nRaster++;
                    AlphaExt x;
                    if constexpr (kAlpha)
                        x = alpha_ext(t, rcpArea, texcoord_word(mp, idxBytes[p]), texcoord_word(mp, idxBytes[128 + p]),
                                      texcoord_word(mp, idxBytes[256 + p]), matId);
                    const int tilesX = ((bbMax & 0xFFFF) - (bbMin & 0xFFFF)) >> 2;
                    const int tilesY = ((bbMax >> 16) - (bbMin >> 16)) >> 2;
                    TinyBox tb;
                    if (kPass == kPassOpaque && det > 0 && tiny_box(t, vp.halfW, vp.halfH, bbMin, bbMax, tb)) {
                        shade_tiny(r, tb, vp.keys, vp.width);
                    } else if (tilesX * tilesY <= kSmallTiles) {
                        // tile index -> row by a multiply-shift (exact for tile < 16, tilesX <= 16), and
                        // whether the shading reads the keys before its atomics (keyReadTiles)
                        r.pad = (uint32_t)tilesX | (row_magic(tilesX) << 8) |
                                (a.keyReadTiles == 0 || (uint32_t)(tilesX * tilesY) <= a.keyReadTiles ? kPadReadKey : 0u);
                        tris[lane].v = r;
                        if constexpr (kAlpha) S.exts[lane].v = x;
                        myTiles = tilesX * tilesY;
                        S.zmax[lane] = triangle_depth_bound(t);
                    } else {
                        bool queued;
                        if constexpr (kAlpha) {
                            r.pad = view | kTriAlpha;
                            queued = enqueue_alpha(r, x, a, chunk);
                            if (!queued) S.exts[lane].v = x;
                        } else {
                            r.pad = view;
                            queued = enqueue_big(r, a, chunk);
                        }
                        if (!queued) {
                            tris[lane].v = r;
                            overflow = true;
                        }
                    }
                }
            }
            if (clipped) {  // rare: the clip-space vertices are transformed again
                const uint32_t i0 = preload64_index(idxBytes[p]), i1 = preload64_index(idxBytes[128 + p]),
                               i2 = preload64_index(idxBytes[256 + p]);
                const uint32_t partial = (S.code[i0] | S.code[i1] | S.code[i2]) & 0x3Fu;
                auto clip_vertex = [&](uint32_t v) {
                    const float4 c = kShaded ? make_float4(P[v], P[64 + v], P[128 + v], P[192 + v])
                                             : clip_position(P[v], P[64 + v], P[128 + v], v < nvr, vp);
                    return Vtx{ c.x, c.y, c.z, c.w };
                };
                clip_and_queue(clip_vertex(i0), clip_vertex(i1), clip_vertex(i2), partial, a, vp, view, chunk, cullMode, g, p,
                               nRaster, kAlpha ? matId : ~0u, mp, idxBytes);
            }
            __syncwarp();

            // Once half of the warps have run out of work items, the warps still busy are the
            // kernel's tail (in a sparse frame, a few visible meshlets are all of it). A packet whose
            // small triangles cover more than kPacketTiles tiles would then keep this warp busy for
            // many steps while the others idle: its triangles of more than kSpreadTiles tiles go to
            // the queue, whose chunks spread over all warps of the chunk stage. (Sparser budgets, or
            // a second level once 90 % of the warps are idle, cost the dense frame more than they
            // gain in the sparse one.)
            bool spread = false;
            if (__reduce_add_sync(0xFFFFFFFFu, (unsigned)myTiles) > kPacketTiles) {
                unsigned long long idle = 0;
                if (lane == 0) idle = *(volatile unsigned long long*)idleWarps;
                spread = __shfl_sync(0xFFFFFFFFu, idle, 0) * 2 >= numWarps;
            }
            if (spread && myTiles > kSpreadTiles) {
                TriRec r = tris[lane].v;
                bool queued;
                if constexpr (kAlpha) {
                    r.pad = view | kTriAlpha;
                    queued = enqueue_alpha(r, S.exts[lane].v, a, chunk);
                } else {
                    r.pad = view;
                    queued = enqueue_big(r, a, chunk);
                }
                if (queued) myTiles = 0;
            }

            // Small triangles: the warp walks the concatenated tile lists of all of them, two
            // tiles (32 pixels) per step, so tiny triangles share steps.
            int incl = myTiles;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            const int excl = incl - myTiles;
            const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            for (int k = 0; k < myTiles; k++) S.owner[excl + k] = (uint8_t)lane;
            __syncwarp();
            // 32 tiles at a time: lane j tests tile b + j of the list (empty or hidden tiles are
            // dropped), then the live ones are shaded two per step.
            const uint32_t tw = vp.width >> 2;
            for (int b = 0; b < total; b += 32) {
                const int t = b + lane;
                const uint32_t own = t < total ? S.owner[t] : 0u;
                const int ownerExcl = __shfl_sync(0xFFFFFFFFu, excl, own);
                bool live = false;
                uint32_t tpx = 0, tpy = 0, tmin = 0;
                if (t < total) {
                    const TriRec& r = tris[own].v;
                    const int tile = t - ownerExcl;
                    const int tilesX = r.pad & 0xFF, magic = (r.pad >> 8) & 0x1FF;
                    const int ty = (tile * magic) >> 8, tx = tile - ty * tilesX;
                    tpx = (r.bbMin & 0xFFFF) + tx * 4, tpy = (r.bbMin >> 16) + ty * 4;
                    live = tile_live(r, tpx, tpy, vp.tileMin, tw, &tmin, S.zmax[own]);
                }
                const unsigned liveMask = __ballot_sync(0xFFFFFFFFu, live);
                if constexpr (kAlpha) {
                    const DevMaterial& mt = a.materials[matId];
                    shade_live_tiles_alpha([&](uint32_t q) -> const TriRec& { return tris[q].v; },
                                           [&](uint32_t q) -> const AlphaExt& { return S.exts[q].v; }, own, mt.tex,
                                           mt.alpha_cutoff << 24, liveMask, tpx, tpy, tmin, vp.keys, vp.tileMin, vp.width,
                                           lane);
                } else if constexpr (kOver) {
                    shade_live_tiles_overdraw([&](uint32_t q) -> const TriRec& { return tris[q].v; }, own, liveMask, tpx, tpy,
                                              vp.keys, a.counts, vp.width, lane);
                } else {
                    shade_live_tiles([&](uint32_t q) -> const TriRec& { return tris[q].v; },
                                     [&](uint32_t q) { return (tris[q].v.pad & kPadReadKey) != 0u; }, own, liveMask, tpx, tpy,
                                     tmin, vp.keys, vp.tileMin, vp.width, lane);
                }
            }
            // Triangles the full queue turned away are rasterized here by the whole warp.
            unsigned ovMask = __ballot_sync(0xFFFFFFFFu, overflow);
            while (ovMask) {
                const int src = __ffs(ovMask) - 1;
                ovMask &= ovMask - 1;
                const TriRec r = tris[src].v;
                const uint32_t x0 = r.bbMin & 0xFFFF, y0 = r.bbMin >> 16;
                const int tx = (int)(((r.bbMax & 0xFFFF) - x0) >> 2), ty = (int)(((r.bbMax >> 16) - y0) >> 2);
                if constexpr (kAlpha) {
                    const DevMaterial& mt = a.materials[matId];
                    raster_region_alpha(&tris[src].v, &S.exts[src].v, mt.tex, mt.alpha_cutoff << 24, x0, y0, tx, ty, vp.keys,
                                        vp.tileMin, vp.width, lane);
                } else if constexpr (kOver) {
                    raster_region_overdraw(r, x0, y0, tx, ty, vp.keys, a.counts, vp.width, lane);
                } else {
                    raster_region(r, x0, y0, tx, ty, vp.keys, vp.tileMin, vp.width, lane, a.keyReadTiles);
                }
            }
            __syncwarp();
        }
        __syncwarp();
    }
    // perf counters (Rasterizer.h:366-370)
    nRaster = __reduce_add_sync(0xFFFFFFFFu, nRaster);
    if (lane == 0) {
        atomicAdd(idleWarps, 1ull);
        if (nProcessed) atomicAdd(&a.s.control[3], (unsigned long long)nProcessed);
        if (nRaster) atomicAdd(&a.s.control[4], (unsigned long long)nRaster);
        if (nClipped) atomicAdd(&a.s.control[5], (unsigned long long)nClipped);
    }
}

// Chunk stage: warps take runs of up to kChunkRun consecutive chunks (chunk_shape: w x h tiles) of the queued
// triangles from a global cursor (control[8], zeroed by the mesh stage), locate the run's first
// chunk by binary search over the queue's chunk prefix and walk the rest sequentially. A queued
// triangle carries its view in pad (batched draws) or belongs to the single view; an alpha-tested
// one (kTriAlpha) has its AlphaExt in the next slot, which owns no chunks and is never selected.
constexpr uint32_t kChunkRun = 8;
constexpr uint32_t kRunsPerWarp = 4;  // a shorter run when the queue holds fewer chunks than this many runs a warp

// A chunk of the alpha-tested triangle whose record (and AlphaExt after it) is at q, kept out of
// line so that the opaque chunks keep the kernel's registers.
__device__ __noinline__ void raster_chunk_alpha(const TriRec* q, const DevMaterial* materials, uint32_t x0, uint32_t y0,
                                                int tilesX, int tilesY, unsigned long long* keys, uint32_t* tileMin,
                                                uint32_t width, int lane) {
    const AlphaExt* xp = (const AlphaExt*)&q[1];
    const DevMaterial& mt = materials[xp->material & ~kTriAlpha];
    raster_region_alpha(q, xp, mt.tex, mt.alpha_cutoff << 24, x0, y0, tilesX, tilesY, keys, tileMin, width, lane,
                        kDiv16[tilesX]);
}

template <bool kOver>
__global__ void __launch_bounds__(256, 5) k_raster_big(const TriRec* __restrict__ big, const unsigned long long* __restrict__ bigBase,
                                                    unsigned long long* control, uint32_t capacity,
                                                    unsigned long long* keys, uint32_t* tileMin, uint32_t width,
                                                    const ViewParams* __restrict__ views, uint32_t chunk,
                                                    const DevMaterial* __restrict__ materials, unsigned long long* counts,
                                                    uint32_t readTiles) {
    const unsigned long long q = control[1];
    if (blockIdx.x == 0 && threadIdx.x == 0)  // the next draw's second cursor, alpha list and idle-warp counts
        control[7] = control[9] = control[10] = control[11] = control[12] = 0;
    const uint32_t n = (uint32_t)min((unsigned long long)capacity, q >> 40);
    if (n == 0) return;
    const int lane = threadIdx.x & 31;
    const TriRec& last = big[n - 1];
    const int lastTX = (int)(((last.bbMax & 0xFFFF) - (last.bbMin & 0xFFFF)) >> 2);
    const int lastTY = (int)(((last.bbMax >> 16) - (last.bbMin >> 16)) >> 2);
    const uint32_t cw = chunk & 0xFF, ch = chunk >> 8;
    const unsigned long long total = bigBase[n - 1] + (unsigned long long)((lastTX + cw - 1) / cw) * ((lastTY + ch - 1) / ch);
    // a sparse queue (few big triangles) is spread with shorter runs so that every warp gets work
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long run = max(1ull, min((unsigned long long)kChunkRun, total / (warps * kRunsPerWarp)));
    while (true) {
        unsigned long long w0 = 0;
        if (lane == 0) w0 = atomicAdd(&control[8], run);
        w0 = __shfl_sync(0xFFFFFFFFu, w0, 0);
        if (w0 >= total) break;
        const unsigned long long w1 = min(w0 + run, total);
        // largest slot with bigBase[slot] <= w0
        uint32_t slot = 0, hi = n - 1;
        while (slot < hi) {
            uint32_t mid = (slot + hi + 1) >> 1;
            if (bigBase[mid] <= w0) slot = mid; else hi = mid - 1;
        }
        TriRec r = big[slot];
        unsigned long long base = bigBase[slot];
        unsigned long long next = slot + 1 < n ? bigBase[slot + 1] : total;
        // the run's chunk of the triangle: one division where the run starts, then stepped
        auto chunks_x = [&](const TriRec& t) { return ((((t.bbMax & 0xFFFF) - (t.bbMin & 0xFFFF)) >> 2) + cw - 1) / cw; };
        uint32_t chunksX = chunks_x(r);
        uint32_t cy = (uint32_t)(w0 - base) / chunksX, cx = (uint32_t)(w0 - base) - cy * chunksX;
        for (unsigned long long w = w0; w < w1; w++) {
            if (w != w0) {
                if (w >= next) {  // the run crossed into the next triangle(s): its chunk 0
                    while (w >= next) {
                        slot++;
                        base = next;
                        next = slot + 1 < n ? bigBase[slot + 1] : total;
                        if (w < next) r = big[slot];
                    }
                    chunksX = chunks_x(r);
                    cx = 0, cy = 0;
                } else if (++cx == chunksX) {
                    cx = 0, cy++;
                }
            }
            unsigned long long* vkeys = keys;
            uint32_t* vtiles = tileMin;
            uint32_t vwidth = width;
            if (views) {
                const ViewParams& v = views[r.pad & ~kTriAlpha];
                vkeys = v.keys, vtiles = v.tileMin, vwidth = v.width;
            }
            const uint32_t minX = r.bbMin & 0xFFFF, minY = r.bbMin >> 16, maxX = r.bbMax & 0xFFFF, maxY = r.bbMax >> 16;
            const uint32_t x0 = minX + cx * (cw * 4), y0 = minY + cy * (ch * 4);
            const uint32_t x1 = min(x0 + cw * 4, maxX), y1 = min(y0 + ch * 4, maxY);
            // Empty and hidden tiles of the chunk are rejected inside raster_region.
            const int tilesX = (int)((x1 - x0) >> 2), tilesY = (int)((y1 - y0) >> 2);
            if constexpr (kOver) {
                raster_region_overdraw(r, x0, y0, tilesX, tilesY, vkeys, counts, vwidth, lane, kDiv16[tilesX]);
            } else if (r.pad & kTriAlpha) {
                raster_chunk_alpha(big + slot, materials, x0, y0, tilesX, tilesY, vkeys, vtiles, vwidth, lane);
            } else {
                raster_region(r, x0, y0, tilesX, tilesY, vkeys, vtiles, vwidth, lane, readTiles, kDiv16[tilesX]);
            }
        }
    }
}

// Keys from a depth layer (pre-existing depth: low word kKeyEmptyLow) and, when kept, each tile's
// depth bound as the minimum over its 16 pixels (a tile is 16 consecutive words; the grid stride
// is a multiple of 16, so a half-warp always covers one tile).
__global__ void k_init_keys(const uint32_t* __restrict__ depth, unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ tileMin, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t hi = float_order(__uint_as_float(depth[i]));
        keys[i] = ((unsigned long long)hi << 32) | kKeyEmptyLow;
        if (tileMin) {
            const unsigned half = 0xFFFFu << (threadIdx.x & 16);
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) hi = min(hi, __shfl_xor_sync(half, hi, o));
            if ((i & 15) == 0) tileMin[i >> 4] = hi;
        }
    }
}

__global__ void k_clear(uint32_t* __restrict__ l0, uint32_t* __restrict__ l1, unsigned long long* __restrict__ keys,
                        uint32_t* __restrict__ tileMin, uint32_t n, uint32_t color, uint32_t depthBits) {
    const uint32_t hi = float_order(__uint_as_float(depthBits));
    const unsigned long long key = ((unsigned long long)hi << 32) | kKeyEmptyLow;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) * 4; i < n; i += gridDim.x * blockDim.x * 4) {
        // n is a multiple of 16 (4x4 tiles), so the 16-byte vectors never straddle the end
        *(uint4*)&l0[i] = make_uint4(color, color, color, color);
        if (l1) *(uint4*)&l1[i] = make_uint4(depthBits, depthBits, depthBits, depthBits);
        if (keys) {
            *(ulonglong2*)&keys[i] = make_ulonglong2(key, key);
            *(ulonglong2*)&keys[i + 2] = make_ulonglong2(key, key);
        }
        if (tileMin && (i & 15) == 0) tileMin[i >> 4] = hi;
    }
}

__global__ void k_fill(uint32_t* __restrict__ dst, uint32_t n, uint32_t v) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = v;
}

__global__ void k_finalize(const unsigned long long* __restrict__ keys, uint32_t* __restrict__ l0,
                           uint32_t* __restrict__ l1, uint32_t n) {
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) * 2; i < n; i += gridDim.x * blockDim.x * 2) {
        const ulonglong2 k = *(const ulonglong2*)&keys[i];
        const unsigned long long kk[2] = { k.x, k.y };
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const uint32_t low = (uint32_t)kk[j];
            if (low == kKeyEmptyLow) continue;
            l1[i + j] = __float_as_uint(float_unorder((uint32_t)(kk[j] >> 32)));
            if (l0) l0[i + j] = rank_surface_id(0xFFFFFFFEu - low);  // l0 null: depth only
        }
    }
}

// OverdrawShader results: layer 0 += the counters (two saturating 16-bit halves, as the
// reference's _mm512_adds_epu16 accumulate them), layer 1 = the maximum depth where a sample
// raised it.
__global__ void k_finalize_overdraw(const unsigned long long* __restrict__ keys, const unsigned long long* __restrict__ counts,
                                    uint32_t* __restrict__ l0, uint32_t* __restrict__ l1, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long c = counts[i];
        const uint32_t old = l0[i];
        const unsigned long long lo = (old & 0xFFFFu) + (c & 0xFFFFFFFFull), hi = (old >> 16) + (c >> 32);
        l0[i] = (uint32_t)min(lo, 0xFFFFull) | ((uint32_t)min(hi, 0xFFFFull) << 16);
        const unsigned long long k = keys[i];
        if ((uint32_t)k != kKeyEmptyLow) l1[i] = __float_as_uint(float_unorder((uint32_t)(k >> 32)));
    }
}

// Framebuffer::GetPixels de-tiling (ImageHelpers.cpp:109-147) into a row-major device buffer.
__global__ void k_detile(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint32_t width, uint32_t height,
                         uint32_t stride) {
    const uint32_t n = width * height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t y = i / width, x = i - y * width;
        dst[(size_t)y * stride + x] = src[pixel_offset(x, y, width)];
    }
}

static int grid_for(uint32_t n, int perThread, int block) {
    long long g = ((long long)n / perThread + block - 1) / block;
    return (int)max(1ll, min(g, 152ll * 16));
}

uint32_t order_stride(uint32_t count) {
    if (count <= 2) return 1;
    uint32_t s = (uint32_t)((double)count * 0.6180339887498949) | 1u;
    while (std::gcd(s, count) != 1u) s += 2;
    return s % count;
}

// The dynamic shared memory limit of a mesh-stage pass is an attribute of the kernel in one
// device's context: it is raised per device (and only when a larger size is needed), under a lock
// because draws may come from several host threads.
static void raise_smem_limit(int pass, const void* kernel, size_t bytes) {
    static std::mutex mu;
    static size_t setSize[64][5] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (bytes <= setSize[dev][pass]) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
        setSize[dev][pass] = bytes;
}

void launch_draw(const DrawArgs& args, cudaStream_t st, int numSMs) {
    DrawArgs a = args;
    if (!a.views) {
        a.orderStride = order_stride(a.count);
        // Single-view draws skip the key read for triangles above 4 tiles (1080p, 100k meshlets:
        // 1.378 -> 1.320 ms); batched draws of many small views lose by it (64 views 5.93 -> 6.34
        // ms), because their tiles are mostly covered partially, and keep every read.
        a.keyReadTiles = 4;
    }
    const uint32_t warps = a.warpsPerBlock ? a.warpsPerBlock : kWarpsPerBlock;
    const size_t smem = warps * sizeof(WarpSmem), smemAlpha = warps * sizeof(WarpSmemAlpha);
    if (smem > 48 * 1024)
        raise_smem_limit(a.counts ? kPassOverdraw : kPassOpaque,
                         a.counts ? (const void*)k_draw_meshlets<kPassOverdraw> : (const void*)k_draw_meshlets<kPassOpaque>,
                         smem);
    if (a.s.alphaList && smemAlpha > 48 * 1024) raise_smem_limit(kPassAlpha, (const void*)k_draw_meshlets<kPassAlpha>, smemAlpha);
    const uint32_t chunk = chunk_shape(a);
    const int grid = numSMs * (32 / warps);  // 64 registers a thread leave room for 32 resident warps per SM
    if (a.counts) {  // OverdrawShader: one pass, every meshlet
        {
            LaunchScope ls("k_draw_meshlets_overdraw", st);
            k_draw_meshlets<kPassOverdraw><<<grid, warps * 32, smem, st>>>(a);
        }
        LaunchScope ls("k_raster_big_overdraw", st);
        k_raster_big<true><<<numSMs * 8, 256, 0, st>>>(a.s.big, a.s.bigBase, a.s.control, a.s.bigCapacity, a.keys, nullptr,
                                                       a.width, a.views, chunk, a.materials, a.counts, 0u);
        return;
    }
    if (a.shaded) {  // meshlets shaded by a user mesh shader
        if (smem > 48 * 1024) raise_smem_limit(3, (const void*)k_draw_meshlets<kPassOpaque, true>, smem);
        if (a.s.alphaList && smemAlpha > 48 * 1024) raise_smem_limit(4, (const void*)k_draw_meshlets<kPassAlpha, true>, smemAlpha);
        {
            LaunchScope ls("k_draw_meshlets_shaded", st);
            k_draw_meshlets<kPassOpaque, true><<<grid, warps * 32, smem, st>>>(a);
        }
        if (a.s.alphaList) {
            LaunchScope ls("k_draw_meshlets_shaded_alpha", st);
            k_draw_meshlets<kPassAlpha, true><<<grid, warps * 32, smemAlpha, st>>>(a);
        }
    } else {
        {
            LaunchScope ls("k_draw_meshlets", st);
            k_draw_meshlets<kPassOpaque><<<grid, warps * 32, smem, st>>>(a);
        }
        if (a.s.alphaList) {  // the scene has alpha-tested materials
            LaunchScope ls("k_draw_meshlets_alpha", st);
            k_draw_meshlets<kPassAlpha><<<grid, warps * 32, smemAlpha, st>>>(a);
        }
    }
    {
        LaunchScope ls("k_raster_big", st);
        k_raster_big<false><<<numSMs * 8, 256, 0, st>>>(a.s.big, a.s.bigBase, a.s.control, a.s.bigCapacity, a.keys,
                                                        a.tileMin, a.width, a.views, chunk, a.materials, nullptr,
                                                        a.keyReadTiles);
    }
}

void launch_init_keys(const uint32_t* depthLayer, unsigned long long* keys, uint32_t* tileMin, uint32_t n, cudaStream_t st) {
    LaunchScope ls("k_init_keys", st);
    k_init_keys<<<grid_for(n, 1, 256), 256, 0, st>>>(depthLayer, keys, tileMin, n);
}

void launch_clear(uint32_t* l0, uint32_t* l1, unsigned long long* keys, uint32_t* tileMin, uint32_t n, uint32_t color,
                  uint32_t depthBits, cudaStream_t st) {
    LaunchScope ls("k_clear", st);
    k_clear<<<grid_for(n, 4, 256), 256, 0, st>>>(l0, l1, keys, tileMin, n, color, depthBits);
}

void launch_fill(uint32_t* dst, uint32_t n, uint32_t value, cudaStream_t st) {
    LaunchScope ls("k_fill", st);
    k_fill<<<grid_for(n, 1, 256), 256, 0, st>>>(dst, n, value);
}

void launch_finalize(const unsigned long long* keys, uint32_t* l0, uint32_t* l1, uint32_t n, cudaStream_t st) {
    LaunchScope ls("k_finalize", st);
    k_finalize<<<grid_for(n, 2, 256), 256, 0, st>>>(keys, l0, l1, n);
}

void launch_finalize_overdraw(const unsigned long long* keys, const unsigned long long* counts, uint32_t* l0, uint32_t* l1,
                              uint32_t n, cudaStream_t st) {
    LaunchScope ls("k_finalize_overdraw", st);
    k_finalize_overdraw<<<grid_for(n, 1, 256), 256, 0, st>>>(keys, counts, l0, l1, n);
}

void launch_detile(const uint32_t* src, uint32_t* dst, uint32_t width, uint32_t height, uint32_t stride, cudaStream_t st) {
    LaunchScope ls("k_detile", st);
    k_detile<<<grid_for(width * height, 1, 256), 256, 0, st>>>(src, dst, width, height, stride);
}

}  // namespace swr
