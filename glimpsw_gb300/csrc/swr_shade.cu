// Meshlet culling (ShadingContext::CullMeshlets), the Hi-Z depth pyramid (texutil::DownsampleDepth)
// and the vis-buffer resolve (ShadingContext::Resolve) for sm_103a.
//
// The translation unit is compiled with -fmad=false, so every float expression below is evaluated
// in source order with one rounding per operation, as the reference's C++ is written; fmaf()
// stands for the reference's explicit simd::fma. simd::approx_rcp / approx_rsqrt / approx_sqrt
// (the AVX-512 instructions VRCP14PS and VRSQRT14PS) are reproduced bit for bit by the integer
// segment tables of include/swr/approx14.h.
//
// Resolve layout: a half-warp shades one 4x4 tile (lane = pixel), so the reference's tile-wide
// decisions (`any(mipLevel > 0)` filter choice, normal-map enable, light skipping, sky branch)
// become ballots over the half-warp, evaluated over all 16 pixels like the 16 AVX-512 lanes.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swr/approx14.h"
#include "../../include/swr/hostmath.h"
#include "swr_device.cuh"
#include "swr_internal.h"
#include "swr_neural.h"
#include "swr_sample.cuh"
#include "swr_surface.cuh"

namespace swr {
namespace {


// =========================================================================== culling
struct CullArgs {
    const uint8_t* meshlets;
    uint32_t first, count;
    uint16_t* bitmap;
    unsigned int* visibleCount;
    float planes[5][4];
    float objectToPrevView[16];
    float objectToWorldScale;
    float projFactors[3];
    float frameW, frameH;
    const uint32_t* depthData;  // R32f Hi-Z storage or null
    uint32_t mipOffsets[16];
    uint32_t mipLevels, rowShift;
    // backface-cone culling (cone_culled): camera centre in object space, materials
    uint32_t cone;
    float eye[3];
    const DevMaterial* materials;
    uint32_t numMaterials;
};

// ShadingContext::CullMeshlets (Shading.cpp:775-869) + ProjectSphere (264-279), one meshlet per
// thread; a warp's ballot gives two of the reference's 16-bit masks. With a.cone, meshlets that
// pass the frustum test and face away as a whole (cone_culled) are dropped before the Hi-Z test.
__global__ void __launch_bounds__(256) k_cull(CullArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool visible = i < a.count;
    if (visible) {
        const float* b = (const float*)(a.meshlets + (size_t)(a.first + i) * kMeshletSize);  // BoundCenter, BoundRadius
        const float4 s = *(const float4*)b;
        const F3 c = { s.x, s.y, s.z };
        const float r = s.w;
        for (int k = 0; k < 5; k++) {
            float dist = fmaf(c.x, a.planes[k][0], fmaf(c.y, a.planes[k][1], c.z * a.planes[k][2])) + a.planes[k][3];
            visible = visible && (dist > -r);
        }
        if (a.cone && visible)
            visible = !cone_culled((const uint8_t*)b, a.eye[0], a.eye[1], a.eye[2], a.materials, a.numMaterials);
        if (a.depthData != nullptr && visible) {
            float vw;
            F3 vs = xform4(a.objectToPrevView, c, vw);
            const float rvs = r * a.objectToWorldScale;
            // ProjectSphere
            float cx = vs.x, cy = vs.y, cz = vs.z * -1.0f;
            bool projMask = cz >= rvs + a.projFactors[0];
            if (projMask) {
                float crx = cx * rvs, cry = cy * rvs, crz = cz * rvs;
                float vx = approx_sqrt(cx * cx + cz * cz - rvs * rvs);
                float vy = approx_sqrt(cy * cy + cz * cz - rvs * rvs);
                float sx = a.projFactors[1] * 0.5f, sy = a.projFactors[2] * 0.5f;
                float bb0 = (vx * cx - crz) * approx_rcp(vx * cz + crx) * sx + 0.5f;
                float bb1 = (vy * cy + crz) * approx_rcp(vy * cz - cry) * sy + 0.5f;
                float bb2 = (vx * cx + crz) * approx_rcp(vx * cz - crx) * sx + 0.5f;
                float bb3 = (vy * cy - crz) * approx_rcp(vy * cz + cry) * sy + 0.5f;
                float bw = (bb2 - bb0) * a.frameW, bh = (bb3 - bb1) * a.frameH;
                int32_t mip = ilog2_x86(vmax(bw, bh));
                mip = min(max(mip, 1), (int32_t)a.mipLevels - 1);
                int32_t x0 = max(trunc2i(bb0 * a.frameW), 0) >> mip;
                int32_t y0 = max(trunc2i(bb1 * a.frameH), 0) >> mip;
                int32_t x1 = min(trunc2i(bb2 * a.frameW), (int32_t)a.frameW - 1) >> mip;
                int32_t y1 = min(trunc2i(bb3 * a.frameH), (int32_t)a.frameH - 1) >> mip;
                float depthSphere = a.projFactors[0] / (-vs.z - rvs);
                float depthVisible = FLT_MAX;
                const uint32_t level = (uint32_t)(mip - 1);
                const int32_t stride = (int32_t)a.rowShift - (int32_t)level;
                const uint32_t* base = a.depthData + a.mipOffsets[level & 15];
                for (int32_t y = y0; y <= y1; y++)
                    for (int32_t x = x0; x <= x1; x++)
                        depthVisible = vmin(depthVisible, __uint_as_float(base[texel_offset(x, y, stride)]));
                visible = depthSphere > depthVisible;
            }
        }
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, visible);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t w0 = i & ~31u;
    if (lane == 0 && w0 < a.count) {
        a.bitmap[w0 / 16] = (uint16_t)(m & 0xFFFF);
        if (w0 + 16 < a.count) a.bitmap[w0 / 16 + 1] = (uint16_t)(m >> 16);
        if (a.visibleCount) atomicAdd(a.visibleCount, (unsigned)__popc(m));
    }
}

// =========================================================================== Hi-Z
// texutil::DownsampleDepth (ImageHelpers.cpp:150-247). Mip m texels hold the min of the frame
// depths they cover (FLT_MAX where they cover none). The reference writes mip m (m <= root-4) in
// 8x8-texel blocks of 2^(m+4)-pixel regions whose origin lies inside the frame, and mip root-3
// as one 4x4 tile. Two launches write exactly those texels: k_hiz_local makes levels 0-3 of one
// 128x128-pixel region per block in shared memory, k_hiz_tail the levels above in one block,
// level by level. A texel is the min of its four children in the order vmin(vmin(00, 01),
// vmin(10, 11)); a child whose origin lies outside the frame counts as FLT_MAX.
struct HizOffsets { uint32_t off[16]; };  // MipOffsets of the levels written (0 for levels the texture lacks)
constexpr uint32_t kHizRegion = 128;      // pixels per side of a k_hiz_local block (level 3's 8x8 texels)

__global__ void __launch_bounds__(256) k_hiz_local(const float* __restrict__ depth, uint32_t fbW, uint32_t fbH,
                                                   uint32_t* __restrict__ tex, HizOffsets offs, int32_t rowShift,
                                                   uint32_t nLocal) {
    __shared__ float s0[64 * 64], s1[32 * 32], s2[16 * 16], s3[8 * 8];
#pragma unroll
    for (uint32_t m = 0; m < 4; m++) {
        if (m >= nLocal) break;
        float* dst = m == 0 ? s0 : (m == 1 ? s1 : (m == 2 ? s2 : s3));
        const float* src = m == 1 ? s0 : (m == 2 ? s1 : s2);
        const uint32_t side = 64u >> m, gx0 = blockIdx.x * side, gy0 = blockIdx.y * side;
        for (uint32_t i = threadIdx.x; i < side * side; i += blockDim.x) {
            const uint32_t lx = i % side, ly = i / side, gx = gx0 + lx, gy = gy0 + ly;
            const uint32_t x = gx * 2, y = gy * 2;
            float v;
            if (m == 0) {
                auto d = [&](uint32_t px, uint32_t py) -> float {
                    return (px < fbW && py < fbH) ? depth[pixel_offset(px, py, fbW)] : FLT_MAX;
                };
                v = vmin(vmin(d(x, y), d(x, y + 1)), vmin(d(x + 1, y), d(x + 1, y + 1)));
            } else {
                // children at mip m-1 cover 2^m pixels; one whose origin is outside the frame covers none
                auto c = [&](uint32_t cx, uint32_t cy) -> float {
                    if ((cx << m) >= fbW || (cy << m) >= fbH) return FLT_MAX;
                    return src[(cy - gy0 * 2) * (side * 2) + (cx - gx0 * 2)];
                };
                v = vmin(vmin(c(x, y), c(x, y + 1)), vmin(c(x + 1, y), c(x + 1, y + 1)));
            }
            dst[ly * side + lx] = v;
            if (((gx & ~7u) << (m + 1)) < fbW && ((gy & ~7u) << (m + 1)) < fbH)  // the 8x8 block's region is in the frame
                tex[offs.off[m] + texel_offset(gx, gy, rowShift - (int32_t)m)] = __float_as_uint(v);
        }
        __syncthreads();
    }
}

// The levels above k_hiz_local's (first = 4 .. last = root-3) in one block, out of shared memory:
// the texels of level first-1 whose origin lies in the frame are read once (the others count as
// FLT_MAX), then each level is computed from the previous one in shared memory and written out.
// lvl[k] holds level first-1+k as a (fbW >> (first+k) rounded up) x (fbH >> ...) array.
__host__ __device__ inline uint32_t hiz_extent(uint32_t n, uint32_t level) { return (n + (2u << level) - 1) >> (level + 1); }

__global__ void __launch_bounds__(1024) k_hiz_tail(uint32_t fbW, uint32_t fbH, uint32_t* tex, HizOffsets offs,
                                                   int32_t rowShift, uint32_t first, uint32_t last, uint32_t root) {
    extern __shared__ float lvl[];
    {  // level first-1 from the texture
        const uint32_t m = first - 1, w = hiz_extent(fbW, m), h = hiz_extent(fbH, m);
        const int32_t stride = rowShift - (int32_t)m;
        for (uint32_t t = threadIdx.x; t < w * h; t += blockDim.x)
            lvl[t] = __uint_as_float(tex[offs.off[m] + texel_offset(t % w, t / w, stride)]);
    }
    __syncthreads();
    float* src = lvl;
    for (uint32_t m = first; m <= last; m++) {
        const uint32_t sw = hiz_extent(fbW, m - 1), sh = hiz_extent(fbH, m - 1);
        const uint32_t dw = hiz_extent(fbW, m), dh = hiz_extent(fbH, m);
        float* dst = src + sw * sh;
        uint32_t regionsX = 1, regionsY = 1, blockTexels = 16;
        if (m + 4 <= root) {
            const uint32_t region = 1u << (m + 4);
            regionsX = (fbW + region - 1) / region, regionsY = (fbH + region - 1) / region, blockTexels = 64;
        }
        const uint32_t bs = blockTexels == 64 ? 8 : 4, n = regionsX * regionsY * blockTexels;
        for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) {
            const uint32_t blk = t / blockTexels, within = t - blk * blockTexels;
            const uint32_t by = blk / regionsX, bx = blk - by * regionsX;
            const uint32_t tx = bx * bs + within % bs, ty = by * bs + within / bs;
            // children at mip m-1 cover 2^m pixels; one whose origin is outside the frame covers none
            auto c = [&](uint32_t x, uint32_t y) -> float { return (x < sw && y < sh) ? src[y * sw + x] : FLT_MAX; };
            const uint32_t x = tx * 2, y = ty * 2;
            const float v = vmin(vmin(c(x, y), c(x, y + 1)), vmin(c(x + 1, y), c(x + 1, y + 1)));
            tex[offs.off[m] + texel_offset(tx, ty, rowShift - (int32_t)m)] = __float_as_uint(v);
            if (tx < dw && ty < dh) dst[ty * dw + tx] = v;
        }
        __syncthreads();
        src = dst;
    }
}

// =========================================================================== resolve
struct ResolveArgs {
    const uint8_t* meshlets;
    uint32_t numMeshlets;
    const DevMaterial* materials;
    uint32_t numMaterials;
    uint32_t* color;        // layer 0 (surface ids in, RGBA8 out)
    const float* depth;     // layer 1
    uint32_t width, height;
    float objectToClip[16];
    float objectToWorld[9];
    float invProj[16];
    float viewPos[3];
    float exposure;
    const swr_light* lights;  // device copy
    uint32_t numLights;
    DevTexture sky;
    int hasSky;
    uint32_t debugLayer;    // SWR_DEBUG_* of the debug mode
};

// Neural resolve: the emit pass records, per pixel, the texels of the levels the model decodes
// (4 slots: the nearest texel, or the bilinear quad's 00 10 01 11 texels; ~0 = none) and counts
// them per material; the shade pass reads the decoded texels from the same slots. Within a 4x4
// tile, a slot whose texel a lower lane's slot of the same quad position already requests holds
// kReqRedirect | that slot instead and is not decoded: a magnified texture gives most of a tile's
// pixels the same quad.
enum { kResolvePlain = 0, kResolveEmit = 1, kResolveNeural = 2, kResolveDebug = 3 };
constexpr unsigned long long kReqRedirect = 1ull << 63;  // | slot; ~0 (none) has the bit too
struct NeuralResolve {
    const DevTexture* tex;             // model textures (data == nullptr: not decoded)
    uint32_t numMaterials, decodedLevels;  // texture levels below decodedLevels are decoded
    unsigned long long* pixelReq;      // [pixel * 4 + k] material<<32 | level<<28 | ty<<14 | tx
    uint32_t* counts;                  // [material]
    const uint2* decoded;              // [pixel * 4 + k] layer-0 RGBA8, layer-1 RGBA8
    uint4* surf;                       // [pixel * 2 + 0..1] the emit pass's surface record (kSurf*)
};
// The emit pass's per-pixel surface record, which spares the second pass the reconstruction of a
// tile whose pixels all have it (kSurfFast): word 0-1 barycentrics b1, b2; 2-4 the vertices'
// normal/tangent words; 5-6 the decoded quad's filter fractions; 7 flags.
enum : uint32_t {
    kSurfFast = 1u,        // sampled from decoded texels, or untextured (albedo and NMR 0)
    kSurfDecoded = 2u,     // a decoded material sample: fetch it
    kSurfNearest = 4u, kSurfInX = 8u, kSurfInY = 16u, kSurfTwoLayers = 32u,
    kSurfHand = 1u << 31,  // the bitangent's sign bit
};

__device__ __forceinline__ uint32_t sat_u8(int32_t v) { return (uint32_t)min(max(min(max(v, -32768), 32767), 0), 255); }
__device__ __forceinline__ float unpack_f11(uint32_t x) { x <<= 17; return __uint_as_float((x & 0x0FFE0000u) + 0x38000000u); }
__device__ __forceinline__ float unpack_f10(uint32_t x) { x <<= 18; return __uint_as_float((x & 0x0FFC0000u) + 0x38000000u); }
__device__ __forceinline__ F3 unpack_r11(uint32_t p) { return { unpack_f11(p >> 21), unpack_f11(p >> 10), unpack_f10(p) }; }

// SampleOctLevel<EnvSampler>(dir, 1) on an R11G11B10 map (Texture.h:467-480; level 1 has no fraction).
__device__ F3 sample_env(const DevTexture& t, F3 dir) {
    float w = approx_rcp(fabsf(dir.x) + fabsf(dir.y) + fabsf(dir.z));
    float tt = vmax(-dir.z * w, 0.0f);
    float u = fmaf(dir.x, w, mulsign(tt, dir.x)) * 0.5f + 0.5f;
    float v = fmaf(dir.y, w, mulsign(tt, dir.y)) * 0.5f + 0.5f;
    int32_t m = min(max(1, 0), (int32_t)t.mip_levels - 1);
    int32_t x = min(max(round2i(u * t.scale_lerp_u), 0), t.mask_lerp_u);
    int32_t y = min(max(round2i(v * t.scale_lerp_v), 0), t.mask_lerp_v);
    int32_t stride = (int32_t)t.row_shift - m;
    x >>= m, y >>= m;
    const uint32_t* base = t.data + t.mip_offsets[m & 15];
    int32_t xf = max(x - 127, 0), yf = max(y - 127, 0);
    int32_t tx = xf >> 8, ty = yf >> 8;
    bool inX = ((tx + 1) << m) < (int32_t)t.width, inY = ((ty + 1) << m) < (int32_t)t.height;
    uint32_t i00 = texel_offset(tx, ty, stride), i01 = texel_offset(tx, ty + (inY ? 1 : 0), stride);
    F3 c00 = unpack_r11(base[i00]), c10 = unpack_r11(base[i00 + 8]), c01 = unpack_r11(base[i01]), c11 = unpack_r11(base[i01 + 8]);
    const float fs = 1.0f / 256;
    float fx = (float)(xf & 255) * fs, fy = (float)(yf & 255) * fs;
    if (!inX) fx = 0;
    F3 ra = { c00.x + (c10.x - c00.x) * fx, c00.y + (c10.y - c00.y) * fx, c00.z + (c10.z - c00.z) * fx };
    F3 rb = { c01.x + (c11.x - c01.x) * fx, c01.y + (c11.y - c01.y) * fx, c01.z + (c11.z - c01.z) * fx };
    return { ra.x + (rb.x - ra.x) * fy, ra.y + (rb.y - ra.y) * fy, ra.z + (rb.z - ra.z) * fy };
}

// Turbo colormap (Google Research 2019, polynomial fit; Shading.cpp:249-260) in the reference's
// Horner order.
__device__ __forceinline__ F3 colormap_turbo(float x) {
    constexpr float c[18] = {
        0.13572138f, 4.61539260f,  -42.66032258f, 132.13108234f, -152.94239396f, 59.28637943f,
        0.09140261f, 2.19418839f,  4.84296658f,   -14.18503333f, 4.27729857f,    2.82956604f,
        0.10667330f, 12.64194608f, -60.58204836f, 110.36276771f, -89.90310912f,  27.34824973f,
    };
    auto poly = [&](int k) { return x * (x * (x * (x * (x * c[k + 5] + c[k + 4]) + c[k + 3]) + c[k + 2]) + c[k + 1]) + c[k]; };
    return { poly(0), poly(6), poly(12) };
}

// RGBA8u::Unpack of the RGB bytes (Texture.h:28-36).
__device__ __forceinline__ F3 unpack_rgb8(uint32_t p) {
    const float s = 1.0f / 255;
    return { (float)(p & 255) * s, (float)((p >> 8) & 255) * s, (float)((p >> 16) & 255) * s };
}

// ResolveDebug's colour of one non-sky pixel (Shading.cpp:748-768) as RGBA8u::Pack({c, 1}); data is
// the pixel's layer-0 word, the surface values are read for layers 1-3 only.
__device__ __forceinline__ uint32_t debug_pixel(uint32_t layer, uint32_t data, uint32_t albedo, F3 N, float metallic,
                                                float roughness) {
    F3 c = { 0.0f, 0.0f, 0.0f };
    if (layer == SWR_DEBUG_BASE_COLOR) c = unpack_rgb8(albedo);
    else if (layer == SWR_DEBUG_NORMALS) c = { N.x * 0.5f + 0.5f, N.y * 0.5f + 0.5f, N.z * 0.5f + 0.5f };
    else if (layer == SWR_DEBUG_METALLIC_ROUGHNESS) c = { metallic, roughness, 0.0f };
    else if (layer == SWR_DEBUG_MESHLET_ID) c = unpack_rgb8((data / 128u) * 123456789u);
    else if (layer == SWR_DEBUG_TRIANGLE_ID) c = unpack_rgb8(data * 123456789u);
    else if (layer == SWR_DEBUG_OVERDRAW_PIXEL) c = colormap_turbo((float)(data >> 16) / 30.0f);
    else if (layer == SWR_DEBUG_OVERDRAW_QUAD) c = colormap_turbo(((float)(data >> 16) + (float)(data & 0xFFFF) * 0.5f) / 30.0f);
    return sat_u8(round2i(c.x * 255.0f)) | (sat_u8(round2i(c.y * 255.0f)) << 8) | (sat_u8(round2i(c.z * 255.0f)) << 16) |
           (255u << 24);
}

template <int kMode>
__global__ void __launch_bounds__(256) k_resolve(ResolveArgs a, NeuralResolve nr) {
    const uint32_t lane = threadIdx.x & 31, l = lane & 15, half = lane >> 4;
    const unsigned hm = 0xFFFFu << (16 * half);
    const uint32_t tilesX = a.width >> 2, numTiles = tilesX * (a.height >> 2);
    const uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    if (tile >= numTiles) return;  // whole half-warps leave together
    const uint32_t ty = tile / tilesX, tx = tile - ty * tilesX;
    const uint32_t x0 = tx * 4, y0 = ty * 4;
    const uint32_t px = x0 + (l & 3), py = y0 + (l >> 2);
    const uint32_t off = pixel_offset(x0, y0, a.width) + l;

    const uint32_t id = a.color[off];
    const float d = a.depth[off];
    const bool isSky = d <= 0.0f;
    const float fpx = (float)(int32_t)px, fpy = (float)(int32_t)py;
    float qw;
    F3 q = xform4(a.invProj, { fpx, fpy, isSky ? 1.0f : d }, qw);
    const float rw = 1.0f / qw;
    const F3 world = { q.x * rw, q.y * rw, q.z * rw };
    const float W = (float)a.width, H = (float)a.height;
    const float scaleU = 2.0f / W, scaleV = 2.0f / H;
    const float su = fpx * scaleU + (0.5f * scaleU - 1.0f), sv = fpy * scaleV + (0.5f * scaleV - 1.0f);
    const unsigned skyBits = (__ballot_sync(hm, isSky) >> (16 * half)) & 0xFFFF;

    F3 color = { 0.f, 0.f, 0.f };
    unsigned long long req[4] = { ~0ull, ~0ull, ~0ull, ~0ull };
    // ResolveDebug: sky pixels get a checkerboard of 4x4 tiles; layers other than the surface
    // ones need no surface
    const uint32_t background = ((x0 ^ y0) & 4) ? 0xFFA0A0A0u : 0xFFFFFFFFu;
    if constexpr (kMode == kResolveDebug) {
        if (skyBits == 0xFFFF || a.debugLayer - 1u >= 3u) {
            a.color[off] = isSky ? background : debug_pixel(a.debugLayer, id, 0u, F3{}, 0.0f, 0.0f);
            return;
        }
    }
    if constexpr (kMode == kResolveEmit) {
        if (skyBits == 0xFFFF) {
            uint4* dst = (uint4*)(nr.pixelReq + (size_t)off * 4);
            dst[0] = dst[1] = make_uint4(~0u, ~0u, ~0u, ~0u);
            return;
        }
    }
    if (skyBits != 0xFFFF) {
        uint32_t ntg[3] = {}, hand = 0, albedo = 0, nmr = 0;
        float b[3];
        bool fast = false;  // the neural pass found the emit pass's records for the whole tile
        if constexpr (kMode == kResolveNeural) {
            uint4 s0 = make_uint4(0u, 0u, 0u, 0u), s1 = make_uint4(0u, 0u, 0u, 0u);
            if (!isSky) s0 = nr.surf[(size_t)off * 2], s1 = nr.surf[(size_t)off * 2 + 1];
            fast = (__ballot_sync(hm, isSky || (s1.w & kSurfFast)) & hm) == hm;
            if (fast) {
                const float nan = __int_as_float(0x7FFFFFFF);  // what the full path gives sky pixels
                b[1] = isSky ? nan : __uint_as_float(s0.x);
                b[2] = isSky ? nan : __uint_as_float(s0.y);
                b[0] = 1 - b[1] - b[2];
                ntg[0] = s0.z, ntg[1] = s0.w, ntg[2] = s1.x;
                hand = s1.w & kSurfHand;
                if (!isSky && (s1.w & kSurfDecoded)) {
                    const ulonglong2* rq = (const ulonglong2*)(nr.pixelReq + (size_t)off * 4);
                    const ulonglong2 r01 = rq[0], r23 = rq[1];
                    auto at = [&](unsigned long long r, uint32_t k) {
                        const size_t slot = (r != ~0ull && (r & kReqRedirect)) ? (size_t)(uint32_t)r : (size_t)off * 4 + k;
                        return nr.decoded[slot];
                    };
                    const bool inX = s1.w & kSurfInX, inY = s1.w & kSurfInY;
                    const uint2 d00 = at(r01.x, 0);
                    uint2 r0 = d00;
                    if (!(s1.w & kSurfNearest)) {
                        const uint2 d10 = inX ? at(r01.y, 1) : d00, d01 = inY ? at(r23.x, 2) : d00;
                        const uint2 d11 = inY ? (inX ? at(r23.y, 3) : d01) : d10;
                        r0.x = filter_rgba8(d00.x, d10.x, d01.x, d11.x, s1.y, s1.z);
                        r0.y = filter_rgba8(d00.y, d10.y, d01.y, d11.y, s1.y, s1.z);
                    }
                    albedo = r0.x;
                    if (s1.w & kSurfTwoLayers) nmr = r0.y;
                }
            }
        }
        if (!fast) {
        // ---- ResolveSurface (Shading.cpp:471-579): waterfall over the tile's surface ids
        F3 pos[3] = {};
        uint32_t tc[3] = {}, matId = 0;
        uint32_t sflags = kSurfFast, sfx = 0, sfy = 0;  // the emit pass's record of this pixel
        unsigned pending = (~skyBits) & 0xFFFF;
        while (pending) {
            const int src = __ffs(pending) - 1;
            const uint32_t sid = __shfl_sync(hm, id, src + 16 * half);
            const unsigned iter = (__ballot_sync(hm, id == sid) >> (16 * half)) & 0xFFFF;
            pending &= ~iter;
            const uint32_t mId = sid / 128, tri = sid % 128;
            if (((iter >> l) & 1) && mId < a.numMeshlets) {
                const uint8_t* mp = a.meshlets + (size_t)mId * kMeshletSize;
                const float* P = (const float*)(mp + kOffPositions);
                const uint32_t* TC = (const uint32_t*)(mp + kOffTexCoords);
                const uint32_t* NT = (const uint32_t*)(mp + kOffNormalTangents);
                const uint8_t* I = mp + kOffIndices;
                const unsigned long long handBits = *(const unsigned long long*)(mp + kOffHandedness);
#pragma unroll
                for (int vi = 0; vi < 3; vi++) {
                    const uint32_t idx = I[vi * 128 + tri] & 63;
                    pos[vi] = { P[idx], P[64 + idx], P[128 + idx] };
                    tc[vi] = TC[idx];
                    ntg[vi] = NT[idx];
                    if (vi == 0 && ((handBits >> idx) & 1)) hand = 1u << 31;
                }
                matId = *(const uint32_t*)(mp + kOffMaterialId);
            }
        }
        // IntersectTriangle (Shading.cpp:417-464)
        float w0, w1, w2;
        F3 c0 = xform4(a.objectToClip, pos[0], w0), c1 = xform4(a.objectToClip, pos[1], w1), c2 = xform4(a.objectToClip, pos[2], w2);
        const float iw0 = 1.0f / w0, iw1 = 1.0f / w1, iw2 = 1.0f / w2;
        const float p0x = c0.x * iw0, p0y = c0.y * iw0, p1x = c1.x * iw1, p1y = c1.y * iw1, p2x = c2.x * iw2, p2y = c2.y * iw2;
        const float m0x = p2x - p1x, m0y = p2y - p1y, m1x = p0x - p1x, m1y = p0y - p1y;
        const float invDet = 1.0f / (m0x * m1y - m1x * m0y);
        const float s0 = invDet * iw0, s1 = invDet * iw1, s2 = invDet * iw2;
        float dx[3] = { (p1y - p2y) * s0, (p2y - p0y) * s1, (p0y - p1y) * s2 };
        float dy[3] = { (p2x - p1x) * s0, (p0x - p2x) * s1, (p1x - p0x) * s2 };
        float dxs = dx[0] + dx[1] + dx[2], dys = dy[0] + dy[1] + dy[2];
        const float r0x = su - p0x, r0y = sv - p0y;
        const float interpInvW = iw0 + r0x * dxs + r0y * dys;
        const float interpW = 1.0f / interpInvW;
        b[1] = interpW * (r0x * dx[1] + r0y * dy[1]);
        b[2] = interpW * (r0x * dx[2] + r0y * dy[2]);
        b[0] = 1 - b[1] - b[2];
        const float kx = 2.0f / W, ky = -(2.0f / H);
#pragma unroll
        for (int k = 0; k < 3; k++) dx[k] *= kx, dy[k] *= ky;
        dxs *= kx, dys *= ky;
        const float wdx = 1.0f / (interpInvW + dxs), wdy = 1.0f / (interpInvW + dys);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            dx[k] = wdx * (b[k] * interpInvW + dx[k]) - b[k];
            dy[k] = wdy * (b[k] * interpInvW + dy[k]) - b[k];
        }
        const float t0x = h2f(tc[0] & 0xFFFF), t0y = h2f(tc[0] >> 16);
        const float t10x = h2f(tc[1] & 0xFFFF) - t0x, t10y = h2f(tc[1] >> 16) - t0y;
        const float t20x = h2f(tc[2] & 0xFFFF) - t0x, t20y = h2f(tc[2] >> 16) - t0y;
        const float texU = t0x + t10x * b[1] + t20x * b[2];
        const float texV = t0y + t10y * b[1] + t20y * b[2];
        const float g0 = t10x * dx[1] + t20x * dx[2], g1 = t10y * dx[1] + t20y * dx[2];
        const float g2 = t10x * dy[1] + t20x * dy[2], g3 = t10y * dy[1] + t20y * dy[2];

        // waterfall over materials: filter chosen over the whole tile per material
        unsigned pm = (__ballot_sync(hm, !isSky && matId != 0xFFFFFFFFu) >> (16 * half)) & 0xFFFF;
        while (pm) {
            const int src = __ffs(pm) - 1;
            const uint32_t mid = __shfl_sync(hm, matId, src + 16 * half);
            const unsigned iter = (__ballot_sync(hm, matId == mid) >> (16 * half)) & 0xFFFF;
            pm &= ~iter;
            if (mid >= a.numMaterials || !a.materials[mid].has_texture) continue;
            const DevTexture& tex = a.materials[mid].tex;
            const float ssu = tex.scale_u * tex.scale_u, ssv = tex.scale_v * tex.scale_v;
            const float ddx2 = fmaf(g0, g0, g1 * g1) * ssu, ddy2 = fmaf(g2, g2, g3 * g3) * ssv;
            const int32_t mip = ilog2_x86(vmax(ddx2, ddy2)) >> 1;
            const bool nearest = __ballot_sync(hm, mip > 0) & hm;
            if ((iter >> l) & 1) {
                if constexpr (kMode == kResolvePlain || kMode == kResolveDebug) {
                    albedo = sample_rgba8(tex, texU, texV, 0, mip, nearest);
                    if (tex.num_layers >= 2) nmr = sample_rgba8(tex, texU, texV, 1, mip, nearest);
                } else {
                    const TexelQuad q = texel_quad(tex, texU, texV, mip, nearest);
                    // decoded when the model covers the level and its texture has this texture's size
                    const bool dec = mid < nr.numMaterials && q.m < (int32_t)nr.decodedLevels && nr.tex[mid].data != nullptr &&
                                     nr.tex[mid].width == tex.width && nr.tex[mid].height == tex.height;
                    if constexpr (kMode == kResolveEmit) {
                        uint32_t nq = 0;
                        sflags = dec ? kSurfFast | kSurfDecoded | (nearest ? kSurfNearest : 0u) | (q.inX ? kSurfInX : 0u) |
                                           (q.inY ? kSurfInY : 0u) | (tex.num_layers >= 2 ? kSurfTwoLayers : 0u)
                                     : 0u;  // sampled from the plain texture: the second pass reconstructs
                        sfx = q.fx, sfy = q.fy;
                        if (dec) {
                            const unsigned long long b = ((unsigned long long)mid << 32) | ((uint32_t)q.m << 28);
                            const uint32_t x0 = (uint32_t)q.tx, y0 = (uint32_t)q.ty;
                            req[0] = b | (y0 << 14) | x0, nq = 1;
                            if (!nearest) {
                                if (q.inX) req[1] = b | (y0 << 14) | (x0 + 1), nq++;
                                if (q.inY) req[2] = b | ((y0 + 1) << 14) | x0, nq++;
                                if (q.inX && q.inY) req[3] = b | ((y0 + 1) << 14) | (x0 + 1), nq++;
                            }
                        }
                        const unsigned grp = iter << (16 * half);
                        nq = 0;
#pragma unroll
                        for (int k = 0; k < 4; k++) {  // requests equal to a lower lane's at the same position
                            const unsigned peers = __match_any_sync(grp, req[k]);
                            const int lead = __ffs(peers) - 1;
                            const uint32_t leadOff = __shfl_sync(grp, off, lead);
                            if (req[k] == ~0ull) continue;
                            if (lead != (int)lane) req[k] = kReqRedirect | ((unsigned long long)leadOff * 4 + k);
                            else nq++;
                        }
                        const uint32_t total = __reduce_add_sync(grp, nq);
                        if (total && (int)lane == __ffs(grp) - 1) atomicAdd(&nr.counts[mid], total);
                    } else if (dec) {
                        // a slot's decoded texel, or the one of the slot it redirects to
                        const ulonglong2* rq = (const ulonglong2*)(nr.pixelReq + (size_t)off * 4);
                        const ulonglong2 r01 = rq[0], r23 = rq[1];
                        auto at = [&](unsigned long long r, uint32_t k) {
                            const size_t slot = (r != ~0ull && (r & kReqRedirect)) ? (size_t)(uint32_t)r : (size_t)off * 4 + k;
                            return nr.decoded[slot];
                        };
                        const uint2 d00 = at(r01.x, 0);
                        uint2 r0 = d00;
                        if (!nearest) {
                            const uint2 d10 = q.inX ? at(r01.y, 1) : d00, d01 = q.inY ? at(r23.x, 2) : d00;
                            const uint2 d11 = q.inY ? (q.inX ? at(r23.y, 3) : d01) : d10;
                            r0.x = filter_rgba8(d00.x, d10.x, d01.x, d11.x, q.fx, q.fy);
                            r0.y = filter_rgba8(d00.y, d10.y, d01.y, d11.y, q.fx, q.fy);
                        }
                        albedo = r0.x;
                        if (tex.num_layers >= 2) nmr = r0.y;
                    } else {
                        albedo = sample_rgba8(tex, texU, texV, 0, mip, nearest);
                        if (tex.num_layers >= 2) nmr = sample_rgba8(tex, texU, texV, 1, mip, nearest);
                    }
                }
            }
        }
        if constexpr (kMode == kResolveEmit) {
            uint4* dst = (uint4*)(nr.pixelReq + (size_t)off * 4);
            dst[0] = make_uint4((uint32_t)req[0], (uint32_t)(req[0] >> 32), (uint32_t)req[1], (uint32_t)(req[1] >> 32));
            dst[1] = make_uint4((uint32_t)req[2], (uint32_t)(req[2] >> 32), (uint32_t)req[3], (uint32_t)(req[3] >> 32));
            nr.surf[(size_t)off * 2] = make_uint4(__float_as_uint(b[1]), __float_as_uint(b[2]), ntg[0], ntg[1]);
            nr.surf[(size_t)off * 2 + 1] = make_uint4(ntg[2], sfx, sfy, sflags | hand);
            return;
        }
        }  // !fast
        F3 nrm[3], tan[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint32_t p = ntg[k];
            const float s = 1.0f / 255;
            nrm[k] = unmap_oct((float)(p & 255) * s, (float)((p >> 8) & 255) * s);
            tan[k] = unmap_oct((float)((p >> 16) & 255) * s, (float)(p >> 24) * s);
        }
        const float* M = a.objectToWorld;
        auto bl = [&](const F3* v) {
            return F3{ fmaf(v[0].x, b[0], fmaf(v[1].x, b[1], v[2].x * b[2])), fmaf(v[0].y, b[0], fmaf(v[1].y, b[1], v[2].y * b[2])),
                       fmaf(v[0].z, b[0], fmaf(v[1].z, b[1], v[2].z * b[2])) };
        };
        auto m3 = [&](F3 n) {
            return F3{ fmaf(n.x, M[0], fmaf(n.y, M[3], n.z * M[6])), fmaf(n.x, M[1], fmaf(n.y, M[4], n.z * M[7])),
                       fmaf(n.x, M[2], fmaf(n.y, M[5], n.z * M[8])) };
        };
        const F3 nws = normalize3(m3(bl(nrm)));
        F3 N = nws;
        if (__ballot_sync(hm, (nmr & 0xFFFF) != 0) & hm) {
            const F3 tws = normalize3(m3(bl(tan)));
            F3 bws = { fmaf(nws.y, tws.z, -nws.z * tws.y), fmaf(nws.z, tws.x, -nws.x * tws.z), fmaf(nws.x, tws.y, -nws.y * tws.x) };
            bws = { __uint_as_float(__float_as_uint(bws.x) ^ hand), __uint_as_float(__float_as_uint(bws.y) ^ hand),
                    __uint_as_float(__float_as_uint(bws.z) ^ hand) };
            const float tx_ = (float)(nmr & 255) * (1.0f / 127.5f) - 1.0f;
            const float ty_ = (float)((nmr >> 8) & 255) * (1.0f / 127.5f) - 1.0f;
            const float tz_ = approx_sqrt(1.0f - (tx_ * tx_ + ty_ * ty_));
            N = normalize3({ tx_ * tws.x + ty_ * bws.x + tz_ * nws.x, tx_ * tws.y + ty_ * bws.y + tz_ * nws.y,
                             tx_ * tws.z + ty_ * bws.z + tz_ * nws.z });
        }
        const float metallic = (float)((nmr >> 16) & 255) * (1.0f / 255);
        const float roughness = (float)((nmr >> 24) & 255) * (1.0f / 255);
        if constexpr (kMode == kResolveDebug) {
            a.color[off] = isSky ? background : debug_pixel(a.debugLayer, id, albedo, N, metallic, roughness);
            return;
        }

        // ---- EvalLighting (Shading.cpp:602-645)
        const float invPi = 0.3183098861837907f;
        uint32_t rb1 = ((albedo << 8) & 0xFF00FF00u) + 0x00FF00FFu, ag1 = (albedo & 0xFF00FF00u) + 0x00FF00FFu;
        uint32_t rb2 = (((rb1 & 0xFFFF) * (rb1 & 0xFFFF)) >> 16) | ((((rb1 >> 16) * (rb1 >> 16)) >> 16) << 16);
        uint32_t ag2 = (((ag1 & 0xFFFF) * (ag1 & 0xFFFF)) >> 16) | ((((ag1 >> 16) * (ag1 >> 16)) >> 16) << 16);
        const float s65 = 1.0f / 65535;
        const F3 base = { (float)(rb2 & 65535) * s65, (float)(ag2 & 65535) * s65, (float)(rb2 >> 16) * s65 };
        const float alphaR = vmax(roughness * roughness, 1e-4f);
        const float f0d = 0.16f * 0.5f * 0.5f;
        const F3 f0 = { lerpf(f0d, base.x, metallic), lerpf(f0d, base.y, metallic), lerpf(f0d, base.z, metallic) };
        const float dm = 1.0f - metallic;
        const F3 diffuse = { base.x * dm, base.y * dm, base.z * dm };
        const F3 vp = { a.viewPos[0], a.viewPos[1], a.viewPos[2] };
        const F3 viewDir = normalize3({ vp.x - world.x, vp.y - world.y, vp.z - world.z });
        const float NoV = fabsf(dot3(N, viewDir)) + 1e-5f;
        const float exposure = a.exposure * 0.001f;
        for (uint32_t i = 0; i < a.numLights; i++) {
            const swr_light& li = a.lights[i];
            F3 ld = li.type == 0 ? F3{ -li.direction[0], -li.direction[1], -li.direction[2] }
                                 : normalize3({ li.position[0] - world.x, li.position[1] - world.y, li.position[2] - world.z });
            const float NoL = dot3(N, ld);
            if ((__ballot_sync(hm, NoL < 1e-4f) & hm) == hm) continue;
            float att = 1.0f;
            if (li.type != 0) {
                const F3 p2l = { li.position[0] - world.x, li.position[1] - world.y, li.position[2] - world.z };
                const float d2 = dot3(p2l, p2l);
                const float f = d2 * li.inv_radius_sq;
                const float sm = vmax(1.0f - f * f, 0.0f);
                att = (sm * sm) * approx_rcp(vmax(d2, 1e-4f));
                if (li.type == 2) {
                    const float cd = dot3({ -li.direction[0], -li.direction[1], -li.direction[2] }, normalize3(p2l));
                    const float sa = vmin(vmax(cd * li.spot_scale + li.spot_offset, 0.0f), 1.0f);
                    att *= sa * sa;
                }
            }
            att = att * li.intensity * exposure;
            if ((__ballot_sync(hm, NoL * att < 1e-4f) & hm) == hm) continue;
            const F3 h = normalize3({ viewDir.x + ld.x, viewDir.y + ld.y, viewDir.z + ld.z });
            const float NoH = vmin(vmax(dot3(N, h), 0.0f), 1.0f);
            const float LoH = vmin(vmax(dot3(ld, h), 0.0f), 1.0f);
            const float aa = NoH * alphaR;
            const float k = alphaR * approx_rcp(1.0f - NoH * NoH + aa * aa);
            const float D = k * k * invPi;
            const float V = 0.5f / lerpf(2.0f * NoL * NoV, NoL + NoV, alphaR);
            const float x = 1.0f - LoH;
            const float f = (x * x) * (x * x) * x;
            const F3 F = { f + f0.x * (1.0f - f), f + f0.y * (1.0f - f), f + f0.z * (1.0f - f) };
            const float DV = D * V;
            const float wgt = vmax(NoL * att, 0.0f);
            color.x += (diffuse.x * invPi + DV * F.x) * li.color[0] * wgt;
            color.y += (diffuse.y * invPi + DV * F.y) * li.color[1] * wgt;
            color.z += (diffuse.z * invPi + DV * F.z) * li.color[2] * wgt;
        }
        color.x += base.x * 0.05f;
        color.y += base.y * 0.05f;
        color.z += base.z * 0.05f;
    }
    if (skyBits != 0 && a.hasSky && isSky) color = sample_env(a.sky, { world.x - a.viewPos[0], world.y - a.viewPos[1], world.z - a.viewPos[2] });
    // Tonemap_Unreal (Shading.cpp:221-226) + RGBA8u::Pack
    const float e = a.exposure;
    const F3 c = { color.x * e, color.y * e, color.z * e };
    const uint32_t r = sat_u8(round2i(c.x / (c.x + 0.155f) * 1.019f * 255.0f));
    const uint32_t g = sat_u8(round2i(c.y / (c.y + 0.155f) * 1.019f * 255.0f));
    const uint32_t bch = sat_u8(round2i(c.z / (c.z + 0.155f) * 1.019f * 255.0f));
    a.color[off] = r | (g << 8) | (bch << 16) | (255u << 24);
}

}  // namespace
}  // namespace swr

using namespace swr;

namespace {
// ShadingContext::Resolve's per-frame constants (Shading.cpp:658-690); the lights are copied to a
// stream-ordered device allocation that the caller frees after the launch.
swr_status build_resolve_args(swr_framebuffer fb, const swr_shading_context* ctx, ResolveArgs& a, const char* fn) {
    if (!fb || !ctx || !ctx->scene) return swr_internal_fail(SWR_EINVAL, (std::string(fn) + ": NULL argument").c_str());
    if (ctx->num_lights && !ctx->lights) return swr_internal_fail(SWR_EINVAL, (std::string(fn) + ": lights is NULL").c_str());
    if (ctx->skybox && ctx->skybox->format != SWR_FORMAT_R11G11B10F)
        return swr_internal_fail(SWR_EINVAL, (std::string(fn) + ": the skybox must be R11G11B10f").c_str());
    swr_status fst = swr_internal_finalize(fb);  // pending draws reach layers 0 and 1 first
    if (fst != SWR_OK) return fst;
    cudaStream_t st = swr_internal_stream();
    a = {};
    a.meshlets = ctx->scene->meshlets;
    a.numMeshlets = ctx->scene->count;
    a.materials = ctx->scene->materials;
    a.numMaterials = ctx->scene->num_materials;
    a.color = fb->layers;
    a.depth = (const float*)(fb->layers + fb->layer_stride);
    a.width = fb->width, a.height = fb->height;
    memcpy(a.objectToClip, ctx->object_to_clip, sizeof(a.objectToClip));
    memcpy(a.objectToWorld, ctx->object_to_world, sizeof(a.objectToWorld));
    if (!swr_hostmath::inverse_screen_proj(ctx->world_to_clip, fb->width, fb->height, a.invProj))
        return swr_internal_fail(SWR_EINVAL, (std::string(fn) + ": singular world_to_clip").c_str());
    memcpy(a.viewPos, ctx->view_pos, sizeof(a.viewPos));
    a.exposure = ctx->exposure;
    if (ctx->skybox) a.sky = ctx->skybox->d, a.hasSky = 1;
    if (ctx->num_lights) {
        swr_light* dl = nullptr;
        cudaError_t e = cudaMallocAsync(&dl, ctx->num_lights * sizeof(swr_light), st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dl, ctx->lights, ctx->num_lights * sizeof(swr_light), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, fn);
        a.lights = dl;
    }
    a.numLights = ctx->num_lights;
    return SWR_OK;
}
}  // namespace

extern "C" {

swr_status swr_cull_meshlets(swr_scene s, uint32_t first, uint32_t count, uint16_t* bitmap_device, const float proj[16],
                             const float view[16], const float model[16], const float prev_view[16], float frame_width,
                             float frame_height, swr_texture depth_map, uint32_t* visible_count) {
    return swr_cull_meshlets_ex(s, first, count, bitmap_device, proj, view, model, prev_view, frame_width, frame_height,
                                depth_map, visible_count, 0u);
}

swr_status swr_cull_meshlets_ex(swr_scene s, uint32_t first, uint32_t count, uint16_t* bitmap_device, const float proj[16],
                                const float view[16], const float model[16], const float prev_view[16], float frame_width,
                                float frame_height, swr_texture depth_map, uint32_t* visible_count, uint32_t flags) {
    if (!s || !bitmap_device || !proj || !view || !model || !prev_view)
        return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets: NULL argument");
    if (flags & ~(uint32_t)SWR_CULL_BACKFACE_CONE) return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets_ex: unknown flags");
    if ((uint64_t)first + count > s->count) return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets: range outside the scene");
    if (depth_map && depth_map->format != SWR_FORMAT_R32F)
        return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets: the depth map must be R32f");
    if (!(frame_width >= 1.0f && frame_width <= 65536.0f && frame_height >= 1.0f && frame_height <= 65536.0f))
        return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets: frame size outside [1, 65536]");
    // Texel reads stay inside the map when it is at least half the frame in each dimension (the
    // frame driver's sizing, Main.cpp:54-56) and has two levels (mip clamps to [1, levels-1]).
    if (depth_map && ((float)(depth_map->d.width * 2) < frame_width || (float)(depth_map->d.height * 2) < frame_height ||
                      depth_map->d.mip_levels < 2))
        return swr_internal_fail(SWR_EINVAL, "swr_cull_meshlets: depth map smaller than half the frame or without mips");
    cudaStream_t st = swr_internal_stream();
    CullArgs a = {};
    a.meshlets = s->meshlets;
    a.first = first, a.count = count;
    a.bitmap = bitmap_device;
    float objToPrev[16], pv[16], objToClip[16], planes[6][4];
    swr_hostmath::mat4_mul(prev_view, model, objToPrev);
    swr_hostmath::mat4_mul(proj, view, pv);
    swr_hostmath::mat4_mul(pv, model, objToClip);
    swr_hostmath::frustum_planes(objToClip, planes);
    memcpy(a.planes, planes, sizeof(a.planes));  // planes 0..4 (the reference skips the last, Shading.cpp:806)
    if (flags & SWR_CULL_BACKFACE_CONE) {
        a.cone = swr_hostmath::cone_camera(objToClip, a.eye) ? 1u : 0u;
        a.materials = s->materials;
        a.numMaterials = s->num_materials;
    }
    memcpy(a.objectToPrevView, objToPrev, sizeof(objToPrev));
    a.objectToWorldScale = swr_hostmath::column0_length(model);
    a.projFactors[0] = proj[3 * 4 + 2], a.projFactors[1] = proj[0], a.projFactors[2] = proj[1 * 4 + 1];
    a.frameW = frame_width, a.frameH = frame_height;
    if (depth_map) {
        a.depthData = depth_map->d.data;
        memcpy(a.mipOffsets, depth_map->d.mip_offsets, sizeof(a.mipOffsets));
        a.mipLevels = depth_map->d.mip_levels;
        a.rowShift = depth_map->d.row_shift;
    }
    unsigned int* cnt = nullptr;
    cudaError_t e = cudaSuccess;
    if (visible_count) {
        e = cudaMallocAsync(&cnt, sizeof(unsigned int), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned int), st);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_cull_meshlets");
        a.visibleCount = cnt;
    }
    if (count) {
        LaunchScope ls("k_cull", st);
        k_cull<<<(count + 255) / 256, 256, 0, st>>>(a);
        e = cudaGetLastError();
    }
    if (visible_count) {
        unsigned int h = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(cnt, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        *visible_count = h;
    }
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_cull_meshlets");
    return SWR_OK;
}

swr_status swr_downsample_depth(swr_framebuffer fb, swr_texture dest) {
    if (!fb || !dest) return swr_internal_fail(SWR_EINVAL, "swr_downsample_depth: NULL argument");
    if (dest->format != SWR_FORMAT_R32F) return swr_internal_fail(SWR_EINVAL, "swr_downsample_depth: destination must be R32f");
    swr_status fst = swr_internal_finalize(fb);
    if (fst != SWR_OK) return fst;
    const uint32_t root = 32 - __builtin_clz(std::max(fb->width, fb->height));
    if (root < 4) return swr_internal_fail(SWR_EINVAL, "swr_downsample_depth: framebuffer smaller than 16 pixels");
    cudaStream_t st = swr_internal_stream();
    const float* depth = (const float*)(fb->layers + fb->layer_stride);
    uint32_t* tex = (uint32_t*)dest->d.data;
    auto blocks = [&](uint32_t m, uint32_t& rx, uint32_t& ry, uint32_t& bt) {
        if (m + 4 <= root) {
            const uint32_t region = 1u << (m + 4);
            rx = (fb->width + region - 1) / region, ry = (fb->height + region - 1) / region, bt = 64;
        } else {
            rx = ry = 1, bt = 16;
        }
    };
    // Levels the texture does not have use MipOffsets[m] = 0, as the reference's zero-filled table
    // does (for non-square frames its root tile lands at the start of mip 0). Every written texel
    // must fall inside the texture's storage.
    auto mipOff = [&](uint32_t m) { return m < dest->d.mip_levels ? dest->d.mip_offsets[m] : 0u; };
    for (uint32_t m = 0; m + 3 <= root; m++) {
        uint32_t rx, ry, bt;
        blocks(m, rx, ry, bt);
        const uint32_t side = bt == 64 ? 8 : 4;
        const int32_t stride = (int32_t)dest->d.row_shift - (int32_t)m;
        const uint64_t maxX = (uint64_t)rx * side - 1, maxY = (uint64_t)ry * side - 1;
        if (stride < 0 || mipOff(m) + 7 + (maxX << 3) + (maxY << stride) >= dest->words)
            return swr_internal_fail(SWR_EINVAL, "swr_downsample_depth: destination too small for this framebuffer");
    }
    HizOffsets offs = {};
    for (uint32_t m = 0; m + 3 <= root && m < 16; m++) offs.off[m] = mipOff(m);
    const uint32_t nLocal = std::min(4u, root - 3);  // levels with 8x8-texel blocks inside 128-pixel regions
    {
        LaunchScope ls("k_hiz_local", st);
        const dim3 grid((fb->width + kHizRegion - 1) / kHizRegion, (fb->height + kHizRegion - 1) / kHizRegion);
        k_hiz_local<<<grid, 256, 0, st>>>(depth, fb->width, fb->height, tex, offs, (int32_t)dest->d.row_shift, nLocal);
    }
    if (root - 3 >= nLocal) {
        size_t smem = 0;  // levels nLocal-1 .. root-3, texels whose origin lies in the frame
        for (uint32_t m = nLocal - 1; m <= root - 3; m++)
            smem += (size_t)hiz_extent(fb->width, m) * hiz_extent(fb->height, m) * sizeof(float);
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_hiz_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        LaunchScope ls("k_hiz_tail", st);
        k_hiz_tail<<<1, 1024, smem, st>>>(fb->width, fb->height, tex, offs, (int32_t)dest->d.row_shift, nLocal, root - 3,
                                           root);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_downsample_depth");
    return SWR_OK;
}

swr_status swr_resolve(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx) {
    (void)r;
    ResolveArgs a = {};
    swr_status s = build_resolve_args(fb, ctx, a, "swr_resolve");
    if (s != SWR_OK) return s;
    cudaStream_t st = swr_internal_stream();
    const uint32_t tiles = (fb->width / 4) * (fb->height / 4);
    cudaError_t e;
    {
        LaunchScope ls("k_resolve", st);
        k_resolve<kResolvePlain><<<(tiles * 16 + 255) / 256, 256, 0, st>>>(a, NeuralResolve{});
        e = cudaGetLastError();
    }
    if (a.lights) cudaFreeAsync((void*)a.lights, st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_resolve");
    fb->keys_valid = false;  // layer 0 now holds colour; a later draw rebuilds its keys from depth
    return SWR_OK;
}

swr_status swr_resolve_debug(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx, uint32_t layer) {
    (void)r;
    if (layer > SWR_DEBUG_OVERDRAW_QUAD) return swr_internal_fail(SWR_EINVAL, "swr_resolve_debug: unknown debug layer");
    ResolveArgs a = {};
    swr_status s = build_resolve_args(fb, ctx, a, "swr_resolve_debug");
    if (s != SWR_OK) return s;
    a.debugLayer = layer;
    cudaStream_t st = swr_internal_stream();
    const uint32_t tiles = (fb->width / 4) * (fb->height / 4);
    cudaError_t e;
    {
        LaunchScope ls("k_resolve_debug", st);
        k_resolve<kResolveDebug><<<(tiles * 16 + 255) / 256, 256, 0, st>>>(a, NeuralResolve{});
        e = cudaGetLastError();
    }
    if (a.lights) cudaFreeAsync((void*)a.lights, st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_resolve_debug");
    fb->keys_valid = false;  // layer 0 now holds colour
    return SWR_OK;
}

swr_status swr_resolve_neural(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx, swr_neural n,
                              swr_neural_stats* stats) {
    (void)r;
    if (!n) return swr_internal_fail(SWR_EINVAL, "swr_resolve_neural: NULL model");
    ResolveArgs a = {};
    swr_status s = build_resolve_args(fb, ctx, a, "swr_resolve_neural");
    if (s != SWR_OK) return s;
    cudaStream_t st = swr_internal_stream();
    const uint32_t M = n->d.numMaterials;
    const size_t slots = (size_t)fb->width * fb->height * 4;
    cudaError_t e = cudaSuccess;
    if (n->scratchSlots < slots) {
        if (n->pixelReq) cudaFree(n->pixelReq);
        if (n->sorted) cudaFree(n->sorted);
        if (n->decoded) cudaFree(n->decoded);
        if (n->surf) cudaFree(n->surf);
        n->pixelReq = n->sorted = nullptr, n->decoded = nullptr, n->surf = nullptr, n->scratchSlots = 0;
        e = cudaMalloc(&n->pixelReq, slots * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&n->sorted, slots * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&n->decoded, slots * sizeof(uint2));
        if (e == cudaSuccess) e = cudaMalloc(&n->surf, slots / 4 * 2 * sizeof(uint4));
        if (e != cudaSuccess) {
            if (a.lights) cudaFreeAsync((void*)a.lights, st);
            return swr_internal_cuda_fail(e, "swr_resolve_neural: scratch");
        }
        n->scratchSlots = slots;
    }
    neural_sync_half(n, st);
    uint32_t* counts = n->counters;
    uint32_t* cursor = counts + (M + 1);
    uint32_t* reqOffset = cursor + (M + 1);
    uint32_t* tileOffset = reqOffset + (M + 1);
    uint32_t* levelCount = tileOffset + (M + 1);
    NeuralResolve nr = {};
    nr.tex = n->d.tex, nr.numMaterials = M, nr.decodedLevels = n->d.levels + 2;
    nr.pixelReq = n->pixelReq, nr.counts = counts, nr.decoded = n->decoded, nr.surf = n->surf;
    const uint32_t tiles = (fb->width / 4) * (fb->height / 4), blocks = (tiles * 16 + 255) / 256;
    e = cudaMemsetAsync(counts, 0, 2 * (M + 1) * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(levelCount, 0, kNeuralMaxDecoded * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        LaunchScope ls("k_resolve_emit", st);
        k_resolve<kResolveEmit><<<blocks, 256, 0, st>>>(a, nr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        LaunchScope ls("k_neural_offsets", st);
        launch_neural_offsets(counts, reqOffset, tileOffset, M, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        LaunchScope ls("k_neural_scatter", st);
        launch_neural_scatter(n->pixelReq, (uint32_t)slots, reqOffset, cursor, n->sorted, levelCount, M, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        NeuralDecodeArgs d = {};
        d.n = n->d;
        d.sorted = n->sorted, d.reqOffset = reqOffset, d.tileOffset = tileOffset;
        d.out = n->decoded;
        d.status = n->status;
        LaunchScope ls("k_neural_decode", st);
        launch_neural_decode(d, neural_decode_blocks_per_sm() * neural_num_sms(), st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        LaunchScope ls("k_resolve_neural", st);
        k_resolve<kResolveNeural><<<blocks, 256, 0, st>>>(a, nr);
        e = cudaGetLastError();
    }
    if (a.lights) cudaFreeAsync((void*)a.lights, st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_resolve_neural");
    fb->keys_valid = false;
    if (stats) {
        uint32_t v[2] = {};
        e = cudaMemcpyAsync(&v[0], reqOffset + M, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&v[1], tileOffset + M, 4, cudaMemcpyDeviceToHost, st);
        uint32_t status = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&status, n->status, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(stats->level_texels, levelCount, kNeuralMaxDecoded * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_resolve_neural: stats");
        stats->requests = v[0], stats->tiles = v[1];
        if (status) {
            cudaMemsetAsync(n->status, 0, 4, st);
            return swr_internal_fail(SWR_ETIMEOUT, "swr_resolve_neural: a tensor-core wait timed out");
        }
    }
    return SWR_OK;
}

}  // extern "C"
