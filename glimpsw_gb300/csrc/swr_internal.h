// Host-side object definitions behind the opaque handles of swr_gb300.h.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/swr_gb300.h"

namespace swr {

// Device copy of a Texture2D header (Texture.h:314-329) with its storage pointer.
struct DevTexture {
    uint32_t width, height, mip_levels, num_layers;
    uint32_t row_shift, layer_stride;
    float scale_u, scale_v, scale_lerp_u, scale_lerp_v;
    int32_t mask_u, mask_v, mask_lerp_u, mask_lerp_v;
    uint32_t mip_offsets[16];
    const uint32_t* data;
};

// Device copy of a Material (Scene.h:7-14).
struct DevMaterial {
    uint32_t has_texture;
    uint32_t is_double_sided;
    uint32_t alpha_cutoff;
    uint32_t pad;
    DevTexture tex;
};

// True if a material's meshlets take the alpha-tested vis-buffer shader: FragmentShaderId 1 for
// AlphaCutoff < 255 (Shading.cpp:305). A cutoff of 0 passes every texel and a material without a
// texture is taken to pass every fragment (the reference dereferences the texture unconditionally),
// so both draw as opaque.
inline __host__ __device__ bool material_alpha_tested(const DevMaterial& m) {
    return m.alpha_cutoff - 1u < 254u && m.has_texture;
}
// FS_EncodeGBuffer (Shading.cpp:357-359) alpha-tests every material with a texture (a cutoff of 0
// passes every texel and stays opaque).
inline __host__ __device__ bool material_alpha_tested_all(const DevMaterial& m) {
    return m.alpha_cutoff != 0u && m.has_texture;
}

#ifdef __CUDACC__
// Backface-cone culling of one meshlet record (no counterpart in the reference's CullMeshlets; the
// records carry meshoptimizer's cone, Scene.h:18-19, Scene.cpp:240-244): every triangle faces away
// from the camera at eye (object space) when dot(normalize(ConeApex - eye), ConeAxis) >= ConeCutoff.
// The test here is conservative by a margin, so that no triangle the rasterizer would keep is
// culled despite float rounding: the cosine must exceed the cutoff by kConeMargin (about 1.8
// degrees of the view direction), and the camera must be at least four times the apex's reach
// (|centre - apex| + radius) away, so that each triangle's plane is seen at more than a degree.
// Double-sided materials draw both faces and are never culled. Degenerate cones (cutoff 1) never
// pass.
constexpr float kConeMargin = 1.0f / 32.0f;
__device__ __forceinline__ bool cone_culled(const uint8_t* rec, float ex, float ey, float ez, const DevMaterial* materials,
                                            uint32_t numMaterials) {
    const float* f = (const float*)rec;  // BoundCenter, BoundRadius, ConeApex, ConeAxis, ConeCutoff
    const float cm = f[10] + kConeMargin;
    if (!(cm < 1.0f)) return false;
    const uint32_t mat = *(const uint32_t*)(rec + 48);
    if (mat < numMaterials && materials[mat].is_double_sided) return false;
    const float dx = f[4] - ex, dy = f[5] - ey, dz = f[6] - ez;
    const float l2 = dx * dx + dy * dy + dz * dz;
    const float proj = dx * f[7] + dy * f[8] + dz * f[9];
    const float a2 = f[7] * f[7] + f[8] * f[8] + f[9] * f[9];
    if (!(proj > 0.0f) || !(a2 > 0.5f)) return false;
    const float cx = f[0] - f[4], cy = f[1] - f[5], cz = f[2] - f[6];
    const float reach = sqrtf(cx * cx + cy * cy + cz * cz) + f[3];
    return proj * proj >= cm * cm * l2 * a2 && l2 >= 16.0f * reach * reach;
}
#endif

// A triangle ready to rasterize: edge equations at pixel (0,0), depth plane and tie-break rank.
struct TriRec {
    int32_t E0, E1, E2;
    int32_t A12, B12, A20, B20, A01, B01;
    float Z0, Z10, Z20;
    uint32_t bbMin, bbMax;  // packed (x | y << 16), 4-aligned, [min, max)
    uint32_t lowword;       // 0xFFFFFFFE - rank
    uint32_t pad;
};
static_assert(sizeof(TriRec) == 64, "TriRec");

// TriRec::pad bit of a queued triangle whose material is alpha-tested (FS_EncodeSurfaceId<true>);
// the rest of pad is the view index.
constexpr uint32_t kTriAlpha = 0x80000000u;

// What the alpha test of a queued triangle needs besides its TriRec; stored in the queue slot
// after it. Its bbMin/bbMax words overlay TriRec::bbMin/bbMax and are zero, so the slot owns no
// chunks of its own.
struct AlphaExt {
    float W0, W0S, W1S, W2S;     // perspective terms (TriangleEdgeVars, Rasterizer.cpp:320-328)
    float ru[3], rv[3];          // TriangleClipData rows of a clipped triangle (Rasterizer.cpp:455-458)
    uint32_t tc0, tc1;           // packed half2 texcoords of vertices 0 and 1
    uint32_t zero0, zero1;       // = 0 (bbMin, bbMax of the overlaid TriRec)
    uint32_t tc2;                // texcoord of vertex 2
    uint32_t material;           // material index | kTriAlpha when clipped
};
static_assert(sizeof(AlphaExt) == sizeof(TriRec) && offsetof(AlphaExt, zero0) == offsetof(TriRec, bbMin) &&
                  offsetof(AlphaExt, zero1) == offsetof(TriRec, bbMax), "AlphaExt overlays TriRec");

// Per-rasterizer device scratch, reused by every draw.
struct DrawScratch {
    unsigned long long* control;   // [0] meshlet work counter, [1] big-triangle queue (slots<<40 | chunks),
                                   // [2] status flags, [3..6] perf counters, [7] the second pass's work
                                   // counter of a single-view draw, [8] chunk-stage cursor,
                                   // [9] alpha list length, [10] alpha-pass cursor,
                                   // [11] / [12] warps done in the opaque / alpha pass
    TriRec* big;                   // queue of triangles rasterized by the chunk kernel
    unsigned long long* bigBase;   // first chunk index of each queued triangle
    uint32_t bigCapacity;
    uint32_t* alphaList;           // work items of alpha-tested meshlets (nullptr: the draw has none)
    uint32_t alphaCapacity;
};

enum : unsigned long long { kStatusBigOverflow = 1ull, kStatusClipOverflow = 2ull };

// One view of a draw: its transform, viewport, vis-buffer keys and meshlet range.
struct ViewParams {
    float m[16];
    int32_t halfW, halfH;
    uint32_t width, height;
    float bx, by;
    uint32_t meshletOffset, count;
    unsigned long long* keys;
    const uint32_t* groupMasks;  // batched views: bit l of word g is the cull result of draw position
                                 // 32 g + l (nullptr: every meshlet visible)
    uint32_t* tileMin;      // per 4x4 tile: lower bound of its keys' depth words (nullptr: no tile culling)
    uint32_t orderStride;   // draw order: position p draws meshlet (p * orderStride) mod count (order_stride)
    uint32_t pad;
};
static_assert(sizeof(ViewParams) == 128, "ViewParams");

struct DrawArgs {
    const uint8_t* meshlets;
    const DevMaterial* materials;
    uint32_t numMaterials;
    // single view (views == nullptr)
    uint32_t meshletOffset;
    uint32_t count;
    const uint16_t* cullBitmap;
    float m[16];
    int halfW, halfH;
    uint32_t width, height;
    float bx, by;
    int clipMode;     // 1: clip non-trivial triangles (Mode B), 0: drop them
    int countClipped; // count non-trivial triangles in TrianglesClipped
    unsigned long long* keys;
    uint32_t* tileMin;  // per 4x4 tile depth lower bound (nullptr: no tile culling)
    DrawScratch s;
    // batched views: work item i of [0, viewStart[numViews]) is meshlet i - viewStart[v] of view v
    const ViewParams* views;
    const uint32_t* viewStart;
    uint32_t numViews;
    // tuning: chunk width in 4x4 tiles (0 = 8), chunk height (0 = the width) and warps per block (0 = 8)
    uint32_t chunkTiles;
    uint32_t chunkTilesY;
    uint32_t warpsPerBlock;
    // OverdrawShader draws (single view): per-pixel counters (covered << 32 | other samples of
    // covered tiles), keys hold the maximum depth; nullptr for vis-buffer draws
    unsigned long long* counts;
    // single view: order_stride(count), set by launch_draw
    uint32_t orderStride;
    // the shading steps read a pixel's key before its atomicMax only for triangles of at most this
    // many tiles (0: for all); set by launch_draw
    uint32_t keyReadTiles;
    // single view: swr_shaded_meshlet records of a user mesh shader (record i = meshlet i of the
    // draw) in place of ShadeMeshlet's transform; nullptr for the built-in mesh shader
    const uint8_t* shaded;
    // FS_EncodeGBuffer's alpha test: every material with a texture is alpha-tested with its cutoff
    uint32_t alphaAll;
};

// swr_shaded_meshlet (ShadedMeshlet, Rasterizer.h:82-99) offsets.
constexpr uint32_t kShadedSize = 1472, kShadedIndices = 64, kShadedPositions = 448;

// The mesh stage draws a view's meshlets in the order p -> (p * stride) mod count: a Weyl sequence
// with stride near count / golden ratio (coprime to count), so neighbouring positions, fetched
// together or by warps running at the same time, hold meshlets far apart in the record order. In a
// spatially coherent order (meshlets built from a mesh, a grid) a fetch of 32 positions can
// otherwise be 32 visible neighbours close to the camera, all for one warp, and concurrent warps
// contend for the same pixels' keys. Keys are order-independent, so the image is the same for
// every order. Work is fetched kBatchGroup positions at a time in batches (whose views' position
// ranges are padded to multiples of it); single-view draws start at kDrawGroup positions and adapt
// the group to the share of visible meshlets, and the alpha pass takes kDrawGroup list entries.
constexpr uint32_t kDrawGroup = 4, kBatchGroup = 32;
uint32_t order_stride(uint32_t count);
// Meshlet drawn at position p of a view of count meshlets (order_stride).
__device__ __forceinline__ uint32_t draw_order(uint32_t p, uint32_t count, uint32_t stride) {
    return (uint32_t)(((unsigned long long)p * stride) % count);
}

void launch_draw(const DrawArgs& a, cudaStream_t st, int numSMs);
void launch_init_keys(const uint32_t* depthLayer, unsigned long long* keys, uint32_t* tileMin, uint32_t n, cudaStream_t st);
void launch_clear(uint32_t* layer0, uint32_t* layer1, unsigned long long* keys, uint32_t* tileMin, uint32_t n,
                  uint32_t color, uint32_t depthBits, cudaStream_t st);
void launch_fill(uint32_t* dst, uint32_t n, uint32_t value, cudaStream_t st);
void launch_finalize(const unsigned long long* keys, uint32_t* layer0, uint32_t* layer1, uint32_t n, cudaStream_t st);
void launch_finalize_overdraw(const unsigned long long* keys, const unsigned long long* counts, uint32_t* layer0,
                              uint32_t* layer1, uint32_t n, cudaStream_t st);
void launch_detile(const uint32_t* src, uint32_t* dst, uint32_t width, uint32_t height, uint32_t stride, cudaStream_t st);

}  // namespace swr

// Error reporting and the calling thread's stream, shared by all translation units (swr_api.cu).
swr_status swr_internal_fail(swr_status code, const char* msg);
swr_status swr_internal_cuda_fail(cudaError_t e, const char* what);
cudaStream_t swr_internal_stream();
// The current device and its SM count (queried once per device, then cached). Returns SWR_ECUDA
// with the message set if either query fails.
swr_status swr_internal_device(int* dev, int* sms);
// SM count of the current device, 148 if the query fails (launch sizing only).
int swr_internal_sm_count();
// Profiling on/off for this thread (returns the previous state) and extra launches to count
// (kernels replayed inside a CUDA graph).
bool swr_internal_set_profiling(bool on);
void swr_internal_count_launches(unsigned long long n);

namespace swr {
// Kernel tracing: every launch is counted; while profiling is enabled each launch is bracketed
// by CUDA events on its stream (the GPU counterpart of the reference's Tracy zones).
struct LaunchScope {
    LaunchScope(const char* name, cudaStream_t st);
    ~LaunchScope();
    cudaStream_t st;
    int rec;
};
}  // namespace swr

struct swr_framebuffer_t {
    uint32_t width, height, tile_stride, layer_stride, num_layers;
    uint32_t* layers;              // num_layers * layer_stride words (+64 pad)
    unsigned long long* keys;      // one vis-buffer key per pixel, tiled like the layers
    uint32_t* tileMin;             // per 4x4 tile: lower bound of its keys' depth words
    unsigned long long* counts;    // OverdrawShader counters, allocated by its first draw
    bool keys_valid;               // keys and tileMin reflect the depth layer
    uint8_t layers_stale;          // the keys hold draws not yet written to the layers: kStale*
};
enum : uint8_t { kStaleNone = 0, kStaleDepth = 1, kStaleAll = 2 };  // kStaleDepth: depth-only views of a batch
// swr_draw_meshlets with SWR_SHADER_DEFERRED (swr_gbuffer.cu).
swr_status swr_internal_draw_deferred(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* ctx);
// Writes pending vis-buffer draws from the keys to layers 0 and 1 (k_finalize); every reader or
// writer of the layers calls it first, so consecutive draws into one framebuffer finalize once.
swr_status swr_internal_finalize(swr_framebuffer fb);

struct swr_scene_t {
    uint8_t* meshlets;
    uint32_t count, capacity;
    swr::DevMaterial* materials;
    uint32_t num_materials;
    bool hasAlpha;                 // some material selects FS_EncodeSurfaceId<true> (swr::material_alpha_tested)
    bool hasAlphaAll;              // some material is alpha-tested under FS_EncodeGBuffer (material_alpha_tested_all)
    uint8_t* fsIds;                // device: FragmentShaderId of each material under ShadeMeshlet
    uint64_t version;              // bumped when meshlets or materials move (recorded draw graphs re-capture)
};

struct swr_texture_t {
    uint32_t format;
    swr::DevTexture d;             // d.data is the device storage
    size_t words;
};

struct swr_rasterizer_t {
    int enable_binning, enable_clipping, enable_guardband;
    swr::DrawScratch scratch;
    // Queue sizing: the status word of each draw is copied to pinned memory; a later draw that
    // sees an overflow reported sizes the queue for every triangle of a draw.
    unsigned long long* hostStatus;   // pinned
    cudaEvent_t statusEvent;
    bool statusPending;
    bool sawOverflow;
    uint32_t fixedCapacity;           // 0: automatic sizing
};
