// Shader hooks of the GPU meshlet rasterizer: the reference's mesh-shader / fragment-shader binding
// (ShadedMeshlet, FragmentVars and GetDispatchTable<&MeshFn, &FragFn...>, Rasterizer.h:82-138,
// 178-196, 342-364) as header-only CUDA templates. A translation unit compiled with nvcc for
// sm_103a includes this header, writes its shaders as __device__ functors and calls
// swr::DrawMeshlets<MeshFn, Ctx, FragFn...>(...); the functors are instantiated into kernels of that
// translation unit, which drive libswr_gb300's C entry points (swr_gb300.h) for visibility.
//
// The reference calls a fragment shader for every 4x4 tile a triangle covers, in draw order, and the
// shader does its own depth test against the depth layer. A GPU draw cannot order its fragments, so
// the stages are split as GPU vis-buffer renderers split them:
//  1. mesh stage: MeshFn shades each meshlet into a swr_shaded_meshlet record (clip positions,
//     indices, PrimCount, CullMode, FragmentShaderId), as the reference's MeshFn does;
//  2. visibility: libswr_gb300 rasterizes the records with the reference's fixed-point edges and
//     depth test (GREATER; equal depths go to the first-submitted triangle), including the alpha test
//     of alpha-tested materials, and writes the depth layer;
//  3. fragment stage: for every 4x4 tile, each triangle that is visible in some of its pixels is
//     rebuilt with the raster's own setup code (swr/raster_math.cuh, same bits) and the fragment
//     shader FragFn[FragmentShaderId] is called once for it by the 16 threads of a half-warp, thread
//     l standing for the reference's vector lane l (pixel (l % 4, l / 4) of the tile). Its
//     FragmentVars carry the reference's values: perspective-correct barycentrics (rcp14 and one
//     Newton step, remapped through the clipper's TriangleClipData), Depth, MeshletId, PrimId,
//     VertexId; TileMask holds the pixels where the triangle is the visible one.
// A fragment shader therefore sees exactly the fragments that end up visible, and the library has
// already done the depth test and written the depth: a shader restated from the reference drops its
// own depth test (LoadTile(depth) / compare) and writes its other layers with StoreTile. The final
// framebuffer equals the reference's for shaders whose output at a pixel is a function of its
// front-most fragment (depth-tested shaders such as FS_EncodeSurfaceId and FS_EncodeGBuffer);
// shaders that accumulate over every fragment (FS_Overdraw) need the library's built-in tables.
//
// Requirements: draws into one framebuffer shade disjoint meshlet ranges (the fragment stage finds a
// pixel's draw by its meshlet), single view, and the mesh shader is called by the 32 lanes of a warp
// together (swr::mesh_lane() tells each lane which vertices to write).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <tuple>
#include <type_traits>

#include "../swr_gb300.h"
#include "raster_math.cuh"

namespace swr {

// ShadedMeshlet (Rasterizer.h:82-99), same layout.
using ShadedMeshlet = swr_shaded_meshlet;
enum : uint8_t { kFaceCullNone = 0, kFaceCullFrontCCW = 1, kFaceCullFrontCW = 2 };  // FaceCullMode

// Lane of the calling thread inside the warp running a mesh shader (vertices lane and lane + 32).
__device__ __forceinline__ uint32_t mesh_lane() { return threadIdx.x & 31; }

// The framebuffer as the fragment stage sees it: 4x4-tiled 32-bit layers (Rasterizer.h:10-78).
struct FragmentFramebuffer {
    uint32_t* layers;
    uint32_t layer_stride, width, height, num_layers;
    __device__ uint32_t* GetLayerData(uint32_t layer) const { return layers + (size_t)layer * layer_stride; }
    __device__ uint32_t* GetColorBuffer() const { return layers; }
    __device__ float* GetDepthBuffer() const { return (float*)(layers + layer_stride); }
};

// FragmentVars (Rasterizer.h:115-138) for one thread: the thread is lane `Lane` of the tile's 16.
struct FragmentVars {
    uint32_t MeshletId;    // the scene's meshlet index (the reference's is draw-relative)
    uint32_t PrimId;
    uint32_t VertexId[3];  // index bytes of the primitive (Mesh::Indices)
    uint32_t TileOffset;   // tiled word offset of the tile's first pixel
    uint32_t TileMask;     // pixels (bits 0-15) where this triangle is the visible one
    uint32_t Lane;         // this thread's pixel: (Lane % 4, Lane / 4) of the tile
    uint32_t PixelX, PixelY;
    float Bary[3];         // perspective-correct barycentrics { 1 - u - v, u, v }
    float Depth;

    __device__ bool Active() const { return (TileMask >> Lane) & 1u; }
    // BaryLerp (Rasterizer.h:101-113): fma(v0, b0, fma(v1, b1, v2 * b2)) per component.
    __device__ float Interpolate(float v0, float v1, float v2) const {
        return ffma(v0, Bary[0], ffma(v1, Bary[1], fmul(v2, Bary[2])));
    }
    __device__ float2 Interpolate(float2 v0, float2 v1, float2 v2) const {
        return make_float2(Interpolate(v0.x, v1.x, v2.x), Interpolate(v0.y, v1.y, v2.y));
    }
    __device__ float3 Interpolate(float3 v0, float3 v1, float3 v2) const {
        return make_float3(Interpolate(v0.x, v1.x, v2.x), Interpolate(v0.y, v1.y, v2.y), Interpolate(v0.z, v1.z, v2.z));
    }
    __device__ float4 Interpolate(float4 v0, float4 v1, float4 v2) const {
        return make_float4(Interpolate(v0.x, v1.x, v2.x), Interpolate(v0.y, v1.y, v2.y), Interpolate(v0.z, v1.z, v2.z),
                           Interpolate(v0.w, v1.w, v2.w));
    }
    // LoadTile / StoreTile (Rasterizer.h:128-137): this lane's word of a layer; stores only where
    // the triangle is visible.
    __device__ uint32_t LoadTile(const uint32_t* layer) const { return layer[TileOffset + Lane]; }
    __device__ float LoadTile(const float* layer) const { return layer[TileOffset + Lane]; }
    __device__ void StoreTile(uint32_t* layer, uint32_t v) const {
        if (Active()) layer[TileOffset + Lane] = v;
    }
    __device__ void StoreTile(float* layer, float v) const {
        if (Active()) layer[TileOffset + Lane] = v;
    }
    // texutil::dFdx / dFdy (Texture.h:258-275): p[l | 1] - p[l & ~1] and p[l | 4] - p[l & ~4] across the
    // tile's lanes (every lane of the half-warp takes part).
    __device__ float dFdx(float p) const {
        const float q = __shfl_xor_sync(half_mask(), p, 1);
        return (Lane & 1) ? fsub(p, q) : fsub(q, p);
    }
    __device__ float dFdy(float p) const {
        const float q = __shfl_xor_sync(half_mask(), p, 4);
        return (Lane & 4) ? fsub(p, q) : fsub(q, p);
    }
    // simd::any over the tile's 16 lanes.
    __device__ bool TileAny(bool p) const { return (__ballot_sync(half_mask(), p) & half_mask()) != 0; }
    __device__ static unsigned half_mask() { return 0xFFFFu << (threadIdx.x & 16); }
};

// Built-in mesh shader tag: ShadeMeshlet (Shading.cpp:281-307), fused into the library's raster
// (no shaded records); the fragment stage transforms the visible triangles' vertices again.
struct ShadeMeshletFn {};

namespace hook {

// Mesh stage: one warp per meshlet; MeshFn fills a shared-memory record, copied out coalesced.
template <class Ctx, class MeshFn>
__global__ void __launch_bounds__(256) k_mesh_shader(const __grid_constant__ Ctx ctx, uint32_t count, ShadedMeshlet* out) {
    __shared__ __align__(64) ShadedMeshlet rec[8];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    ShadedMeshlet& s = rec[warp];
    for (uint32_t idx = blockIdx.x * (blockDim.x >> 5) + warp; idx < count; idx += warps) {
        if (lane == 0) s.prim_count = 0, s.cull_mode = kFaceCullFrontCCW, s.fragment_shader_id = 0;
        __syncwarp();
        MeshFn{}(ctx, idx, s);
        __syncwarp();
        const uint4* src = (const uint4*)&s;
        uint4* dst = (uint4*)(out + idx);
        for (uint32_t i = lane; i < sizeof(ShadedMeshlet) / 16; i += 32) dst[i] = src[i];
        __syncwarp();
    }
}

// Clip position of vertex slot s of draw-relative meshlet m.
__device__ __forceinline__ float4 hook_vertex(const swr_fragment_source& src, uint32_t m, uint32_t s) {
    if (src.shaded) {
        const float* P = (const float*)((const uint8_t*)src.shaded + (size_t)m * sizeof(ShadedMeshlet) + 448);
        return make_float4(P[s], P[64 + s], P[128 + s], P[192 + s]);
    }
    const uint8_t* mp = (const uint8_t*)src.meshlets + (size_t)(src.meshlet_offset + m) * 1728u;
    const uint32_t nv = mp[44], nvr = min((nv + 15u) & ~15u, 64u);  // ShadeMeshlet's 16-vertex chunks
    const float* P = (const float*)(mp + 64);
    return s < nvr ? clip_transform(P[s], P[64 + s], P[128 + s], src.object_to_clip) : make_float4(0.f, 0.f, 0.f, 0.f);
}

template <class F0, class F1, class F2, class F3, class Ctx>
__device__ __forceinline__ void call_fragment(uint32_t id, const Ctx& ctx, const FragmentFramebuffer& fb, FragmentVars& v) {
    switch (id & 3) {  // GetDispatchTable fills the 4 slots round-robin (Rasterizer.h:356-360)
    case 0: F0{}(ctx, fb, v); break;
    case 1: F1{}(ctx, fb, v); break;
    case 2: F2{}(ctx, fb, v); break;
    default: F3{}(ctx, fb, v); break;
    }
}

// Rebuilds the triangle of vis-buffer rank R (TrianglePacket::Setup, the clipper and
// TriangleEdgeVars::Setup exactly as the raster ran them) and calls its fragment shader for the
// tile at (tx, ty), visible pixels `mask`. Called by the 16 lanes of a half-warp.
template <class F0, class F1, class F2, class F3, class Ctx>
__device__ void shade_tile_triangle(const swr_fragment_source& src, const Ctx& ctx, const FragmentFramebuffer& fb,
                                    uint32_t R, uint32_t mask, uint32_t tx, uint32_t ty, uint32_t l) {
    const RankFields f = decode_rank(R);
    const uint32_t m = f.meshlet - src.meshlet_offset;
    const uint8_t* rec = (const uint8_t*)src.meshlets + (size_t)f.meshlet * 1728u;
    const uint8_t* idx = src.shaded ? (const uint8_t*)src.shaded + (size_t)m * sizeof(ShadedMeshlet) + 64 : rec + 1344;
    const uint32_t raw0 = idx[f.prim], raw1 = idx[128 + f.prim], raw2 = idx[256 + f.prim];
    const float4 c0 = hook_vertex(src, m, preload64_index(raw0));
    const float4 c1 = hook_vertex(src, m, preload64_index(raw1));
    const float4 c2 = hook_vertex(src, m, preload64_index(raw2));
    Setup t;
    uint32_t bbMin, bbMax;
    float ru[3] = { 0.f, 0.f, 0.f }, rv[3] = { 0.f, 0.f, 0.f };
    if (!f.clipped) {
        tri_setup_ndc(project(c0.x, c0.y, c0.z, c0.w), project(c1.x, c1.y, c1.z, c1.w), project(c2.x, c2.y, c2.z, c2.w),
                      src.half_w, src.half_h, kCullNone, t, bbMin, bbMax);
    } else {
        const uint32_t codes = (vertex_code(c0, src.guard_x, src.guard_y) | vertex_code(c1, src.guard_x, src.guard_y) |
                                vertex_code(c2, src.guard_x, src.guard_y)) & 0x3Fu;
        ClipPoly P;
        clip_polygon({ c0.x, c0.y, c0.z, c0.w }, { c1.x, c1.y, c1.z, c1.w }, { c2.x, c2.y, c2.z, c2.w }, codes, src.guard_x,
                     src.guard_y, 6, P);
        Vtx a0, a1, a2;
        clip_fan(P, f.fan, a0, a1, a2, ru, rv);
        tri_setup(a0, a1, a2, src.half_w, src.half_h, kCullNone, t, bbMin, bbMax);
    }
    const Edges e = edge_vars(t, src.half_w, src.half_h);
    FragmentVars v;
    v.MeshletId = f.meshlet;
    v.PrimId = f.prim;
    v.VertexId[0] = raw0, v.VertexId[1] = raw1, v.VertexId[2] = raw2;
    v.TileOffset = (tx << 2) + ty * src.width;
    v.TileMask = mask;
    v.Lane = l;
    v.PixelX = tx + (l & 3), v.PixelY = ty + (l >> 2);
    int32_t e0, e1, e2;
    edge_values(e, v.PixelX, v.PixelY, e0, e1, e2);
    const float u = __int2float_rn(e1), w = __int2float_rn(e2);
    v.Depth = fragment_depth(e, u, w);
    float bu, bv;
    perspective_bary(u, w, t.W0, fmul(t.W0, e.rcpArea), fmul(t.W1, e.rcpArea), fmul(t.W2, e.rcpArea), f.clipped != 0,
                     ru, rv, bu, bv);
    v.Bary[0] = fsub(fsub(1.0f, bu), bv), v.Bary[1] = bu, v.Bary[2] = bv;
    uint32_t fsId;
    if (src.shaded) {
        fsId = ((const ShadedMeshlet*)src.shaded)[m].fragment_shader_id;
    } else {
        const uint32_t mat = *(const uint32_t*)(rec + 48);
        fsId = mat < src.num_materials ? src.material_fs_ids[mat] : 0u;
    }
    call_fragment<F0, F1, F2, F3>(fsId, ctx, fb, v);
}

// Fragment stage: a half-warp per 4x4 tile; the tile's visible triangles of the draw are shaded one
// after another (pixels grouped by rank), then the tile's keys are marked shaded.
template <class Ctx, class F0, class F1, class F2, class F3>
__global__ void __launch_bounds__(256) k_shade_fragments(const __grid_constant__ swr_fragment_source src,
                                                         const __grid_constant__ Ctx ctx) {
    const uint32_t lane = threadIdx.x & 31, l = lane & 15;
    const unsigned half = 0xFFFFu << (lane & 16);
    const uint32_t tilesX = src.width >> 2, tiles = tilesX * (src.height >> 2);
    const FragmentFramebuffer fb = { src.layers, src.layer_stride, src.width, src.height, src.num_layers };
    const uint32_t halves = (gridDim.x * blockDim.x) >> 4;
    for (uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 4; tile < tiles; tile += halves) {
        const uint32_t ty = (tile / tilesX) << 2, tx = (tile - (tile / tilesX) * tilesX) << 2;
        uint64_t* kp = src.keys + (tx << 2) + ty * src.width + l;
        const uint64_t key = *kp;
        const uint32_t low = (uint32_t)key, rank = 0xFFFFFFFEu - low;
        const bool mine = low != kKeyEmptyLow && (rank >> 11) - src.meshlet_offset < src.count;
        unsigned pend = (__ballot_sync(half, mine) & half) >> (lane & 16);
        while (pend) {
            const uint32_t R = __shfl_sync(half, rank, (lane & 16) | (__ffs(pend) - 1));
            const unsigned mask = (__ballot_sync(half, mine && rank == R) & half) >> (lane & 16);
            shade_tile_triangle<F0, F1, F2, F3>(src, ctx, fb, R, mask, tx, ty, l);
            pend &= ~mask;
        }
        if (mine) *kp = (key & 0xFFFFFFFF00000000ull) | kKeyEmptyLow;  // shaded: later draws see plain depth
    }
}

template <class... F>
struct FragTable {  // GetDispatchTable's round-robin of up to 4 entry points
    static_assert(sizeof...(F) >= 1 && sizeof...(F) <= 4, "1 to 4 fragment entry points");
    using L = std::tuple<F...>;
    template <size_t i>
    using at = typename std::tuple_element<i % sizeof...(F), L>::type;
};

}  // namespace hook

// Runs the fragment stage of a draw over src (from swr_fragment_source_get).
template <class Ctx, class... FragFn>
swr_status ShadeFragments(const swr_fragment_source& src, const Ctx& ctx, cudaStream_t st) {
    using T = hook::FragTable<FragFn...>;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t tiles = (src.width >> 2) * (src.height >> 2);
    const uint32_t blocks = (uint32_t)std::max(1, std::min((int)((tiles + 15) / 16), (sms > 0 ? sms : 148) * 8));
    hook::k_shade_fragments<Ctx, typename T::template at<0>, typename T::template at<1>, typename T::template at<2>,
                            typename T::template at<3>><<<blocks, 256, 0, st>>>(src, ctx);
    return cudaGetLastError() == cudaSuccess ? SWR_OK : SWR_ECUDA;  // the launch's error, if any, is consumed
}

// Rasterizer::DrawMeshlets(fb, count, ShaderBinding{GetDispatchTable<&MeshFn, &FragFn...>(), &ctx})
// (Rasterizer.h:213, 342-364) on the calling thread's library stream (swr_get_stream):
//  - MeshFn: a functor `void operator()(const Ctx&, uint32_t idx, swr::ShadedMeshlet& out) const`
//    called by the 32 lanes of a warp for draw-relative meshlet idx (out starts with PrimCount 0,
//    FrontCCW, FragmentShaderId 0), or swr::ShadeMeshletFn for the library's ShadeMeshlet;
//  - FragFn...: 1 to 4 functors `void operator()(const Ctx&, const swr::FragmentFramebuffer&,
//    swr::FragmentVars&) const`, selected by FragmentShaderId (round-robin as GetDispatchTable);
//  - sctx: the library-side context (scene, meshlet offset; for ShadeMeshletFn also object_to_clip
//    and cull_bitmap); ctx: the shaders' own context, copied to the kernels by value.
// With ShadeMeshletFn, alpha_test_all selects FS_EncodeGBuffer's alpha test (every textured
// material) instead of FS_EncodeSurfaceId's (materials with AlphaCutoff < 255).
template <class MeshFn, class Ctx, class... FragFn>
swr_status DrawMeshlets(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* sctx, const Ctx& ctx,
                        int alpha_test_all = 0) {
    cudaStream_t st = (cudaStream_t)swr_get_stream();
    if (count == 0) return SWR_OK;
    swr_fragment_source src;
    swr_status s;
    if constexpr (std::is_same<MeshFn, ShadeMeshletFn>::value) {
        s = swr_draw_meshlets_hooked(r, fb, count, sctx, alpha_test_all);
        if (s == SWR_OK) s = swr_fragment_source_get(r, fb, count, nullptr, sctx, &src);
        if (s == SWR_OK) s = ShadeFragments<Ctx, FragFn...>(src, ctx, st);
        return s;
    } else {
        ShadedMeshlet* buf = nullptr;
        if (cudaMallocAsync((void**)&buf, (size_t)count * sizeof(ShadedMeshlet), st) != cudaSuccess) return SWR_ENOMEM;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const uint32_t blocks = std::max(1u, std::min((count + 7) / 8, (uint32_t)(sms > 0 ? sms : 148) * 8u));
        hook::k_mesh_shader<Ctx, MeshFn><<<blocks, 256, 0, st>>>(ctx, count, buf);
        s = cudaGetLastError() == cudaSuccess ? SWR_OK : SWR_ECUDA;
        if (s == SWR_OK) s = swr_draw_shaded_meshlets(r, fb, count, buf, sctx);
        if (s == SWR_OK) s = swr_fragment_source_get(r, fb, count, buf, sctx, &src);
        if (s == SWR_OK) s = ShadeFragments<Ctx, FragFn...>(src, ctx, st);
        cudaFreeAsync(buf, st);
        return s;
    }
}

}  // namespace swr
