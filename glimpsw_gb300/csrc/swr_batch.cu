// Batched multi-view rendering: many views of different resolutions and meshlet ranges drawn by one
// persistent launch of the mesh stage, the whole frame (clear, frustum culling, draw, chunk raster)
// captured once into a CUDA graph and replayed; each view's layers are written from its keys by
// their next reader, as after a single draw (depth-only views: the depth layer alone). The
// reference renders one view per
// DrawMeshlets call (Main.cpp:216-245); each view of a batch gives exactly the vis-buffer of that
// call sequence (clear, CullMeshlets without depth map, DrawMeshlets), since keys stay per view.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/swr/hostmath.h"
#include "swr_device.cuh"
#include "swr_internal.h"

namespace swr {
namespace {

struct BatchView {              // device table for the batched clear and cull kernels
    float planes[5][4];         // CullMeshlets frustum planes 0..4 (Shading.cpp:806)
    uint32_t* layer0;
    uint32_t* layer1;
    unsigned long long* keys;
    uint32_t* groupMasks;       // one word per 32 draw positions (ViewParams::groupMasks)
    uint32_t pixels;            // width * height
    uint32_t* tileMin;          // per 4x4 tile depth bound
    uint32_t frustum, cone;     // tests of the batched cull: frustum planes, backface cone
    float eye[3];               // camera centre in object space (cone_camera)
};

// Framebuffer::Clear(color, depth) for every view; keys and tile depth bounds restart from the
// cleared depth.
__global__ void k_clear_views(const BatchView* __restrict__ views, uint32_t color, uint32_t depthBits) {
    const BatchView& v = views[blockIdx.y];
    const uint32_t hi = float_order(__uint_as_float(depthBits));
    const unsigned long long key = ((unsigned long long)hi << 32) | kKeyEmptyLow;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < v.pixels; i += gridDim.x * blockDim.x) {
        v.layer0[i] = color;
        v.layer1[i] = depthBits;
        v.keys[i] = key;
        if ((i & 15) == 0) v.tileMin[i >> 4] = hi;
    }
}

// CullMeshlets without a depth map (Shading.cpp:797-809, 865): frustum planes 0..4 and, when enabled,
// the backface-cone test (cone_culled). One draw position per thread for every view (all views of
// a batch draw the same meshlets in the same order): its meshlet's bounding sphere is loaded once
// and tested against each view's planes, kept in shared memory kCullViews views at a time. A warp's
// ballot is the view's mask of 32 consecutive positions, stored by the lane numbered after the view,
// so the mesh stage tests a fetched group with one word.
constexpr uint32_t kCullViews = 32;

__global__ void __launch_bounds__(256) k_cull_views(const BatchView* __restrict__ views, uint32_t numViews,
                                                    const uint8_t* __restrict__ meshlets, uint32_t first, uint32_t count,
                                                    uint32_t orderStride, const DevMaterial* __restrict__ materials,
                                                    uint32_t numMaterials) {
    __shared__ BatchView sv[kCullViews];
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    const bool valid = q < count;
    const uint8_t* rec = meshlets + (size_t)(first + (valid ? draw_order(q, count, orderStride) : 0u)) * kMeshletSize;
    const float4 s = valid ? *(const float4*)rec : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t group = q / 32;
    for (uint32_t v0 = 0; v0 < numViews; v0 += kCullViews) {
        const uint32_t nv = min(kCullViews, numViews - v0);
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < nv * (uint32_t)(sizeof(BatchView) / 4); k += blockDim.x)
            ((uint32_t*)sv)[k] = ((const uint32_t*)(views + v0))[k];
        __syncthreads();
        unsigned mine = 0;  // the mask of view v0 + lane
        for (uint32_t j = 0; j < nv; j++) {
            const BatchView& v = sv[j];
            bool visible = valid;
            if (visible && v.frustum) {
                for (int k = 0; k < 5; k++) {
                    float dist = fadd(ffma(s.x, v.planes[k][0], ffma(s.y, v.planes[k][1], fmul(s.z, v.planes[k][2]))), v.planes[k][3]);
                    visible = visible && (dist > -s.w);
                }
            }
            if (v.cone && visible) visible = !cone_culled(rec, v.eye[0], v.eye[1], v.eye[2], materials, numMaterials);
            const unsigned m = __ballot_sync(0xFFFFFFFFu, visible);
            if (lane == j) mine = m;
        }
        if (lane < nv && group * 32 < count) sv[lane].groupMasks[group] = mine;
    }
}

}  // namespace
}  // namespace swr

using namespace swr;

struct swr_batch_t {
    swr_rasterizer rast;
    swr_scene scene;
    uint32_t first, count, numViews;
    uint32_t cullFlags;  // SWR_CULL_FRUSTUM | SWR_CULL_BACKFACE_CONE
    uint32_t maxPixels;
    std::vector<swr_framebuffer> fbs;
    std::vector<uint8_t> depthOnly;  // per view: only the depth layer is written
    ViewParams* dViews = nullptr;
    BatchView* dBatch = nullptr;
    uint32_t* dViewStart = nullptr;
    uint32_t* dGroupMasks = nullptr;  // per view: the cull's masks of 32 draw positions
    DrawScratch scratch = {};
    uint32_t chunkTiles = 0, chunkTilesY = 0, warpsPerBlock = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long kernelNodes = 0;
    uint64_t sceneVersion = 0;     // scene->version the graph was recorded with
};

namespace {

int sm_count() { return swr_internal_sm_count(); }

swr_status upload_views(swr_batch b, const swr_view_desc* views) {
    std::vector<ViewParams> vp(b->numViews);
    std::vector<BatchView> bv(b->numViews);
    const uint32_t words = (b->count + 31) / 32;  // group masks per view
    for (uint32_t i = 0; i < b->numViews; i++) {
        const swr_view_desc& d = views[i];
        swr_framebuffer fb = b->fbs[i];
        float pv[16], objToClip[16], planes[6][4];
        swr_hostmath::mat4_mul(d.proj, d.view, pv);
        swr_hostmath::mat4_mul(pv, d.model, objToClip);
        swr_hostmath::frustum_planes(objToClip, planes);
        ViewParams& v = vp[i];
        memset(&v, 0, sizeof(v));
        memcpy(v.m, objToClip, sizeof(v.m));
        v.halfW = (int32_t)fb->width / 2, v.halfH = (int32_t)fb->height / 2;
        v.width = fb->width, v.height = fb->height;
        // binned or unbinned semantics follow the rasterizer's flags, as swr_draw_meshlets does
        v.bx = (float)SWR_MAX_RENDER_SIZE / (float)fb->width;
        v.by = (float)SWR_MAX_RENDER_SIZE / (float)fb->height;
        if (!b->rast->enable_binning && !b->rast->enable_guardband) v.bx = v.by = 1.0f;
        v.meshletOffset = b->first;
        v.count = b->count;
        v.orderStride = order_stride(b->count);
        v.keys = fb->keys;
        v.tileMin = fb->tileMin;
        v.groupMasks = b->cullFlags ? b->dGroupMasks + (size_t)i * words : nullptr;
        BatchView& w = bv[i];
        memset(&w, 0, sizeof(w));
        memcpy(w.planes, planes, sizeof(w.planes));
        w.layer0 = fb->layers;
        w.layer1 = fb->layers + fb->layer_stride;
        w.keys = fb->keys;
        w.tileMin = fb->tileMin;
        w.groupMasks = b->dGroupMasks + (size_t)i * words;
        w.pixels = fb->width * fb->height;
        w.frustum = (b->cullFlags & SWR_CULL_FRUSTUM) ? 1u : 0u;
        w.cone = ((b->cullFlags & SWR_CULL_BACKFACE_CONE) && swr_hostmath::cone_camera(objToClip, w.eye)) ? 1u : 0u;
        b->depthOnly[i] = d.depth_only != 0;
    }
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync(b->dViews, vp.data(), vp.size() * sizeof(ViewParams), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->dBatch, bv.data(), bv.size() * sizeof(BatchView), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host staging vectors die here
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch: view upload");
    return SWR_OK;
}

// The frame, recorded once on a private stream into a graph (event tracing is paused while
// capturing; the graph's kernels are counted at every replay).
swr_status capture(swr_batch b) {
    // the alpha pass's work list: one entry per (view, meshlet) work item
    const uint32_t items = b->count * b->numViews;
    if (b->scene->hasAlpha && b->scratch.alphaCapacity < items) {
        cudaFree(b->scratch.alphaList);
        b->scratch.alphaList = nullptr, b->scratch.alphaCapacity = 0;
        cudaError_t e = cudaMalloc(&b->scratch.alphaList, (size_t)std::max(items, 1u) * sizeof(uint32_t));
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch: alpha work list");
        b->scratch.alphaCapacity = std::max(items, 1u);
    }
    b->sceneVersion = b->scene->version;
    // The clear (bound by HBM writes) and the cull (by the records' sphere loads) are independent:
    // they run as two branches of the graph, joined before the mesh stage.
    cudaStream_t cs = nullptr, cs2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (cs) cudaStreamDestroy(cs);
        if (cs2) cudaStreamDestroy(cs2);
        if (fork) cudaEventDestroy(fork);
        return swr_internal_cuda_fail(e, "swr_batch: capture streams");
    }
    const bool prof = swr_internal_set_profiling(false);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const bool began = e == cudaSuccess;
    if (e == cudaSuccess) e = cudaEventRecord(fork, cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs2, fork, 0);
    if (e == cudaSuccess) {
        const uint32_t nv = b->numViews;
        const int blocksX = (int)std::min<uint32_t>((b->maxPixels + 255) / 256, 1024u);
        k_clear_views<<<dim3(blocksX, nv), 256, 0, cs2>>>(b->dBatch, 0xFF000000u, 0u);
        e = cudaEventRecord(join, cs2);
        if (b->cullFlags && b->count)
            k_cull_views<<<(b->count + 255) / 256, 256, 0, cs>>>(b->dBatch, nv, b->scene->meshlets, b->first, b->count,
                                                                order_stride(b->count), b->scene->materials,
                                                                b->scene->num_materials);
        cudaMemsetAsync(b->scratch.control, 0, 3 * sizeof(unsigned long long), cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, join, 0);
        DrawArgs a = {};
        a.meshlets = b->scene->meshlets;
        a.materials = b->scene->materials;
        a.numMaterials = b->scene->num_materials;
        a.clipMode = (!b->rast->enable_binning && b->rast->enable_clipping) ? 1 : 0;
        a.countClipped = (b->rast->enable_binning || b->rast->enable_clipping) ? 1 : 0;
        a.s = b->scratch;
        if (!b->scene->hasAlpha) a.s.alphaList = nullptr;  // no alpha pass
        a.views = b->dViews;
        a.viewStart = b->dViewStart;
        a.numViews = nv;
        a.chunkTiles = b->chunkTiles;
        a.chunkTilesY = b->chunkTilesY;
        a.warpsPerBlock = b->warpsPerBlock;
        launch_draw(a, cs, sm_count());
    }
    if (began) {  // a failed step still ends the capture before the streams go
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess) e = ec;
        if (e == cudaSuccess) b->graph = g;
        else if (g) cudaGraphDestroy(g);
    }
    swr_internal_set_profiling(prof);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e == cudaSuccess) {
        size_t n = 0;
        cudaGraphGetNodes(b->graph, nullptr, &n);
        std::vector<cudaGraphNode_t> nodes(n);
        cudaGraphGetNodes(b->graph, nodes.data(), &n);
        b->kernelNodes = 0;
        for (cudaGraphNode_t node : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(node, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) b->kernelNodes++;
        }
    }
    cudaStreamDestroy(cs);
    cudaStreamDestroy(cs2);
    cudaEventDestroy(fork);
    cudaEventDestroy(join);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch: graph capture");
    return SWR_OK;
}

void drop_graph(swr_batch b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr, b->graph = nullptr;
}

}  // namespace

extern "C" {

swr_status swr_batch_create(swr_rasterizer r, swr_scene s, uint32_t first, uint32_t count, const swr_view_desc* views,
                            uint32_t num_views, int frustum_cull, swr_batch* out) {
    if (!r || !s || !views || !out || num_views == 0) return swr_internal_fail(SWR_EINVAL, "swr_batch_create: bad argument");
    if ((uint64_t)first + count > s->count) return swr_internal_fail(SWR_EINVAL, "swr_batch_create: range outside the scene");
    if (num_views > 4096) return swr_internal_fail(SWR_EINVAL, "swr_batch_create: at most 4096 views");
    for (uint32_t i = 0; i < num_views; i++)
        if (!views[i].fb) return swr_internal_fail(SWR_EINVAL, "swr_batch_create: view without framebuffer");
    const uint64_t padded = ((uint64_t)count + kBatchGroup - 1) / kBatchGroup * kBatchGroup;  // a view's work positions
    if (padded * num_views >= (1ull << 32)) return swr_internal_fail(SWR_EINVAL, "swr_batch_create: too many work items");
    swr_batch b = new (std::nothrow) swr_batch_t();
    if (!b) return swr_internal_fail(SWR_ENOMEM, "swr_batch_create: host allocation failed");
    b->rast = r, b->scene = s, b->first = first, b->count = count, b->numViews = num_views, b->cullFlags = (uint32_t)frustum_cull & (SWR_CULL_FRUSTUM | SWR_CULL_BACKFACE_CONE);
    uint64_t totalTris = 0;
    for (uint32_t i = 0; i < num_views; i++) {
        b->fbs.push_back(views[i].fb);
        b->depthOnly.push_back(views[i].depth_only != 0);
        b->maxPixels = std::max(b->maxPixels, views[i].fb->width * views[i].fb->height);
        totalTris += (uint64_t)count * 32;
    }
    const uint32_t words = (count + 31) / 32;
    std::vector<uint32_t> start(num_views + 1);
    for (uint32_t i = 0; i <= num_views; i++) start[i] = i * (uint32_t)padded;
    cudaError_t e = cudaMalloc(&b->dViews, num_views * sizeof(ViewParams));
    if (e == cudaSuccess) e = cudaMalloc(&b->dBatch, num_views * sizeof(BatchView));
    if (e == cudaSuccess) e = cudaMalloc(&b->dViewStart, (num_views + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->dGroupMasks, (size_t)num_views * words * sizeof(uint32_t) + 16);
    if (e == cudaSuccess) e = cudaMemcpy(b->dViewStart, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    // the batch's own queue: a quarter of the triangles of every view; overflow is rasterized in place
    b->scratch.bigCapacity = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(totalTris, 1u << 18), 1u << 26);
    if (e == cudaSuccess) e = cudaMalloc(&b->scratch.control, 16 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->scratch.control, 0, 16 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->scratch.big, (size_t)b->scratch.bigCapacity * sizeof(TriRec));
    if (e == cudaSuccess) e = cudaMalloc(&b->scratch.bigBase, (size_t)b->scratch.bigCapacity * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        swr_batch_destroy(b);
        return swr_internal_cuda_fail(e, "swr_batch_create");
    }
    swr_status st = upload_views(b, views);
    if (st != SWR_OK) {
        swr_batch_destroy(b);
        return st;
    }
    *out = b;
    return SWR_OK;
}

swr_status swr_batch_set_views(swr_batch b, const swr_view_desc* views, uint32_t num_views) {
    if (!b || !views || num_views != b->numViews) return swr_internal_fail(SWR_EINVAL, "swr_batch_set_views: bad argument");
    for (uint32_t i = 0; i < num_views; i++)
        if (views[i].fb != b->fbs[i]) return swr_internal_fail(SWR_EINVAL, "swr_batch_set_views: framebuffers must not change");
    return upload_views(b, views);
}

swr_status swr_batch_set_tuning(swr_batch b, uint32_t chunk_tiles, uint32_t warps_per_block) {
    if (!b) return swr_internal_fail(SWR_EINVAL, "swr_batch_set_tuning: NULL batch");
    if (chunk_tiles && chunk_tiles != 2 && chunk_tiles != 4 && chunk_tiles != 8 && chunk_tiles != 16)
        return swr_internal_fail(SWR_EINVAL, "swr_batch_set_tuning: chunk_tiles must be 2, 4, 8 or 16 (8-64 px bins)");
    if (warps_per_block && warps_per_block != 4 && warps_per_block != 8 && warps_per_block != 16)
        return swr_internal_fail(SWR_EINVAL, "swr_batch_set_tuning: warps_per_block must be 4, 8 or 16");
    if (chunk_tiles != b->chunkTiles || b->chunkTilesY != 0 || warps_per_block != b->warpsPerBlock) drop_graph(b);
    b->chunkTiles = chunk_tiles, b->chunkTilesY = 0, b->warpsPerBlock = warps_per_block;
    return SWR_OK;
}

swr_status swr_batch_set_chunk_shape(swr_batch b, uint32_t chunk_w_tiles, uint32_t chunk_h_tiles) {
    if (!b) return swr_internal_fail(SWR_EINVAL, "swr_batch_set_chunk_shape: NULL batch");
    auto valid = [](uint32_t c) { return c == 2 || c == 4 || c == 8 || c == 16; };
    if (!valid(chunk_w_tiles) || !valid(chunk_h_tiles))
        return swr_internal_fail(SWR_EINVAL, "swr_batch_set_chunk_shape: chunk sides must be 2, 4, 8 or 16 tiles (8-64 px)");
    if (chunk_w_tiles != b->chunkTiles || chunk_h_tiles != b->chunkTilesY) drop_graph(b);
    b->chunkTiles = chunk_w_tiles, b->chunkTilesY = chunk_h_tiles;
    return SWR_OK;
}

swr_status swr_batch_render(swr_batch b) {
    if (!b) return swr_internal_fail(SWR_EINVAL, "swr_batch_render: NULL batch");
    if (b->exec && b->sceneVersion != b->scene->version) drop_graph(b);  // meshlets or materials moved
    if (!b->exec) {
        swr_status st = capture(b);
        if (st != SWR_OK) return st;
    }
    cudaStream_t st = swr_internal_stream();
    cudaError_t e;
    {
        LaunchScope ls("swr_batch_graph", st);
        e = cudaGraphLaunch(b->exec, st);
    }
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch_render");
    if (b->kernelNodes > 1) swr_internal_count_launches(b->kernelNodes - 1);
    for (uint32_t i = 0; i < b->numViews; i++) {  // the layers are written by their next reader
        b->fbs[i]->keys_valid = true;
        b->fbs[i]->layers_stale = b->depthOnly[i] ? kStaleDepth : kStaleAll;
    }
    return SWR_OK;
}

swr_status swr_batch_get_counters(swr_batch b, uint64_t out[SWR_NUM_COUNTERS]) {
    if (!b || !out) return swr_internal_fail(SWR_EINVAL, "swr_batch_get_counters: bad argument");
    unsigned long long c[16];
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync(c, b->scratch.control, sizeof(c), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch_get_counters");
    out[0] = c[3], out[1] = c[4], out[2] = c[5], out[3] = c[6];
    return SWR_OK;
}

swr_status swr_batch_reset_counters(swr_batch b) {
    if (!b) return swr_internal_fail(SWR_EINVAL, "swr_batch_reset_counters: NULL batch");
    cudaError_t e = cudaMemsetAsync(b->scratch.control + 3, 0, 4 * sizeof(unsigned long long), swr_internal_stream());
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_batch_reset_counters");
    return SWR_OK;
}

swr_status swr_batch_destroy(swr_batch b) {
    if (!b) return SWR_OK;
    drop_graph(b);
    cudaFree(b->dViews);
    cudaFree(b->dBatch);
    cudaFree(b->dViewStart);
    cudaFree(b->dGroupMasks);
    cudaFree(b->scratch.control);
    cudaFree(b->scratch.big);
    cudaFree(b->scratch.bigBase);
    cudaFree(b->scratch.alphaList);
    delete b;
    return SWR_OK;
}

}  // extern "C"
