// C ABI of libswr_gb300 (include/swr_gb300.h): handles, validation, errors and the host-side
// orchestration of the raster kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/swr/hostmath.h"
#include "swr_device.cuh"
#include "swr_internal.h"

using namespace swr;

namespace {

thread_local std::string t_lastError;
thread_local cudaStream_t t_stream = cudaStreamPerThread;

swr_status fail(swr_status code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_lastError = buf;
    return code;
}

swr_status cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? SWR_ENOMEM : SWR_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SWR_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

#define SWR_CHECK_LAUNCH(what)                           \
    do {                                                 \
        cudaError_t e_ = cudaGetLastError();             \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

int num_sms() { return swr_internal_sm_count(); }

constexpr uint32_t kDefaultBigCapacity = 1u << 18;

swr_status ensure_scratch(swr_rasterizer r) {
    DrawScratch& s = r->scratch;
    if (s.control != nullptr) return SWR_OK;
    SWR_CUDA(cudaMalloc(&s.control, 16 * sizeof(unsigned long long)));
    SWR_CUDA(cudaMemset(s.control, 0, 16 * sizeof(unsigned long long)));
    s.bigCapacity = kDefaultBigCapacity;
    // stream-ordered allocations, so size_queue can replace them with cudaFreeAsync
    SWR_CUDA(cudaMallocAsync(&s.big, (size_t)s.bigCapacity * sizeof(TriRec), t_stream));
    SWR_CUDA(cudaMallocAsync(&s.bigBase, (size_t)s.bigCapacity * sizeof(unsigned long long), t_stream));
    SWR_CUDA(cudaStreamSynchronize(t_stream));
    SWR_CUDA(cudaMallocHost(&r->hostStatus, sizeof(unsigned long long)));
    *r->hostStatus = 0;
    SWR_CUDA(cudaEventCreateWithFlags(&r->statusEvent, cudaEventDisableTiming));
    return SWR_OK;
}

// Sizes the large-triangle queue for a draw of `count` meshlets: a quarter of their triangles by
// default, all of them once a draw has overflowed. Reallocation is stream-ordered. A full queue
// never loses triangles (the draw kernel rasterizes them itself); it only costs time.
swr_status size_queue(swr_rasterizer r, uint32_t count) {
    if (r->statusPending && cudaEventQuery(r->statusEvent) == cudaSuccess) {
        r->statusPending = false;
        if (*r->hostStatus & kStatusBigOverflow) r->sawOverflow = true;
    }
    uint64_t want = (uint64_t)count * (r->sawOverflow ? 128u : 32u);
    want = std::min<uint64_t>(std::max<uint64_t>(want, kDefaultBigCapacity), 1u << 26);
    DrawScratch& s = r->scratch;
    if (r->fixedCapacity) {
        if (s.bigCapacity != r->fixedCapacity) s.bigCapacity = std::min(r->fixedCapacity, s.bigCapacity);
        if (s.bigCapacity == r->fixedCapacity) return SWR_OK;
        want = r->fixedCapacity;
    }
    if (want <= s.bigCapacity) return SWR_OK;
    SWR_CUDA(cudaFreeAsync(s.big, t_stream));
    SWR_CUDA(cudaFreeAsync(s.bigBase, t_stream));
    s.big = nullptr, s.bigBase = nullptr, s.bigCapacity = 0;
    SWR_CUDA(cudaMallocAsync(&s.big, (size_t)want * sizeof(TriRec), t_stream));
    SWR_CUDA(cudaMallocAsync(&s.bigBase, (size_t)want * sizeof(unsigned long long), t_stream));
    s.bigCapacity = (uint32_t)want;
    return SWR_OK;
}

// The alpha pass's work list holds one entry per work item of a draw (stream-ordered growth).
swr_status size_alpha_list(swr_rasterizer r, uint32_t count) {
    DrawScratch& s = r->scratch;
    if (count <= s.alphaCapacity) return SWR_OK;
    const uint32_t want = std::max(count, 1u << 16);
    if (s.alphaList) SWR_CUDA(cudaFreeAsync(s.alphaList, t_stream));
    s.alphaList = nullptr, s.alphaCapacity = 0;
    SWR_CUDA(cudaMallocAsync(&s.alphaList, (size_t)want * sizeof(uint32_t), t_stream));
    s.alphaCapacity = want;
    return SWR_OK;
}

}  // namespace

// ------------------------------------------------------------------ tracing
namespace {
struct ProfRec {
    const char* name;
    cudaEvent_t start, stop;
};
thread_local bool t_profiling = false;
thread_local std::vector<ProfRec> t_prof;
std::atomic<unsigned long long> g_launches{ 0 };
}  // namespace

swr::LaunchScope::LaunchScope(const char* name, cudaStream_t s) : st(s), rec(-1) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!t_profiling) return;
    ProfRec r{ name, nullptr, nullptr };
    if (cudaEventCreate(&r.start) != cudaSuccess || cudaEventCreate(&r.stop) != cudaSuccess) return;
    cudaEventRecord(r.start, st);
    t_prof.push_back(r);
    rec = (int)t_prof.size() - 1;
}
swr::LaunchScope::~LaunchScope() {
    if (rec >= 0) cudaEventRecord(t_prof[rec].stop, st);
}

bool swr_internal_set_profiling(bool on) {
    bool prev = t_profiling;
    t_profiling = on;
    return prev;
}
void swr_internal_count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

swr_status swr_internal_fail(swr_status code, const char* msg) { return fail(code, "%s", msg); }
swr_status swr_internal_cuda_fail(cudaError_t e, const char* what) { return cuda_fail(e, what); }
cudaStream_t swr_internal_stream() { return t_stream; }

namespace {
constexpr int kMaxDevices = 64;
std::atomic<int> g_smCount[kMaxDevices];  // 0: not queried yet
}  // namespace

swr_status swr_internal_device(int* dev, int* sms) {
    cudaError_t e = cudaGetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (*dev < 0 || *dev >= kMaxDevices) return fail(SWR_EINVAL, "device ordinal %d above %d", *dev, kMaxDevices - 1);
    int n = g_smCount[*dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, *dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute(MultiProcessorCount)");
        if (n <= 0) return fail(SWR_ECUDA, "device %d reports %d SMs", *dev, n);
        g_smCount[*dev].store(n, std::memory_order_relaxed);
    }
    *sms = n;
    return SWR_OK;
}

int swr_internal_sm_count() {
    int dev = 0, n = 0;
    return swr_internal_device(&dev, &n) == SWR_OK ? n : 148;
}

extern "C" {

const char* swr_last_error(void) { return t_lastError.c_str(); }

swr_status swr_set_stream(void* cuda_stream) {
    t_stream = cuda_stream ? (cudaStream_t)cuda_stream : cudaStreamPerThread;
    return SWR_OK;
}
void* swr_get_stream(void) { return (void*)t_stream; }

swr_status swr_synchronize(void) {
    SWR_CUDA(cudaStreamSynchronize(t_stream));
    return SWR_OK;
}

uint64_t swr_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

swr_status swr_profile_enable(int enable) {
    t_profiling = enable != 0;
    return SWR_OK;
}

swr_status swr_profile_collect(uint32_t max_records, const char** names, float* ms, uint32_t* count) {
    if (!count || (max_records && (!names || !ms))) return fail(SWR_EINVAL, "swr_profile_collect: bad argument");
    uint32_t n = 0;
    for (ProfRec& r : t_prof) {
        cudaError_t e = cudaEventSynchronize(r.stop);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.start, r.stop);
        if (e != cudaSuccess) return cuda_fail(e, "swr_profile_collect");
        if (n < max_records) names[n] = r.name, ms[n] = t;
        n++;
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    t_prof.clear();
    *count = n;
    return SWR_OK;
}

// ------------------------------------------------------------------ rasterizer
swr_status swr_rasterizer_create(uint32_t num_threads, swr_rasterizer* out) {
    (void)num_threads;
    if (!out) return fail(SWR_EINVAL, "swr_rasterizer_create: out is NULL");
    swr_rasterizer r = new (std::nothrow) swr_rasterizer_t();
    if (!r) return fail(SWR_ENOMEM, "swr_rasterizer_create: host allocation failed");
    r->enable_binning = 1, r->enable_clipping = 1, r->enable_guardband = 1;  // Rasterizer.h:206-208
    swr_status st = ensure_scratch(r);
    if (st != SWR_OK) {
        swr_rasterizer_destroy(r);
        return st;
    }
    *out = r;
    return SWR_OK;
}

swr_status swr_rasterizer_destroy(swr_rasterizer r) {
    if (!r) return SWR_OK;
    cudaFree(r->scratch.control);
    cudaFree(r->scratch.big);  // cudaFree synchronises for stream-ordered allocations
    cudaFree(r->scratch.bigBase);
    cudaFree(r->scratch.alphaList);
    if (r->hostStatus) cudaFreeHost(r->hostStatus);
    if (r->statusEvent) cudaEventDestroy(r->statusEvent);
    delete r;
    return SWR_OK;
}

swr_status swr_rasterizer_set_flags(swr_rasterizer r, int enable_binning, int enable_clipping, int enable_guardband) {
    if (!r) return fail(SWR_EINVAL, "swr_rasterizer_set_flags: NULL rasterizer");
    r->enable_binning = enable_binning != 0;
    r->enable_clipping = enable_clipping != 0;
    r->enable_guardband = enable_guardband != 0;
    return SWR_OK;
}

swr_status swr_rasterizer_set_queue_capacity(swr_rasterizer r, uint32_t triangles) {
    if (!r) return fail(SWR_EINVAL, "swr_rasterizer_set_queue_capacity: NULL rasterizer");
    r->fixedCapacity = triangles;
    return SWR_OK;
}

swr_status swr_rasterizer_get_counters(swr_rasterizer r, uint64_t out[SWR_NUM_COUNTERS]) {
    if (!r || !out) return fail(SWR_EINVAL, "swr_rasterizer_get_counters: NULL argument");
    unsigned long long c[16];
    SWR_CUDA(cudaMemcpyAsync(c, r->scratch.control, sizeof(c), cudaMemcpyDeviceToHost, t_stream));
    SWR_CUDA(cudaStreamSynchronize(t_stream));
    out[SWR_COUNTER_TRIANGLES_PROCESSED] = c[3];
    out[SWR_COUNTER_TRIANGLES_RASTERIZED] = c[4];
    out[SWR_COUNTER_TRIANGLES_CLIPPED] = c[5];
    out[SWR_COUNTER_BIN_QUEUE_FLUSHES] = c[6];
    return SWR_OK;
}

swr_status swr_rasterizer_reset_counters(swr_rasterizer r) {
    if (!r) return fail(SWR_EINVAL, "swr_rasterizer_reset_counters: NULL rasterizer");
    SWR_CUDA(cudaMemsetAsync(r->scratch.control + 3, 0, 4 * sizeof(unsigned long long), t_stream));
    return SWR_OK;
}

// ------------------------------------------------------------------ framebuffer
swr_status swr_framebuffer_create(uint32_t width, uint32_t height, uint32_t num_layers, swr_framebuffer* out) {
    if (!out) return fail(SWR_EINVAL, "swr_framebuffer_create: out is NULL");
    if (width == 0 || height == 0 || width % 4 || height % 4)
        return fail(SWR_EINVAL, "swr_framebuffer_create: %ux%u is not a non-zero multiple of 4", width, height);
    if (width > SWR_MAX_RENDER_SIZE || height > SWR_MAX_RENDER_SIZE)
        return fail(SWR_EINVAL, "swr_framebuffer_create: %ux%u exceeds MaxRenderSize %u", width, height, SWR_MAX_RENDER_SIZE);
    if (num_layers < 2 || num_layers > 8)
        return fail(SWR_EINVAL, "swr_framebuffer_create: num_layers %u outside [2, 8]", num_layers);
    swr_framebuffer fb = new (std::nothrow) swr_framebuffer_t();
    if (!fb) return fail(SWR_ENOMEM, "swr_framebuffer_create: host allocation failed");
    fb->width = width, fb->height = height, fb->tile_stride = width / 4;
    fb->layer_stride = (width * height + 63) & ~63u;  // CreateFramebuffer, Rasterizer.h:69
    fb->num_layers = num_layers;
    cudaError_t e = cudaMalloc(&fb->layers, ((size_t)fb->layer_stride * num_layers + 64) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&fb->keys, (size_t)fb->layer_stride * 8);
    if (e == cudaSuccess) e = cudaMalloc(&fb->tileMin, (size_t)fb->layer_stride / 16 * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(fb->layers, 0, ((size_t)fb->layer_stride * num_layers + 64) * 4, t_stream);
    if (e != cudaSuccess) {
        swr_framebuffer_destroy(fb);
        return cuda_fail(e, "swr_framebuffer_create");
    }
    fb->keys_valid = false;
    *out = fb;
    return SWR_OK;
}

swr_status swr_framebuffer_destroy(swr_framebuffer fb) {
    if (!fb) return SWR_OK;
    cudaFree(fb->layers);
    cudaFree(fb->keys);
    cudaFree(fb->tileMin);
    cudaFree(fb->counts);
    delete fb;
    return SWR_OK;
}

}  // extern "C"

swr_status swr_internal_finalize(swr_framebuffer fb) {
    if (fb->layers_stale == kStaleNone) return SWR_OK;
    launch_finalize(fb->keys, fb->layers_stale == kStaleDepth ? nullptr : fb->layers, fb->layers + fb->layer_stride,
                    fb->width * fb->height, t_stream);
    SWR_CHECK_LAUNCH("finalize the vis-buffer layers");
    fb->layers_stale = kStaleNone;
    return SWR_OK;
}

extern "C" {

swr_status swr_framebuffer_clear(swr_framebuffer fb, uint32_t color, float depth) {
    if (!fb) return fail(SWR_EINVAL, "swr_framebuffer_clear: NULL framebuffer");
    fb->layers_stale = kStaleNone;  // every layer word is overwritten
    uint32_t d;
    memcpy(&d, &depth, 4);
    launch_clear(fb->layers, fb->layers + fb->layer_stride, fb->keys, fb->tileMin, fb->width * fb->height, color, d,
                 t_stream);
    SWR_CHECK_LAUNCH("swr_framebuffer_clear");
    fb->keys_valid = true;
    return SWR_OK;
}

swr_status swr_framebuffer_clear_layer(swr_framebuffer fb, uint32_t layer, uint32_t value) {
    if (!fb || layer >= fb->num_layers) return fail(SWR_EINVAL, "swr_framebuffer_clear_layer: bad framebuffer or layer");
    swr_status st = swr_internal_finalize(fb);
    if (st != SWR_OK) return st;
    launch_fill(fb->layers + (size_t)layer * fb->layer_stride, fb->width * fb->height, value, t_stream);
    SWR_CHECK_LAUNCH("swr_framebuffer_clear_layer");
    if (layer <= 1) fb->keys_valid = false;
    return SWR_OK;
}

swr_status swr_framebuffer_get_pixels_device(swr_framebuffer fb, uint32_t layer, uint32_t* dest_device) {
    if (!fb || layer >= fb->num_layers || !dest_device)
        return fail(SWR_EINVAL, "swr_framebuffer_get_pixels_device: bad argument");
    swr_status st = swr_internal_finalize(fb);
    if (st != SWR_OK) return st;
    launch_detile(fb->layers + (size_t)layer * fb->layer_stride, dest_device, fb->width, fb->height, fb->width, t_stream);
    SWR_CHECK_LAUNCH("swr_framebuffer_get_pixels_device");
    return SWR_OK;
}

swr_status swr_framebuffer_get_pixels(swr_framebuffer fb, uint32_t layer, uint32_t* dest, uint32_t stride) {
    if (!fb || layer >= fb->num_layers || !dest || stride < fb->width)
        return fail(SWR_EINVAL, "swr_framebuffer_get_pixels: bad argument");
    swr_status st = swr_internal_finalize(fb);
    if (st != SWR_OK) return st;
    const uint32_t* src = fb->layers + (size_t)layer * fb->layer_stride;
    // Pinned host memory the device can address is written by the detiling kernel itself, over the
    // host link, with no staging copy; other memory goes through a device buffer and a copy.
    cudaPointerAttributes pa = {};
    if (cudaPointerGetAttributes(&pa, dest) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
        launch_detile(src, (uint32_t*)pa.devicePointer, fb->width, fb->height, stride, t_stream);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(t_stream);
        if (e != cudaSuccess) return cuda_fail(e, "swr_framebuffer_get_pixels");
        return SWR_OK;
    }
    cudaGetLastError();  // an unregistered pointer is not an error
    uint32_t* tmp = nullptr;
    SWR_CUDA(cudaMallocAsync(&tmp, (size_t)fb->width * fb->height * 4, t_stream));
    launch_detile(src, tmp, fb->width, fb->height, fb->width, t_stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(dest, (size_t)stride * 4, tmp, (size_t)fb->width * 4, (size_t)fb->width * 4, fb->height,
                              cudaMemcpyDeviceToHost, t_stream);
    cudaFreeAsync(tmp, t_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t_stream);
    if (e != cudaSuccess) return cuda_fail(e, "swr_framebuffer_get_pixels");
    return SWR_OK;
}

swr_status swr_framebuffer_layer_data(swr_framebuffer fb, uint32_t layer, void** out_device_ptr) {
    if (!fb || layer >= fb->num_layers || !out_device_ptr) return fail(SWR_EINVAL, "swr_framebuffer_layer_data: bad argument");
    swr_status st = swr_internal_finalize(fb);
    if (st != SWR_OK) return st;
    *out_device_ptr = fb->layers + (size_t)layer * fb->layer_stride;
    return SWR_OK;
}

swr_status swr_framebuffer_invalidate(swr_framebuffer fb) {
    if (!fb) return fail(SWR_EINVAL, "swr_framebuffer_invalidate: NULL framebuffer");
    swr_status st = swr_internal_finalize(fb);
    if (st != SWR_OK) return st;
    fb->keys_valid = false;
    return SWR_OK;
}

swr_status swr_framebuffer_size(swr_framebuffer fb, uint32_t* width, uint32_t* height, uint32_t* layer_stride,
                                uint32_t* num_layers) {
    if (!fb) return fail(SWR_EINVAL, "swr_framebuffer_size: NULL framebuffer");
    if (width) *width = fb->width;
    if (height) *height = fb->height;
    if (layer_stride) *layer_stride = fb->layer_stride;
    if (num_layers) *num_layers = fb->num_layers;
    return SWR_OK;
}

// ------------------------------------------------------------------ scene
swr_status swr_scene_create(swr_scene* out) {
    if (!out) return fail(SWR_EINVAL, "swr_scene_create: out is NULL");
    swr_scene s = new (std::nothrow) swr_scene_t();
    if (!s) return fail(SWR_ENOMEM, "swr_scene_create: host allocation failed");
    *out = s;
    return SWR_OK;
}

swr_status swr_scene_destroy(swr_scene s) {
    if (!s) return SWR_OK;
    cudaFree(s->meshlets);
    cudaFree(s->materials);
    cudaFree(s->fsIds);
    delete s;
    return SWR_OK;
}

swr_status swr_scene_upload_meshlets(swr_scene s, const void* meshlets, uint32_t first, uint32_t count) {
    if (!s || (!meshlets && count)) return fail(SWR_EINVAL, "swr_scene_upload_meshlets: bad argument");
    uint64_t end = (uint64_t)first + count;
    if (end > SWR_MAX_MESHLETS)
        return fail(SWR_EINVAL, "swr_scene_upload_meshlets: %llu meshlets exceed the limit %u", (unsigned long long)end,
                    SWR_MAX_MESHLETS);
    // Records are not inspected on the host (that would cost a cache miss per meshlet); kernels
    // clamp NumVertices to 64 and NumTriangles to 128, the sizes of the record's arrays.
    if (end > s->capacity) {
        uint32_t cap = (uint32_t)std::max<uint64_t>(end, (uint64_t)s->capacity * 3 / 2);
        cap = std::min(cap, SWR_MAX_MESHLETS);
        uint8_t* p = nullptr;
        SWR_CUDA(cudaMalloc(&p, (size_t)cap * kMeshletSize));
        if (s->meshlets) {
            SWR_CUDA(cudaMemcpyAsync(p, s->meshlets, (size_t)s->count * kMeshletSize, cudaMemcpyDeviceToDevice, t_stream));
            SWR_CUDA(cudaStreamSynchronize(t_stream));
            cudaFree(s->meshlets);
        }
        s->meshlets = p;
        s->capacity = cap;
        s->version++;
    }
    if (count)
        SWR_CUDA(cudaMemcpyAsync(s->meshlets + (size_t)first * kMeshletSize, meshlets, (size_t)count * kMeshletSize,
                                 cudaMemcpyHostToDevice, t_stream));
    s->count = std::max(s->count, (uint32_t)end);
    return SWR_OK;
}

swr_status swr_scene_set_materials(swr_scene s, const swr_material* materials, uint32_t count) {
    if (!s || (!materials && count)) return fail(SWR_EINVAL, "swr_scene_set_materials: bad argument");
    std::vector<DevMaterial> h(count);
    std::vector<uint8_t> fsIds(count);
    bool hasAlpha = false, hasAlphaAll = false;
    for (uint32_t i = 0; i < count; i++) {
        DevMaterial& d = h[i];
        memset(&d, 0, sizeof(d));
        d.is_double_sided = materials[i].is_double_sided != 0;
        d.alpha_cutoff = materials[i].alpha_cutoff;
        if (materials[i].texture) {
            d.has_texture = 1;
            d.tex = materials[i].texture->d;
        }
        hasAlpha = hasAlpha || material_alpha_tested(d);
        hasAlphaAll = hasAlphaAll || material_alpha_tested_all(d);
        fsIds[i] = material_alpha_tested(d) ? 1 : 0;
    }
    cudaFree(s->materials);
    cudaFree(s->fsIds);
    s->materials = nullptr;
    s->fsIds = nullptr;
    s->num_materials = 0;
    s->hasAlpha = hasAlpha;
    s->hasAlphaAll = hasAlphaAll;
    s->version++;
    if (count) {
        SWR_CUDA(cudaMalloc(&s->materials, count * sizeof(DevMaterial)));
        SWR_CUDA(cudaMemcpy(s->materials, h.data(), count * sizeof(DevMaterial), cudaMemcpyHostToDevice));
        SWR_CUDA(cudaMalloc(&s->fsIds, count));
        SWR_CUDA(cudaMemcpy(s->fsIds, fsIds.data(), count, cudaMemcpyHostToDevice));
    }
    s->num_materials = count;
    return SWR_OK;
}

swr_status swr_scene_meshlets_device(swr_scene s, const void** out) {
    if (!s || !out) return fail(SWR_EINVAL, "swr_scene_meshlets_device: bad argument");
    *out = s->meshlets;
    return SWR_OK;
}

swr_status swr_scene_meshlet_count(swr_scene s, uint32_t* out) {
    if (!s || !out) return fail(SWR_EINVAL, "swr_scene_meshlet_count: bad argument");
    *out = s->count;
    return SWR_OK;
}

// ------------------------------------------------------------------ draw
}  // extern "C"

namespace {

enum class DrawKind { VisBuffer, Overdraw, Hooked };

// One draw's visibility: the mesh stage (ShadeMeshlet, or the records of a user mesh shader) and the
// chunk stage into the framebuffer's keys. Vis-buffer draws leave the layers pending
// (layers_stale); overdraw draws finalize their counters; hooked draws start from keys with no
// pending fragments, so that the fragment stage (swr_fragment_source_get) finds this draw's alone.
swr_status draw_impl(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* ctx, DrawKind kind,
                     const void* shaded, bool alphaAll, const char* what) {
    if (!r || !fb || !ctx || !ctx->scene) return fail(SWR_EINVAL, "%s: NULL argument", what);
    const bool overdraw = kind == DrawKind::Overdraw;
    swr_scene sc = ctx->scene;
    if ((uint64_t)ctx->meshlet_offset + count > sc->count)
        return fail(SWR_EINVAL, "%s: meshlets [%u, %llu) outside the scene's %u", what, ctx->meshlet_offset,
                    (unsigned long long)ctx->meshlet_offset + count, sc->count);
    if (count == 0) return SWR_OK;
    const bool hasAlpha = !overdraw && (alphaAll ? sc->hasAlphaAll : sc->hasAlpha);
    swr_status st = ensure_scratch(r);
    if (st == SWR_OK) st = size_queue(r, count);
    if (st == SWR_OK && hasAlpha) st = size_alpha_list(r, count);
    if (st != SWR_OK) return st;
    if (overdraw && !fb->counts) SWR_CUDA(cudaMalloc(&fb->counts, (size_t)fb->layer_stride * 8));
    if ((overdraw || kind == DrawKind::Hooked) && (st = swr_internal_finalize(fb)) != SWR_OK) return st;
    if (!fb->keys_valid || kind == DrawKind::Hooked) {
        launch_init_keys(fb->layers + fb->layer_stride, fb->keys, fb->tileMin, fb->width * fb->height, t_stream);
        SWR_CHECK_LAUNCH("draw: init keys");
        fb->keys_valid = true;
    }
    DrawArgs a = {};
    a.meshlets = sc->meshlets;
    a.materials = sc->materials;
    a.numMaterials = sc->num_materials;
    a.meshletOffset = ctx->meshlet_offset;
    a.count = count;
    a.cullBitmap = shaded ? nullptr : ctx->cull_bitmap;
    memcpy(a.m, ctx->object_to_clip, sizeof(a.m));
    a.halfW = (int)fb->width / 2, a.halfH = (int)fb->height / 2;
    a.width = fb->width, a.height = fb->height;
    // DrawMeshletsST honours EnableGuardband (Rasterizer.cpp:155-156); the binned path does not (509).
    a.bx = (float)SWR_MAX_RENDER_SIZE / (float)fb->width;
    a.by = (float)SWR_MAX_RENDER_SIZE / (float)fb->height;
    if (!r->enable_binning && !r->enable_guardband) a.bx = a.by = 1.0f;
    a.clipMode = (!r->enable_binning && r->enable_clipping) ? 1 : 0;
    a.countClipped = (r->enable_binning || r->enable_clipping) ? 1 : 0;
    a.keys = fb->keys;
    a.tileMin = fb->tileMin;
    a.s = r->scratch;
    a.shaded = (const uint8_t*)shaded;
    a.alphaAll = alphaAll ? 1u : 0u;
    if (!hasAlpha) a.s.alphaList = nullptr;  // no alpha pass
    if (overdraw) {  // no depth test: no tile depth bounds; counters restart per draw
        a.tileMin = nullptr;
        a.counts = fb->counts;
        SWR_CUDA(cudaMemsetAsync(fb->counts, 0, (size_t)fb->width * fb->height * 8, t_stream));
    }
    SWR_CUDA(cudaMemsetAsync(r->scratch.control, 0, 3 * sizeof(unsigned long long), t_stream));
    launch_draw(a, t_stream, num_sms());
    SWR_CHECK_LAUNCH(what);
    if (!r->statusPending) {
        SWR_CUDA(cudaMemcpyAsync(r->hostStatus, r->scratch.control + 2, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, t_stream));
        SWR_CUDA(cudaEventRecord(r->statusEvent, t_stream));
        r->statusPending = true;
    }
    if (overdraw) {
        launch_finalize_overdraw(fb->keys, fb->counts, fb->layers, fb->layers + fb->layer_stride, fb->width * fb->height,
                                 t_stream);
        fb->keys_valid = false;  // the keys hold the maximum depth of all samples, not vis-buffer keys
        SWR_CHECK_LAUNCH("swr_draw_meshlets: finalize");
    } else {
        fb->layers_stale = kStaleAll;  // written by the next reader of the layers
    }
    return SWR_OK;
}

}  // namespace

extern "C" {

swr_status swr_draw_meshlets(swr_rasterizer r, swr_framebuffer fb, uint32_t count, uint32_t shader_table,
                             const swr_shading_context* ctx) {
    if (shader_table == SWR_SHADER_DEFERRED) return swr_internal_draw_deferred(r, fb, count, ctx);
    if (shader_table != SWR_SHADER_VISBUFFER && shader_table != SWR_SHADER_OVERDRAW)
        return fail(SWR_EINVAL, "swr_draw_meshlets: unknown shader table %u", shader_table);
    return draw_impl(r, fb, count, ctx, shader_table == SWR_SHADER_OVERDRAW ? DrawKind::Overdraw : DrawKind::VisBuffer,
                     nullptr, false, "swr_draw_meshlets");
}

swr_status swr_draw_meshlets_hooked(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* ctx,
                                    int alpha_test_all) {
    return draw_impl(r, fb, count, ctx, DrawKind::Hooked, nullptr, alpha_test_all != 0, "swr_draw_meshlets_hooked");
}

swr_status swr_draw_shaded_meshlets(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const void* shaded_device,
                                    const swr_shading_context* ctx) {
    if (!shaded_device && count) return fail(SWR_EINVAL, "swr_draw_shaded_meshlets: NULL records");
    if (((uintptr_t)shaded_device & 15) != 0) return fail(SWR_EINVAL, "swr_draw_shaded_meshlets: records not 16-byte aligned");
    return draw_impl(r, fb, count, ctx, DrawKind::Hooked, shaded_device, false, "swr_draw_shaded_meshlets");
}

swr_status swr_fragment_source_get(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const void* shaded_device,
                                   const swr_shading_context* ctx, swr_fragment_source* out) {
    if (!r || !fb || !ctx || !ctx->scene || !out) return fail(SWR_EINVAL, "swr_fragment_source_get: NULL argument");
    if (!fb->keys_valid) return fail(SWR_EINVAL, "swr_fragment_source_get: no hooked draw into this framebuffer");
    swr_scene sc = ctx->scene;
    if (fb->layers_stale != kStaleNone) {  // the draw's depth; layer 0 is the fragment stage's
        launch_finalize(fb->keys, nullptr, fb->layers + fb->layer_stride, fb->width * fb->height, t_stream);
        SWR_CHECK_LAUNCH("swr_fragment_source_get: depth");
        fb->layers_stale = kStaleNone;
    }
    memset(out, 0, sizeof(*out));
    out->keys = (uint64_t*)fb->keys;
    out->layers = fb->layers;
    out->width = fb->width, out->height = fb->height, out->layer_stride = fb->layer_stride, out->num_layers = fb->num_layers;
    out->meshlets = sc->meshlets;
    out->shaded = shaded_device;
    out->material_fs_ids = sc->fsIds;
    out->num_materials = sc->num_materials;
    out->meshlet_offset = ctx->meshlet_offset, out->count = count;
    memcpy(out->object_to_clip, ctx->object_to_clip, sizeof(out->object_to_clip));
    out->guard_x = (float)SWR_MAX_RENDER_SIZE / (float)fb->width;
    out->guard_y = (float)SWR_MAX_RENDER_SIZE / (float)fb->height;
    if (!r->enable_binning && !r->enable_guardband) out->guard_x = out->guard_y = 1.0f;
    out->half_w = (int32_t)fb->width / 2, out->half_h = (int32_t)fb->height / 2;
    out->clip_mode = (!r->enable_binning && r->enable_clipping) ? 1u : 0u;
    return SWR_OK;
}

}  // extern "C"
