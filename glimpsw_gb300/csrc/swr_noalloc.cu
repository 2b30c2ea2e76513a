// swr_draw_meshlets_noalloc: the vis-buffer draw for callers that cannot allocate device memory.
//
// Some callers own every byte of device memory themselves (a renderer with its own pooled
// allocator, a runtime that forbids cudaMalloc after start-up, code running inside a host
// callback where CUDA allocation calls are not allowed). They cannot create the handles of the
// regular API, which allocate. This entry point takes raw device pointers for all inputs and
// outputs and keeps its working memory (vis-buffer keys, the large-triangle queue, control
// words and expanded material records) in one file-scope device array of fixed size, so the
// call itself allocates nothing. It reuses the regular draw kernels unchanged.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "swr_device.cuh"
#include "swr_internal.h"

namespace swr {
namespace {

constexpr size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Limits of the static working memory (about 9.3 MiB, held by every GPU that loads the library
// until the process exits).
constexpr uint32_t kNoAllocMaxPixels = 1u << 20;     // e.g. 1280x720 or 1024x1024
constexpr uint32_t kNoAllocMaxMaterials = 1024;
constexpr uint32_t kNoAllocQueue = 16384;            // large triangles; more are rasterized in place

constexpr size_t kOffControl = 0;                    // 16 x u64
constexpr size_t kOffMaterials = 256;
constexpr size_t kOffQueue = kOffMaterials + align256(kNoAllocMaxMaterials * sizeof(DevMaterial));
constexpr size_t kOffBases = kOffQueue + align256((size_t)kNoAllocQueue * sizeof(TriRec));
constexpr size_t kOffKeys = kOffBases + align256((size_t)kNoAllocQueue * sizeof(unsigned long long));
constexpr size_t kNoAllocBytes = kOffKeys + (size_t)kNoAllocMaxPixels * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

// In host code g_noallocScratch names a host-side stand-in, not device memory: the device address
// is looked up with the device current and cached per device, together with the identity of the
// context it was looked up in. A cudaDeviceReset ends that context; the next call sees a new
// context and looks the address up again.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Identity of the calling thread's current context (0 if none is current or the driver does not
// tell; the address is then looked up at every call).
unsigned long long current_context_id() {
    static CtxGetCurrentFn getCurrent = nullptr;
    static CtxGetIdFn getId = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getCurrent = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getId = (CtxGetIdFn)f;
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!getCurrent || !getId || getCurrent(&c) != CUDA_SUCCESS || !c || getId(c, &id) != CUDA_SUCCESS) return 0;
    return id + 1;
}

struct DeviceScratch {
    unsigned char* ptr;
    unsigned long long context;
};
std::mutex g_mu;
DeviceScratch g_scratch[64] = {};

// The working array's device address and the SM count of the current device.
swr_status scratch_for_current_device(unsigned char** out, int* sms) {
    int dev = 0;
    swr_status st = swr_internal_device(&dev, sms);
    if (st != SWR_OK) return st;
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceScratch& d = g_scratch[dev];
    const unsigned long long ctx = current_context_id();
    if (!d.ptr || ctx == 0 || ctx != d.context) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_draw_meshlets_noalloc: cudaGetSymbolAddress");
        d.ptr = (unsigned char*)p;
        d.context = current_context_id();  // the lookup made the context current if none was
    }
    *out = d.ptr;
    return SWR_OK;
}

// Material records for the draw kernel from one flag byte per material (bit 0: double-sided; the
// other bits are reserved). The entry point takes no textures, so no material is alpha-tested: every
// meshlet draws with the opaque shader, FragmentShaderId 0.
__global__ void k_expand_material_flags(const uint8_t* __restrict__ flags, uint32_t n, DevMaterial* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        DevMaterial m = {};
        m.is_double_sided = flags[i] & 1;
        m.alpha_cutoff = 255;
        out[i] = m;
    }
}

}  // namespace
}  // namespace swr

using namespace swr;

extern "C" swr_status swr_draw_meshlets_noalloc(const void* meshlets, uint32_t meshlet_offset, uint32_t count,
                                                const uint8_t* material_flags, uint32_t num_materials,
                                                const uint16_t* cull_bitmap, const float object_to_clip[16],
                                                uint32_t* surface_ids, float* depth, uint32_t width, uint32_t height,
                                                int enable_binning, int enable_clipping, int enable_guardband) {
    if (!meshlets || !object_to_clip || !surface_ids || !depth || (num_materials && !material_flags))
        return swr_internal_fail(SWR_EINVAL, "swr_draw_meshlets_noalloc: NULL argument");
    if (width == 0 || height == 0 || width % 4 || height % 4 || width > SWR_MAX_RENDER_SIZE || height > SWR_MAX_RENDER_SIZE)
        return swr_internal_fail(SWR_EINVAL, "swr_draw_meshlets_noalloc: size must be a non-zero multiple of 4, at most 2896");
    if ((uint64_t)width * height > kNoAllocMaxPixels)
        return swr_internal_fail(SWR_ECAPACITY, "swr_draw_meshlets_noalloc: width*height exceeds the 1048576 pixels of "
                                                "its static working memory; use swr_draw_meshlets");
    if (num_materials > kNoAllocMaxMaterials)
        return swr_internal_fail(SWR_ECAPACITY, "swr_draw_meshlets_noalloc: more than 1024 materials");
    if ((uint64_t)meshlet_offset + count > SWR_MAX_MESHLETS)
        return swr_internal_fail(SWR_EINVAL, "swr_draw_meshlets_noalloc: meshlet range above 2^21");
    if (count == 0) return SWR_OK;

    unsigned char* base = nullptr;
    int sms = 0;
    swr_status st = scratch_for_current_device(&base, &sms);
    if (st != SWR_OK) return st;
    cudaStream_t stream = swr_internal_stream();
    const uint32_t n = width * height;
    unsigned long long* keys = (unsigned long long*)(base + kOffKeys);
    DevMaterial* mats = (DevMaterial*)(base + kOffMaterials);

    // The array keeps the previous call's contents: the control words (work and queue counters,
    // status, perf counters) restart at zero and the keys are rebuilt from the caller's depth.
    cudaError_t e = cudaMemsetAsync(base + kOffControl, 0, 16 * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_draw_meshlets_noalloc: clear control words");
    if (num_materials) {
        LaunchScope ls("k_expand_material_flags", stream);
        k_expand_material_flags<<<(num_materials + 255) / 256, 256, 0, stream>>>(material_flags, num_materials, mats);
    }
    launch_init_keys((const uint32_t*)depth, keys, nullptr, n, stream);

    DrawArgs a = {};
    a.meshlets = (const uint8_t*)meshlets;
    a.materials = mats;
    a.numMaterials = num_materials;
    a.meshletOffset = meshlet_offset;
    a.count = count;
    a.cullBitmap = cull_bitmap;
    memcpy(a.m, object_to_clip, sizeof(a.m));
    a.halfW = (int)width / 2, a.halfH = (int)height / 2;
    a.width = width, a.height = height;
    a.bx = (float)SWR_MAX_RENDER_SIZE / (float)width;
    a.by = (float)SWR_MAX_RENDER_SIZE / (float)height;
    if (!enable_binning && !enable_guardband) a.bx = a.by = 1.0f;
    a.clipMode = (!enable_binning && enable_clipping) ? 1 : 0;
    a.countClipped = (enable_binning || enable_clipping) ? 1 : 0;
    a.keys = keys;
    a.s.control = (unsigned long long*)(base + kOffControl);
    a.s.big = (TriRec*)(base + kOffQueue);
    a.s.bigBase = (unsigned long long*)(base + kOffBases);
    a.s.bigCapacity = kNoAllocQueue;
    launch_draw(a, stream, sms);
    launch_finalize(keys, surface_ids, (uint32_t*)depth, n, stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_draw_meshlets_noalloc");
    return SWR_OK;
}
