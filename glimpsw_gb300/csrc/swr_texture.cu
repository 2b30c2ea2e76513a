// Textures (Texture.h:314-636): TiledY8 storage, SetPixels and GenerateMips on the device.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>

#include "swr_device.cuh"
#include "swr_internal.h"

namespace swr {

// Texture2D::GetTexelOffset, TiledY8 (Texture.h:493-501).
__device__ __forceinline__ uint32_t texel_offset(uint32_t x, uint32_t y, uint32_t stride) {
    return (y & 7) | (x << 3) | ((y & ~7u) << stride);
}

// pixfmt helpers (Texture.h:28-67, 139-182).
__device__ __forceinline__ float4 unpack_rgba8(uint32_t p) {
    const float s = 1.0f / 255;
    return make_float4(fmul((float)(p & 255), s), fmul((float)((p >> 8) & 255), s), fmul((float)((p >> 16) & 255), s),
                       fmul((float)(p >> 24), s));
}
__device__ __forceinline__ uint32_t sat_u8(int32_t v) {
    int32_t s = min(max(v, -32768), 32767);  // packs_epi32
    return (uint32_t)min(max(s, 0), 255);    // packus_epi16
}
__device__ __forceinline__ uint32_t pack_rgba8(float4 v) {
    return sat_u8(round2i(fmul(v.x, 255.0f))) | (sat_u8(round2i(fmul(v.y, 255.0f))) << 8) |
           (sat_u8(round2i(fmul(v.z, 255.0f))) << 16) | (sat_u8(round2i(fmul(v.w, 255.0f))) << 24);
}
__device__ __forceinline__ float unpack_f11(uint32_t x) { x <<= 17; return __uint_as_float((x & 0x0FFE0000u) + 0x38000000u); }
__device__ __forceinline__ float unpack_f10(uint32_t x) { x <<= 18; return __uint_as_float((x & 0x0FFC0000u) + 0x38000000u); }
__device__ __forceinline__ uint32_t pack_f11(float x) {
    x = vmax(x, 1.0f / (1 << 15));
    x = vmin(x, 130048.0f);
    return ((__float_as_uint(x) >> 17) & 0x3FFF) - 0x1C00;
}
__device__ __forceinline__ uint32_t pack_f10(float x) {
    x = vmax(x, 1.0f / (1 << 15));
    x = vmin(x, 129024.0f);
    return ((__float_as_uint(x) >> 18) & 0x1FFF) - 0x0E00;
}

// SetPixels for TiledY8 (Texture.h:336-354): row-major source to tiled storage.
__global__ void k_set_pixels(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint32_t width,
                             uint32_t height, uint32_t rowShift) {
    const uint32_t n = width * height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t y = i / width, x = i - y * width;
        dst[texel_offset(x, y, rowShift)] = src[i];
    }
}

// GenerateMip (Texture.h:577-596): 2x2 box filter on unpacked texels, ((c00 + c10) + c01 + c11) * 0.25.
__global__ void k_generate_mip(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint32_t w, uint32_t h,
                               uint32_t sstride, uint32_t dstride, uint32_t format) {
    const uint32_t n = w * h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t y = i / w, x = i - y * w;
        uint32_t p00 = src[texel_offset(2 * x, 2 * y, sstride)], p10 = src[texel_offset(2 * x + 1, 2 * y, sstride)];
        uint32_t p01 = src[texel_offset(2 * x, 2 * y + 1, sstride)], p11 = src[texel_offset(2 * x + 1, 2 * y + 1, sstride)];
        uint32_t out;
        if (format == SWR_FORMAT_RGBA8U) {
            float4 a = unpack_rgba8(p00), b = unpack_rgba8(p10), c = unpack_rgba8(p01), d = unpack_rgba8(p11);
            float4 avg = make_float4(fmul(fadd(fadd(fadd(a.x, b.x), c.x), d.x), 0.25f),
                                     fmul(fadd(fadd(fadd(a.y, b.y), c.y), d.y), 0.25f),
                                     fmul(fadd(fadd(fadd(a.z, b.z), c.z), d.z), 0.25f),
                                     fmul(fadd(fadd(fadd(a.w, b.w), c.w), d.w), 0.25f));
            out = pack_rgba8(avg);
        } else if (format == SWR_FORMAT_R11G11B10F) {
            float r = fmul(fadd(fadd(fadd(unpack_f11(p00 >> 21), unpack_f11(p10 >> 21)), unpack_f11(p01 >> 21)), unpack_f11(p11 >> 21)), 0.25f);
            float g = fmul(fadd(fadd(fadd(unpack_f11(p00 >> 10), unpack_f11(p10 >> 10)), unpack_f11(p01 >> 10)), unpack_f11(p11 >> 10)), 0.25f);
            float b = fmul(fadd(fadd(fadd(unpack_f10(p00), unpack_f10(p10)), unpack_f10(p01)), unpack_f10(p11)), 0.25f);
            out = pack_f11(r) << 21 | pack_f11(g) << 10 | pack_f10(b);
        } else if (format == SWR_FORMAT_RG16F) {
            auto lo = [](uint32_t p) { return __half2float(__ushort_as_half((unsigned short)(p & 0xFFFF))); };
            auto hi = [](uint32_t p) { return __half2float(__ushort_as_half((unsigned short)(p >> 16))); };
            const float r = fmul(fadd(fadd(fadd(lo(p00), lo(p10)), lo(p01)), lo(p11)), 0.25f);
            const float g = fmul(fadd(fadd(fadd(hi(p00), hi(p10)), hi(p01)), hi(p11)), 0.25f);
            out = (uint32_t)__half_as_ushort(__float2half_rn(r)) | ((uint32_t)__half_as_ushort(__float2half_rn(g)) << 16);
        } else {
            out = __float_as_uint(fmul(fadd(fadd(fadd(__uint_as_float(p00), __uint_as_float(p10)), __uint_as_float(p01)),
                                            __uint_as_float(p11)), 0.25f));
        }
        dst[texel_offset(x, y, dstride)] = out;
    }
}

static int grid_for(uint32_t n) { return (int)std::max(1u, std::min((n + 255) / 256, 152u * 16)); }

}  // namespace swr

using namespace swr;

extern "C" {

// CreateTexture2D (Texture.h:599-636).
swr_status swr_texture_create(uint32_t format, uint32_t width, uint32_t height, uint32_t max_levels,
                              uint32_t num_layers, swr_texture* out) {
    if (!out) return swr_internal_fail(SWR_EINVAL, "swr_texture_create: out is NULL");
    if (format > SWR_FORMAT_RG16F) return swr_internal_fail(SWR_EINVAL, "swr_texture_create: unknown format");
    if (width < 8 || height < 4 || (width & (width - 1)) || (height & (height - 1)) || width > 16384 || height > 16384)
        return swr_internal_fail(SWR_EINVAL, "swr_texture_create: sizes must be powers of two, width >= 8, height >= 4");
    if (max_levels == 0 || max_levels > 16 || num_layers == 0 || num_layers > 64)
        return swr_internal_fail(SWR_EINVAL, "swr_texture_create: max_levels in [1,16], num_layers in [1,64]");
    swr_texture t = new (std::nothrow) swr_texture_t();
    if (!t) return swr_internal_fail(SWR_ENOMEM, "swr_texture_create: host allocation failed");
    DevTexture& d = t->d;
    memset(&d, 0, sizeof(d));
    uint32_t stride = 0, mip = 0;
    for (; mip < max_levels; mip++) {
        if ((width >> mip) < 4 || (height >> mip) < 4) break;
        d.mip_offsets[mip] = stride;
        stride += ((width >> mip) * (height >> mip) + 63) & ~63u;
    }
    if ((uint64_t)stride * num_layers >= 0x7FFFFFFFull) {
        delete t;
        return swr_internal_fail(SWR_EINVAL, "swr_texture_create: texture exceeds 2^31 texels");
    }
    d.width = width, d.height = height, d.mip_levels = mip, d.num_layers = num_layers;
    d.row_shift = (uint32_t)__builtin_ctz(std::max(width, 8u));
    d.layer_stride = stride;
    d.scale_u = (float)width, d.scale_v = (float)height;
    d.mask_u = (int32_t)width - 1, d.mask_v = (int32_t)height - 1;
    d.mask_lerp_u = (int32_t)(width << 8) - 1, d.mask_lerp_v = (int32_t)(height << 8) - 1;
    d.scale_lerp_u = (float)(d.mask_lerp_u + 1), d.scale_lerp_v = (float)(d.mask_lerp_v + 1);
    t->format = format;
    t->words = (size_t)stride * num_layers + 64;
    uint32_t* p = nullptr;
    cudaError_t e = cudaMalloc(&p, t->words * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, t->words * 4, swr_internal_stream());
    if (e != cudaSuccess) {
        cudaFree(p);
        delete t;
        return swr_internal_cuda_fail(e, "swr_texture_create");
    }
    d.data = p;
    *out = t;
    return SWR_OK;
}

swr_status swr_texture_destroy(swr_texture t) {
    if (!t) return SWR_OK;
    cudaFree((void*)t->d.data);
    delete t;
    return SWR_OK;
}

swr_status swr_texture_set_pixels(swr_texture t, const uint32_t* pixels, uint32_t stride, uint32_t layer) {
    if (!t || !pixels || layer >= t->d.num_layers || stride < t->d.width)
        return swr_internal_fail(SWR_EINVAL, "swr_texture_set_pixels: bad argument");
    cudaStream_t st = swr_internal_stream();
    uint32_t* tmp = nullptr;
    size_t bytes = (size_t)t->d.width * t->d.height * 4;
    cudaError_t e = cudaMallocAsync(&tmp, bytes, st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(tmp, (size_t)t->d.width * 4, pixels, (size_t)stride * 4, (size_t)t->d.width * 4, t->d.height,
                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        LaunchScope ls("k_set_pixels", st);
        k_set_pixels<<<grid_for(t->d.width * t->d.height), 256, 0, st>>>(
            tmp, (uint32_t*)t->d.data + (size_t)layer * t->d.layer_stride, t->d.width, t->d.height, t->d.row_shift);
        e = cudaGetLastError();
    }
    if (tmp) cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the source is caller-owned host memory
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_texture_set_pixels");
    return SWR_OK;
}

swr_status swr_texture_set_pixels_device(swr_texture t, const uint32_t* pixels_device, uint32_t stride, uint32_t layer) {
    if (!t || !pixels_device || layer >= t->d.num_layers || stride != t->d.width)
        return swr_internal_fail(SWR_EINVAL, "swr_texture_set_pixels_device: bad argument (stride must equal the width)");
    cudaStream_t st = swr_internal_stream();
    LaunchScope ls("k_set_pixels", st);
    k_set_pixels<<<grid_for(t->d.width * t->d.height), 256, 0, st>>>(
        pixels_device, (uint32_t*)t->d.data + (size_t)layer * t->d.layer_stride, t->d.width, t->d.height, t->d.row_shift);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_texture_set_pixels_device");
    return SWR_OK;
}

swr_status swr_texture_generate_mips(swr_texture t) {
    if (!t) return swr_internal_fail(SWR_EINVAL, "swr_texture_generate_mips: NULL texture");
    cudaStream_t st = swr_internal_stream();
    const DevTexture& d = t->d;
    for (uint32_t layer = 0; layer < d.num_layers; layer++) {
        for (uint32_t level = 1; level < d.mip_levels; level++) {
            uint32_t w = d.width >> level, h = d.height >> level;
            uint32_t* base = (uint32_t*)d.data + (size_t)layer * d.layer_stride;
            LaunchScope ls("k_generate_mip", st);
            k_generate_mip<<<grid_for(w * h), 256, 0, st>>>(base + d.mip_offsets[level - 1], base + d.mip_offsets[level], w, h,
                                                           d.row_shift - level + 1, d.row_shift - level, t->format);
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_texture_generate_mips");
    return SWR_OK;
}

swr_status swr_texture_info(swr_texture t, uint32_t* mip_levels, uint32_t* layer_stride, uint32_t mip_offsets[16]) {
    if (!t) return swr_internal_fail(SWR_EINVAL, "swr_texture_info: NULL texture");
    if (mip_levels) *mip_levels = t->d.mip_levels;
    if (layer_stride) *layer_stride = t->d.layer_stride;
    if (mip_offsets) memcpy(mip_offsets, t->d.mip_offsets, sizeof(t->d.mip_offsets));
    return SWR_OK;
}

swr_status swr_texture_get_data(swr_texture t, uint32_t* dest, size_t words) {
    if (!t || !dest || words > t->words) return swr_internal_fail(SWR_EINVAL, "swr_texture_get_data: bad argument");
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync(dest, t->d.data, words * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_texture_get_data");
    return SWR_OK;
}

swr_status swr_texture_set_data(swr_texture t, const uint32_t* src, size_t words) {
    if (!t || !src || words > t->words) return swr_internal_fail(SWR_EINVAL, "swr_texture_set_data: bad argument");
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync((void*)t->d.data, src, words * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_texture_set_data");
    return SWR_OK;
}

}  // extern "C"
