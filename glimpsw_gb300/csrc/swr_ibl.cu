// Image-based lighting precompute (Shading.cpp:35-219): the diffuse irradiance map
// (GenerateIrradianceMap / PrefilterDiffuseIrradiance), the GGX-prefiltered radiance map with one
// roughness per mip level (GenerateRadianceMap / PrefilterEnvMap, Karis 2014) and the split-sum
// environment BRDF table (GenerateEnvBRDFLut / IntegrateBRDF). The reference computes them on the
// CPU and its frame driver never calls them. The radiance map has enough texels for one GPU thread
// each. The irradiance map (4,096 texels of 32,400 samples at 64x64) and the BRDF table have too few
// to fill the GPU that way, so their blocks work on 32 texels (one per lane) at a time: all warps but
// the first compute sample terms of those texels into shared memory and the first adds them in
// sample order.
//
// Exactness: every texel is an independent sum in the reference's order (its 16-lane tile
// decisions, `any(NoL > 0)` and SampleOctLevel's `any(mipFrac > 0)`, give the same value as a
// per-lane decision, because the lanes they add are exact zeros), with the reference's float
// operations in source order. The scalar terms the reference computes once per sample step
// (cosf / sinf of the irradiance integral's angles, the Hammersley points and simd::sincos of their
// azimuths) are computed on the host in the same operations and handed to the kernels as tables.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "swr_internal.h"
#include "swr_sample.cuh"
#include "swr_surface.cuh"

namespace swr {
namespace {

constexpr float kPi = 3.141592653589793f, kTau = 6.283185307179586f, kInvPi = 0.3183098861837907f;

// The per-sample scalars of the three integrals.
struct IblTables {
    const float* cosPhi;     // PrefilterDiffuseIrradiance: cosf(phi), sinf(phi) of each phi step
    const float* sinPhi;
    const float* cosTheta;   // cosf(theta), sinf(theta) of each theta step
    const float* sinTheta;
    uint32_t numPhi, numTheta;
    float irradianceScale;   // simd::pi * 1.0f / sampleCount
    const float* ham;        // Hammersley(i, n): Xi.y, cos(phi), sin(phi) with phi = 2 pi Xi.x (n = 128 | 1024)
};

__device__ __forceinline__ float unpack_f11_(uint32_t x) { x <<= 17; return __uint_as_float((x & 0x0FFE0000u) + 0x38000000u); }
__device__ __forceinline__ float unpack_f10_(uint32_t x) { x <<= 18; return __uint_as_float((x & 0x0FFC0000u) + 0x38000000u); }
__device__ __forceinline__ F3 unpack_r11g11b10(uint32_t p) { return { unpack_f11_(p >> 21), unpack_f11_(p >> 10), unpack_f10_(p) }; }
// R11G11B10f::Pack (Texture.h:146-167): clamping only.
__device__ __forceinline__ uint32_t pack_r11g11b10(F3 c) {
    auto f11 = [](float x) {
        x = vmax(x, 1.0f / (1 << 15));
        x = vmin(x, 130048.0f);
        return ((__float_as_uint(x) >> 17) & 0x3FFF) - 0x1C00;
    };
    auto f10 = [](float x) {
        x = vmax(x, 1.0f / (1 << 15));
        x = vmin(x, 129024.0f);
        return ((__float_as_uint(x) >> 18) & 0x1FFF) - 0x0E00;
    };
    return f11(c.x) << 21 | f11(c.y) << 10 | f10(c.z);
}

// SampleLevel<EnvSampler> (Texture.h:412-459: ClampToEdge, linear in both directions) of an
// R11G11B10 texture at (u, v), mip m, with SampleLinear's float path (Texture.h:506-575).
__device__ F3 sample_env_level(const DevTexture& t, float u, float v, int32_t mipIn) {
    int32_t ix = min(max(round2i(u * t.scale_lerp_u), 0), t.mask_lerp_u);
    int32_t iy = min(max(round2i(v * t.scale_lerp_v), 0), t.mask_lerp_v);
    const int32_t m = min(max(mipIn, 0), (int32_t)t.mip_levels - 1);
    const int32_t stride = (int32_t)t.row_shift - m;
    ix >>= m, iy >>= m;
    const uint32_t* base = t.data + t.mip_offsets[m & 15];
    const int32_t xf = max(ix - 127, 0), yf = max(iy - 127, 0);
    const int32_t tx = xf >> 8, ty = yf >> 8;
    const bool inX = ((tx + 1) << m) < (int32_t)t.width, inY = ((ty + 1) << m) < (int32_t)t.height;
    const uint32_t i00 = texel_offset(tx, ty, stride), i01 = texel_offset(tx, ty + (inY ? 1 : 0), stride);
    const F3 c00 = unpack_r11g11b10(base[i00]), c10 = unpack_r11g11b10(base[i00 + 8]);
    const F3 c01 = unpack_r11g11b10(base[i01]), c11 = unpack_r11g11b10(base[i01 + 8]);
    const float fs = 1.0f / 256;
    float fx = (float)(xf & 255) * fs;
    const float fy = (float)(yf & 255) * fs;
    if (!inX) fx = 0;
    const F3 ra = { c00.x + (c10.x - c00.x) * fx, c00.y + (c10.y - c00.y) * fx, c00.z + (c10.z - c00.z) * fx };
    const F3 rb = { c01.x + (c11.x - c01.x) * fx, c01.y + (c11.y - c01.y) * fx, c01.z + (c11.z - c01.z) * fx };
    return { ra.x + (rb.x - ra.x) * fy, ra.y + (rb.y - ra.y) * fy, ra.z + (rb.z - ra.z) * fy };
}

// SampleOctLevel<EnvSampler> (Texture.h:467-480): between mips trunc(level) and trunc(level) + 1.
__device__ F3 sample_oct_level(const DevTexture& t, F3 dir, float level) {
    float u, v;
    map_oct(dir, u, v);
    const int32_t baseMip = trunc2i(level);
    const F3 b = sample_env_level(t, u, v, baseMip);
    const float frac = level - (float)baseMip;
    if (frac > 0.0f && baseMip < (int32_t)t.mip_levels - 1) {
        const F3 l = sample_env_level(t, u, v, baseMip + 1);
        return { b.x + (l.x - b.x) * frac, b.y + (l.y - b.y) * frac, b.z + (l.z - b.z) * frac };
    }
    return b;
}

// TonemapSample / TonemapSampleInv (Shading.cpp:36-44).
__device__ __forceinline__ F3 tonemap_sample(F3 c, float sign) {
    const float luma = dot3(c, { 0.299f, 0.587f, 0.114f });
    const float r = approx_rcp(sign > 0 ? 1.0f + luma : 1.0f - luma);
    return { c.x * r, c.y * r, c.z * r };
}

// The tangent frame of ImportanceSampleGGX / PrefilterDiffuseIrradiance around N (Shading.cpp:64-67, 74-77).
__device__ __forceinline__ void tangent_frame(F3 N, F3& tx, F3& ty) {
    const bool nz = fabsf(N.z) < 0.999f;
    const F3 up = { nz ? 0.0f : 1.0f, 0.0f, nz ? 1.0f : 0.0f };
    tx = normalize3(cross3(up, N));
    ty = cross3(N, tx);
}

// ImportanceSampleGGX (Shading.cpp:56-70) with the sample's Xi.y and simd::cos / sin of its azimuth.
__device__ __forceinline__ F3 importance_sample_ggx(float xiY, float cphi, float sphi, float roughness, F3 N, F3 tx, F3 ty) {
    const float a = roughness * roughness;
    const float cosTheta = __fsqrt_rn((1.0f - xiY) / (1.0f + (a * a - 1.0f) * xiY));
    const float sinTheta = __fsqrt_rn(1.0f - cosTheta * cosTheta);
    const F3 H = { cphi * sinTheta, sphi * sinTheta, cosTheta };
    return { tx.x * H.x + ty.x * H.y + N.x * H.z, tx.y * H.x + ty.y * H.y + N.y * H.z, tx.z * H.x + ty.z * H.y + N.z * H.z };
}

// D_GGX (Shading.cpp:19-23).
__device__ __forceinline__ float d_ggx(float NoH, float roughness) {
    const float a = NoH * roughness;
    const float k = roughness * approx_rcp(1.0f - NoH * NoH + a * a);
    return k * k * kInvPi;
}

// simd::approx_log2 (SIMD.h:416-419).
__device__ __forceinline__ float approx_log2(float x) {
    return fmaf(__uint2float_rn(__float_as_uint(x)), 1.1920928955078125e-7f, -126.94269504f);
}

// Sums n sample terms of C channels for the block's 32 texels (lane l = texel l) in sample order.
// Warps 1 to W - 1 compute the terms k = base + j * (W - 1) + warp - 1 (j < S) of each chunk of
// (W - 1) * S samples into one of two shared buffers; after the chunk's barrier warp 0 adds them in
// order while the others compute the next chunk. Warp 0 only adds: its 3 dependent adds a term take
// a small fraction of the time the other warps spend on a chunk, so it never holds up a barrier. A
// buffer is written again two chunks later, after the next barrier, which warp 0 reaches only when
// it has added it. Returns the sums in warp 0's lanes.
template <int W, int S, int C, class TermFn>
__device__ __forceinline__ void ordered_block_sum(uint32_t n, TermFn term, float (&acc)[C], float* buf) {
    constexpr uint32_t K = (W - 1) * S;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < C; c++) acc[c] = 0.0f;
    for (uint32_t base = 0, it = 0; base < n; base += K, it++) {
        float* b = buf + (it & 1) * (K * C * 32);
        if (warp > 0) {
            for (uint32_t j = 0; j < S; j++) {
                const uint32_t r = j * (W - 1) + warp - 1;
                if (base + r < n) {
                    float t[C];
                    term(base + r, t);
                    for (int c = 0; c < C; c++) b[(r * C + c) * 32 + lane] = t[c];
                }
            }
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t m = min(K, n - base);
            for (uint32_t r = 0; r < m; r++)
                for (int c = 0; c < C; c++) acc[c] = acc[c] + b[(r * C + c) * 32 + lane];
        }
    }
}

constexpr int kIrrWarps = 32, kIrrSteps = 2, kBrdfWarps = 8, kBrdfSteps = 4;

// GenerateIrradianceMap (Shading.cpp:177-186) with PrefilterDiffuseIrradiance (72-102): level 0 of
// out. Sample k is phi step k / numTheta, theta step k % numTheta; its term s * cos(theta) *
// sin(theta) is added to the texel's sum in that order, as the reference's nested loops do.
__global__ void __launch_bounds__(kIrrWarps * 32) k_ibl_irradiance(DevTexture env, DevTexture out, uint32_t* outData, IblTables tb) {
    __shared__ float buf[2 * (kIrrWarps - 1) * kIrrSteps * 3 * 32];
    const uint32_t n = out.width * out.height;
    const uint32_t i = min(blockIdx.x * 32 + (threadIdx.x & 31), n - 1);  // lanes past the end repeat the last texel
    const uint32_t x = i % out.width, y = i / out.width;
    const float u = ((float)x + 0.5f) * (1.0f / (float)out.width), v = ((float)y + 0.5f) * (1.0f / (float)out.height);
    const F3 N = unmap_oct(u, v);
    F3 right, up;
    tangent_frame(N, right, up);
    float color[3];
    ordered_block_sum<kIrrWarps, kIrrSteps, 3>(tb.numPhi * tb.numTheta, [&](uint32_t k, float (&t)[3]) {
        const uint32_t p = k / tb.numTheta, q = k - p * tb.numTheta;
        const float cp = tb.cosPhi[p], sp = tb.sinPhi[p];
        const F3 tmp = { cp * right.x + sp * up.x, cp * right.y + sp * up.y, cp * right.z + sp * up.z };
        const float ct = tb.cosTheta[q], st = tb.sinTheta[q];
        const F3 dir = { ct * N.x + st * tmp.x, ct * N.y + st * tmp.y, ct * N.z + st * tmp.z };
        const F3 s = tonemap_sample(sample_oct_level(env, dir, 2.0f), 1.0f);
        t[0] = s.x * ct * st, t[1] = s.y * ct * st, t[2] = s.z * ct * st;
    }, color, buf);
    if (threadIdx.x >= 32 || blockIdx.x * 32 + threadIdx.x >= n) return;
    const float k = tb.irradianceScale;
    const F3 r = tonemap_sample({ color[0] * k, color[1] * k, color[2] * k }, -1.0f);
    outData[out.mip_offsets[0] + texel_offset((int32_t)x, (int32_t)y, (int32_t)out.row_shift)] = pack_r11g11b10(r);
}

// GenerateRadianceMap (Shading.cpp:187-201) with PrefilterEnvMap (105-147, 128 samples): every mip
// level of out, level L prefiltered at roughness L / (MipLevels - 1).
__global__ void k_ibl_radiance(DevTexture env, DevTexture out, uint32_t* outData, IblTables tb, uint32_t totalTexels) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= totalTexels) return;
    uint32_t level = 0, j = i;
    while (j >= (out.width >> level) * (out.height >> level)) j -= (out.width >> level) * (out.height >> level), level++;
    const uint32_t w = out.width >> level, h = out.height >> level;
    const uint32_t x = j % w, y = j / w;
    const float u = ((float)x + 0.5f) * (1.0f / (float)w), v = ((float)y + 0.5f) * (1.0f / (float)h);
    const F3 R = unmap_oct(u, v);
    const float roughness = vmax((float)level / ((float)out.mip_levels - 1.0f), 0.01f);  // std::max
    F3 tx, ty;
    tangent_frame(R, tx, ty);
    const uint32_t numSamples = 128;
    const float omegaP = 4.0f * kPi / (float)(6u * env.width * env.width);
    F3 pre = { 0.0f, 0.0f, 0.0f };
    float total = 0.0f;
    for (uint32_t s = 0; s < numSamples; s++) {
        const F3 H = importance_sample_ggx(tb.ham[3 * s], tb.ham[3 * s + 1], tb.ham[3 * s + 2], roughness, R, tx, ty);
        const float VoH = dot3(R, H);
        const float NoH = vmax(VoH, 0.0f);
        const F3 L = { 2.0f * VoH * H.x - R.x, 2.0f * VoH * H.y - R.y, 2.0f * VoH * H.z - R.z };
        const float NoL = vmax(dot3(R, L), 0.0f);
        if (NoL > 0.0f) {
            const float pdf = d_ggx(NoH, roughness) / 4.0f + 0.001f;
            const float omegaS = 1.0f / ((float)numSamples * pdf);
            const float mip = vmax(0.5f * approx_log2(omegaS / omegaP), 0.0f);
            const F3 c = tonemap_sample(sample_oct_level(env, L, mip), 1.0f);
            pre = { pre.x + c.x * NoL, pre.y + c.y * NoL, pre.z + c.z * NoL };
            total += NoL;
        }
    }
    const F3 r = tonemap_sample({ pre.x / total, pre.y / total, pre.z / total }, -1.0f);
    outData[out.mip_offsets[level & 15] + texel_offset((int32_t)x, (int32_t)y, (int32_t)out.row_shift - (int32_t)level)] =
        pack_r11g11b10(r);
}

// GenerateEnvBRDFLut (Shading.cpp:202-210) with IntegrateBRDF (149-175, 1024 samples): RG16f texel
// (scale, bias) at NoV = u, roughness = v. A sample with NoL <= 0 adds +0, as the reference's lanes
// with Gv = 0 do (Shading.cpp:167).
__global__ void __launch_bounds__(kBrdfWarps * 32) k_ibl_env_brdf(DevTexture out, uint32_t* outData, IblTables tb) {
    __shared__ float buf[2 * (kBrdfWarps - 1) * kBrdfSteps * 2 * 32];
    const uint32_t n = out.width * out.height;
    const uint32_t i = min(blockIdx.x * 32 + (threadIdx.x & 31), n - 1);
    const uint32_t x = i % out.width, y = i / out.width;
    const float NoV = ((float)x + 0.5f) * (1.0f / (float)out.width), roughness = ((float)y + 0.5f) * (1.0f / (float)out.height);
    const F3 N = { 0.0f, 0.0f, 1.0f };
    const F3 V = { __fsqrt_rn(1.0f - NoV * NoV), 0.0f, NoV };
    F3 tx, ty;
    tangent_frame(N, tx, ty);
    const uint32_t sampleCount = 1024;
    float acc[2];
    ordered_block_sum<kBrdfWarps, kBrdfSteps, 2>(sampleCount, [&](uint32_t s, float (&t)[2]) {
        const F3 H = importance_sample_ggx(tb.ham[3 * s], tb.ham[3 * s + 1], tb.ham[3 * s + 2], roughness, N, tx, ty);
        const float VdH = dot3(V, H);
        const F3 L = { 2.0f * VdH * H.x - V.x, 2.0f * VdH * H.y - V.y, 2.0f * VdH * H.z - V.z };
        const float VoH = vmax(0.0f, VdH), NoL = vmax(0.0f, L.z), NoH = vmax(0.0f, H.z);
        t[0] = 0.0f, t[1] = 0.0f;
        if (NoL > 0.0f) {
            // V_SmithGGXCorrelatedFast (Shading.cpp:24-28) with roughness^2
            const float r2 = roughness * roughness;
            const float a = 2.0f * NoL * NoV, b = NoL + NoV;
            const float G = 0.5f / fmaf(r2, b, fmaf(-r2, a, a));
            const float Gv = G * 4.0f * VoH * NoL / NoH;
            const float om = 1.0f - VoH;
            const float Fc = (om * om) * (om * om) * om;  // pow5
            t[0] = Gv * (1.0f - Fc), t[1] = Gv * Fc;
        }
    }, acc, buf);
    if (threadIdx.x >= 32 || blockIdx.x * 32 + threadIdx.x >= n) return;
    const uint32_t hx = __half_as_ushort(__float2half_rn(acc[0] * (1.0f / sampleCount)));
    const uint32_t hy = __half_as_ushort(__float2half_rn(acc[1] * (1.0f / sampleCount)));
    outData[out.mip_offsets[0] + texel_offset((int32_t)x, (int32_t)y, (int32_t)out.row_shift)] = hx | (hy << 16);
}

// ---------------------------------------------------------------------------- host tables
// simd::sincos_2pi (SIMD.h:390-409): sin and cos of 2 pi x by the reference's polynomials.
void sincos_2pi(float x, float& s, float& c) {
    x = x + 0.25f;
    x = x - std::nearbyint(x);
    const float x1 = std::fabs(x) - 0.25f;
    const float x2 = x1 * x1;
    s = std::fma(x2, std::fma(x2, std::fma(x2, -70.993433272f, 81.340768887f), -41.337142371f), 6.283164044f) * x1;
    c = std::fma(x2, std::fma(x2, std::fma(x2, -78.216131988f, 64.660541218f), -19.735752060f), 0.999993295f);
    uint32_t cb, xb;
    memcpy(&cb, &c, 4);
    memcpy(&xb, &x, 4);
    cb ^= xb & 0x80000000u;  // mulsign(r_cos, x)
    memcpy(&c, &cb, 4);
}

// Hammersley(i, n) (Shading.cpp:46-54), with simd::cos / sin (SIMD.h:411-413) of phi = 2 pi Xi.x
// (ImportanceSampleGGX, Shading.cpp:59): Xi.y, cos(phi), sin(phi) per sample.
std::vector<float> hammersley_table(uint32_t n) {
    std::vector<float> t(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        uint32_t bits = i;
        bits = (bits << 16) | (bits >> 16);
        bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
        bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
        bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
        bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
        const float xiX = (float)i / (float)n;
        const float xiY = (float)(bits * (1.0 / 4294967295.0));
        const float phi = (float)(2.0 * (double)kPi * (double)xiX);
        float s, c;
        sincos_2pi(phi * 0.15915494309189535f, s, c);
        t[3 * i] = xiY, t[3 * i + 1] = c, t[3 * i + 2] = s;
    }
    return t;
}

// The phi / theta steps of PrefilterDiffuseIrradiance (release build: 360 x 90) with their cosf / sinf.
void irradiance_steps(std::vector<float>& cp, std::vector<float>& sp, std::vector<float>& ct, std::vector<float>& st,
                      float& scale) {
    const float halfPi = (float)((double)kPi * 0.5);
    const float deltaPhi = (float)((double)kTau / 360.0), deltaTheta = (float)((double)halfPi / 90.0);
    for (float phi = 0.0f; phi < kTau; phi += deltaPhi) cp.push_back(cosf(phi)), sp.push_back(sinf(phi));
    for (float theta = 0.0f; theta < halfPi; theta += deltaTheta) ct.push_back(cosf(theta)), st.push_back(sinf(theta));
    const uint32_t sampleCount = (uint32_t)(cp.size() * ct.size());
    scale = kPi * 1.0f / (float)sampleCount;
}

// Uploads the tables (stream-ordered; freed after the kernels by cudaFreeAsync).
swr_status upload(const std::vector<float>& h, float** d, cudaStream_t st) {
    cudaError_t e = cudaMallocAsync((void**)d, h.size() * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_ibl: tables");
}

swr_status check_env(swr_texture env, const char* what) {
    if (!env) return swr_internal_fail(SWR_EINVAL, what);
    if (env->format != SWR_FORMAT_R11G11B10F || env->d.num_layers < 1)
        return swr_internal_fail(SWR_EINVAL, "swr_ibl: the environment map must be an R11G11B10 octahedral texture");
    return SWR_OK;
}

}  // namespace
}  // namespace swr

using namespace swr;

extern "C" {

swr_status swr_ibl_irradiance_map(swr_texture env, swr_texture out) {
    swr_status s = check_env(env, "swr_ibl_irradiance_map: NULL environment map");
    if (s != SWR_OK) return s;
    if (!out || out->format != SWR_FORMAT_R11G11B10F)
        return swr_internal_fail(SWR_EINVAL, "swr_ibl_irradiance_map: the output must be an R11G11B10 texture");
    std::vector<float> cp, sp, ct, stt;
    IblTables tb = {};
    irradiance_steps(cp, sp, ct, stt, tb.irradianceScale);
    cudaStream_t st = swr_internal_stream();
    float *dcp = nullptr, *dsp = nullptr, *dct = nullptr, *dst = nullptr;
    if ((s = upload(cp, &dcp, st)) != SWR_OK || (s = upload(sp, &dsp, st)) != SWR_OK || (s = upload(ct, &dct, st)) != SWR_OK ||
        (s = upload(stt, &dst, st)) != SWR_OK)
        return s;
    tb.cosPhi = dcp, tb.sinPhi = dsp, tb.cosTheta = dct, tb.sinTheta = dst;
    tb.numPhi = (uint32_t)cp.size(), tb.numTheta = (uint32_t)ct.size();
    const uint32_t n = out->d.width * out->d.height;
    {
        LaunchScope ls("k_ibl_irradiance", st);
        k_ibl_irradiance<<<(n + 31) / 32, kIrrWarps * 32, 0, st>>>(env->d, out->d, (uint32_t*)out->d.data, tb);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(dcp, st), cudaFreeAsync(dsp, st), cudaFreeAsync(dct, st), cudaFreeAsync(dst, st);
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_ibl_irradiance_map");
}

swr_status swr_ibl_radiance_map(swr_texture env, swr_texture out) {
    swr_status s = check_env(env, "swr_ibl_radiance_map: NULL environment map");
    if (s != SWR_OK) return s;
    if (!out || out->format != SWR_FORMAT_R11G11B10F || out->d.mip_levels < 2)
        return swr_internal_fail(SWR_EINVAL, "swr_ibl_radiance_map: the output must be an R11G11B10 texture with mips");
    IblTables tb = {};
    cudaStream_t st = swr_internal_stream();
    float* dh = nullptr;
    if ((s = upload(hammersley_table(128), &dh, st)) != SWR_OK) return s;
    tb.ham = dh;
    uint32_t total = 0;
    for (uint32_t l = 0; l < out->d.mip_levels; l++) total += (out->d.width >> l) * (out->d.height >> l);
    {
        LaunchScope ls("k_ibl_radiance", st);
        k_ibl_radiance<<<(total + 127) / 128, 128, 0, st>>>(env->d, out->d, (uint32_t*)out->d.data, tb, total);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(dh, st);
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_ibl_radiance_map");
}

swr_status swr_ibl_env_brdf_lut(swr_texture out) {
    if (!out || out->format != SWR_FORMAT_RG16F)
        return swr_internal_fail(SWR_EINVAL, "swr_ibl_env_brdf_lut: the output must be an RG16f texture");
    IblTables tb = {};
    cudaStream_t st = swr_internal_stream();
    float* dh = nullptr;
    swr_status s = upload(hammersley_table(1024), &dh, st);
    if (s != SWR_OK) return s;
    tb.ham = dh;
    const uint32_t n = out->d.width * out->d.height;
    {
        LaunchScope ls("k_ibl_env_brdf", st);
        k_ibl_env_brdf<<<(n + 31) / 32, kBrdfWarps * 32, 0, st>>>(out->d, (uint32_t*)out->d.data, tb);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(dh, st);
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_ibl_env_brdf_lut");
}

}  // extern "C"
