// Learned texture decoder on the sm_103a tensor cores: training step (forward, backward and
// weight gradients), Adam, latent initialisation and export, and the inference decoder that the
// neural resolve feeds with texel requests grouped by material.
//
// Latent level k has the resolution of texture level k + 2. A texel (texture level L, x, y) of a
// material is decoded from latent level max(L - 2, 0): levels L >= 2 sit on latent texel centres
// (one tap), levels 1 and 0 are magnified 2x / 4x from latent level 0 (bilinear, wrap, at the
// texel centre). The 8 latent channels are rounded to BF16 and run through an MLP of 11 inputs
// (the 8 channels, a constant 1 carrying the first bias, and one-hot flags for L = 0 and L = 1,
// so the network can add the detail of the magnified levels) -> 64 -> 64 -> 8 (GELU) whose
// outputs are albedo RGB, normal XY, metallic, roughness and AO in [0, 1]. The training target of
// a texel is the plain sampler's point sample of that texel (SampleLevel<SurfaceSampler> with
// nearest filtering, Texture.h:412-459); AO has no source channel (layer 1 holds NX, NY, M, R;
// Scene.h:9, Scene.cpp:31-34) and is trained towards a constant 1.
//
// One CTA of 128 threads works on 128-sample tiles: thread t owns sample row t, which is TMEM
// lane t of every accumulator (M = 128). Every matrix product is a tcgen05.mma issued by thread 0
// from shared-memory operands in the slab layout of swr_tc.cuh, FP32 accumulation in TMEM,
// completion signalled through tcgen05.commit on an mbarrier that every thread waits on with a
// one-second limit (a timeout sets a status bit, skips the remaining work and still frees TMEM).
//
// Training tile, 6 round trips through the tensor cores:
//   z1 = X0 W1^T            h1 = gelu(z1)      (X0 = [latents, 1, L==0, L==1, 0...], K = 16)
//   z2 = H1 W2^T + b2       h2 = gelu(z2)
//   y  = H2 W3^T + b3       dy = (2 / 1024) (y - target)   (mean over the tile's 8 x 128 outputs)
//   dh2 = (DY W3) * gelu'(z2);  dh1 = (DH2 W2) * gelu'(z1);  dx0 = DH1 W1
//   G_a += [DH2 | DH1]^T [H1 | X0]   -> dW2 (rows 0-63, cols 0-63), dW1 (rows 64-127, cols 64-79)
//   G_b += [H2 | 1 | ...]^T [DY | DH2] -> dW3^T (rows 0-63, cols 0-15), db3 and db2 (row 64)
// The weight-gradient products read the activation slabs as MN-major operands (features = M/N,
// samples = K), so no transposed copy is written. G_a and G_b stay in TMEM over all tiles of the
// CTA and are written out once per CTA; dx0 is scattered into the latent gradient with vector
// atomics at the bilinear weights (the FP16/BF16 roundings of the forward pass are treated as
// identity in the backward pass).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "swr_device.cuh"
#include "swr_neural.h"
#include "swr_tc.cuh"

namespace swr {
namespace {

using namespace tc;

constexpr uint32_t kSlab = 2048;                    // 128 rows x 16 bytes
// training kernel shared memory
constexpr uint32_t kSQ = kNeuralImage;              // H1 (8 slabs) | X0 (2 slabs)
constexpr uint32_t kSR = kSQ + 10 * kSlab;          // H2 (8) | ONES (1) -- P must follow directly
constexpr uint32_t kSP = kSR + 9 * kSlab;           // DY (2) | DH2 (8) | DH1 (8)
constexpr uint32_t kSBar = kSP + 18 * kSlab;
constexpr uint32_t kTrainSmem = kSBar + 64;
constexpr uint32_t kTrainTmemCols = 256, kT0 = 0, kTGa = 64, kTGb = 144;
// decode kernel shared memory: one activation buffer holds X0 (slabs 0-1), then H1, then H2 (each
// is dead once the MMA reading it has completed), so 7 CTAs fit on an SM
constexpr uint32_t kDX = kNeuralFwdImage;           // X0 (2 slabs) / H1 (8) / H2 (8)
constexpr uint32_t kDH1 = kDX;
constexpr uint32_t kDH2 = kDX;
constexpr uint32_t kDBar = kDX + 8 * kSlab;
constexpr uint32_t kDecodeSmem = kDBar + 64;
constexpr uint32_t kDecodeTmemCols = 64;
constexpr float kGradScale = 2.0f / 1024.0f;        // d(mean over 128 samples x 8 outputs)/dy

static_assert(kSQ % 16 == 0 && kSR % 16 == 0 && kSP % 16 == 0 && kDX % 16 == 0, "operands must be 16-byte aligned");
static_assert(kTrainSmem <= 227 * 1024 && kDecodeSmem <= 227 * 1024, "shared memory");
static_assert(kTGb + 80 <= kTrainTmemCols, "TMEM columns");

// Texture2D tiled texel address (columns of 8 rows; Texture.h:314-329).
__device__ __forceinline__ uint32_t texel_offset(int32_t x, int32_t y, int32_t stride) {
    return (uint32_t)((y & 7) | (x << 3) | ((y & ~7) << stride));
}
__device__ __forceinline__ uint32_t hash32(uint32_t x) {  // integer finaliser (lowbias32)
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
// GELU in its tanh form (Hendrycks & Gimpel, 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))),
// with the hardware tanh.approx.f32; the derivative is that of the same expression.
constexpr float kGeluA = 0.7978845608028654f, kGeluB = 0.044715f;
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float x) {
    const float t = tanh_hw(kGeluA * x * fmaf(kGeluB, x * x, 1.0f));
    const float h = 0.5f * x;
    return fmaf(h, t, h);
}
// 2 gelu(x) = x + x tanh(sqrt(2/pi) x (1 + 0.044715 x^2)): four instructions and the tanh. The
// inference kernel keeps its activations doubled and its next layer's weights halved (exact for
// BF16 weights of normal magnitude), so the products, hence z2 and y, are those of gelu.
constexpr float kGeluAB = kGeluA * kGeluB;
__device__ __forceinline__ float gelu_x2(float x) {
    const float t = tanh_hw(x * fmaf(kGeluAB, x * x, kGeluA));
    return fmaf(x, t, x);
}
// gelu_x2 of two values with the packed FP32 instructions (FMUL2 / FFMA2, sm_100): the same
// IEEE operations on each value, in half the instructions.
__device__ __forceinline__ float2 gelu_x2_pair(float2 x) {
    const float2 p = __ffma2_rn(make_float2(kGeluAB, kGeluAB), __fmul2_rn(x, x), make_float2(kGeluA, kGeluA));
    const float2 u = __fmul2_rn(x, p);
    return __ffma2_rn(x, make_float2(tanh_hw(u.x), tanh_hw(u.y)), x);
}
// gelu_x2 in place over 16 values, a pair at a time (kBias: b[j] is added first).
template <bool kBias>
__device__ __forceinline__ void gelu_x2_16(float (&v)[16], const float* b) {
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
        float2 x = make_float2(v[j], v[j + 1]);
        if constexpr (kBias) x = __fadd2_rn(x, make_float2(b[j], b[j + 1]));
        x = gelu_x2_pair(x);
        v[j] = x.x, v[j + 1] = x.y;
    }
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float x2 = x * x;
    const float t = tanh_hw(kGeluA * x * fmaf(kGeluB, x2, 1.0f));
    const float dt = 0.5f * x * fmaf(-t, t, 1.0f) * kGeluA * fmaf(3.0f * kGeluB, x2, 1.0f);
    return fmaf(0.5f, t, 0.5f) + dt;
}
__device__ __forceinline__ float half_round(float v) { return __half2float(__float2half_rn(v)); }
__device__ __forceinline__ float h2f(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)h)); }

struct Sample {
    uint32_t level, tx, ty;
};
__device__ __forceinline__ Sample unpack_sample(uint32_t p) { return { p >> 28, p & 0x3FFFu, (p >> 14) & 0x3FFFu }; }

// Bilinear taps of the latent grid at a texel centre: texture level L reads latent level
// max(L-2, 0) at x = (tx + 0.5) / s - 0.5 with s = 4, 2, 1 for L = 0, 1, >= 2 (exact in float),
// wrapping; idx are texel indices inside the material's latent block. For s = 1 the fractions are
// 0 and only idx[0] carries weight.
struct Taps {
    uint32_t idx[4];  // (x0,y0) (x1,y0) (x0,y1) (x1,y1)
    float fx, fy;
};
__device__ __forceinline__ Taps latent_taps(const NeuralDev& n, Sample s) {
    const uint32_t l = s.level >= 2 ? s.level - 2 : 0;
    const float inv = s.level == 0 ? 0.125f : s.level == 1 ? 0.25f : 0.5f;  // 1 / (2 s)
    const int32_t LW = (int32_t)n.levelW[l], LH = (int32_t)n.levelH[l];
    const float lx = (float)(2 * s.tx + 1) * inv - 0.5f, ly = (float)(2 * s.ty + 1) * inv - 0.5f;
    const float flx = floorf(lx), fly = floorf(ly);
    Taps q;
    q.fx = lx - flx, q.fy = ly - fly;
    int32_t x0 = (int32_t)flx, y0 = (int32_t)fly;
    if (x0 < 0) x0 += LW;
    if (y0 < 0) y0 += LH;
    const int32_t x1 = x0 + 1 == LW ? 0 : x0 + 1, y1 = y0 + 1 == LH ? 0 : y0 + 1;
    const uint32_t b = n.levelOffset[l];
    q.idx[0] = b + y0 * LW + x0, q.idx[1] = b + y0 * LW + x1;
    q.idx[2] = b + y1 * LW + x0, q.idx[3] = b + y1 * LW + x1;
    return q;
}
// v = (c00 (1-fx) + c10 fx)(1-fy) + (c01 (1-fx) + c11 fx) fy, per channel, in this order.
// Two channels at a time with the packed FP32 instructions: the same operations per channel.
__device__ __forceinline__ void interpolate(const float (&c)[4][8], float fx, float fy, float* x0) {
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    const float2 GX = make_float2(gx, gx), FX = make_float2(fx, fx), GY = make_float2(gy, gy), FY = make_float2(fy, fy);
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
        const float2 c0 = make_float2(c[0][k], c[0][k + 1]), c1 = make_float2(c[1][k], c[1][k + 1]);
        const float2 c2 = make_float2(c[2][k], c[2][k + 1]), c3 = make_float2(c[3][k], c[3][k + 1]);
        const float2 top = __fadd2_rn(__fmul2_rn(c0, GX), __fmul2_rn(c1, FX));
        const float2 bot = __fadd2_rn(__fmul2_rn(c2, GX), __fmul2_rn(c3, FX));
        const float2 r = __fadd2_rn(__fmul2_rn(top, GY), __fmul2_rn(bot, FY));
        x0[k] = r.x, x0[k + 1] = r.y;
    }
}

// Point-sampled texel of both layers as 8 targets in [0, 1]; AO = 1.
__device__ __forceinline__ void fetch_targets(const DevTexture& t, Sample s, float* out) {
    const int32_t stride = (int32_t)t.row_shift - (int32_t)s.level;
    const uint32_t off = t.mip_offsets[s.level & 15] + texel_offset((int32_t)s.tx, (int32_t)s.ty, stride);
    const uint32_t a0 = t.data[off];
    const uint32_t a1 = t.num_layers >= 2 ? t.data[(size_t)t.layer_stride + off] : 0u;
    const float k = 1.0f / 255.0f;
    out[0] = (float)(a0 & 255) * k, out[1] = (float)((a0 >> 8) & 255) * k, out[2] = (float)((a0 >> 16) & 255) * k;
    out[3] = (float)(a1 & 255) * k, out[4] = (float)((a1 >> 8) & 255) * k, out[5] = (float)((a1 >> 16) & 255) * k;
    out[6] = (float)(a1 >> 24) * k, out[7] = 1.0f;
}

__device__ Sample draw_sample(const NeuralTrainArgs& a, const DevTexture& t, uint32_t slot, uint32_t s) {
    if (a.samples) return unpack_sample(a.samples[(size_t)slot * a.samplesPerMaterial + s]);
    const uint32_t h = hash32(a.seedLo ^ hash32(a.seedHi + hash32(a.step * 0x9E3779B9u + slot)));
    const uint32_t r0 = hash32(h ^ (s * 0x68E31DA4u + 1u)), r1 = hash32(r0 + 0xB5297A4Du), r2 = hash32(r1 ^ 0x1B56C4E9u);
    // texture level l of the L decoded ones with weight 2^(levelShift (L-1-l)): levelShift 2 =
    // proportional to the level's texel count, 1 = to its edge length, 0 = uniform over levels
    const uint32_t L = a.n.levels + 2, sh = a.levelShift;
    uint32_t total = 0;
    for (uint32_t l = 0; l < L; l++) total += 1u << (sh * (L - 1 - l));
    uint32_t pick = r0 % total, level = 0;
    while (level + 1 < L && pick >= (1u << (sh * (L - 1 - level)))) pick -= 1u << (sh * (L - 1 - level)), level++;
    return { level, r1 % (t.width >> level), r2 % (t.height >> level) };
}

// The columns 8-15 of an input row: the bias input and the magnified-level flags.
__device__ __forceinline__ void level_inputs(uint32_t level, float* v) {
    v[0] = 1.0f, v[1] = level == 0 ? 1.0f : 0.0f, v[2] = level == 1 ? 1.0f : 0.0f;
    v[3] = v[4] = v[5] = v[6] = v[7] = 0.0f;
}
// Corners with zero weight are not read (their value would be multiplied by 0).
__device__ __forceinline__ bool tap_used(const Taps& q, int k) {
    return (k & 1 ? q.fx != 0.0f : true) && (k & 2 ? q.fy != 0.0f : true);
}

__device__ __forceinline__ void load_latent_f32(const float* L, const Taps& q, float (&c)[4][8]) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!tap_used(q, k)) {
#pragma unroll
            for (int j = 0; j < 8; j++) c[k][j] = 0.0f;
            continue;
        }
        const float4 u = *(const float4*)(L + (size_t)q.idx[k] * 8), v = *(const float4*)(L + (size_t)q.idx[k] * 8 + 4);
        c[k][0] = half_round(u.x), c[k][1] = half_round(u.y), c[k][2] = half_round(u.z), c[k][3] = half_round(u.w);
        c[k][4] = half_round(v.x), c[k][5] = half_round(v.y), c[k][6] = half_round(v.z), c[k][7] = half_round(v.w);
    }
}
__device__ __forceinline__ void load_latent_f16(const uint16_t* L, const Taps& q, float (&c)[4][8]) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!tap_used(q, k)) {
#pragma unroll
            for (int j = 0; j < 8; j++) c[k][j] = 0.0f;
            continue;
        }
        const uint4 u = *(const uint4*)(L + (size_t)q.idx[k] * 8);
        const uint32_t w[4] = { u.x, u.y, u.z, u.w };
#pragma unroll
        for (int j = 0; j < 4; j++) c[k][2 * j] = h2f(w[j] & 0xFFFF), c[k][2 * j + 1] = h2f(w[j] >> 16);
    }
}

// Synchronise the CTA (publishing its shared-memory operand writes to the tensor cores), let
// thread 0 issue `issue()` and commit, and wait for completion. Returns the CTA-uniform status.
template <class F>
__device__ __forceinline__ bool tc_round(bool ok, uint64_t* bar, uint32_t& phase, uint64_t limitNs, F&& issue) {
    fence_proxy_async();
    fence_before_sync();
    ok = __syncthreads_and(ok);
    fence_after_sync();
    if (!ok) return false;
    if (threadIdx.x == 0) {
        issue();
        mma_commit(bar);
    }
    ok = mbar_wait_drained(bar, phase, limitNs);
    phase ^= 1;
    ok = __syncthreads_and(ok);  // every thread leaves with the same verdict
    fence_after_sync();
    return ok;
}

__global__ void __launch_bounds__(128) k_neural_train(const __grid_constant__ NeuralTrainArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* barMma = (uint64_t*)(sm + kSBar);
    uint64_t* barLoad = barMma + 1;
    uint32_t* tmemSlot = (uint32_t*)(barMma + 2);
    float* red = (float*)(barMma + 3);
    const uint32_t t = threadIdx.x, warp = t >> 5;
    const uint32_t slot = blockIdx.x / a.ctasPerMaterial, sub = blockIdx.x - slot * a.ctasPerMaterial;
    const uint32_t mat = a.materials[slot];
    const DevTexture& tex = a.n.tex[mat];
    const uint32_t tilesPerMat = a.samplesPerMaterial / 128;
    const uint32_t tBegin = sub * tilesPerMat / a.ctasPerMaterial, tEnd = (sub + 1) * tilesPerMat / a.ctasPerMaterial;

    if (t == 0) {
        mbar_init(barMma, 1);
        mbar_init(barLoad, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmemSlot, kTrainTmemCols);
        tmem_relinquish();
    }
    {
        const float one[8] = { 1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f }, zero[8] = {};
        store_row8(sm + kSR, 128, 8, t, one);   // ONES slab: feature 0 = 1
        store_row8(sm + kSP, 128, 1, t, zero);  // DY columns 8-15
    }
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (t == 0) {
        mbar_arrive_expect_tx(barLoad, kNeuralImage);
        bulk_g2s(sm, a.n.image + (size_t)mat * kNeuralImage, kNeuralImage, barLoad);
    }
    const uint32_t tmem = *tmemSlot;
    const uint32_t tRow = tmem + ((warp * 32) << 16);
    const uint32_t sb = smem_u32(sm);
    bool ok = mbar_wait_drained(barLoad, 0, a.n.waitNs);
    uint32_t phase = 0;
    float lossAcc = 0.f;
    const float* b2 = (const float*)(sm + kIB2);
    const float* b3 = (const float*)(sm + kIB3);
    const size_t matLatent = (size_t)mat * a.n.texelsPerMaterial;
    const float* latent = a.latent + matLatent * 8;
    float* latentGrad = a.latentGrad + matLatent * 8;
    const uint32_t iFwd128x64 = idesc_bf16(128, 64, false, false), iFwd128x16 = idesc_bf16(128, 16, false, false);
    const uint32_t iGrad = idesc_bf16(128, 80, true, true);

    for (uint32_t tile = tBegin; tile < tEnd && ok; tile++) {
        const Sample smp = draw_sample(a, tex, slot, tile * 128 + t);
        float target[8];
        fetch_targets(tex, smp, target);
        const Taps q = latent_taps(a.n, smp);
        float x0[8];
        {
            float c[4][8];
            load_latent_f32(latent, q, c);
            interpolate(c, q.fx, q.fy, x0);
        }
        store_row8(sm + kSQ, 128, 8, t, x0);
        {
            float li[8];
            level_inputs(smp.level, li);
            store_row8(sm + kSQ, 128, 9, t, li);  // X0 columns 8-15
        }
        // ---- layer 1
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
            mma_bf16(tmem + kT0, desc_kmajor(sb + kSQ + 8 * kSlab, 128), desc_kmajor(sb + kIW1, 64), iFwd128x64, 0);
        });
        float z1[64];
#pragma unroll
        for (int c = 0; c < 4; c++) tmem_ld16(tRow + kT0 + 16 * c, z1 + 16 * c);
#pragma unroll
        for (int s = 0; s < 8; s++) {
            float h[8];
#pragma unroll
            for (int j = 0; j < 8; j++) h[j] = gelu(z1[8 * s + j]);
            store_row8(sm + kSQ, 128, s, t, h);
        }
        // ---- layer 2
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem + kT0, desc_kmajor(sb + kSQ + 2 * k * kSlab, 128), desc_kmajor(sb + kIW2 + 2 * k * 1024, 64),
                         iFwd128x64, k);
        });
        float z2[64];
#pragma unroll
        for (int c = 0; c < 4; c++) tmem_ld16(tRow + kT0 + 16 * c, z2 + 16 * c);
#pragma unroll
        for (int s = 0; s < 8; s++) {
            float h[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                z2[8 * s + j] += b2[8 * s + j];
                h[j] = gelu(z2[8 * s + j]);
            }
            store_row8(sm + kSR, 128, s, t, h);
        }
        // ---- layer 3 and the loss gradient
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem + kT0, desc_kmajor(sb + kSR + 2 * k * kSlab, 128), desc_kmajor(sb + kIW3 + 2 * k * 256, 16),
                         iFwd128x16, k);
        });
        {
            float y[16], dy[8];
            tmem_ld16(tRow + kT0, y);
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const float e = (y[c] + b3[c]) - target[c];
                lossAcc += e * e;
                dy[c] = e * kGradScale;
            }
            store_row8(sm + kSP, 128, 0, t, dy);
        }
        // ---- dh2 = (DY W3) * gelu'(z2)
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
            mma_bf16(tmem + kT0, desc_kmajor(sb + kSP, 128), desc_kmajor(sb + kIW3t, 64), iFwd128x64, 0);
        });
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v[16];
            tmem_ld16(tRow + kT0 + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] *= gelu_grad(z2[16 * c + j]);
            store_row8(sm + kSP, 128, 2 + 2 * c, t, v);
            store_row8(sm + kSP, 128, 3 + 2 * c, t, v + 8);
        }
        // ---- dh1 = (DH2 W2) * gelu'(z1)
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem + kT0, desc_kmajor(sb + kSP + (2 + 2 * k) * kSlab, 128),
                         desc_kmajor(sb + kIW2t + 2 * k * 1024, 64), iFwd128x64, k);
        });
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v[16];
            tmem_ld16(tRow + kT0 + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] *= gelu_grad(z1[16 * c + j]);
            store_row8(sm + kSP, 128, 10 + 2 * c, t, v);
            store_row8(sm + kSP, 128, 11 + 2 * c, t, v + 8);
        }
        // ---- dx0 = DH1 W1, and the weight-gradient accumulators
        const uint32_t acc = tile > tBegin ? 1u : 0u;
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem + kT0, desc_kmajor(sb + kSP + (10 + 2 * k) * kSlab, 128),
                         desc_kmajor(sb + kIW1t + 2 * k * 256, 16), iFwd128x16, k);
#pragma unroll
            for (uint32_t i = 0; i < 8; i++)
                mma_bf16(tmem + kTGa, desc_mnmajor(sb + kSP + 2 * kSlab + i * 256, 128), desc_mnmajor(sb + kSQ + i * 256, 128),
                         iGrad, acc | (i > 0));
#pragma unroll
            for (uint32_t i = 0; i < 8; i++)
                mma_bf16(tmem + kTGb, desc_mnmajor(sb + kSR + i * 256, 128), desc_mnmajor(sb + kSP + i * 256, 128), iGrad,
                         acc | (i > 0));
        });
        {
            float d[16];
            tmem_ld16(tRow + kT0, d);
            const float gx = 1.0f - q.fx, gy = 1.0f - q.fy;
            const float w[4] = { gx * gy, q.fx * gy, gx * q.fy, q.fx * q.fy };
            if (ok) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (!tap_used(q, k)) continue;
                    float* g = latentGrad + (size_t)q.idx[k] * 8;
                    atomicAdd((float4*)g, make_float4(w[k] * d[0], w[k] * d[1], w[k] * d[2], w[k] * d[3]));
                    atomicAdd((float4*)(g + 4), make_float4(w[k] * d[4], w[k] * d[5], w[k] * d[6], w[k] * d[7]));
                }
            }
        }
    }
    ok = __syncthreads_and(ok);

    // ---- this CTA's parameter gradients
    float* out = a.partial + (size_t)blockIdx.x * kNeuralParams;
    if (!ok || tEnd == tBegin) {
        for (uint32_t i = t; i < kNeuralParams; i += 128) out[i] = 0.f;
    } else {  // every entry is written below (W1 columns 11-15 multiply zero inputs: 0)
        float v[16];
        if (warp < 2) {  // rows 0-63: dW2 row o = t, dW3^T row i = t
#pragma unroll
            for (int c = 0; c < 4; c++) {
                tmem_ld16(tRow + kTGa + 16 * c, v);
#pragma unroll
                for (int j = 0; j < 16; j++) out[kPW2 + t * 64 + 16 * c + j] = v[j];
            }
            tmem_ld16(tRow + kTGb, v);
#pragma unroll
            for (int o = 0; o < 8; o++) out[kPW3 + o * 64 + t] = v[o];
        } else {  // rows 64-127: dW1 row o = t - 64; row 64 of G_b: db3, db2
            tmem_ld16(tRow + kTGa + 64, v);
#pragma unroll
            for (int j = 0; j < 16; j++) out[kPW1 + (t - 64) * 16 + j] = v[j];
            if (warp == 2) {
                tmem_ld16(tRow + kTGb, v);
                if (t == 64)
                    for (int o = 0; o < 8; o++) out[kPB3 + o] = v[o];
#pragma unroll
                for (int c = 1; c < 5; c++) {
                    tmem_ld16(tRow + kTGb + 16 * c, v);
                    if (t == 64)
                        for (int j = 0; j < 16; j++) out[kPB2 + 16 * (c - 1) + j] = v[j];
                }
            }
        }
    }
    // ---- loss
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lossAcc += __shfl_xor_sync(0xFFFFFFFFu, lossAcc, o);
    if ((t & 31) == 0) red[warp] = lossAcc;
    fence_before_sync();
    __syncthreads();
    if (t == 0) {
        atomicAdd(a.loss, red[0] + red[1] + red[2] + red[3]);
        atomicAdd(a.loss + 1, (float)(128 * (tEnd - tBegin)));
        if (!ok) atomicOr(a.status, 1u);
    }
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tmem, kTrainTmemCols);
    }
}

// Position(s) of parameter i in the BF16 operand image.
__device__ __forceinline__ void image_store(uint8_t* img, uint32_t i, float w) {
    const unsigned short b = __bfloat16_as_ushort(__float2bfloat16_rn(w));
    if (i < kPW2) {
        const uint32_t o = i / 16, j = i % 16;
        *(unsigned short*)(img + kIW1 + slab_offset(64, o, j)) = b;
        *(unsigned short*)(img + kIW1t + slab_offset(16, j, o)) = b;
    } else if (i < kPB2) {
        const uint32_t o = (i - kPW2) / 64, k = (i - kPW2) % 64;
        *(unsigned short*)(img + kIW2 + slab_offset(64, o, k)) = b;
        *(unsigned short*)(img + kIW2t + slab_offset(64, k, o)) = b;
    } else if (i < kPW3) {
        *(float*)(img + kIB2 + (i - kPB2) * 4) = w;
    } else if (i < kPB3) {
        const uint32_t o = (i - kPW3) / 64, k = (i - kPW3) % 64;
        *(unsigned short*)(img + kIW3 + slab_offset(16, o, k)) = b;
        *(unsigned short*)(img + kIW3t + slab_offset(64, k, o)) = b;
    } else if (i < kNeuralParams) {
        *(float*)(img + kIB3 + (i - kPB3) * 4) = w;
    }
}

__global__ void k_neural_image(const float* params, uint8_t* image) {
    const uint32_t mat = blockIdx.x;
    for (uint32_t i = threadIdx.x; i < kNeuralParams; i += blockDim.x)
        image_store(image + (size_t)mat * kNeuralImage, i, params[(size_t)mat * kNeuralParams + i]);
}

// One Adam update: m, v moments; w -= lr m / (1 - b1^t) / (sqrt(v / (1 - b2^t)) + eps), written as
// w -= lrm m / (sqrt(v) s2 + eps) with lrm = lr / (1 - b1^t) and s2 = 1 / sqrt(1 - b2^t) from the host,
// square root and quotient on the SFU (sqrt.approx, div.approx: a few ulp, irrelevant to Adam).
__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void adam_update(float g, float& m, float& v, float& w, float b1, float b2, float lrm, float s2,
                                            float eps) {
    m = fmaf(b1, m, (1.0f - b1) * g);
    v = fmaf(b2, v, (1.0f - b2) * g * g);
    w -= __fdividef(lrm * m, fmaf(sqrt_approx(v), s2, eps));
}

// Adam on the parameters of the step's materials (sum of the CTAs' partial gradients in a fixed
// order), then the new BF16 image.
__global__ void k_neural_adam_params(const __grid_constant__ NeuralAdamArgs a) {
    const uint32_t slot = blockIdx.y, mat = a.materials[slot];
    float* p = a.params + (size_t)mat * kNeuralParams;
    float* m = a.m + (size_t)mat * kNeuralParams;
    float* v = a.v + (size_t)mat * kNeuralParams;
    const float* part = a.partial + (size_t)slot * a.ctasPerMaterial * kNeuralParams;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // one parameter per thread
    if (i < kNeuralParams) {
        float g = 0.f;
        uint32_t c = 0;
        for (; c + 8 <= a.ctasPerMaterial; c += 8) {  // 8 loads in flight, summed in CTA order
            float q[8];
#pragma unroll
            for (int k = 0; k < 8; k++) q[k] = part[(size_t)(c + k) * kNeuralParams + i];
#pragma unroll
            for (int k = 0; k < 8; k++) g += q[k];
        }
        for (; c < a.ctasPerMaterial; c++) g += part[(size_t)c * kNeuralParams + i];
        float mi = m[i], vi = v[i], w = p[i];
        adam_update(g, mi, vi, w, a.beta1, a.beta2, a.lrm[slot], a.s2[slot], a.eps);
        m[i] = mi, v[i] = vi, p[i] = w;
        image_store(a.image + (size_t)mat * kNeuralImage, i, w);
    }
}

// Adam on the latents of the step's materials, one float4 per thread; clears the gradient.
__global__ void __launch_bounds__(256) k_neural_adam_latent(const __grid_constant__ NeuralAdamArgs a) {
    const uint32_t slot = blockIdx.y, mat = a.materials[slot];
    const size_t n4 = (size_t)a.texelsPerMaterial * 2, base = (size_t)mat * n4;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n4) return;
    float4* G = (float4*)a.latentGrad + base + i;
    float4* M = (float4*)a.latentM + base + i;
    float4* V = (float4*)a.latentV + base + i;
    float4* P = (float4*)a.latent + base + i;
    const float4 g = *G;
    float4 m = *M, v = *V, p = *P;
    *G = make_float4(0.f, 0.f, 0.f, 0.f);
    const float lrm = a.lrm[slot], s2 = a.s2[slot];
    adam_update(g.x, m.x, v.x, p.x, a.beta1, a.beta2, lrm, s2, a.eps);
    adam_update(g.y, m.y, v.y, p.y, a.beta1, a.beta2, lrm, s2, a.eps);
    adam_update(g.z, m.z, v.z, p.z, a.beta1, a.beta2, lrm, s2, a.eps);
    adam_update(g.w, m.w, v.w, p.w, a.beta1, a.beta2, lrm, s2, a.eps);
    *M = m, *V = v, *P = p;
}

// Latent level l texel (x, y) starts as texture level l + 2 texel (x, y): channels R G B (layer
// 0), NX NY M R (layer 1) mapped to [-1, 1], channel 7 = 0. Materials without a texture get zeros.
__global__ void k_neural_latent_init(const __grid_constant__ NeuralDev n, float* latent) {
    const uint32_t mat = blockIdx.y;
    const DevTexture& t = n.tex[mat];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n.texelsPerMaterial; i += gridDim.x * blockDim.x) {
        float* o = latent + ((size_t)mat * n.texelsPerMaterial + i) * 8;
        if (t.data == nullptr) {
            for (int c = 0; c < 8; c++) o[c] = 0.f;
            continue;
        }
        uint32_t l = 0;
        while (l + 1 < n.levels && i >= n.levelOffset[l + 1]) l++;
        const uint32_t r = i - n.levelOffset[l], x = r % n.levelW[l], y = r / n.levelW[l];
        const uint32_t L = l + 2;
        const uint32_t off = t.mip_offsets[L] + texel_offset((int32_t)x, (int32_t)y, (int32_t)t.row_shift - (int32_t)L);
        const uint32_t a0 = t.data[off], a1 = t.num_layers >= 2 ? t.data[(size_t)t.layer_stride + off] : 0u;
        const uint32_t s[7] = { a0 & 255, (a0 >> 8) & 255, (a0 >> 16) & 255, a1 & 255, (a1 >> 8) & 255, (a1 >> 16) & 255, a1 >> 24 };
        for (int c = 0; c < 7; c++) o[c] = (float)s[c] * (2.0f / 255.0f) - 1.0f;
        o[7] = 0.f;
    }
}

__global__ void k_neural_export(const float* latent, uint16_t* half, size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        half[i] = __half_as_ushort(__float2half_rn(latent[i]));
}

// ---------------------------------------------------------------------------- inference
__device__ __forceinline__ uint32_t unorm8(float v) {
    return (uint32_t)__float2int_rn(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f);
}

__global__ void __launch_bounds__(128) k_neural_decode(const __grid_constant__ NeuralDecodeArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const uint32_t numMat = a.n.numMaterials;
    const uint32_t total = a.tileOffset[numMat];
    const uint32_t tb = (uint32_t)((uint64_t)blockIdx.x * total / gridDim.x);
    const uint32_t te = (uint32_t)((uint64_t)(blockIdx.x + 1) * total / gridDim.x);
    if (tb >= te) return;
    uint64_t* barMma = (uint64_t*)(sm + kDBar);
    uint64_t* barLoad = barMma + 1;
    uint32_t* tmemSlot = (uint32_t*)(barMma + 2);
    const uint32_t t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        mbar_init(barMma, 1);
        mbar_init(barLoad, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmemSlot, kDecodeTmemCols);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmemSlot;
    const uint32_t tRow = tmem + ((warp * 32) << 16);
    const uint32_t sb = smem_u32(sm);
    const float* b2 = (const float*)(sm + kIB2);
    const float* b3 = (const float*)(sm + kIB3);
    const uint32_t i64 = idesc_bf16(128, 64, false, false), i16 = idesc_bf16(128, 16, false, false);
    // first material with tiles at or after tb
    uint32_t lo = 0, hi = numMat;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (a.tileOffset[mid + 1] <= tb) lo = mid + 1;
        else hi = mid;
    }
    uint32_t mat = lo, loaded = 0xFFFFFFFFu, phase = 0, loadPhase = 0;
    bool ok = true;
    for (uint32_t tile = tb; tile < te && ok; tile++) {
        while (tile >= a.tileOffset[mat + 1]) mat++;
        if (mat != loaded) {
            ok = __syncthreads_and(ok);  // the previous tile's readers of the image are done
            if (t == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(barLoad, kNeuralFwdImage);
                bulk_g2s(sm, a.n.image + (size_t)mat * kNeuralImage, kNeuralFwdImage, barLoad);
            }
            ok = mbar_wait_drained(barLoad, loadPhase, a.n.waitNs) && ok;
            loadPhase ^= 1;
            loaded = mat;
            // W2 and W3 halved in place: the activations they weigh are 2 gelu (gelu_x2)
            __nv_bfloat162* w = (__nv_bfloat162*)(sm + kIW2);
            const __nv_bfloat162 half2 = __floats2bfloat162_rn(0.5f, 0.5f);
            for (uint32_t i = t; i < (kIB2 - kIW2) / 4; i += blockDim.x) w[i] = __hmul2(w[i], half2);
        }
        const uint32_t first = a.reqOffset[mat] + (tile - a.tileOffset[mat]) * 128;
        const bool valid = first + t < a.reqOffset[mat + 1];
        const unsigned long long req = valid ? a.sorted[first + t] : 0ull;
        const Sample smp = unpack_sample((uint32_t)req);
        const Taps q = latent_taps(a.n, smp);
        float x0[8];
        {
            float c[4][8];
            load_latent_f16(a.n.latentHalf + (size_t)mat * a.n.texelsPerMaterial * 8, q, c);
            interpolate(c, q.fx, q.fy, x0);
        }
        store_row8(sm + kDX, 128, 0, t, x0);
        {
            float li[8];  // bias and level inputs (the buffer held H2 of the last tile)
            level_inputs(smp.level, li);
            store_row8(sm + kDX, 128, 1, t, li);
        }
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
            mma_bf16(tmem, desc_kmajor(sb + kDX, 128), desc_kmajor(sb + kIW1, 64), i64, 0);
        });
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v[16];
            tmem_ld16(tRow + 16 * c, v);
            gelu_x2_16<false>(v, nullptr);
            store_row8(sm + kDH1, 128, 2 * c, t, v);
            store_row8(sm + kDH1, 128, 2 * c + 1, t, v + 8);
        }
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem, desc_kmajor(sb + kDH1 + 2 * k * kSlab, 128), desc_kmajor(sb + kIW2 + 2 * k * 1024, 64), i64, k);
        });
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v[16];
            tmem_ld16(tRow + 16 * c, v);
            gelu_x2_16<true>(v, b2 + 16 * c);
            store_row8(sm + kDH2, 128, 2 * c, t, v);
            store_row8(sm + kDH2, 128, 2 * c + 1, t, v + 8);
        }
        ok = tc_round(ok, barMma, phase, a.n.waitNs, [&] {
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                mma_bf16(tmem, desc_kmajor(sb + kDH2 + 2 * k * kSlab, 128), desc_kmajor(sb + kIW3 + 2 * k * 256, 16), i16, k);
        });
        float y[16];
        tmem_ld16(tRow, y);
        if (valid && ok) {
            uint32_t u[8];
#pragma unroll
            for (int c = 0; c < 8; c++) u[c] = unorm8(y[c] + b3[c]);
            a.out[req >> 32] = make_uint2(u[0] | (u[1] << 8) | (u[2] << 16) | (u[7] << 24), u[3] | (u[4] << 8) | (u[5] << 16) | (u[6] << 24));
        }
    }
    ok = __syncthreads_and(ok);
    if (t == 0 && !ok) atomicOr(a.status, 1u);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tmem, kDecodeTmemCols);
    }
}

// Exclusive prefix of the per-material request counts and of their 128-request tiles
// (numMaterials <= 1024, one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_neural_offsets(const uint32_t* counts, uint32_t* reqOffset, uint32_t* tileOffset,
                                                         uint32_t n) {
    __shared__ uint32_t sr[1024], st[1024];
    const uint32_t t = threadIdx.x;
    const uint32_t c = t < n ? counts[t] : 0u;
    sr[t] = c, st[t] = (c + 127) / 128;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1) {
        const uint32_t a = t >= o ? sr[t - o] : 0u, b = t >= o ? st[t - o] : 0u;
        __syncthreads();
        sr[t] += a, st[t] += b;
        __syncthreads();
    }
    if (t < n) reqOffset[t] = sr[t] - c, tileOffset[t] = st[t] - (c + 127) / 128;
    if (t == n - 1) reqOffset[n] = sr[t], tileOffset[n] = st[t];
}

// Groups the per-pixel requests (material<<32 | level<<28 | ty<<14 | tx, or ~0) by material. A
// block takes kScatterSlots consecutive slots: shared-memory counters rank each request among the
// block's requests of its material, then one global atomic per (block, material) reserves the
// block's run in that material's list (the per-material cursors see few, uncontended atomics).
constexpr uint32_t kScatterThreads = 256, kScatterPerThread = 4, kScatterSlots = kScatterThreads * kScatterPerThread;
__global__ void __launch_bounds__(kScatterThreads) k_neural_scatter(const unsigned long long* pixelReq, uint32_t slots,
                                                                    const uint32_t* reqOffset, uint32_t* cursor,
                                                                    unsigned long long* sorted, uint32_t* levelCount,
                                                                    uint32_t numMaterials) {
    extern __shared__ uint32_t sMat[];  // [numMaterials] counts, then [numMaterials] run starts
    __shared__ uint32_t sLevel[kNeuralMaxDecoded];
    uint32_t* sCount = sMat;
    uint32_t* sBase = sMat + numMaterials;
    for (uint32_t m = threadIdx.x; m < numMaterials; m += kScatterThreads) sCount[m] = 0;
    if (threadIdx.x < kNeuralMaxDecoded) sLevel[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t first = blockIdx.x * kScatterSlots + threadIdx.x;
    unsigned long long r[kScatterPerThread];
    uint32_t rank[kScatterPerThread];
#pragma unroll
    for (uint32_t k = 0; k < kScatterPerThread; k++) {  // slot first + k * 256: coalesced loads
        const uint32_t i = first + k * kScatterThreads;
        r[k] = i < slots ? pixelReq[i] : ~0ull;
        if (r[k] >> 63) r[k] = ~0ull;  // none, or a redirect to another slot's request
        if (r[k] != ~0ull) {
            rank[k] = atomicAdd(&sCount[(uint32_t)(r[k] >> 32)], 1u);
            atomicAdd(&sLevel[((uint32_t)r[k] >> 28) & 15u], 1u);
        }
    }
    __syncthreads();
    for (uint32_t m = threadIdx.x; m < numMaterials; m += kScatterThreads)
        if (sCount[m]) sBase[m] = reqOffset[m] + atomicAdd(&cursor[m], sCount[m]);
    if (threadIdx.x < kNeuralMaxDecoded && sLevel[threadIdx.x]) atomicAdd(&levelCount[threadIdx.x], sLevel[threadIdx.x]);
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < kScatterPerThread; k++) {
        if (r[k] == ~0ull) continue;
        const uint32_t i = first + k * kScatterThreads;
        sorted[sBase[(uint32_t)(r[k] >> 32)] + rank[k]] = ((unsigned long long)i << 32) | (uint32_t)r[k];
    }
}

}  // namespace

void launch_neural_train(const NeuralTrainArgs& a, uint32_t blocks, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_neural_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
        attr = true;
    }
    k_neural_train<<<blocks, 128, kTrainSmem, st>>>(a);
}
void launch_neural_adam(const NeuralAdamArgs& a, cudaStream_t st) {
    k_neural_adam_params<<<dim3((kNeuralParams + 127) / 128, a.numSlots), 128, 0, st>>>(a);
    const uint32_t n4 = a.texelsPerMaterial * 2;
    k_neural_adam_latent<<<dim3((n4 + 255) / 256, a.numSlots), 256, 0, st>>>(a);
}
uint32_t neural_decode_blocks_per_sm() {
    static int per = 0;
    if (!per) {
        // shared memory bound (the kernel's other limits are looser): per-SM capacity over the
        // CTA's dynamic part plus the per-block reservation; TMEM (512 columns) bounds it too
        int dev = 0, smem = 0, reserved = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        per = smem / (int)(kDecodeSmem + (uint32_t)reserved);
        per = std::max(1, std::min(per, (int)(512 / kDecodeTmemCols)));
    }
    return (uint32_t)per;
}
void launch_neural_decode(const NeuralDecodeArgs& a, uint32_t blocks, cudaStream_t st) {
    neural_decode_blocks_per_sm();
    k_neural_decode<<<blocks, 128, kDecodeSmem, st>>>(a);
}
// The bounded-wait path on demand (see launch_wait_selftest): an mbarrier armed with expect_tx for a
// copy that is never issued, so only the time limit can end the wait. The CTA holds TMEM while it
// waits, as the decoder's CTAs do, and frees it on the way out.
__global__ void __launch_bounds__(128) k_wait_selftest(uint32_t* status, uint64_t limitNs) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemSlot;
    const uint32_t warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmemSlot, 32);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    bool ok = true;
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, 16);  // the one arrival, with 16 bytes that never come
        ok = mbar_wait(&bar, 0, limitNs);
        if (!ok) atomicOr(status, 1u);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0) tmem_dealloc(tmemSlot, 32);
}

void launch_wait_selftest(uint32_t* status, uint64_t limitNs, cudaStream_t st) {
    k_wait_selftest<<<1, 128, 0, st>>>(status, limitNs);
}

void launch_neural_image(float* params, uint8_t* image, uint32_t numMaterials, cudaStream_t st) {
    k_neural_image<<<numMaterials, 256, 0, st>>>(params, image);
}
void launch_neural_latent_init(const NeuralDev& n, float* latent, cudaStream_t st) {
    k_neural_latent_init<<<dim3(std::min<uint32_t>((n.texelsPerMaterial + 255) / 256, 512), n.numMaterials), 256, 0, st>>>(n, latent);
}
void launch_neural_export(const float* latent, uint16_t* half, size_t count, cudaStream_t st) {
    k_neural_export<<<(uint32_t)std::min<size_t>((count + 255) / 256, 8192), 256, 0, st>>>(latent, half, count);
}
void launch_neural_offsets(const uint32_t* counts, uint32_t* reqOffset, uint32_t* tileOffset, uint32_t numMaterials,
                           cudaStream_t st) {
    k_neural_offsets<<<1, 1024, 0, st>>>(counts, reqOffset, tileOffset, numMaterials);
}
void launch_neural_scatter(const unsigned long long* pixelReq, uint32_t slots, const uint32_t* reqOffset, uint32_t* cursor,
                           unsigned long long* sorted, uint32_t* levelCount, uint32_t numMaterials, cudaStream_t st) {
    k_neural_scatter<<<(slots + kScatterSlots - 1) / kScatterSlots, kScatterThreads, 2 * numMaterials * sizeof(uint32_t), st>>>(
        pixelReq, slots, reqOffset, cursor, sorted, levelCount, numMaterials);
}

}  // namespace swr
