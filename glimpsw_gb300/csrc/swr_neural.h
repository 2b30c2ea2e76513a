// Learned texture decoder shared definitions: the per-material parameter block, the BF16 operand
// image the tensor-core kernels copy into shared memory, the per-material latent pyramid, and the
// kernels' argument blocks. The decoder has no counterpart in the reference; the plain sampler
// (SampleLevel<SurfaceSampler>, Texture.h:412-459) produces its training targets and stays the
// fallback for texture levels the latents do not cover.
#pragma once
#include <cstdint>

#include "swr_internal.h"

namespace swr {

constexpr uint32_t kNeuralChannels = 8;     // latent channels
constexpr uint32_t kNeuralHidden = 64;      // two hidden layers of 64 (GELU)
constexpr uint32_t kNeuralOutputs = 8;      // albedo RGB, normal XY, metallic, roughness, AO
constexpr uint32_t kNeuralMaxLevels = 4;    // latent levels; latent level k has texture level k+2's size
constexpr uint32_t kNeuralMaxDecoded = kNeuralMaxLevels + 2;  // decoded texture levels 0 .. levels+1
constexpr uint32_t kNeuralDownscale = 4;    // texture level 0 texels per latent level 0 texel, per axis
constexpr uint32_t kNeuralMaxStepMaterials = 64;

// FP32 parameter block of one material (padded layout; 5384 live parameters):
//   W1[64][16]: columns 0-7 weigh the latent channels, column 8 is b1 (the input vector carries a
//               constant 1 there), columns 9 and 10 weigh the level-0 / level-1 flags, columns
//               11-15 are zero and stay zero;
//   W2[64][64], b2[64], W3[8][64], b3[8].
constexpr uint32_t kPW1 = 0, kPW2 = 1024, kPB2 = 5120, kPW3 = 5184, kPB3 = 5696, kNeuralParams = 5704;

// BF16 operand image of one material (slab layout of swr_tc.cuh, K-major B operands):
//   W1 [64 n][16 k], W2 [64][64], W3 [16][64] (rows 8-15 zero), b2 f32[64], b3 f32[16]   forward part
//   W3t [64][16] (= W3^T), W2t [64][64] (= W2^T), W1t [16][64] (= W1^T)                    backward part
constexpr uint32_t kIW1 = 0, kIW2 = 2048, kIW3 = 10240, kIB2 = 12288, kIB3 = 12544, kNeuralFwdImage = 12800;
constexpr uint32_t kIW3t = 12800, kIW2t = 14848, kIW1t = 23040, kNeuralImage = 25088;

// Kernel view of a model.
struct NeuralDev {
    uint32_t numMaterials, levels;
    uint32_t texelsPerMaterial;                 // latent texels over all levels
    uint32_t levelOffset[kNeuralMaxLevels];     // first texel of each level inside a material block
    uint32_t levelW[kNeuralMaxLevels], levelH[kNeuralMaxLevels];
    const DevTexture* tex;                      // per material (layer 0 RGBA, layer 1 NX NY M R)
    const uint16_t* latentHalf;                 // FP16 [material][texel][8]
    const uint8_t* image;                       // [material][kNeuralImage]
    uint64_t waitNs;                            // limit of each bounded tensor-core / copy wait
};

struct NeuralTrainArgs {
    NeuralDev n;
    const float* latent;        // FP32 master [material][texel][8]
    float* latentGrad;          // same shape, accumulated by the step
    float* partial;             // [block][kNeuralParams] parameter gradients of each block
    const uint32_t* samples;    // optional explicit samples [slot][samplesPerMaterial]: level<<28 | ty<<14 | tx
    float* loss;                // [0] += squared error, [1] += samples
    uint32_t* status;           // bit 0: a tensor-core wait timed out
    uint32_t materials[kNeuralMaxStepMaterials];
    uint32_t numSlots, samplesPerMaterial, ctasPerMaterial;
    uint32_t seedLo, seedHi, step;
    uint32_t levelShift;        // level l drawn with weight 2^(levelShift (levels-1-l))
};

struct NeuralAdamArgs {
    float* params;              // [material][kNeuralParams]
    float* m;
    float* v;
    const float* partial;
    uint8_t* image;
    float* latent;
    float* latentM;
    float* latentV;
    float* latentGrad;
    uint32_t texelsPerMaterial;
    uint32_t ctasPerMaterial, numSlots;
    float lr, beta1, beta2, eps;
    uint32_t materials[kNeuralMaxStepMaterials];
    float lrm[kNeuralMaxStepMaterials];   // lr / (1 - beta1^t) per slot (t: the material's step count)
    float s2[kNeuralMaxStepMaterials];    // 1 / sqrt(1 - beta2^t) per slot
};

struct NeuralDecodeArgs {
    NeuralDev n;
    const unsigned long long* sorted;   // requests grouped by material: slot<<32 | level<<28 | ty<<14 | tx
    const uint32_t* reqOffset;          // [numMaterials + 1] first request of each material
    const uint32_t* tileOffset;         // [numMaterials + 1] first 128-request tile of each material
    uint2* out;                         // [slot] decoded (layer 0 RGBA8 with AO in alpha, layer 1 RGBA8)
    uint32_t* status;
};

void launch_neural_train(const NeuralTrainArgs& a, uint32_t blocks, cudaStream_t st);
void launch_neural_adam(const NeuralAdamArgs& a, cudaStream_t st);
void launch_neural_decode(const NeuralDecodeArgs& a, uint32_t blocks, cudaStream_t st);
uint32_t neural_decode_blocks_per_sm();  // resident decode CTAs per SM (shared memory and TMEM bound)
void launch_neural_image(float* params, uint8_t* image, uint32_t numMaterials, cudaStream_t st);
void launch_neural_latent_init(const NeuralDev& n, float* latent, cudaStream_t st);
void launch_neural_export(const float* latent, uint16_t* half, size_t count, cudaStream_t st);
// One CTA announces a 16-byte copy on an mbarrier and issues none, waits at most limitNs with TMEM
// allocated, then frees the TMEM and sets status bit 0 if the wait gave up.
void launch_wait_selftest(uint32_t* status, uint64_t limitNs, cudaStream_t st);
void launch_neural_offsets(const uint32_t* counts, uint32_t* reqOffset, uint32_t* tileOffset, uint32_t numMaterials,
                           cudaStream_t st);
void launch_neural_scatter(const unsigned long long* pixelReq, uint32_t slots, const uint32_t* reqOffset,
                           uint32_t* cursor, unsigned long long* sorted, uint32_t* levelCount, uint32_t numMaterials,
                           cudaStream_t st);

}  // namespace swr

struct swr_neural_t;
namespace swr {
void neural_sync_half(swr_neural_t* n, cudaStream_t st);  // FP16 latents up to date with the master copy
int neural_num_sms();
}  // namespace swr

struct swr_neural_t {
    swr::NeuralDev d;                        // device view (pointers below)
    std::vector<swr::DevTexture> texHost;
    swr::DevTexture* tex;
    float *latent, *latentM, *latentV, *latentGrad;
    uint16_t* latentHalf;
    float *params, *paramM, *paramV;
    uint8_t* image;
    float* partial;
    size_t partialFloats;
    float* loss;                             // device [2]
    uint32_t* status;                        // device
    std::vector<uint32_t> steps;             // Adam step count per material
    uint64_t seed;
    uint32_t trainCalls;
    bool halfStale;                          // latentHalf behind the master copy
    // neural resolve scratch (grow-only)
    unsigned long long* pixelReq;
    unsigned long long* sorted;
    uint2* decoded;
    uint4* surf;                             // two words per pixel: the emit pass's surface records
    size_t scratchSlots;
    uint32_t* counters;                      // counts | cursors | reqOffset | tileOffset, numMaterials+1 each,
                                             // then 4 per-level request counts
};
