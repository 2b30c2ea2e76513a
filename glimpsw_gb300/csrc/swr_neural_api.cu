// C ABI of the learned texture decoder: model creation (latents initialised from the textures,
// seeded parameters), training steps, gradient and decode entry points for testing, parameter
// and latent access. The neural resolve itself is in swr_shade.cu next to the plain resolve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "swr_neural.h"

using namespace swr;

namespace {

int num_sms() { return swr_internal_sm_count(); }

constexpr uint64_t kDefaultWaitNs = 1000000000ull;  // 1 s per bounded wait

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
float uniform_pm(uint64_t& s, float a) { return (float)((double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * a; }

// Seeded initial parameters of one material: Glorot-uniform weights, zero biases except b3 = 0.5
// (the middle of the [0, 1] outputs); padding entries zero.
void init_params(float* p, uint64_t seed, uint32_t mat) {
    uint64_t s = seed * 0x2545F4914F6CDD1Dull + mat * 0x9E3779B97F4A7C15ull + 1;
    std::fill(p, p + kNeuralParams, 0.0f);
    const float a1 = std::sqrt(6.0f / (8 + 64)), a2 = std::sqrt(6.0f / (64 + 64)), a3 = std::sqrt(6.0f / (64 + 8));
    for (uint32_t o = 0; o < 64; o++)
        for (uint32_t j = 0; j < 8; j++) p[kPW1 + o * 16 + j] = uniform_pm(s, a1);
    for (uint32_t i = 0; i < 64 * 64; i++) p[kPW2 + i] = uniform_pm(s, a2);
    for (uint32_t i = 0; i < 8 * 64; i++) p[kPW3 + i] = uniform_pm(s, a3);
    for (uint32_t o = 0; o < 8; o++) p[kPB3 + o] = 0.5f;
}

bool has_texture(const swr_neural_t* n, uint32_t m) { return n->texHost[m].data != nullptr; }

template <class T>
cudaError_t dev_alloc(T** p, size_t count) {
    return cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
}

void free_model(swr_neural_t* n) {
    void* ptrs[] = { n->tex, n->latent, n->latentM, n->latentV, n->latentGrad, n->latentHalf, n->params, n->paramM,
                     n->paramV, n->image, n->partial, n->loss, n->status, n->pixelReq, n->sorted, n->decoded, n->surf,
                     n->counters };
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete n;
}

swr_status ensure_partial(swr_neural_t* n, size_t floats) {
    if (n->partialFloats >= floats) return SWR_OK;
    if (n->partial) cudaFree(n->partial);
    n->partial = nullptr;
    n->partialFloats = 0;
    cudaError_t e = dev_alloc(&n->partial, floats);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural: gradient buffer");
    n->partialFloats = floats;
    return SWR_OK;
}

swr_status check_status(swr_neural_t* n, cudaStream_t st, const char* what) {
    uint32_t s = 0;
    cudaError_t e = cudaMemcpyAsync(&s, n->status, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, what);
    if (s) {
        cudaMemsetAsync(n->status, 0, 4, st);
        return swr_internal_fail(SWR_ETIMEOUT, "swr_neural: a tensor-core wait timed out");
    }
    return SWR_OK;
}

NeuralTrainArgs train_args(swr_neural_t* n) {
    NeuralTrainArgs a = {};
    a.n = n->d;
    a.latent = n->latent;
    a.latentGrad = n->latentGrad;
    a.partial = n->partial;
    a.loss = n->loss;
    a.status = n->status;
    a.seedLo = (uint32_t)n->seed, a.seedHi = (uint32_t)(n->seed >> 32);
    return a;
}

}  // namespace

namespace swr {
// Brings the FP16 inference latents up to date with the FP32 master copy.
void neural_sync_half(swr_neural_t* n, cudaStream_t st) {
    if (!n->halfStale) return;
    LaunchScope ls("k_neural_export", st);
    launch_neural_export(n->latent, n->latentHalf, (size_t)n->d.numMaterials * n->d.texelsPerMaterial * 8, st);
    n->halfStale = false;
}
int neural_num_sms() { return num_sms(); }
}  // namespace swr

extern "C" {

swr_status swr_neural_create(const swr_texture* textures, uint32_t num_materials, uint32_t latent_levels, uint64_t seed,
                             swr_neural* out) {
    if (!textures || !out) return swr_internal_fail(SWR_EINVAL, "swr_neural_create: NULL argument");
    *out = nullptr;
    if (num_materials == 0 || num_materials > 1024)
        return swr_internal_fail(SWR_EINVAL, "swr_neural_create: num_materials must be in [1, 1024]");
    if (latent_levels == 0 || latent_levels > kNeuralMaxLevels)
        return swr_internal_fail(SWR_EINVAL, "swr_neural_create: latent_levels must be in [1, 4]");
    uint32_t W = 0, H = 0;
    const uint32_t align = kNeuralDownscale << (latent_levels - 1);
    for (uint32_t i = 0; i < num_materials; i++) {
        const swr_texture t = textures[i];
        if (!t) continue;
        if (t->format != SWR_FORMAT_RGBA8U)
            return swr_internal_fail(SWR_EINVAL, "swr_neural_create: textures must be RGBA8");
        if (t->d.num_layers > 2) return swr_internal_fail(SWR_EINVAL, "swr_neural_create: textures have 1 or 2 layers");
        if (t->d.width % align || t->d.height % align || t->d.mip_levels < latent_levels + 2)
            return swr_internal_fail(SWR_EINVAL, "swr_neural_create: texture size not a multiple of 4 << (latent_levels-1) "
                                                 "or fewer than latent_levels + 2 mips");
        if (t->d.width > 16384 || t->d.height > 16384)
            return swr_internal_fail(SWR_EINVAL, "swr_neural_create: texture larger than 16384");
        if (W == 0) W = t->d.width, H = t->d.height;
        if (t->d.width != W || t->d.height != H)
            return swr_internal_fail(SWR_EINVAL, "swr_neural_create: all textures must have the same size");
    }
    if (W == 0) return swr_internal_fail(SWR_EINVAL, "swr_neural_create: no material has a texture");

    swr_neural_t* n = new swr_neural_t();
    n->seed = seed;
    n->d.numMaterials = num_materials;
    n->d.levels = latent_levels;
    uint32_t off = 0;
    for (uint32_t l = 0; l < latent_levels; l++) {
        n->d.levelOffset[l] = off;
        n->d.levelW[l] = (W >> l) / kNeuralDownscale;
        n->d.levelH[l] = (H >> l) / kNeuralDownscale;
        off += n->d.levelW[l] * n->d.levelH[l];
    }
    n->d.texelsPerMaterial = off;
    n->texHost.resize(num_materials);
    for (uint32_t i = 0; i < num_materials; i++) {
        if (textures[i]) n->texHost[i] = textures[i]->d;
        else memset(&n->texHost[i], 0, sizeof(DevTexture));
    }
    n->steps.assign(num_materials, 0);
    const size_t latentFloats = (size_t)num_materials * off * 8;
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    chk(dev_alloc(&n->tex, num_materials));
    chk(dev_alloc(&n->latent, latentFloats));
    chk(dev_alloc(&n->latentM, latentFloats));
    chk(dev_alloc(&n->latentV, latentFloats));
    chk(dev_alloc(&n->latentGrad, latentFloats));
    chk(dev_alloc(&n->latentHalf, latentFloats));
    chk(dev_alloc(&n->params, (size_t)num_materials * kNeuralParams));
    chk(dev_alloc(&n->paramM, (size_t)num_materials * kNeuralParams));
    chk(dev_alloc(&n->paramV, (size_t)num_materials * kNeuralParams));
    chk(dev_alloc(&n->image, (size_t)num_materials * kNeuralImage));
    chk(dev_alloc(&n->loss, 2));
    chk(dev_alloc(&n->status, 1));
    chk(dev_alloc(&n->counters, 4 * (size_t)(num_materials + 1) + kNeuralMaxDecoded));
    if (e != cudaSuccess) {
        free_model(n);
        return e == cudaErrorMemoryAllocation ? swr_internal_fail(SWR_ENOMEM, "swr_neural_create: out of device memory")
                                              : swr_internal_cuda_fail(e, "swr_neural_create");
    }
    std::vector<float> p((size_t)num_materials * kNeuralParams);
    for (uint32_t i = 0; i < num_materials; i++) init_params(&p[(size_t)i * kNeuralParams], seed, i);
    chk(cudaMemcpy(n->tex, n->texHost.data(), num_materials * sizeof(DevTexture), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(n->params, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice));
    chk(cudaMemsetAsync(n->paramM, 0, p.size() * sizeof(float), st));
    chk(cudaMemsetAsync(n->paramV, 0, p.size() * sizeof(float), st));
    chk(cudaMemsetAsync(n->latent, 0, latentFloats * sizeof(float), st));
    chk(cudaMemsetAsync(n->latentM, 0, latentFloats * sizeof(float), st));
    chk(cudaMemsetAsync(n->latentV, 0, latentFloats * sizeof(float), st));
    chk(cudaMemsetAsync(n->latentGrad, 0, latentFloats * sizeof(float), st));
    chk(cudaMemsetAsync(n->image, 0, (size_t)num_materials * kNeuralImage, st));
    chk(cudaMemsetAsync(n->status, 0, 4, st));
    n->d.tex = n->tex;
    n->d.latentHalf = n->latentHalf;
    n->d.image = n->image;
    n->d.waitNs = kDefaultWaitNs;
    if (e == cudaSuccess) {
        {
            LaunchScope ls("k_neural_image", st);
            launch_neural_image(n->params, n->image, num_materials, st);
        }
        {
            LaunchScope ls("k_neural_latent_init", st);
            launch_neural_latent_init(n->d, n->latent, st);
        }
        n->halfStale = true;
        neural_sync_half(n, st);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        free_model(n);
        return swr_internal_cuda_fail(e, "swr_neural_create");
    }
    *out = n;
    return SWR_OK;
}

swr_status swr_neural_set_wait_limit(swr_neural n, uint64_t limit_ns) {
    if (!n) return swr_internal_fail(SWR_EINVAL, "swr_neural_set_wait_limit: NULL handle");
    if (limit_ns == 0 || limit_ns > 60000000000ull)
        return swr_internal_fail(SWR_EINVAL, "swr_neural_set_wait_limit: the limit must be 1 ns to 60 s");
    n->d.waitNs = limit_ns;
    return SWR_OK;
}

swr_status swr_selftest_bounded_wait(uint64_t limit_ns) {
    if (limit_ns == 0 || limit_ns > 1000000000ull)
        return swr_internal_fail(SWR_EINVAL, "swr_selftest_bounded_wait: the limit must be 1 ns to 1 s");
    cudaStream_t st = swr_internal_stream();
    uint32_t* status = nullptr;
    cudaError_t e = cudaMalloc(&status, sizeof(uint32_t));
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_selftest_bounded_wait: status word");
    uint32_t s = 0;
    e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        LaunchScope ls("k_wait_selftest", st);
        launch_wait_selftest(status, limit_ns, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(status);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_selftest_bounded_wait");
    if (s & 1u) return swr_internal_fail(SWR_ETIMEOUT, "swr_selftest_bounded_wait: the wait gave up at its limit");
    return SWR_OK;
}

swr_status swr_neural_destroy(swr_neural n) {
    if (!n) return swr_internal_fail(SWR_EINVAL, "swr_neural_destroy: NULL handle");
    cudaStreamSynchronize(swr_internal_stream());
    free_model(n);
    return SWR_OK;
}

swr_status swr_neural_get_info(swr_neural n, swr_neural_info* info) {
    if (!n || !info) return swr_internal_fail(SWR_EINVAL, "swr_neural_get_info: NULL argument");
    memset(info, 0, sizeof(*info));
    info->num_materials = n->d.numMaterials;
    info->latent_levels = n->d.levels;
    info->texels_per_material = n->d.texelsPerMaterial;
    for (uint32_t l = 0; l < n->d.levels; l++)
        info->level_offset[l] = n->d.levelOffset[l], info->level_width[l] = n->d.levelW[l], info->level_height[l] = n->d.levelH[l];
    for (uint32_t m = 0; m < n->d.numMaterials; m++) {
        if (!has_texture(n, m)) continue;
        const DevTexture& t = n->texHost[m];
        const uint64_t layers = std::max<uint32_t>(t.num_layers, 1);
        info->latent_bytes += (uint64_t)n->d.texelsPerMaterial * 8 * 2;
        info->weight_bytes += kNeuralFwdImage;
        info->plain_bytes += (uint64_t)t.layer_stride * 4 * layers;
        const uint32_t firstPlain = n->d.levels + 2;  // levels the sampler still reads
        if (firstPlain < t.mip_levels) info->fallback_bytes += (uint64_t)(t.layer_stride - t.mip_offsets[firstPlain]) * 4 * layers;
    }
    return SWR_OK;
}

swr_status swr_neural_train(swr_neural n, uint32_t steps, uint32_t batch, uint32_t materials_per_step,
                            uint32_t level_weighting, float learning_rate, float* mean_loss) {
    if (!n) return swr_internal_fail(SWR_EINVAL, "swr_neural_train: NULL handle");
    std::vector<uint32_t> trainable;
    for (uint32_t m = 0; m < n->d.numMaterials; m++)
        if (has_texture(n, m)) trainable.push_back(m);
    const uint32_t G = materials_per_step;
    if (G == 0 || G > kNeuralMaxStepMaterials || G > trainable.size())
        return swr_internal_fail(SWR_EINVAL, "swr_neural_train: materials_per_step must be in [1, min(64, textured materials)]");
    if (batch == 0 || batch % (G * 128))
        return swr_internal_fail(SWR_EINVAL, "swr_neural_train: batch must be a multiple of 128 * materials_per_step");
    if (!(learning_rate > 0.0f)) return swr_internal_fail(SWR_EINVAL, "swr_neural_train: learning rate must be > 0");
    if (level_weighting > 2) return swr_internal_fail(SWR_EINVAL, "swr_neural_train: level_weighting must be 0, 1 or 2");
    if (steps == 0) return SWR_OK;
    const uint32_t spm = batch / G, tiles = spm / 128;
    const uint32_t cpm = std::max<uint32_t>(1, std::min<uint32_t>(tiles, (2 * num_sms() + G - 1) / G));
    swr_status s = ensure_partial(n, (size_t)G * cpm * kNeuralParams);
    if (s != SWR_OK) return s;
    cudaStream_t st = swr_internal_stream();
    NeuralTrainArgs a = train_args(n);
    a.partial = n->partial;
    a.numSlots = G, a.samplesPerMaterial = spm, a.ctasPerMaterial = cpm;
    a.levelShift = level_weighting;
    NeuralAdamArgs d = {};
    d.params = n->params, d.m = n->paramM, d.v = n->paramV, d.partial = n->partial, d.image = n->image;
    d.latent = n->latent, d.latentM = n->latentM, d.latentV = n->latentV, d.latentGrad = n->latentGrad;
    d.texelsPerMaterial = n->d.texelsPerMaterial;
    d.ctasPerMaterial = cpm, d.numSlots = G;
    d.lr = learning_rate, d.beta1 = 0.9f, d.beta2 = 0.999f, d.eps = 1e-8f;
    cudaError_t e = cudaSuccess;
    for (uint32_t k = 0; k < steps && e == cudaSuccess; k++) {
        for (uint32_t i = 0; i < G; i++) {
            const uint32_t m = trainable[(n->trainCalls * (uint64_t)G + i) % trainable.size()];
            a.materials[i] = d.materials[i] = m;
            const uint32_t tstep = ++n->steps[m];
            d.lrm[i] = (float)((double)learning_rate / (1.0 - std::pow(0.9, (double)tstep)));
            d.s2[i] = (float)(1.0 / std::sqrt(1.0 - std::pow(0.999, (double)tstep)));
        }
        a.step = n->trainCalls++;
        if (k + 1 == steps && mean_loss) e = cudaMemsetAsync(n->loss, 0, 8, st);
        {
            LaunchScope ls("k_neural_train", st);
            launch_neural_train(a, G * cpm, st);
        }
        {
            LaunchScope ls("k_neural_adam", st);
            launch_neural_adam(d, st);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    n->halfStale = true;
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_train");
    if (mean_loss) {
        float l[2] = {};
        e = cudaMemcpyAsync(l, n->loss, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_train");
        *mean_loss = l[1] > 0 ? l[0] / (l[1] * 8.0f) : 0.0f;
        return check_status(n, st, "swr_neural_train");
    }
    return SWR_OK;
}

swr_status swr_neural_gradients(swr_neural n, uint32_t material, const uint32_t* samples_device, uint32_t count,
                                float* param_grad, float* latent_grad, float* loss) {
    if (!n || !samples_device || !param_grad) return swr_internal_fail(SWR_EINVAL, "swr_neural_gradients: NULL argument");
    if (material >= n->d.numMaterials || !has_texture(n, material))
        return swr_internal_fail(SWR_EINVAL, "swr_neural_gradients: material out of range or without texture");
    if (count == 0 || count % 128) return swr_internal_fail(SWR_EINVAL, "swr_neural_gradients: count must be a positive multiple of 128");
    {
        std::vector<uint32_t> h(count);
        cudaError_t e = cudaMemcpy(h.data(), samples_device, count * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_gradients: samples");
        const DevTexture& t = n->texHost[material];
        for (uint32_t v : h) {
            const uint32_t lvl = v >> 28, x = v & 0x3FFF, y = (v >> 14) & 0x3FFF;
            if (lvl >= n->d.levels + 2 || x >= (t.width >> lvl) || y >= (t.height >> lvl))
                return swr_internal_fail(SWR_EINVAL, "swr_neural_gradients: sample outside the decoded levels");
        }
    }
    const uint32_t tiles = count / 128;
    const uint32_t cpm = std::min<uint32_t>(tiles, 2 * num_sms());
    swr_status s = ensure_partial(n, (size_t)cpm * kNeuralParams);
    if (s != SWR_OK) return s;
    cudaStream_t st = swr_internal_stream();
    const size_t T8 = (size_t)n->d.texelsPerMaterial * 8;
    float* g = n->latentGrad + (size_t)material * T8;
    cudaError_t e = cudaMemsetAsync(g, 0, T8 * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->loss, 0, 8, st);
    NeuralTrainArgs a = train_args(n);
    a.partial = n->partial;
    a.materials[0] = material;
    a.numSlots = 1, a.samplesPerMaterial = count, a.ctasPerMaterial = cpm;
    a.samples = samples_device;
    if (e == cudaSuccess) {
        LaunchScope ls("k_neural_train", st);
        launch_neural_train(a, cpm, st);
        e = cudaGetLastError();
    }
    std::vector<float> part((size_t)cpm * kNeuralParams);
    float l[2] = {};
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), n->partial, part.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && latent_grad) e = cudaMemcpyAsync(latent_grad, g, T8 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(l, n->loss, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemsetAsync(g, 0, T8 * sizeof(float), st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_gradients");
    for (uint32_t i = 0; i < kNeuralParams; i++) {
        float v = 0.f;
        for (uint32_t c = 0; c < cpm; c++) v += part[(size_t)c * kNeuralParams + i];
        param_grad[i] = v;
    }
    if (loss) *loss = l[0];
    return check_status(n, st, "swr_neural_gradients");
}

// Training checkpoint: a versioned little-endian blob of everything the training trajectory depends
// on (header, per-material Adam step counts, parameters, latents and their Adam moments).
namespace {
constexpr uint32_t kCheckpointMagic = 0x4E525753u;  // "SWRN"
constexpr uint32_t kCheckpointVersion = 1;
struct CheckpointHeader {
    uint32_t magic, version, numMaterials, levels, texelsPerMaterial, paramsPerMaterial;
    uint64_t seed;
    uint64_t trainCalls;
};
static_assert(sizeof(CheckpointHeader) == 40, "checkpoint header");

size_t checkpoint_size(const swr_neural_t* n) {
    const size_t M = n->d.numMaterials, P = (size_t)M * kNeuralParams, T = (size_t)M * n->d.texelsPerMaterial * 8;
    return sizeof(CheckpointHeader) + M * sizeof(uint32_t) + 3 * P * sizeof(float) + 3 * T * sizeof(float);
}
}  // namespace

swr_status swr_neural_save(swr_neural n, void* dst, size_t capacity, size_t* size) {
    if (!n || !size) return swr_internal_fail(SWR_EINVAL, "swr_neural_save: NULL argument");
    const size_t need = checkpoint_size(n);
    *size = need;
    if (!dst) return SWR_OK;
    if (capacity < need) return swr_internal_fail(SWR_ECAPACITY, "swr_neural_save: the buffer is smaller than the checkpoint");
    const size_t M = n->d.numMaterials, P = M * kNeuralParams, T = M * (size_t)n->d.texelsPerMaterial * 8;
    CheckpointHeader h = { kCheckpointMagic, kCheckpointVersion, n->d.numMaterials, n->d.levels, n->d.texelsPerMaterial,
                           kNeuralParams, n->seed, n->trainCalls };
    uint8_t* p = (uint8_t*)dst;
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    memcpy(p, n->steps.data(), M * sizeof(uint32_t));
    p += M * sizeof(uint32_t);
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaSuccess;
    const float* src[6] = { n->params, n->paramM, n->paramV, n->latent, n->latentM, n->latentV };
    const size_t cnt[6] = { P, P, P, T, T, T };
    for (int i = 0; i < 6 && e == cudaSuccess; i++) {
        e = cudaMemcpyAsync(p, src[i], cnt[i] * sizeof(float), cudaMemcpyDeviceToHost, st);
        p += cnt[i] * sizeof(float);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_save");
}

swr_status swr_neural_load(swr_neural n, const void* src, size_t size) {
    if (!n || !src) return swr_internal_fail(SWR_EINVAL, "swr_neural_load: NULL argument");
    CheckpointHeader h;
    if (size < sizeof(h)) return swr_internal_fail(SWR_EINVAL, "swr_neural_load: blob too short");
    memcpy(&h, src, sizeof(h));
    if (h.magic != kCheckpointMagic || h.version != kCheckpointVersion)
        return swr_internal_fail(SWR_EINVAL, "swr_neural_load: not a decoder checkpoint of this version");
    if (h.numMaterials != n->d.numMaterials || h.levels != n->d.levels || h.texelsPerMaterial != n->d.texelsPerMaterial ||
        h.paramsPerMaterial != kNeuralParams)
        return swr_internal_fail(SWR_EINVAL, "swr_neural_load: the checkpoint was saved from a model of another shape");
    if (size != checkpoint_size(n)) return swr_internal_fail(SWR_EINVAL, "swr_neural_load: blob size does not match");
    const size_t M = n->d.numMaterials, P = M * kNeuralParams, T = M * (size_t)n->d.texelsPerMaterial * 8;
    const uint8_t* p = (const uint8_t*)src + sizeof(h);
    cudaStream_t st = swr_internal_stream();
    // the blob stays host memory the caller may free on return: copy synchronously
    cudaError_t e = cudaStreamSynchronize(st);
    float* dst[6] = { n->params, n->paramM, n->paramV, n->latent, n->latentM, n->latentV };
    const size_t cnt[6] = { P, P, P, T, T, T };
    const uint8_t* q = p + M * sizeof(uint32_t);
    for (int i = 0; i < 6 && e == cudaSuccess; i++) {
        e = cudaMemcpyAsync(dst[i], q, cnt[i] * sizeof(float), cudaMemcpyHostToDevice, st);
        q += cnt[i] * sizeof(float);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_load");
    memcpy(n->steps.data(), p, M * sizeof(uint32_t));
    n->seed = h.seed;
    n->trainCalls = (uint32_t)h.trainCalls;
    {
        LaunchScope ls("k_neural_image", st);
        launch_neural_image(n->params, n->image, n->d.numMaterials, st);  // the BF16 operand image of the parameters
    }
    n->halfStale = true;
    e = cudaGetLastError();
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_load");
}

swr_status swr_neural_get_params(swr_neural n, uint32_t material, float* params) {
    if (!n || !params || material >= n->d.numMaterials) return swr_internal_fail(SWR_EINVAL, "swr_neural_get_params: bad argument");
    cudaError_t e = cudaMemcpyAsync(params, n->params + (size_t)material * kNeuralParams, kNeuralParams * sizeof(float),
                                    cudaMemcpyDeviceToHost, swr_internal_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(swr_internal_stream());
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_get_params");
}

swr_status swr_neural_set_params(swr_neural n, uint32_t material, const float* params) {
    if (!n || !params || material >= n->d.numMaterials) return swr_internal_fail(SWR_EINVAL, "swr_neural_set_params: bad argument");
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync(n->params + (size_t)material * kNeuralParams, params, kNeuralParams * sizeof(float),
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
        LaunchScope ls("k_neural_image", st);
        launch_neural_image(n->params, n->image, n->d.numMaterials, st);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_set_params");
}

swr_status swr_neural_get_latents(swr_neural n, uint32_t material, float* latents) {
    if (!n || !latents || material >= n->d.numMaterials) return swr_internal_fail(SWR_EINVAL, "swr_neural_get_latents: bad argument");
    const size_t T8 = (size_t)n->d.texelsPerMaterial * 8;
    cudaError_t e = cudaMemcpyAsync(latents, n->latent + (size_t)material * T8, T8 * sizeof(float), cudaMemcpyDeviceToHost,
                                    swr_internal_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(swr_internal_stream());
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_get_latents");
}

swr_status swr_neural_set_latents(swr_neural n, uint32_t material, const float* latents) {
    if (!n || !latents || material >= n->d.numMaterials) return swr_internal_fail(SWR_EINVAL, "swr_neural_set_latents: bad argument");
    const size_t T8 = (size_t)n->d.texelsPerMaterial * 8;
    cudaStream_t st = swr_internal_stream();
    cudaError_t e = cudaMemcpyAsync(n->latent + (size_t)material * T8, latents, T8 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    n->halfStale = true;
    return e == cudaSuccess ? SWR_OK : swr_internal_cuda_fail(e, "swr_neural_set_latents");
}

swr_status swr_neural_decode(swr_neural n, uint32_t material, const uint32_t* texels_device, uint32_t count, uint32_t* out_device) {
    if (!n || !texels_device || !out_device) return swr_internal_fail(SWR_EINVAL, "swr_neural_decode: NULL argument");
    if (material >= n->d.numMaterials || !has_texture(n, material))
        return swr_internal_fail(SWR_EINVAL, "swr_neural_decode: material out of range or without texture");
    if (count == 0) return SWR_OK;
    cudaStream_t st = swr_internal_stream();
    neural_sync_half(n, st);
    // one material: the request list is the texel list itself, slot i = texel i
    std::vector<unsigned long long> req(count);
    std::vector<uint32_t> tex(count);
    cudaError_t e = cudaMemcpyAsync(tex.data(), texels_device, count * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_decode");
    for (uint32_t i = 0; i < count; i++) {
        const uint32_t lvl = tex[i] >> 28, x = tex[i] & 0x3FFF, y = (tex[i] >> 14) & 0x3FFF;
        const DevTexture& t = n->texHost[material];
        if (lvl >= n->d.levels + 2 || x >= (t.width >> lvl) || y >= (t.height >> lvl))
            return swr_internal_fail(SWR_EINVAL, "swr_neural_decode: texel outside the decoded levels");
        req[i] = ((unsigned long long)i << 32) | tex[i];
    }
    const uint32_t M = n->d.numMaterials, tiles = (count + 127) / 128;
    std::vector<uint32_t> offs(2 * (M + 1));
    for (uint32_t m = 0; m <= M; m++) {
        offs[m] = m <= material ? 0 : count;
        offs[M + 1 + m] = m <= material ? 0 : tiles;
    }
    unsigned long long* dreq = nullptr;
    uint32_t* doff = nullptr;
    e = cudaMallocAsync(&dreq, count * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&doff, offs.size() * 4, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dreq, req.data(), count * sizeof(unsigned long long), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(doff, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        NeuralDecodeArgs a = {};
        a.n = n->d;
        a.sorted = dreq, a.reqOffset = doff, a.tileOffset = doff + M + 1;
        a.out = (uint2*)out_device;
        a.status = n->status;
        LaunchScope ls("k_neural_decode", st);
        launch_neural_decode(a, std::min<uint32_t>(tiles, neural_decode_blocks_per_sm() * num_sms()), st);
        e = cudaGetLastError();
    }
    if (dreq) cudaFreeAsync(dreq, st);
    if (doff) cudaFreeAsync(doff, st);
    if (e != cudaSuccess) return swr_internal_cuda_fail(e, "swr_neural_decode");
    return check_status(n, st, "swr_neural_decode");
}

}  // extern "C"
