// Blackwell (sm_103a) tensor-core building blocks in inline PTX: mbarriers with bounded waits,
// bulk async copies, TMEM allocation, tcgen05.mma (kind::f16, BF16 in, FP32 accumulate in TMEM),
// tcgen05.commit and tcgen05.ld, plus the shared-memory operand layout the neural texture kernels
// use.
//
// Operand layout ("slabs"): a BF16 matrix of R rows x C columns is stored as C/8 slabs of R rows x
// 16 bytes; inside a slab the 8-row x 16-byte core matrices follow each other (row r at byte
// (r/8)*128 + (r%8)*16). Element (r, c) sits at byte (c/8)*R*16 + (r/8)*128 + (r%8)*16 + (c%8)*2.
// A row of 8 columns is one 16-byte vector store, and a warp storing rows 0..31 of a slab writes
// 512 contiguous bytes. The same bytes serve two no-swizzle canonical layouts:
//  * K-major (rows = M or N, columns = K): core matrices step 128 bytes along M/N (SBO) and R*16
//    bytes along K (LBO);
//  * MN-major (rows = K, columns = M or N): core matrices step 128 bytes along K (LBO) and R*16
//    bytes along M/N (SBO).
// So activations written once per sample row feed both the forward MMAs (samples = M, features =
// K) and the weight-gradient MMAs (features = M/N, samples = K) without a transposed copy.
#pragma once
#include <cstdint>

namespace swr {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity to complete; gives up after `limit_ns` nanoseconds
// and returns false (the caller records the failure and leaves without touching the results).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = 1000000000ull) {
    const uint32_t a = smem_u32(bar);
    if (mbar_try_wait(a, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    while (true) {
        for (int i = 0; i < 64; i++)
            if (mbar_try_wait(a, parity)) return true;
        if (global_timer_ns() - t0 > limit_ns) return false;
    }
}

// The wait of a copy or MMA that was issued: when it gives up after limit_ns, the operation is still
// in flight and would land in shared memory or TMEM the CTA is about to release, so this waits for
// the phase once more (at most one further second) before returning false.
__device__ __forceinline__ bool mbar_wait_drained(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_wait(bar, parity, limit_ns)) return true;
    mbar_wait(bar, parity, 1000000000ull);
    return false;
}

// ---------------------------------------------------------------------------- bulk copies
// global -> shared, completion counted in bytes on `bar` (addresses 16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// ---------------------------------------------------------------------------- fences
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---------------------------------------------------------------------------- TMEM
// Executed by one whole warp; the allocated base address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32*(w%4)..+31); the
// wait for the load is part of the same statement, so the registers are valid on return.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------- MMA
// Shared-memory matrix descriptor, no swizzle: start, leading and stride byte offsets (all
// multiples of 16), descriptor version 1 in bits 46-48.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Descriptor of a slab-layout operand with R rows, first slab at `saddr`.
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, uint32_t R) { return sdesc(saddr, R * 16, 128); }
__device__ __forceinline__ uint64_t desc_mnmajor(uint32_t saddr, uint32_t R) { return sdesc(saddr, 128, R * 16); }

// Instruction descriptor for kind::f16: FP32 D, BF16 A and B, dense; a_mn / b_mn select MN-major
// operands; N in bits 17-22 (N/8), M in bits 24-28 (M/16).
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N, bool aMN, bool bMN) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((aMN ? 1u : 0u) << 15) | ((bMN ? 1u : 0u) << 16) | ((N >> 3) << 17) |
           ((M >> 4) << 24);
}

// D[tmem] (+)= A * B^T over one K=16 step (issued by a single thread).
__device__ __forceinline__ void mma_bf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
        "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrives once on `bar` when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// ---------------------------------------------------------------------------- BF16 packing
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}
// Stores 8 consecutive columns (one 16-byte row of a slab) of row `row` of a slab matrix.
__device__ __forceinline__ void store_row8(uint8_t* slabBase, uint32_t R, uint32_t slab, uint32_t row, const float* v) {
    uint4 q;
    q.x = pack_bf16x2(v[0], v[1]);
    q.y = pack_bf16x2(v[2], v[3]);
    q.z = pack_bf16x2(v[4], v[5]);
    q.w = pack_bf16x2(v[6], v[7]);
    *(uint4*)(slabBase + slab * R * 16 + (row >> 3) * 128 + (row & 7) * 16) = q;
}
__host__ __device__ constexpr uint32_t slab_offset(uint32_t R, uint32_t row, uint32_t col) {
    return (col >> 3) * R * 16 + (row >> 3) * 128 + (row & 7) * 16 + (col & 7) * 2;
}

}  // namespace tc
}  // namespace swr
