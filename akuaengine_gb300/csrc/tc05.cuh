// Fifth-generation tensor core (tcgen05) helpers for sm_103a: tensor-memory allocation, MMA issue
// and completion through an mbarrier, tensor-memory loads, and shared-memory operand layout.
//
// Operand layout: no swizzle, K-major.  A tile of R rows x K columns of 16-bit elements is a grid
// of "core matrices" of 8 rows x 8 elements (16 bytes per row, 128 contiguous bytes each).  Core
// matrix (row/8, k/8) starts at (row/8) * SBO + (k/8) * LBO with LBO = 128 bytes (core matrices
// adjacent in K are contiguous) and SBO = K * 16 bytes (the next 8-row group).  One MMA consumes
// K = 16 (two core matrices along K); the k-th step of a wider tile starts 256 bytes further.
//
// Accumulators (FP32) live in tensor memory: for M = 128 and cta_group::1, row m of D is TMEM
// lane m, column n is TMEM column (base + n).  A warp may read only its own 32-lane quarter
// (warp w % 4 -> lanes 32 (w % 4) .. + 31).
//
// Every wait on an mbarrier is bounded: on timeout the caller gets `false`, records an error
// and still releases its tensor memory.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace akua::tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) in a K-major tile with K columns (16-bit elements).
__host__ __device__ constexpr uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t K) {
    return (row >> 3) * (K * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte offsets,
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both operands K-major.
// Bits: D format [4,6) = 1 (F32); A format [7,10) = 1 (BF16); B format [10,13) = 1 (BF16);
// A/B major [15], [16] = 0 (K); N >> 3 at [17,23); M >> 4 at [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// --- tensor memory ------------------------------------------------------------------------------
// Executed by one full warp.  Writes the allocated base address to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// Executed by the warp that allocated.
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes -> visible to the tensor core's (async proxy) reads.
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// --- MMA ----------------------------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier at `bar` completes one phase when all previously issued MMAs of this thread are
// done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(bar))
        : "memory");
}

// --- mbarrier -----------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of `bar`.  Each try_wait suspends for a hardware-chosen time
// (about 4 µs per unsuccessful try on GB300, measured by tests/test_gpu_waits.py); the default
// bound, 2^18 tries (about a second), is far beyond any MMA's latency.  Returns false on timeout.
constexpr uint32_t kWaitTries = 1u << 18;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          uint32_t max_tries = kWaitTries) {
    for (uint32_t t = 0; t < max_tries; ++t)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// --- tensor memory -> registers -----------------------------------------------------------------
// Issues the load of 16 consecutive FP32 columns without waiting; tmem_wait_ld() before use.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// Ties registers written by an asynchronous tensor-memory load to the preceding wait: each passes
// through an (empty, volatile, hence ordered after the wait) statement, so no use of a register
// can be scheduled before the load has landed.
template <int N>
__device__ __forceinline__ void tmem_after_wait(uint32_t (&r)[N]) {
#pragma unroll
    for (int i = 0; i < N; ++i) asm volatile("" : "+r"(r[i]));
}

// 16 consecutive FP32 columns of this thread's TMEM lane.  `taddr` = base + (lane0 << 16) + col,
// lane0 = 32 * (warp % 4).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    tmem_after_wait(r);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace akua::tc
