// Blackwell (sm_103a) primitives written as inline PTX: shared-memory
// mbarriers, bulk global->shared copies (cp.async.bulk), and the 5th
// generation tensor core (tcgen05: TMEM allocation, MMA from shared-memory
// operand descriptors, commit to an mbarrier, TMEM loads).
//
// Operand layout used throughout: BF16 tiles of R rows x K columns, K-major
// ("K contiguous"), no swizzle.  The tile is made of 8x8 core matrices of 128
// contiguous bytes (8 rows of 16 bytes); core matrix (r/8, k/8) starts at
// (r/8) * SBO + (k/8) * LBO with LBO = 128 bytes (next core matrix along K)
// and SBO = K * 16 bytes (next 8-row group).
//
// Every wait is bounded: after TC_WAIT_LIMIT failed polls the caller gets
// `false`, records an error and leaves the loop, so a kernel never spins
// without end.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace omdg {

constexpr int TC_WAIT_LIMIT = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ------------------------------------------------------------------ mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        "  .reg .pred p;\n"
        "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "  selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, int polls) {
    for (int k = 0; k < polls; k++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait_n(bar, parity, TC_WAIT_LIMIT);
}

// A wait of `polls` (the run-time limit, omdg_set_wait_polls) that, when it
// gives up, marks the CTA aborted and then waits up to TC_WAIT_LIMIT polls
// more on the same phase: the copy or MMA this CTA itself issued on the
// barrier finishes before the CTA frees its TMEM and shared memory.
__device__ __forceinline__ void mbar_wait_or_drain(uint64_t* bar, uint32_t parity, int polls, volatile int& abort) {
    if (mbar_wait_n(bar, parity, polls)) return;
    abort = 1;
    mbar_wait_n(bar, parity, TC_WAIT_LIMIT);
}

// ------------------------------------------------------------------ bulk copy
// global -> shared, completion counted in bytes on `bar`; 16-byte aligned
// addresses and a size that is a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Generic-proxy shared-memory writes made visible to the async proxy (MMA).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ------------------------------------------------------------------ tcgen05
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

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Instruction descriptor, kind::f16: BF16 A and B (both K-major), FP32 D.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
    return (1u << 4)                            // D format F32
           | (1u << 7)                          // A format BF16
           | (1u << 10)                         // B format BF16
           | ((uint32_t)(N >> 3) << 17)         // N / 8
           | ((uint32_t)(M >> 4) << 24);        // M / 16
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n"
        "  .reg .pred p;\n"
        "  setp.ne.b32 p, %4, 0;\n"
        "  tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier completes once every MMA this thread issued before has finished.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of the calling thread's TMEM lane.  The values
// are valid after tc_wait_ld on the same array.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

// Waits for this thread's TMEM loads; ties the registers to the wait so that
// no use is scheduled before it.
__device__ __forceinline__ void tc_wait_ld(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// Element offset of (r, k) in an R x K core-matrix tile (see the header).
__host__ __device__ __forceinline__ int tc_tile_off(int r, int k, int K) {
    return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

}  // namespace omdg
