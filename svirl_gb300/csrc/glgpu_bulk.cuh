// Asynchronous bulk copies into shared memory (the Blackwell copy engine, TMA)
// tracked by mbarriers, as inline PTX (sm_90+ instructions, built for sm_103a).
//
//   mbar_init / fence_mbar_init     set up a barrier (count = expected arrivals)
//   mbar_arrive_expect_tx           one arrival that also expects `bytes` of copies
//   mbar_arrive                     one arrival
//   mbar_wait                       wait for a phase, bounded: false if it did not
//                                   complete within `spins` polls
//   bulk_g2s                        global -> shared copy of `bytes` (both addresses
//                                   16-byte aligned, bytes a multiple of 16) that
//                                   signals completion to the barrier
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace glgpu {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity; try_wait itself suspends the
// thread for a while before reporting "not yet", so `spins` polls last far longer
// than any copy.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int spins) {
    for (int t = 0; t < spins; ++t)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

}  // namespace glgpu
