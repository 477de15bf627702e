// mw_async.cuh -- asynchronous global -> shared bulk copies (TMA engine) completed on an
// mbarrier, with a bounded wait.  Used by the contraction kernels that prefetch the next item's
// input block and operator blocks while they compute the current one.
#pragma once

#include <cstdint>

namespace mwg {
namespace {

// ---- asynchronous bulk copies (TMA engine) into shared memory, completed on an mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// global -> shared, 16-byte aligned addresses and a size that is a multiple of 16
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Waits for the copies of the current phase, at most TMA_WAIT_LIMIT polls.  A wait that runs
// out marks the launch failed (the host turns the status into MW_ERR_TIMEOUT) and every later
// wait of the CTA returns at once, so the kernel still ends with all threads on the same path.
constexpr int TMA_WAIT_LIMIT = 1 << 20;

// `code` (non-zero) is what the status word receives: it tells which wait of the kernel ran out.
__device__ __forceinline__ void mbar_wait(uint64_t *bar, uint32_t parity, volatile int *fail, int *status,
                                          int code = 1) {
    if (*fail) return;
    for (int it = 0; it < TMA_WAIT_LIMIT; it++)
        if (mbar_try_wait(bar, parity)) return;
    *fail = 1;
    atomicExch(status, code);
}

}  // namespace
}  // namespace mwg
