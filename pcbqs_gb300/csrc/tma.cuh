// Bulk (TMA) copies into shared memory and bounded mbarrier waits, as inline PTX for sm_103a.
#pragma once
#include <cstdint>

namespace pq {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One arrival that also announces `bytes` of transaction count to be completed by bulk copies.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared, completing `bytes` on `bar`. Both addresses 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Non-blocking probe of phase `phase`.
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Limits below this many SM clocks are polled with the non-blocking probe: try_wait may itself suspend the thread
// until the phase completes (a system-dependent time), which would outlast a short limit.
constexpr unsigned long long PROBE_BELOW_CYCLES = 1ull << 16;

// Wait for phase `phase` of `bar` for at most `limit` SM clocks. Returns false when the limit ran out; the caller
// records the failure and, before its block exits, waits again (with a long limit) for the copies it issued.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, unsigned long long limit) {
    const long long t0 = clock64();
    const bool probe = limit < PROBE_BELOW_CYCLES;
    for (;;) {
        if (probe ? mbar_test_wait(bar, phase) : mbar_try_wait(bar, phase)) return true;
        if ((unsigned long long)(clock64() - t0) > limit) return false;
    }
}

}  // namespace pq
