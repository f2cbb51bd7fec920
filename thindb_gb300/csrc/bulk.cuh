// bulk.cuh — mbarrier and bulk asynchronous copy (cp.async.bulk) helpers in
// inline PTX, shared by the kernels that stream tiles into shared memory.
// Every wait is bounded: a phase that never completes makes the wait return
// false after `cycles` SM clocks, and the caller reports ST_WAIT_TIMEOUT.
#pragma once

#include <cstdint>

namespace tgpu {
namespace {

constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s of SM clock before a phase counts as lost

__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One arrival per phase (the issuing thread's arrive.expect_tx).
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(s_addr(bar)) : "memory");
}

// `count` arrivals per phase.
__device__ __forceinline__ void mbar_init_n(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(bar)), "r"(count) : "memory");
}

// A plain arrival (release: this thread's earlier shared-memory accesses are
// ordered before the phase completes).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(s_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of `bar` to complete: false after `limit`
// SM clocks (0 = WAIT_CYCLES).  A short limit (the test hook
// tgpu_debug_set_wait_limit) checks the clock on every test.
__device__ __noinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = 0) {
    if (mbar_test(bar, parity)) return true;
    if (limit <= 0) limit = WAIT_CYCLES;
    const uint32_t every = limit < (1LL << 20) ? 0u : 63u;
    const long long t0 = clock64();
    for (uint32_t i = 1;; ++i) {
        if (mbar_test(bar, parity)) return true;
        if ((i & every) == 0) {
            if (clock64() - t0 > limit) return false;
            if (every) __nanosleep(32);
        }
    }
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global into this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(s_addr(dst)),
        "l"(src), "r"(bytes), "r"(s_addr(bar))
        : "memory");
}

// Order this thread's earlier generic-proxy accesses to shared memory before
// later bulk copies into it (a stage is refilled only after it was read).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

}  // namespace
}  // namespace tgpu
