// async_copy.cuh -- inline-PTX wrappers for the asynchronous copy engines
// used by the step kernels: mbarriers, 1-D bulk copies (TMA,
// cp.async.bulk) global -> shared with transaction counts, and 16-byte
// cp.async gathers.
#pragma once

#include <cstdint>

namespace tg {
namespace {

constexpr uint32_t kWaitLimit = 1u << 24;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// 1-D bulk copy global -> shared, completion counted on bar (bytes % 16 == 0,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(__cvta_generic_to_global(src))
                 : "memory");
}
// Arrives on bar once this thread's earlier cp.async copies have landed
// (the barrier's expected count includes this arrival).
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait on an mbarrier phase; gives up early when another warp
// raised the abort word.  sleep_ns > 0 backs off between polls (a producer
// that runs ahead waits this way so that its polling does not take issue
// slots from the consumers on its scheduler).
__device__ __forceinline__ bool bounded_wait(uint64_t *bar, uint32_t parity, volatile int *abort_word,
                                             unsigned sleep_ns = 0) {
    for (uint32_t it = 0; it < kWaitLimit; it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && *abort_word) return false;
        if (sleep_ns) __nanosleep(sleep_ns);
    }
    return false;
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// An L2 cache policy for data read once per step (evict first), for the
// bulk copies below: the slab, actuation and incidence blocks then leave L2
// before the state records, which halo gathers and the next step re-read.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// 1-D bulk copy with an L2 cache-policy hint (same rules as bulk_g2s)
__device__ __forceinline__ void bulk_g2s_hint(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                              uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ uint32_t issue_chunks_hint(uint8_t *dst, const uint8_t *src, uint32_t bytes, uint64_t *bar,
                                                      uint64_t pol) {
    constexpr uint32_t kChunk = 32768;
    for (uint32_t o = 0; o < bytes; o += kChunk) {
        uint32_t b = bytes - o < kChunk ? bytes - o : kChunk;
        bulk_g2s_hint(dst + o, src + o, b, bar, pol);
    }
    return bytes;
}

// Bulk copy in pieces of at most 32 KB (each 16-byte aligned, a multiple of
// 16 bytes when the total is); returns the byte count.
__device__ __forceinline__ uint32_t issue_chunks(uint8_t *dst, const uint8_t *src, uint32_t bytes, uint64_t *bar) {
    constexpr uint32_t kChunk = 32768;
    for (uint32_t o = 0; o < bytes; o += kChunk) {
        uint32_t b = bytes - o < kChunk ? bytes - o : kChunk;
        bulk_g2s(dst + o, src + o, b, bar);
    }
    return bytes;
}

}  // namespace
}  // namespace tg
