// bulk.cuh -- 1-D bulk copies (cp.async.bulk, global -> shared) completing on
// mbarriers, with bounded waits.  Shared by the tensor-core class statistics
// (k_chosen.cu) and the tiled sort (k_sort.cu).
//
// Rules the callers keep: source and destination 16-byte aligned, sizes a
// multiple of 16 bytes, at most 2^20 - 1 bytes per phase of a barrier; every
// wait is bounded (about one second of clock) and reports expiry, after which
// the caller records an error flag and stops.  Global memory written by plain
// stores and then read by a bulk copy, and shared memory read or written by
// plain accesses before a bulk copy refills it, are ordered by a CTA barrier
// followed by fence_proxy_async() in the issuing thread.
#pragma once
#include <cstdint>

namespace gsea {

constexpr long long kWaitCycles = 2000000000ll;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; false after ~1 s
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}
// bounded wait that also gives up when another role of the CTA recorded a
// failure in *failed
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t bar, uint32_t parity, const volatile int* failed) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (*failed || clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// orders the issuing thread's earlier plain accesses (and, after a CTA
// barrier, the CTA's) before its later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }
// makes mbarrier initialisation visible to the bulk-copy unit
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

}  // namespace gsea
