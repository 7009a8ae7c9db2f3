// Inline-PTX synchronisation and bulk-copy primitives shared by the sm_103a kernels: acquire/release flags in
// global memory, CTA mbarriers with transaction counts, 1D bulk copies (TMA) into shared memory and the fences
// between the generic and the async proxy.
#pragma once

#include <stdint.h>

namespace sister {
namespace ptx {

__device__ __forceinline__ uint32_t sptr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// a strong load without ordering: the warp does not wait for it until the value is used
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// after relaxed loads that observed released flags: makes the flags' data visible to this thread (acquire pattern)
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
// order this thread's generic-proxy view of global memory (acquired data) before its bulk copies
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
// order this thread's generic-proxy writes of shared memory before bulk copies into the same memory
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
// makes initialised mbarriers visible to the async proxy (the bulk copies' complete_tx)
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(uint32_t a) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
                 : "memory");
}
// 1D bulk copy global -> shared of this CTA, completion counted on mbarrier `bar`
// (both addresses 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// non-blocking test of the phase of parity `par`
__device__ __forceinline__ bool mbar_test(uint32_t a, uint32_t par) {
    uint32_t ok;
    asm volatile("{ .reg .pred p; mbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2; "
                 "selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok)
                 : "r"(a), "r"(par)
                 : "memory");
    return ok != 0;
}
// blocking test: the warp sleeps until the phase completes or about `ns` nanoseconds pass, so waiting
// warps take no issue slots from the warps doing the arithmetic
__device__ __forceinline__ bool mbar_sleep(uint32_t a, uint32_t par, uint32_t ns) {
    uint32_t ok;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3; "
                 "selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok)
                 : "r"(a), "r"(par), "r"(ns)
                 : "memory");
    return ok != 0;
}
constexpr uint32_t kSleepNs = 20000; // suspend hint of one blocking test
// Wait for the phase of parity `par` with a time limit only: used to drain bulk copies still in flight
// before barriers are re-initialised or the CTA exits.
__device__ __forceinline__ void mbar_drain(uint32_t a, uint32_t par, unsigned limit_us) {
    if (mbar_test(a, par)) return;
    const unsigned long long t0 = global_ns();
    while (!mbar_sleep(a, par, kSleepNs) && global_ns() - t0 <= 1000ull * limit_us) {
    }
}

} // namespace ptx
} // namespace sister
