// Shared device-side building blocks for the sm_103a gravity kernels:
// status codes, bounded mbarrier waits, non-tensor TMA bulk copies and the
// packed two-lane FP32 helpers used by the force loops.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nbody_gb300.h"

namespace nbody {

// Upper bound on any spin-wait in these kernels. A wait that runs past it
// records NBODY_ERR_TIMEOUT in the context's status word and gives up; the
// kernel then drains its own copies (again bounded) and returns. Copies from
// L2/HBM land in microseconds, so the bound only trips on a broken invariant.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s
constexpr uint32_t kWaitSpinCheck = 1024;                     // polls between clock reads
constexpr uint32_t kWaitSpinCap = 1u << 30;                   // polls at most, should the clock ever stall

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void record_error(int *status, int code) {
    if (status) atomicCAS(status, NBODY_OK, code);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
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

// Waits for the phase with the given parity to complete, for at most
// limit_ns (and kWaitSpinCap polls). Returns false (and records
// NBODY_ERR_TIMEOUT) on time-out.
__device__ __forceinline__ bool mbar_wait_bounded_ns(uint64_t *bar, uint32_t parity, int *status,
                                                     unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (uint32_t spin = 0; spin < kWaitSpinCap; ++spin) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((spin % kWaitSpinCheck) == kWaitSpinCheck - 1 && global_ns() - t0 > limit_ns) break;
    }
    record_error(status, NBODY_ERR_TIMEOUT);
    return false;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *status) {
    return mbar_wait_bounded_ns(bar, parity, status, kWaitLimitNs);
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) accesses to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Non-tensor bulk copy global -> shared, completing `bytes` on the mbarrier.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void tma_bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// 1/sqrt(x), hardware approximation, flush-to-zero (inputs here are >= eps^2).
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

}  // namespace nbody
