// Bulk-copy (TMA) and mbarrier helpers for sm_100-family GPUs, as inline PTX.
//
// Every wait is bounded: a wait that does not complete within
// DD_WAIT_LIMIT polls reports failure instead of spinning forever, and the
// kernel records DD_ERR_TIMEOUT (dd_report_timeout), lets the copies it has
// issued and not yet waited for land (dd_mbar_drain, bounded by
// DD_DRAIN_LIMIT polls) and returns.  A build with a small DD_WAIT_LIMIT
// makes every wait give up at once while the drain still lets the copies
// land: that is how the timeout path is tested without a fault or a hang.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pridediff_dd.h"

#ifndef DD_WAIT_LIMIT
#define DD_WAIT_LIMIT (1u << 26)
#endif
#ifndef DD_DRAIN_LIMIT
#define DD_DRAIN_LIMIT (1u << 26)
#endif

// Host-visible copy of the timeout status: a word in host-mapped (pinned)
// memory that the caller registers with dd_set_status_sink.  Each translation
// unit holds its own copy of this pointer (file scope) and sets it in
// dd_set_status_sink_tu; kernels write DD_ERR_TIMEOUT there as well as
// into their workspace status word, so the host sees a timeout without a
// synchronisation.
static __device__ int *dd_status_sink = nullptr;

__device__ __forceinline__ void dd_report_timeout(int *status) {
    if (status) atomicExch(status, DD_ERR_TIMEOUT);
    int *sink = dd_status_sink;
    if (sink) atomicExch_system(sink, DD_ERR_TIMEOUT);
}

static inline int dd_set_status_sink_tu(int *sink) {
    return cudaMemcpyToSymbol(dd_status_sink, &sink, sizeof(sink)) == cudaSuccess ? 0 : 1;
}

__device__ __forceinline__ uint32_t dd_smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void dd_mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(dd_smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void dd_fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void dd_mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(dd_smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared, completion signalled on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void dd_bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dd_smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(dd_smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool dd_mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}" : "=r"(ok)
        : "r"(dd_smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Phase parities of a CTA's mbarriers, one bit per barrier.  A bit mask keeps
// them in a register; an array indexed by the buffer number would live in
// local memory and put a load and a store in front of every wait.
struct DdPhases {
    uint32_t bits = 0;
    __device__ __forceinline__ uint32_t parity(int b) const { return (bits >> b) & 1u; }
    __device__ __forceinline__ void flip(int b) { bits ^= 1u << b; }
};

// Bounded wait for the phase with the given parity.  Returns false on timeout.
__device__ __forceinline__ bool dd_mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < DD_WAIT_LIMIT; ++it) {
        if (dd_mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(32);
    }
    return false;
}

// After a timeout: wait (bounded by DD_DRAIN_LIMIT) for the phase of copies
// that were issued and not waited for, so that no bulk copy still writes into
// the CTA's shared memory when it returns.
__device__ __forceinline__ bool dd_mbar_drain(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < DD_DRAIN_LIMIT; ++it) {
        if (dd_mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(32);
    }
    return false;
}
