// mpc_tma.cuh -- Tensor Memory Accelerator (TMA) copies and mbarriers for sm_103a, inline PTX.
//
// The strip kernels of the plane sweep stage their units with bulk tensor copies
// (cp.async.bulk.tensor) that complete on a shared-memory mbarrier, and write them back with
// bulk tensor stores, so that several units are in flight per CTA without spending registers
// or thread instructions on the copies.  Every wait on an mbarrier is bounded by a clock
// limit: a wait that runs out reports failure to the caller, which records an error code in
// global memory and leaves the kernel.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpc {

// a wait on an mbarrier gives up after this many SM clock cycles (about one second)
constexpr long long kWaitLimitCycles = 2000000000LL;

// error codes a kernel leaves in its error word (0 = none)
enum KernelError : unsigned int {
    KERR_NONE = 0,
    KERR_TMA_TIMEOUT = 1,   // a bulk tensor load did not complete within kWaitLimitCycles
    KERR_WAIT_PROBE = 2,    // the wait-limit probe's wait ran out (mpc_wait_limit_check)
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make mbarrier initialisation visible to the async proxy (the TMA unit)
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// order this thread's generic-proxy shared-memory writes before later async-proxy accesses
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Wait for the completion of the phase of parity `parity`; false when kWaitLimitCycles pass first.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_addr(bar);
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kWaitLimitCycles) return false;
    }
}

// 2-D tiled bulk tensor load of one box at coordinates (c0, c1) into shared memory; completes
// on `bar` (transaction bytes).  c0 * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            smem_addr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

// 2-D tiled bulk tensor store of one box from shared memory (bulk async-group completion)
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int c0, int c1, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(map), "r"(c0),
                 "r"(c1), "r"(smem_addr(src))
                 : "memory");
}

// contiguous bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from global
// to shared memory, completing on `bar`
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

// wait until at most N committed bulk groups still read their shared-memory source
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
// wait until at most N committed bulk groups are incomplete
template <int N>
__device__ __forceinline__ void bulk_wait() {
    asm volatile("cp.async.bulk.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace mpc
