// tma.cuh -- mbarrier and Tensor Memory Accelerator (TMA) helpers in inline
// PTX, shared by the tensor-core convolution (tc_conv.cuh) and the
// plane-streaming multigrid stencils (multigrid.cu).
//
// Every wait on an mbarrier is bounded: a kernel that gives up records the
// failure in a device flag and leaves, after waiting (again bounded) for the
// copies it has in flight.  Tensor maps describe this GPU's own memory only,
// and no load uses cluster multicast.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace saras {

__device__ __forceinline__ uint32_t su32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t *m, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(su32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on an mbarrier phase; false (and *err = 1) after the poll limit.
__device__ __forceinline__ bool mbar_wait(uint64_t *m, uint32_t parity, int *err) {
    for (int it = 0; it < (1 << 21); ++it)
        if (mbar_try_wait(m, parity)) return true;
    if (err) atomicExch(err, 1);
    return false;
}
// Bounded wait that lets the thread sleep between polls: each try_wait may
// suspend the thread for up to kWaitHintNs until the phase completes (the
// hardware wakes it), so waiting threads do not take issue slots from the
// ones computing; at most kWaitPolls polls (about a second in all).
constexpr uint32_t kWaitHintNs = 20000;
constexpr int kWaitPolls = 50000;
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(m)), "r"(parity), "r"(kWaitHintNs)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *m, uint32_t parity, int *err) {
    for (int it = 0; it < kWaitPolls; ++it)
        if (mbar_try_wait_sleep(m, parity)) return true;
    if (err) atomicExch(err, 1);
    return false;
}
// One plain arrival.
__device__ __forceinline__ void mbar_arrive(uint64_t *m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(su32(m)) : "memory");
}
// One arrival that also announces `bytes` of asynchronous transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(su32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// Tiled 2D tensor load of one box into shared memory, completing `bytes` of
// transactions on mbarrier m (the box size the tensor map declares).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *m) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(su32(m))
        : "memory");
}

}  // namespace saras
