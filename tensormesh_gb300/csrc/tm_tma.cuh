// Bulk asynchronous copies global -> shared memory (the 1-D form of the
// Tensor Memory Accelerator, cp.async.bulk) completed on an mbarrier, and a
// bounded wait on that barrier.  PTX ISA: "cp.async.bulk", "mbarrier".
//
// A copy needs its global source and shared destination on 16-byte
// boundaries and a size that is a multiple of 16 bytes; stage_range() below
// widens an element range of an array to such a window.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmk {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also announces the bytes the copies will deliver
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// true once the barrier's phase `parity` has completed; false after
// max_iter unsuccessful tries (each try may suspend the thread briefly)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_iter) {
    for (uint32_t i = 0; i < max_iter; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 16-byte window around elements [first, last) of an array of `esize`-byte
// elements: `begin` is the window's first byte offset, `bytes` its size and
// `skip` the number of elements before `first` inside the window
struct StageRange {
    int64_t begin;
    uint32_t bytes;
    int32_t skip;
};
__host__ __device__ inline StageRange stage_range(int64_t first, int64_t last, int esize) {
    const int64_t b0 = first * esize, b1 = last * esize;
    const int64_t lo = b0 & ~int64_t(15), hi = (b1 + 15) & ~int64_t(15);
    return {lo, (uint32_t)(hi - lo), (int32_t)((b0 - lo) / esize)};
}

// shared-memory bytes that hold any window of n elements
__host__ __device__ inline size_t stage_capacity(int64_t n, int esize) {
    return (size_t)(((n * esize + 15) & ~int64_t(15)) + 16);
}

}  // namespace tmk
