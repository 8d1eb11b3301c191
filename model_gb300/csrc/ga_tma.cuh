// ---------------------------------------------------------------------------
// Tensor-memory-accelerator staging: 3-D tiled copies of field boxes from
// global to shared memory (cp.async.bulk.tensor) completed on an mbarrier,
// with a bounded wait.
//
// A field is [i][j][k], k fastest; its tensor map has dimensions
// {NZ, NY, NX} (innermost first), strides NZ*4 and NY*NZ*4 bytes, and a box of
// {BK, BJ, BI} floats.  Coordinates are (k, j, i); the k coordinate is always a
// multiple of 4 (16-byte aligned), j and i are never negative, and points
// outside the field (k < 0, k >= NZ, i >= NX, j >= NY) arrive as zeros.
// ---------------------------------------------------------------------------
#pragma once
#include <cuda.h>
#include <cstdint>

namespace ga {

// the maps of the seven current prognostic fields of one launch (u, v, w,
// theta, qv, qc, qr), passed by value as a __grid_constant__ kernel argument
struct TmaMaps {
    CUtensorMap m[7];
};

// bound of every wait on a staging barrier: 200 ms of wall clock, far above
// any copy's duration; past it the block records the failure and returns
constexpr unsigned long long kTmaWaitNs = 200ull * 1000ull * 1000ull;
constexpr int kErrStaging = 2;  // bit of the context's device error word

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes the initialised barrier visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the barrier; false when kTmaWaitNs passed first
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kTmaWaitNs) return false;
    return true;
}

// one box of a 3-D tensor map into shared memory (dst 128-byte aligned),
// completing `bytes` of the barrier's expected transaction count
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int k, int j, int i, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(k), "r"(j), "r"(i), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace ga
