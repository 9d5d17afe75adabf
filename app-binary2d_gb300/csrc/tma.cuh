// tma.cuh — bulk asynchronous copies (TMA, cp.async.bulk) and mbarriers in
// inline PTX, with bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace b2d {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async proxy.
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Order earlier generic-proxy shared-memory accesses before later bulk copies.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase of parity `parity` to complete; gives up after about one
// second (or 2^26 polls) and returns false, so no wait can hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < (1u << 26); ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > 1000000000ull) break;
    }
    return false;
}

// 1-D bulk copy global -> shared, completing `bytes` on `bar`.  Both addresses
// must be 16-byte aligned and `bytes` a multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Read-set check.  A build with B2D_POISON defined fills every stage kernel's
// dynamic shared memory with quiet NaN before the kernel uses it (each 32-bit
// word, so an FP64 slot reads as NaN too), and the paired kernel also sets the
// stencil points its halo lanes read from outside the staged columns to NaN.
// A slot that a zone's update reads without the kernel having written it, or
// a guard-column value that reaches a zone's update, then turns that zone NaN;
// a poisoned build that reproduces the normal build's states bit for bit shows
// that neither happens.  Without B2D_POISON this is empty.
__device__ __forceinline__ void poison_dynamic_smem(unsigned char* base)
{
#ifdef B2D_POISON
    uint32_t bytes;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(bytes));
    for (uint32_t i = 4 * threadIdx.x; i + 4 <= bytes; i += 4 * blockDim.x)
        *(uint32_t*)(base + i) = 0x7fc00000u;
    __syncthreads();
#else
    (void)base;
#endif
}

__device__ __forceinline__ float poison_or(float v)
{
#ifdef B2D_POISON
    (void)v;
    return __int_as_float(0x7fc00000);
#else
    return v;
#endif
}

}  // namespace b2d
