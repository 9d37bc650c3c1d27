// tma.cuh -- Blackwell asynchronous copies into shared memory (inline PTX):
// mbarrier transaction barriers and 1-D bulk copies (cp.async.bulk; every
// staged object -- spectrum rows, column-pair blocks, twiddle plans -- is one
// contiguous run), plus a bounded barrier wait.
//
// Every wait is bounded by the global nanosecond timer.  On time-out the waiter
// records OCEAN_DEVICE_TIMEOUT in the handle's device status word, waits once
// more (bounded) for its copies in flight, and the block returns as a whole;
// the host reads the status with ocean_device_status().
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ocean {

constexpr unsigned kDeviceTimeout   = 1u;           // status bit: an mbarrier wait timed out
constexpr uint64_t kWaitLimitNs     = 200000000ull; // 0.2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of `bar`: false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    return true;
}

// 1-D bulk copy global -> shared, completing `bytes` transactions on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Block-wide wait executed by thread 0 with the result broadcast through
// shared memory; every thread gets the same answer, so a failing block exits
// as a whole.  On time-out the status word is flagged and thread 0 waits once
// more (bounded) so that copies still in flight land before the block exits.
__device__ __forceinline__ bool block_wait(uint64_t* bar, uint32_t parity, int* flag_smem, unsigned* status)
{
    if (threadIdx.x == 0) {
        bool ok = mbar_wait_bounded(bar, parity);
        if (!ok) {
            atomicOr(status, kDeviceTimeout);
            (void)mbar_wait_bounded(bar, parity);
        }
        *flag_smem = ok ? 1 : 0;
    }
    __syncthreads();
    return *flag_smem != 0;
}

// Ask L2 for [p, p + bytes) (cp.async.bulk.prefetch.L2: a hint, nothing
// waits for it), in 4 KB pieces spread over `nthreads` threads.  p 16-byte
// aligned, bytes a multiple of 16.
__device__ __forceinline__ void l2_prefetch(const void* p, size_t bytes, int tid, int nthreads)
{
    const char* b = static_cast<const char*>(p);
    for (size_t o = (size_t)tid * 4096; o < bytes; o += (size_t)nthreads * 4096) {
        const uint32_t n = (uint32_t)(bytes - o < 4096 ? bytes - o : 4096);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b + o), "r"(n) : "memory");
    }
}

// Drop the L2 lines that lie wholly inside [p, p + bytes), spread over
// `nthreads` threads (discard.global.L2: the lines' contents become undefined
// and are never written back to HBM).  Only for scratch that the calling block
// has consumed and that no other block reads before it is written again; the
// partial lines at either end may hold another block's data and are kept.
__device__ __forceinline__ void l2_discard(const void* p, size_t bytes, int tid, int nthreads)
{
    const uintptr_t b = reinterpret_cast<uintptr_t>(p);
    const uintptr_t e = (b + bytes) & ~uintptr_t(127);
    for (uintptr_t q = ((b + 127) & ~uintptr_t(127)) + (uintptr_t)tid * 128; q < e; q += (uintptr_t)nthreads * 128)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(q) : "memory");
}

// Programmatic dependent launch: let the next kernel in the stream start its
// prologue / wait for the previous kernel's results.
__device__ __forceinline__ void pdl_launch_dependents()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait_prior()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

}  // namespace ocean
