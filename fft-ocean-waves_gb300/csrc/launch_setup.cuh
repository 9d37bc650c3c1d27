// launch_setup.cuh -- per-device one-time set-up of the kernels that need
// more than 48 KB of dynamic shared memory or a persistent grid.
#pragma once
#include <cuda_runtime.h>

#include "per_device.h"

namespace ocean {

// Opt `kernel` into `smem` bytes of dynamic shared memory on the current
// device, once per device (`cache` is the kernel's own PerDevice).
template <class Kernel>
static cudaError_t smem_setup(PerDevice& cache, Kernel kernel, size_t smem)
{
    int dev = 0, done = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int rc = cache.get(dev, &done, (int)cudaErrorInvalidDevice, [&](int* v) -> int {
        const cudaError_t e2 = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        *v = 1;
        return (int)e2;
    });
    return (cudaError_t)rc;
}

// smem_setup, plus the persistent grid of `kernel` on the current device:
// resident CTAs per SM (for `threads` threads and `smem` bytes) x SMs.
template <class Kernel>
static cudaError_t persistent_setup(PerDevice& cache, Kernel kernel, int threads, size_t smem, int* grid)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int rc = cache.get(dev, grid, (int)cudaErrorInvalidDevice, [&](int* v) -> int {
        cudaError_t e2 = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e2 != cudaSuccess) return (int)e2;
        int per_sm = 0, sms = 0;
        if ((e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem)) != cudaSuccess)
            return (int)e2;
        if ((e2 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e2;
        if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
        *v = per_sm * sms;
        return 0;
    });
    return (cudaError_t)rc;
}

}  // namespace ocean
