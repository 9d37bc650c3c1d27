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

// smem_setup, plus the occupancy of `kernel` on the current device: how many
// of its CTAs (`threads` threads, `smem` bytes) fit on one SM.
template <class Kernel>
static cudaError_t persistent_setup(PerDevice& cache, Kernel kernel, int threads, size_t smem, int* per_sm)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int rc = cache.get(dev, per_sm, (int)cudaErrorInvalidDevice, [&](int* v) -> int {
        cudaError_t e2 = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e2 != cudaSuccess) return (int)e2;
        int n = 0;
        if ((e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem)) != cudaSuccess)
            return (int)e2;
        if (n < 1) return (int)cudaErrorInvalidConfiguration;
        *v = n;
        return 0;
    });
    return (cudaError_t)rc;
}

// The current device's SM count (once per device).
static cudaError_t device_sms(int* sms)
{
    static PerDevice cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int rc = cache.get(dev, sms, (int)cudaErrorInvalidDevice, [&](int* v) -> int {
        return (int)cudaDeviceGetAttribute(v, cudaDevAttrMultiProcessorCount, dev);
    });
    return (cudaError_t)rc;
}

// Persistent grid: CTAs per SM (the tuning's cap, 0 = as many as fit) x SMs.
static cudaError_t persistent_grid(int per_sm, int cap, int* grid)
{
    int sms = 0;
    cudaError_t e = device_sms(&sms);
    if (e != cudaSuccess) return e;
    *grid = (cap > 0 && cap < per_sm ? cap : per_sm) * sms;
    return cudaSuccess;
}

}  // namespace ocean
