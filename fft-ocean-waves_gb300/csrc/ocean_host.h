// ocean_host.h -- host-side helpers shared by the C-ABI translation units
// (single tiles in ocean_abi.cpp, batches in ocean_batch.cpp).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "ocean.h"
#include "ocean_internal.h"

namespace ocean {
namespace host {

int    fail(int code, const std::string& msg);               // sets ocean_last_error(), returns code
int    cuda_fail(cudaError_t e, const char* what);
bool   is_pow2(int n);
int    validate(const ocean_params* p);                     // OCEAN_OK or OCEAN_ERR_INVALID
double gravity_of(const ocean_params& p);
H0Args h0_args(const ocean_params& p);
uint64_t splitmix64_at(uint64_t seed, uint64_t i);

int check_device();                                         // sm_103 or OCEAN_ERR_UNSUPPORTED

// Every device (and pinned host) allocation of the library goes through
// dev_alloc, so that ocean_debug_fail_allocations() can make the n-th one fail.
cudaError_t dev_alloc_bytes(void** p, size_t bytes);
cudaError_t host_alloc_bytes(void** p, size_t bytes);
template <class T>
cudaError_t dev_alloc(T** p, size_t bytes)
{
    return dev_alloc_bytes(reinterpret_cast<void**>(p), bytes);
}
template <class T>
cudaError_t host_alloc(T** p, size_t bytes)
{
    return host_alloc_bytes(reinterpret_cast<void**>(p), bytes);
}
int upload_twiddles(float2** d, int N);                     // cudaMalloc + the twiddle plans (on stream 0)

}  // namespace host
}  // namespace ocean
