// ocean_static.cu -- ocean_update_noalloc: one ocean frame without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Some callers of this library cannot allocate device memory on their own:
// plug-in hosts that own the CUDA context and forbid allocation from plug-in
// code, code that runs while the application's allocator is locked or its
// memory pool is exhausted, and callers that must hold a fixed memory budget
// decided at load time.  For them this entry point takes the spectrum h0 and
// the output maps from the caller and keeps the scratch the frame needs -- the
// row-pass intermediate and the column-major maps of the column transforms --
// in fixed arrays compiled into this library, instead of in a handle's
// cudaMalloc'd buffers.
//
// The arrays are file-scope `static __device__` arrays sized for N <= 1024
// (25,190,400 bytes of scratch); every GPU that loads the library holds them
// until the process exits.  In host code their names are only stand-ins: the
// device addresses are obtained with cudaGetSymbolAddress once per device, with
// that device current, on the first call made on that device.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "ocean.h"
#include "ocean_host.h"
#include "ocean_internal.h"

namespace {

constexpr int    kStaticMaxN     = 1024;
constexpr size_t kStaticInterLen = 3 * (size_t)(kStaticMaxN / 2 + 1) * kStaticMaxN;  // float2
constexpr size_t kStaticTmapLen  = 3 * (size_t)kStaticMaxN * kStaticMaxN;            // float
static_assert(kStaticInterLen * 8 + kStaticTmapLen * 4 == 25190400, "documented scratch size");

// The frame's scratch: row-pass intermediate, column-major maps, twiddle
// table, device status word.
static __device__ __align__(256) float2   g_static_inter[kStaticInterLen];
static __device__ __align__(256) float    g_static_tmap[kStaticTmapLen];
constexpr size_t kStaticTwLen    = 4096;   // twiddle plans of N = 1024 (3,648), the largest needed
static __device__ __align__(256) float2   g_static_tw[kStaticTwLen];
static __device__ __align__(256) unsigned g_static_status;

constexpr int kMaxDevices = 64;

struct DeviceScratch {
    bool        ready   = false;
    float2*     inter   = nullptr;   // device addresses of the arrays above
    float*      tmap    = nullptr;
    float2*     tw      = nullptr;
    unsigned*   status  = nullptr;
    int         tw_N    = 0;         // N whose twiddles the table holds
};


std::mutex    g_mu;
DeviceScratch g_dev[kMaxDevices];

// Per-device set-up: resolve the arrays' device addresses (cudaGetSymbolAddress
// with this device current) and clear the status word.
int setup(int dev, DeviceScratch& d, cudaStream_t s)
{
    cudaError_t e;
    if ((e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.inter), g_static_inter)) != cudaSuccess ||
        (e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.tmap), g_static_tmap)) != cudaSuccess ||
        (e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.tw), g_static_tw)) != cudaSuccess ||
        (e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.status), g_static_status)) != cudaSuccess)
        return ocean::host::cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
    if ((e = cudaMemsetAsync(d.status, 0, sizeof(unsigned), s)) != cudaSuccess)
        return ocean::host::cuda_fail(e, "static status clear");
    (void)dev;
    d.ready = true;
    return OCEAN_OK;
}

}  // namespace

using namespace ocean::host;

extern "C" int ocean_update_noalloc(const ocean_params* params, const float* h0_dev, double t,
                                    const ocean_outputs* out, void* stream)
{
    int rc = validate(params);
    if (rc) return rc;
    if (params->N > kStaticMaxN)
        return fail(OCEAN_ERR_INVALID, "ocean_update_noalloc supports N <= " + std::to_string(kStaticMaxN) +
                                           " (its static scratch is sized for that), got N = " +
                                           std::to_string(params->N));
    if (!h0_dev || !out) return fail(OCEAN_ERR_INVALID, "NULL argument");
    if (!std::isfinite(t)) return fail(OCEAN_ERR_INVALID, "time is not finite");
    if (!out->dx || !out->dy || !out->dz || !out->normal_j) return fail(OCEAN_ERR_INVALID, "NULL output pointer");
    const uintptr_t al = reinterpret_cast<uintptr_t>(h0_dev) | reinterpret_cast<uintptr_t>(out->dx) |
                         reinterpret_cast<uintptr_t>(out->dy) | reinterpret_cast<uintptr_t>(out->dz) |
                         reinterpret_cast<uintptr_t>(out->normal_j);
    if (al % 16) return fail(OCEAN_ERR_INVALID, "h0 and output pointers must be 16-byte aligned");
    if ((rc = check_device()) != OCEAN_OK) return rc;
    int         dev = 0;
    cudaError_t e   = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(OCEAN_ERR_UNSUPPORTED, "device ordinal out of range");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int    N = params->N;

    std::lock_guard<std::mutex> lock(g_mu);
    DeviceScratch&              d = g_dev[dev];
    if (!d.ready || d.tw_N != N) {
        // The set-up and a twiddle rebuild are recorded as done when they are
        // enqueued; inside a stream capture they would only run when the graph
        // is launched, and a later direct call would read a stale table.
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
        if (cs != cudaStreamCaptureStatusNone)
            return fail(OCEAN_ERR_INVALID, "ocean_update_noalloc: the first call on a device, and the first call "
                                           "after a change of N, must not be made inside a stream capture");
    }
    if (!d.ready && (rc = setup(dev, d, s)) != OCEAN_OK) return rc;
    if (d.tw_N != N) {                 // the table holds another size's twiddles
        if (ocean::twiddle_len(N) > kStaticTwLen) return fail(OCEAN_ERR_UNSUPPORTED, "twiddle plan exceeds its static array");
        if ((e = ocean::launch_twiddles(N, d.tw, s)) != cudaSuccess) return cuda_fail(e, "static twiddle launch");
        d.tw_N = N;
    }

    // one frame: the same two kernels as ocean_update, scratch from the arrays
    const double g  = gravity_of(*params);
    const double K  = std::sqrt(g / (2.0 * M_PI * (double)params->L));
    const double kt = K * t;
    ocean::RowArgs ra;
    ra.spec            = nullptr;            // G and D formed from h0 on the fly
    ra.h0              = reinterpret_cast<const float4*>(h0_dev);
    ra.inter           = d.inter;
    ra.tw              = d.tw;
    ra.status          = d.status;
    ra.fcs             = nullptr;
    ra.fc0.kt_hi       = (float)kt;
    ra.fc0.kt_lo       = (float)(kt - (double)ra.fc0.kt_hi);
    const double dc    = std::sqrt(g * 0.00001) * t / (2.0 * M_PI);
    ra.fc0.dc_cycles   = (float)(dc - std::nearbyint(dc));
    ra.fc0.literal_conj = (params->flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0;
    ra.tiles           = 1;
    ra.S               = 1;
    ra.wait_first      = 1;                  // the caller's h0 (and a new twiddle table) come from earlier kernels
    if ((e = ocean::launch_row_pass(N, ra, s)) != cudaSuccess) return cuda_fail(e, "row pass launch");
    ocean::ColArgs ca;
    ca.inter     = d.inter;
    ca.tmap      = d.tmap;
    ca.status    = d.status;
    ca.tw        = d.tw;
    ca.units     = nullptr;
    ca.u0.dx     = out->dx;
    ca.u0.dy     = out->dy;
    ca.u0.dz     = out->dz;
    ca.u0.nj     = reinterpret_cast<float4*>(out->normal_j);
    ca.u0.scale  = (float)(0.5 / ((double)N * N));
    ca.u0.lambda = params->choppiness;
    ca.u0.inv2d  = (float)((double)N / (2.0 * (double)params->L));
    ca.u0.pad_   = 0.0f;
    ca.trigger_next = 0;           // the next call's row pass waits for this frame first
    if (const int pairs = ocean::tuning_for(N).col_fused) {
        if ((e = ocean::launch_col_fused(N, pairs, 1, ca, s, true)) != cudaSuccess)
            return cuda_fail(e, "fused column launch");
        return OCEAN_OK;
    }
    if ((e = ocean::launch_col_fft(N, 1, ca, s, true)) != cudaSuccess) return cuda_fail(e, "column transform launch");
    if ((e = ocean::launch_col_out(N, 1, ca, s, true)) != cudaSuccess) return cuda_fail(e, "output launch");
    return OCEAN_OK;
}

extern "C" int ocean_noalloc_device_status(void* stream)
{
    int         dev = 0;
    cudaError_t e   = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(OCEAN_ERR_UNSUPPORTED, "device ordinal out of range");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned*    status;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_dev[dev].ready) return OCEAN_OK;   // no frame has run on this device
        status = g_dev[dev].status;
    }
    unsigned h = 0;
    if ((e = cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(status, 0, sizeof(unsigned), s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "noalloc device status");
    if (h) return fail(OCEAN_ERR_TIMEOUT, "a kernel of ocean_update_noalloc gave up a bounded wait for its TMA copies");
    return OCEAN_OK;
}
