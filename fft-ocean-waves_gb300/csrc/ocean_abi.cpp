// ocean_abi.cpp -- the Ocean handle and the extern "C" entry points of
// include/ocean.h.  Host C++; all device work is in the .cu translation units.
//
// The handle replaces FFTOceanWaves' hot-path state (main.cpp:1589-1599,
// 1640-1646): h0 (m_tilde_h0_k / m_tilde_h0_minus_k), the row-pass
// intermediate (in place of m_tilde_h0_t_* and m_ping_pong), the twiddle
// table (in place of m_twiddle_factors) and, optionally, headless output
// buffers (m_dx, m_dy, m_dz, m_normal_map).
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ocean.h"
#include "ocean_host.h"
#include "ocean_internal.h"

namespace ocean {
namespace host {

thread_local std::string g_err;


int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    return fail(OCEAN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// ocean_debug_fail_allocations: allocations left before the injected failures (< 0: off)
static std::atomic<int> g_alloc_budget{-1};

static bool alloc_injected_failure()
{
    int b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) return true;
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) return false;
    }
    return false;
}

cudaError_t dev_alloc_bytes(void** p, size_t bytes)
{
    if (alloc_injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t host_alloc_bytes(void** p, size_t bytes)
{
    if (alloc_injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocHost(p, bytes);
}

int validate(const ocean_params* p)
{
    if (!p) return fail(OCEAN_ERR_INVALID, "params is NULL");
    if (!is_pow2(p->N) || p->N < OCEAN_MIN_N || p->N > OCEAN_MAX_N)
        return fail(OCEAN_ERR_INVALID, "N must be a power of two in [32, 2048], got " + std::to_string(p->N));
    const float vals[] = {p->L, p->amplitude, p->wind_speed, p->wind_dir_x, p->wind_dir_y,
                          p->choppiness, p->suppression, p->gravity};
    for (float v : vals)
        if (!std::isfinite(v)) return fail(OCEAN_ERR_INVALID, "non-finite ocean parameter");
    if (!(p->L > 0.0f)) return fail(OCEAN_ERR_INVALID, "patch length L must be > 0");
    if (p->amplitude < 0.0f) return fail(OCEAN_ERR_INVALID, "amplitude must be >= 0");
    if (!(p->wind_speed > 0.0f)) return fail(OCEAN_ERR_INVALID, "wind speed must be > 0");
    if (p->wind_dir_x == 0.0f && p->wind_dir_y == 0.0f) return fail(OCEAN_ERR_INVALID, "wind direction is zero");
    if (p->flags & ~OCEAN_FLAG_LITERAL_CONJ) return fail(OCEAN_ERR_INVALID, "unknown flag bits");
    return OCEAN_OK;
}

double gravity_of(const ocean_params& p) { return p.gravity > 0.0f ? (double)p.gravity : 9.81; }

ocean::H0Args h0_args(const ocean_params& p)
{
    const double g  = gravity_of(p);
    const double wn = std::sqrt((double)p.wind_dir_x * p.wind_dir_x + (double)p.wind_dir_y * p.wind_dir_y);
    const double Lp = (double)p.wind_speed * p.wind_speed / g;   // tilde_h0_k_cs.glsl:78
    ocean::H0Args a;
    a.N             = p.N;
    a.two_pi_over_L = (float)(2.0 * M_PI / p.L);
    a.amplitude     = p.amplitude;
    a.inv_Lp2       = (float)(1.0 / (Lp * Lp));
    a.l2            = (float)((double)p.suppression * p.suppression);
    a.wx            = (float)(p.wind_dir_x / wn);
    a.wy            = (float)(p.wind_dir_y / wn);
    return a;
}

int check_device()
{
    int         dev = 0;
    cudaError_t e   = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3)
        return fail(OCEAN_ERR_UNSUPPORTED, "kernels are built for sm_103a only; device is sm_" + std::to_string(major) +
                                               std::to_string(minor));
    return OCEAN_OK;
}

int upload_twiddles(float2** d, int N)
{
    cudaError_t e;
    if ((e = dev_alloc(d, ocean::twiddle_len(N) * sizeof(float2))) != cudaSuccess) {
        *d = nullptr;
        return fail(OCEAN_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    if ((e = ocean::launch_twiddles(N, *d, 0)) != cudaSuccess) return cuda_fail(e, "twiddle plan launch");
    return OCEAN_OK;
}


}  // namespace host
}  // namespace ocean

using namespace ocean::host;

// splitmix64 (Steele, Lea & Flood 2014): i-th draw uses state seed + (i+1)*gamma.
uint64_t ocean::host::splitmix64_at(uint64_t seed, uint64_t i)
{
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct ocean_s {
    ocean_params p{};
    int          N = 0;
    float4*      h0     = nullptr;  // [N][N]
    float2*      spec   = nullptr;  // combined spectrum read by the row pass [spec_len(N)]
    float2*      inter  = nullptr;  // [3][N/2+1][N]: row-pass output
    float*       tmap   = nullptr;  // [3][N][N]: column-transform output, column-major
    unsigned*    status = nullptr;  // device status word (bounded-wait time-outs)
    float2*      tw     = nullptr;  // [N]
    float*       noise  = nullptr;  // [4][N][N], kept for ocean_set_params
    float*       out    = nullptr;  // handle-owned outputs: dx, dy, dz, normal_j
    float2*      adj    = nullptr;  // adjoint scratch: [frames][3][N/2+1][N]
    int          adj_frames = 0;
    double*      sums   = nullptr;  // adjoint parameter sums (4 doubles)
    bool         spec_dirty = true; // the combined spectrum was rebuilt since the last row pass was launched
    bool         rows_pending = false; // a row pass was launched and no column stage since (it writes the
                                       // intermediate that the next row pass would overwrite)
    double       K      = 0.0;      // sqrt(g/(2*pi*L))
    double       w_dc   = 0.0;      // sqrt(g*1e-5): the floored DC frequency

    ~ocean_s()
    {
        cudaFree(h0);
        cudaFree(spec);
        cudaFree(inter);
        cudaFree(tmap);
        cudaFree(status);
        cudaFree(tw);
        cudaFree(noise);
        cudaFree(out);
        cudaFree(adj);
        cudaFree(sums);
    }

    void set_consts()
    {
        const double g = gravity_of(p);
        K    = std::sqrt(g / (2.0 * M_PI * (double)p.L));
        w_dc = std::sqrt(g * 0.00001);  // tilde_h0_t_cs.glsl:76-79 at k = 0
    }

    ocean::FrameConsts frame(double t) const
    {
        ocean::FrameConsts fc;
        const double kt = K * t;
        fc.kt_hi        = (float)kt;
        fc.kt_lo        = (float)(kt - (double)fc.kt_hi);
        const double dc = w_dc * t / (2.0 * M_PI);
        fc.dc_cycles    = (float)(dc - std::nearbyint(dc));
        fc.literal_conj = (p.flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0;
        return fc;
    }

    ocean::ColUnit col_unit(const ocean_outputs& out) const
    {
        ocean::ColUnit u;
        u.dx     = out.dx;
        u.dy     = out.dy;
        u.dz     = out.dz;
        u.nj     = reinterpret_cast<float4*>(out.normal_j);
        u.scale  = (float)(0.5 / ((double)N * N));
        u.lambda = p.choppiness;
        u.inv2d  = (float)((double)N / (2.0 * (double)p.L));
        u.pad_   = 0.0f;
        return u;
    }

    int build_h0(cudaStream_t s)
    {
        cudaError_t e = ocean::launch_h0(h0_args(p), noise, h0, s);
        if (e != cudaSuccess) return cuda_fail(e, "h0 init launch");
        return build_spec(s);
    }

    // The row pass's combined spectrum, after every change of h0 or of the
    // conjugation flag.
    int build_spec(cudaStream_t s)
    {
        cudaError_t e = ocean::launch_spec_combine(N, 1, h0, (p.flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0, spec, s);
        if (e != cudaSuccess) return cuda_fail(e, "spectrum combine launch");
        spec_dirty = true;   // the next row pass must wait for it before reading
        return OCEAN_OK;
    }
};

extern "C" {

const char* ocean_last_error(void) { return g_err.c_str(); }

void ocean_debug_fail_allocations(int32_t after) { g_alloc_budget.store(after < 0 ? -1 : after); }

int ocean_version(void) { return 100; }

int ocean_fill_noise(uint64_t seed, int32_t N, float* host_out)
{
    if (!host_out) return fail(OCEAN_ERR_INVALID, "host_out is NULL");
    if (!is_pow2(N) || N > 65536) return fail(OCEAN_ERR_INVALID, "N must be a power of two");
    const uint64_t n = 4ull * (uint64_t)N * (uint64_t)N;
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t z = splitmix64_at(seed, i);
        host_out[i]      = (float)((double)((z >> 40) + 1) * (1.0 / 16777216.0));
    }
    return OCEAN_OK;
}

int ocean_bit_reversed_indices(int32_t N, int32_t* host_out)
{
    if (!host_out) return fail(OCEAN_ERR_INVALID, "host_out is NULL");
    if (!is_pow2(N) || N < 2 || N > 65536) return fail(OCEAN_ERR_INVALID, "N must be a power of two in [2, 65536]");
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    for (int i = 0; i < N; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b) r |= ((i >> b) & 1) << (lg - 1 - b);
        host_out[i] = r;
    }
    return OCEAN_OK;
}

int ocean_butterfly_table(int32_t N, float* host_out)
{
    if (!host_out) return fail(OCEAN_ERR_INVALID, "host_out is NULL");
    if (!is_pow2(N) || N < 2 || N > 65536) return fail(OCEAN_ERR_INVALID, "N must be a power of two in [2, 65536]");
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    std::vector<int32_t> br(N);
    ocean_bit_reversed_indices(N, br.data());
    for (int s = 0; s < lg; ++s)
        for (int y = 0; y < N; ++y) {
            const long   span = 1L << s;
            const long   k    = ((long)y * (N >> (s + 1))) % N;   // twiddle_factors_cs.glsl:37
            const bool   top  = (y % (2L << s)) < span;             // :44
            float*       o    = host_out + 4 * ((size_t)s * N + y);
            o[0] = (float)std::cos(2.0 * M_PI * (double)k / N);
            o[1] = (float)std::sin(2.0 * M_PI * (double)k / N);
            if (s == 0) {                                           // :50-58, bit-reversed pairs
                o[2] = (float)(top ? br[y] : br[y - 1]);
                o[3] = (float)(top ? br[y + 1] : br[y]);
            } else {                                                // :60-68
                o[2] = (float)(top ? y : y - span);
                o[3] = (float)(top ? y + span : y);
            }
        }
    return OCEAN_OK;
}

int ocean_compute_h0(const ocean_params* params, const float* noise_dev, float* h0_dev, void* stream)
{
    int rc = validate(params);
    if (rc) return rc;
    if (!noise_dev || !h0_dev) return fail(OCEAN_ERR_INVALID, "NULL device pointer");
    if (reinterpret_cast<uintptr_t>(h0_dev) % 16) return fail(OCEAN_ERR_INVALID, "h0_dev must be 16-byte aligned");
    cudaError_t e = ocean::launch_h0(h0_args(*params), noise_dev, reinterpret_cast<float4*>(h0_dev),
                                     static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "h0 init launch");
    return OCEAN_OK;
}

int ocean_create(const ocean_params* params, const float* noise_host, ocean_t** out)
{
    if (!out) return fail(OCEAN_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = validate(params);
    if (rc) return rc;
    if (!noise_host) return fail(OCEAN_ERR_INVALID, "noise_host is NULL");
    if ((rc = check_device()) != OCEAN_OK) return rc;
    cudaError_t e;

    ocean_s* o = new (std::nothrow) ocean_s();
    if (!o) return fail(OCEAN_ERR_NOMEM, "host allocation failed");
    o->p = *params;
    o->N = params->N;
    o->set_consts();
    const size_t N = (size_t)o->N;
    if ((e = dev_alloc(&o->h0, N * N * sizeof(float4))) != cudaSuccess ||
        (e = dev_alloc(&o->spec, ocean::spec_len(o->N) * sizeof(float2))) != cudaSuccess ||
        (e = dev_alloc(&o->inter, ocean::inter_len(o->N) * sizeof(float2))) != cudaSuccess ||
        (e = dev_alloc(&o->tmap, ocean::tmap_len(o->N) * sizeof(float))) != cudaSuccess ||
        (e = dev_alloc(&o->status, sizeof(unsigned))) != cudaSuccess ||
        (e = dev_alloc(&o->noise, 4 * N * N * sizeof(float))) != cudaSuccess) {
        delete o;
        return fail(OCEAN_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    if ((e = cudaMemset(o->status, 0, sizeof(unsigned))) != cudaSuccess) {
        delete o;
        return cuda_fail(e, "status clear");
    }
    if ((rc = upload_twiddles(&o->tw, o->N)) != OCEAN_OK) {
        delete o;
        return rc;
    }
    if ((e = cudaMemcpy(o->noise, noise_host, 4 * N * N * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess) {
        delete o;
        return cuda_fail(e, "upload");
    }
    if ((rc = o->build_h0(0)) != OCEAN_OK) {
        delete o;
        return rc;
    }
    if ((e = cudaStreamSynchronize(0)) != cudaSuccess) {
        delete o;
        return cuda_fail(e, "h0 init");
    }
    *out = o;
    return OCEAN_OK;
}

int ocean_create_seeded(const ocean_params* params, uint64_t seed, ocean_t** out)
{
    if (!out) return fail(OCEAN_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = validate(params);
    if (rc) return rc;
    std::vector<float> nz(4 * (size_t)params->N * params->N);
    ocean_fill_noise(seed, params->N, nz.data());
    return ocean_create(params, nz.data(), out);
}

void ocean_destroy(ocean_t* o) { delete o; }

int ocean_get_params(const ocean_t* o, ocean_params* params)
{
    if (!o || !params) return fail(OCEAN_ERR_INVALID, "NULL argument");
    *params = o->p;
    return OCEAN_OK;
}

int ocean_set_params(ocean_t* o, const ocean_params* params)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    int rc = validate(params);
    if (rc) return rc;
    if (params->N != o->N) return fail(OCEAN_ERR_INVALID, "ocean_set_params cannot change N");
    // frames of this handle may be in flight on any stream: they read the
    // spectrum that is about to be rebuilt
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "ocean_set_params: pending work");
    o->p = *params;
    o->set_consts();
    if ((rc = o->build_h0(0)) != OCEAN_OK) return rc;
    if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return cuda_fail(e, "h0 init");
    return OCEAN_OK;
}

int ocean_get_h0(const ocean_t* o, float* dst, void* stream)
{
    if (!o || !dst) return fail(OCEAN_ERR_INVALID, "NULL argument");
    cudaError_t e = cudaMemcpyAsync(dst, o->h0, (size_t)o->N * o->N * sizeof(float4), cudaMemcpyDefault,
                                    static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "ocean_get_h0");
    return OCEAN_OK;
}

int ocean_set_h0(ocean_t* o, const float* src, void* stream)
{
    if (!o || !src) return fail(OCEAN_ERR_INVALID, "NULL argument");
    cudaError_t e = cudaMemcpyAsync(o->h0, src, (size_t)o->N * o->N * sizeof(float4), cudaMemcpyDefault,
                                    static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "ocean_set_h0");
    return o->build_spec(static_cast<cudaStream_t>(stream));
}

int ocean_get_outputs(ocean_t* o, ocean_outputs* out)
{
    if (!o || !out) return fail(OCEAN_ERR_INVALID, "NULL argument");
    const size_t NN = (size_t)o->N * o->N;
    if (!o->out) {
        cudaError_t e = dev_alloc(&o->out, NN * 7 * sizeof(float));
        if (e != cudaSuccess) {
            o->out = nullptr;
            return fail(OCEAN_ERR_NOMEM, std::string("output allocation failed: ") + cudaGetErrorString(e));
        }
    }
    out->dx       = o->out;
    out->dy       = o->out + NN;
    out->dz       = o->out + 2 * NN;
    out->normal_j = o->out + 3 * NN;
    return OCEAN_OK;
}

int ocean_update_rows(ocean_t* o, double t, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    if (!std::isfinite(t)) return fail(OCEAN_ERR_INVALID, "time is not finite");
    ocean::RowArgs ra;
    ra.spec       = o->spec;
    ra.h0         = o->h0;
    ra.inter      = o->inter;
    ra.tw         = o->tw;
    ra.status     = o->status;
    ra.fcs        = nullptr;
    ra.fc0        = o->frame(t);
    ra.tiles      = 1;
    ra.S          = 1;
    // the row pass overlaps the stream's previous kernel unless that may be
    // the spectrum rebuild (ocean_set_h0 is stream-ordered) or the tuning
    // says otherwise for this N
    ra.wait_first = (o->spec_dirty || o->rows_pending || !ocean::tuning_for(o->N).row_overlap) ? 1 : 0;
    // NVTX ranges name the stages as the reference's GL debug groups do (main.cpp:623,644,665,689)
    nvtxRangePushA("ocean rows: evolution + horizontal FFT");
    cudaError_t e = ocean::launch_row_pass(o->N, ra, static_cast<cudaStream_t>(stream));
    nvtxRangePop();
    if (e != cudaSuccess) return cuda_fail(e, "row pass launch");
    o->spec_dirty   = false;
    o->rows_pending = true;
    return OCEAN_OK;
}

static ocean::ColArgs col_args(const ocean_s* o, const ocean_outputs& out)
{
    ocean::ColArgs ca;
    ca.inter  = o->inter;
    ca.tmap   = o->tmap;
    ca.status = o->status;
    ca.tw     = o->tw;
    ca.units  = nullptr;
    ca.u0     = o->col_unit(out);
    ca.trigger_next = ocean::tuning_for(o->N).row_overlap;
    return ca;
}

// out == NULL: the handle-owned buffers; checks pointers and alignment.
static int resolve_outputs(ocean_t* o, const ocean_outputs* out, ocean_outputs* res)
{
    if (!out) {
        int rc = ocean_get_outputs(o, res);
        if (rc) return rc;
    } else {
        *res = *out;
    }
    if (!res->dx || !res->dy || !res->dz || !res->normal_j) return fail(OCEAN_ERR_INVALID, "NULL output pointer");
    const uintptr_t al = reinterpret_cast<uintptr_t>(res->dx) | reinterpret_cast<uintptr_t>(res->dy) |
                         reinterpret_cast<uintptr_t>(res->dz) | reinterpret_cast<uintptr_t>(res->normal_j);
    if (al % 16) return fail(OCEAN_ERR_INVALID, "output pointers must be 16-byte aligned");
    return OCEAN_OK;
}

int ocean_update_columns(ocean_t* o, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    const ocean_outputs none{};
    nvtxRangePushA("ocean columns: vertical FFT + inversion");
    // every stage is a programmatic dependent of the stream's previous kernel:
    // its launch overlaps that kernel's tail, and it waits for that kernel
    // (griddepcontrol.wait) before it reads or writes anything that kernel may
    // touch
    cudaError_t e = ocean::launch_col_fft(o->N, 1, col_args(o, none), static_cast<cudaStream_t>(stream), true);
    nvtxRangePop();
    if (e != cudaSuccess) return cuda_fail(e, "column transform launch");
    o->rows_pending = false;   // it lets a following kernel start only once its tile is read
    return OCEAN_OK;
}

int ocean_update_outputs(ocean_t* o, const ocean_outputs* out, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    ocean_outputs res;
    int rc = resolve_outputs(o, out, &res);
    if (rc) return rc;
    nvtxRangePushA("ocean outputs: normal map + Jacobian");
    cudaError_t e = ocean::launch_col_out(o->N, 1, col_args(o, res), static_cast<cudaStream_t>(stream), true);
    nvtxRangePop();
    if (e != cudaSuccess) return cuda_fail(e, "output launch");
    return OCEAN_OK;
}

int ocean_update_columns_outputs(ocean_t* o, const ocean_outputs* out, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    ocean_outputs res;
    int rc = resolve_outputs(o, out, &res);
    if (rc) return rc;
    if (const int pairs = ocean::tuning_for(o->N).col_fused) {
        // both column stages in one kernel: the column maps stay on chip
        nvtxRangePushA("ocean columns + outputs: vertical FFT, inversion, normal map + Jacobian");
        cudaError_t e =
            ocean::launch_col_fused(o->N, pairs, 1, col_args(o, res), static_cast<cudaStream_t>(stream), true);
        nvtxRangePop();
        if (e != cudaSuccess) return cuda_fail(e, "fused column launch");
        o->rows_pending = false;   // it lets a following kernel start only once its loads are in
        return OCEAN_OK;
    }
    if ((rc = ocean_update_columns(o, stream)) != OCEAN_OK) return rc;
    return ocean_update_outputs(o, &res, stream);
}

int ocean_update(ocean_t* o, double t, const ocean_outputs* out, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    if (!std::isfinite(t)) return fail(OCEAN_ERR_INVALID, "time is not finite");
    ocean_outputs res;
    int rc = resolve_outputs(o, out, &res);
    if (rc) return rc;
    if ((rc = ocean_update_rows(o, t, stream)) != OCEAN_OK) return rc;
    return ocean_update_columns_outputs(o, &res, stream);
}

int ocean_device_status(ocean_t* o, void* stream)
{
    if (!o) return fail(OCEAN_ERR_INVALID, "ocean is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned     h = 0;
    cudaError_t  e;
    if ((e = cudaMemcpyAsync(&h, o->status, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(o->status, 0, sizeof(unsigned), s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "device status");
    if (h) return fail(OCEAN_ERR_TIMEOUT, "a kernel's bounded wait for its TMA copies timed out");
    return OCEAN_OK;
}

int ocean_backward(ocean_t* o, const double* times, int32_t T, const float* g_dx, const float* g_dy,
                   const float* g_dz, uint32_t flags, ocean_grads* grads, void* stream)
{
    if (!o || !grads || !times) return fail(OCEAN_ERR_INVALID, "NULL argument");
    if (T < 1) return fail(OCEAN_ERR_INVALID, "T must be >= 1");
    if (flags & ~OCEAN_GRAD_ACCUMULATE) return fail(OCEAN_ERR_INVALID, "unknown flag bits");
    for (int j = 0; j < T; ++j)
        if (!std::isfinite(times[j])) return fail(OCEAN_ERR_INVALID, "time is not finite");
    const uintptr_t al = reinterpret_cast<uintptr_t>(g_dx) | reinterpret_cast<uintptr_t>(g_dy) |
                         reinterpret_cast<uintptr_t>(g_dz) | reinterpret_cast<uintptr_t>(grads->dh0);
    if (al % 16) return fail(OCEAN_ERR_INVALID, "gradient pointers must be 16-byte aligned");
    cudaStream_t s  = static_cast<cudaStream_t>(stream);
    const size_t N  = (size_t)o->N, NN = N * N, H = N / 2 + 1;
    const size_t per_frame = 3 * H * N * sizeof(float2);
    int chunk = (int)std::min<size_t>((size_t)ocean::kMaxChunkFrames, std::max<size_t>(1, (512ull << 20) / per_frame));
    chunk     = std::min(chunk, (int)T);
    cudaError_t e;
    if (o->adj_frames < chunk) {
        cudaFree(o->adj);
        o->adj        = nullptr;
        o->adj_frames = 0;
        if ((e = dev_alloc(&o->adj, per_frame * chunk)) != cudaSuccess)
            return fail(OCEAN_ERR_NOMEM, std::string("adjoint scratch allocation failed: ") + cudaGetErrorString(e));
        o->adj_frames = chunk;
    }
    if (!o->sums && (e = dev_alloc(&o->sums, 4 * sizeof(double))) != cudaSuccess) {
        o->sums = nullptr;
        return fail(OCEAN_ERR_NOMEM, std::string("allocation failed: ") + cudaGetErrorString(e));
    }
    if (!(flags & OCEAN_GRAD_ACCUMULATE)) {
        grads->dA = grads->dV = grads->dtheta = grads->dlambda = 0.0;
        if (grads->dh0 && (e = cudaMemsetAsync(grads->dh0, 0, NN * sizeof(float4), s)) != cudaSuccess)
            return cuda_fail(e, "dh0 clear");
    }
    if ((e = cudaMemsetAsync(o->sums, 0, 4 * sizeof(double), s)) != cudaSuccess) return cuda_fail(e, "sums clear");

    const ocean::H0Args ha = h0_args(o->p);
    const double g = gravity_of(o->p), V = o->p.wind_speed, Lw = V * V / g;
    for (int c0 = 0; c0 < T; c0 += chunk) {
        const int n = std::min(chunk, (int)T - c0);
        ocean::AdjColArgs ca;
        ca.gx    = g_dx ? g_dx + (size_t)c0 * NN : nullptr;
        ca.gy    = g_dy ? g_dy + (size_t)c0 * NN : nullptr;
        ca.gz    = g_dz ? g_dz + (size_t)c0 * NN : nullptr;
        ca.inter = o->adj;
        ca.tw    = o->tw;
        ca.scale = (float)(0.5 / (double)NN);
        if ((e = ocean::launch_adj_col(o->N, n, ca, s)) != cudaSuccess) return cuda_fail(e, "adjoint column pass");
        ocean::AdjRowArgs ra;
        ra.inter         = o->adj;
        ra.h0            = o->h0;
        ra.tw            = o->tw;
        ra.dh0           = reinterpret_cast<float4*>(grads->dh0);
        ra.sums          = o->sums;
        ra.T             = n;
        ra.literal_conj  = (o->p.flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0;
        ra.lambda        = o->p.choppiness;
        ra.two_pi_over_L = ha.two_pi_over_L;
        ra.amplitude     = ha.amplitude;
        ra.inv_Lp2       = ha.inv_Lp2;
        ra.l2            = ha.l2;
        ra.wx            = ha.wx;
        ra.wy            = ha.wy;
        ra.wA            = o->p.amplitude > 0.0f ? (float)(0.5 / o->p.amplitude) : 0.0f;
        ra.wV            = (float)(2.0 * V / (g * Lw * Lw * Lw));
        for (int j = 0; j < n; ++j) ra.fc[j] = o->frame(times[c0 + j]);
        if ((e = ocean::launch_adj_row(o->N, ra, s)) != cudaSuccess) return cuda_fail(e, "adjoint row pass");
    }
    double h[4];
    if ((e = cudaMemcpyAsync(h, o->sums, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "adjoint sums");
    grads->dA += h[0];
    grads->dV += h[1];
    grads->dtheta += h[2];
    grads->dlambda += h[3];
    return OCEAN_OK;
}

}  // extern "C"
