// ocean_batch.cpp -- batches of independent tiles (ocean_batch_* in
// include/ocean.h).  No counterpart in the reference, which renders one tile.
//
// Tiles are grouped by N.  Per group: the combined spectrum (G, D) of every
// tile back to back (h0 itself is only a creation-time temporary), one twiddle
// table, and scratch (intermediate + column-major maps) for one wave of units
// (unit = (tile, time sample)).  A wave is as many units as fit a 64 MB scratch
// budget, so its three stages run out of L2: whole tiles with all their
// samples for small N, runs of samples of one tile for large N.  An update is
// a CUDA graph of
//   H2D copy of the per-unit constants (pinned staging -> device)
//   per wave: k_row_pass (persistent; each spectrum row pair is staged once
//             and serves all samples of its tile in the wave) -> k_col_fft ->
//             k_col_out (grids: column pairs / output tiles x units, each a
//             programmatic dependent of the kernel before it)
// captured at creation and replayed by ocean_batch_update.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "ocean.h"
#include "ocean_host.h"
#include "ocean_internal.h"

using namespace ocean::host;

struct ocean_batch_s {
    struct Group {
        int              N = 0;
        std::vector<int> tiles;          // batch tile indices, in slot order
        float2*          spec  = nullptr;
        float2*          inter = nullptr;
        float*           tmap  = nullptr;
        float2*          tw    = nullptr;
        size_t           first_unit = 0; // this group's units start here in the unit arrays
        int              wave_tiles = 1; // tiles per wave (all S samples), or
        int              wave_smp   = 0; // if > 0: samples per wave of a single tile
        int              wave_units = 1; // units the scratch holds
        int              fused      = 0;   // fused column kernel's pairs per CTA (0: two kernels, column maps)
    };
    int                       n_tiles = 0, S = 0;
    std::vector<ocean_params> params;
    std::vector<double>       K, w_dc;
    std::vector<Group>        groups;
    unsigned*                 status = nullptr;
    // per-unit constants, in group order: FrameConsts[units] | ColUnit[units]
    size_t                    units = 0, desc_bytes = 0;
    void*                     d_desc = nullptr;
    void*                     h_desc = nullptr;   // pinned
    cudaStream_t              cap    = nullptr;
    cudaGraph_t               graph  = nullptr;
    cudaGraphExec_t           exec   = nullptr;
    cudaEvent_t               done   = nullptr;
    bool                      launched = false;

    ~ocean_batch_s()
    {
        if (launched) cudaEventSynchronize(done);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (done) cudaEventDestroy(done);
        if (cap) cudaStreamDestroy(cap);
        for (Group& g : groups) {
            cudaFree(g.spec);
            cudaFree(g.inter);
            cudaFree(g.tmap);
            cudaFree(g.tw);
        }
        cudaFree(status);
        cudaFree(d_desc);
        cudaFreeHost(h_desc);
    }

    ocean::FrameConsts* h_fc() { return static_cast<ocean::FrameConsts*>(h_desc); }
    ocean::ColUnit*     h_units()
    {
        return reinterpret_cast<ocean::ColUnit*>(static_cast<char*>(h_desc) + units * sizeof(ocean::FrameConsts));
    }
    ocean::FrameConsts* d_fc() { return static_cast<ocean::FrameConsts*>(d_desc); }
    ocean::ColUnit*     d_units()
    {
        return reinterpret_cast<ocean::ColUnit*>(static_cast<char*>(d_desc) + units * sizeof(ocean::FrameConsts));
    }
};

namespace {

size_t unit_scratch_bytes(int N, int fused)
{
    return ocean::inter_len(N) * sizeof(float2) + (fused ? 0 : ocean::tmap_len(N) * sizeof(float));
}

// Waves of a group: whole tiles (all samples) when a tile's samples fit the
// scratch budget of a wave (the tuning's wave_mib: small enough that a wave's
// three stages run out of the 129 MB L2), else runs of samples of one tile;
// units are tile-major, so a wave's units are contiguous and share their
// tiles' spectra.
void plan_waves(ocean_batch_s::Group& g, int S)
{
    const size_t budget = (size_t)ocean::tuning_for(g.N).wave_mib << 20;
    const size_t U = std::max<size_t>(1, budget / unit_scratch_bytes(g.N, g.fused));
    const size_t T = g.tiles.size();
    if (U >= (size_t)S) {
        g.wave_tiles = (int)std::min(T, U / S);
        g.wave_smp   = 0;
        g.wave_units = g.wave_tiles * S;
    } else {   // equal runs: ceil(S / U) waves per tile
        const int runs = (int)((S + U - 1) / U);
        g.wave_tiles   = 1;
        g.wave_smp     = (S + runs - 1) / runs;
        g.wave_units   = g.wave_smp;
    }
}

// One wave: `tiles` tiles from slot t0, samples s0 .. s0+smp-1 of each.
cudaError_t launch_wave(ocean_batch_s* b, const ocean_batch_s::Group& g, int t0, int tiles, int s0, int smp, bool first)
{
    const size_t u0 = g.first_unit + (size_t)t0 * b->S + s0;   // first unit (batch order)
    ocean::RowArgs ra;
    ra.spec   = g.spec + (size_t)t0 * ocean::spec_len(g.N);
    ra.h0     = nullptr;
    ra.inter  = g.inter;
    ra.tw     = g.tw;
    ra.status = b->status;
    ra.fcs    = b->d_fc() + u0;
    ra.fc0    = ocean::FrameConsts{};
    ra.tiles  = tiles;
    ra.S      = smp;
    // the first wave follows the H2D copy of the constants it reads; later
    // waves follow a k_col_out, whose intermediate they may overwrite once it
    // has started (see k_row_ws)
    ra.wait_first = (first || !ocean::tuning_for(g.N).row_overlap) ? 1 : 0;
    cudaError_t e = ocean::launch_row_pass(g.N, ra, b->cap);
    if (e != cudaSuccess) return e;
    ocean::ColArgs ca;
    ca.inter  = g.inter;
    ca.tmap   = g.tmap;
    ca.status = b->status;
    ca.tw     = g.tw;
    ca.units  = b->d_units() + u0;
    ca.u0     = ocean::ColUnit{};
    ca.trigger_next = ocean::tuning_for(g.N).row_overlap;
    if (g.fused) return ocean::launch_col_fused(g.N, g.fused, tiles * smp, ca, b->cap, true);
    if ((e = ocean::launch_col_fft(g.N, tiles * smp, ca, b->cap, true)) != cudaSuccess) return e;
    return ocean::launch_col_out(g.N, tiles * smp, ca, b->cap, true);
}

int capture(ocean_batch_s* b)
{
    cudaError_t e;
    if ((e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed)) != cudaSuccess)
        return cuda_fail(e, "batch graph capture");
    e = cudaMemcpyAsync(b->d_desc, b->h_desc, b->desc_bytes, cudaMemcpyHostToDevice, b->cap);
    bool first = true;
    for (size_t gi = 0; gi < b->groups.size() && e == cudaSuccess; ++gi) {
        const ocean_batch_s::Group& g = b->groups[gi];
        const int T = (int)g.tiles.size();
        if (g.wave_smp == 0) {
            for (int t0 = 0; t0 < T && e == cudaSuccess; t0 += g.wave_tiles, first = false)
                e = launch_wave(b, g, t0, std::min(g.wave_tiles, T - t0), 0, b->S, first);
        } else {
            for (int t = 0; t < T && e == cudaSuccess; ++t)
                for (int s0 = 0; s0 < b->S && e == cudaSuccess; s0 += g.wave_smp, first = false)
                    e = launch_wave(b, g, t, 1, s0, std::min(g.wave_smp, b->S - s0), first);
        }
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e2    = cudaStreamEndCapture(b->cap, &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(e, "batch graph launch capture");
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "batch graph capture");
    b->graph = graph;
    if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) return cuda_fail(e, "batch graph instantiate");
    return OCEAN_OK;
}

}  // namespace

extern "C" {

int ocean_batch_create(const ocean_params* params, const uint64_t* seeds, int32_t n_tiles, int32_t samples,
                       ocean_batch_t** out)
{
    if (!out) return fail(OCEAN_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!params || !seeds) return fail(OCEAN_ERR_INVALID, "NULL argument");
    if (n_tiles < 1 || samples < 1) return fail(OCEAN_ERR_INVALID, "n_tiles and samples must be >= 1");
    for (int i = 0; i < n_tiles; ++i) {
        int rc = validate(&params[i]);
        if (rc) return fail(rc, "tile " + std::to_string(i) + ": " + ocean_last_error());
    }
    int rc = check_device();
    if (rc) return rc;

    ocean_batch_s* b = new (std::nothrow) ocean_batch_s();
    if (!b) return fail(OCEAN_ERR_NOMEM, "host allocation failed");
    b->n_tiles = n_tiles;
    b->S       = samples;
    b->params.assign(params, params + n_tiles);
    for (const ocean_params& p : b->params) {
        const double g = gravity_of(p);
        b->K.push_back(std::sqrt(g / (2.0 * M_PI * (double)p.L)));
        b->w_dc.push_back(std::sqrt(g * 0.00001));
    }
    // groups, largest N first (its kernels take longest)
    std::map<int, std::vector<int>, std::greater<int>> byN;
    for (int i = 0; i < n_tiles; ++i) byN[params[i].N].push_back(i);
    cudaError_t e;
    size_t      unit0 = 0;
    for (auto& kv : byN) {
        ocean_batch_s::Group g;
        g.N          = kv.first;
        g.tiles      = kv.second;
        g.first_unit = unit0;
        unit0 += g.tiles.size() * (size_t)samples;
        b->groups.push_back(g);
    }
    b->units      = unit0;
    b->desc_bytes = b->units * (sizeof(ocean::FrameConsts) + sizeof(ocean::ColUnit));
    std::vector<float> noise;
    float*             d_noise = nullptr;
    float4*            d_h0    = nullptr;
    const int          maxN    = b->groups.front().N;
    if ((e = dev_alloc(&b->status, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemset(b->status, 0, sizeof(unsigned))) != cudaSuccess ||
        (e = dev_alloc(&b->d_desc, b->desc_bytes)) != cudaSuccess ||
        (e = host_alloc(&b->h_desc, b->desc_bytes)) != cudaSuccess ||
        (e = dev_alloc(&d_noise, 4 * (size_t)maxN * maxN * sizeof(float))) != cudaSuccess ||
        (e = dev_alloc(&d_h0, (size_t)maxN * maxN * sizeof(float4))) != cudaSuccess) {
        cudaFree(d_noise);
        cudaFree(d_h0);
        delete b;
        return fail(OCEAN_ERR_NOMEM, std::string("batch allocation failed: ") + cudaGetErrorString(e));
    }
    for (ocean_batch_s::Group& g : b->groups) {
        const size_t N = (size_t)g.N, NN = N * N, T = g.tiles.size();
        g.fused = ocean::tuning_for(g.N).col_fused;
        plan_waves(g, samples);
        const size_t W = (size_t)g.wave_units;
        if ((e = dev_alloc(&g.spec, T * ocean::spec_len(g.N) * sizeof(float2))) != cudaSuccess ||
            (e = dev_alloc(&g.inter, W * ocean::inter_len(g.N) * sizeof(float2))) != cudaSuccess ||
            (!g.fused && (e = dev_alloc(&g.tmap, W * ocean::tmap_len(g.N) * sizeof(float))) != cudaSuccess)) {
            cudaFree(d_noise);
            cudaFree(d_h0);
            delete b;
            return fail(OCEAN_ERR_NOMEM, std::string("batch allocation failed: ") + cudaGetErrorString(e));
        }
        if ((rc = upload_twiddles(&g.tw, g.N)) != OCEAN_OK) {
            cudaFree(d_noise);
            cudaFree(d_h0);
            delete b;
            return rc;
        }
        noise.resize(4 * NN);
        for (size_t j = 0; j < T; ++j) {
            const int t = g.tiles[j];
            ocean_fill_noise(seeds[t], g.N, noise.data());
            if ((e = cudaMemcpy(d_noise, noise.data(), 4 * NN * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
                (e = ocean::launch_h0(h0_args(params[t]), d_noise, d_h0, 0)) != cudaSuccess ||
                (e = ocean::launch_spec_combine(g.N, 1, d_h0, (params[t].flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0,
                                                g.spec + j * ocean::spec_len(g.N), 0)) != cudaSuccess ||
                (e = cudaStreamSynchronize(0)) != cudaSuccess) {
                cudaFree(d_noise);
                cudaFree(d_h0);
                delete b;
                return cuda_fail(e, "batch h0 init");
            }
        }
    }
    cudaFree(d_noise);
    cudaFree(d_h0);
    if ((e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming)) != cudaSuccess) {
        delete b;
        return cuda_fail(e, "batch stream");
    }
    if ((rc = capture(b)) != OCEAN_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return OCEAN_OK;
}

int ocean_batch_update(ocean_batch_t* b, const double* times, const ocean_outputs* outs, void* stream)
{
    if (!b || !times || !outs) return fail(OCEAN_ERR_INVALID, "NULL argument");
    const size_t n = (size_t)b->n_tiles * b->S;
    for (size_t i = 0; i < n; ++i) {
        if (!std::isfinite(times[i])) return fail(OCEAN_ERR_INVALID, "time is not finite");
        const ocean_outputs& o = outs[i];
        if (!o.dx || !o.dy || !o.dz || !o.normal_j) return fail(OCEAN_ERR_INVALID, "NULL output pointer");
        const uintptr_t al = reinterpret_cast<uintptr_t>(o.dx) | reinterpret_cast<uintptr_t>(o.dy) |
                             reinterpret_cast<uintptr_t>(o.dz) | reinterpret_cast<uintptr_t>(o.normal_j);
        if (al % 16) return fail(OCEAN_ERR_INVALID, "output pointers must be 16-byte aligned");
    }
    cudaError_t e;
    // the previous replay's H2D copy must have read the staging buffer
    if (b->launched && (e = cudaEventSynchronize(b->done)) != cudaSuccess) return cuda_fail(e, "batch wait");
    ocean::FrameConsts* fc = b->h_fc();
    ocean::ColUnit*     cu = b->h_units();
    for (const ocean_batch_s::Group& g : b->groups) {
        for (size_t j = 0; j < g.tiles.size(); ++j) {
            const int           t = g.tiles[j];
            const ocean_params& p = b->params[t];
            for (int s = 0; s < b->S; ++s) {
                const size_t   u  = g.first_unit + j * b->S + s;
                const double   tt = times[(size_t)t * b->S + s];
                const double   kt = b->K[t] * tt;
                ocean::FrameConsts f;
                f.kt_hi          = (float)kt;
                f.kt_lo          = (float)(kt - (double)f.kt_hi);
                const double dc  = b->w_dc[t] * tt / (2.0 * M_PI);
                f.dc_cycles      = (float)(dc - std::nearbyint(dc));
                f.literal_conj   = (p.flags & OCEAN_FLAG_LITERAL_CONJ) ? 1 : 0;
                fc[u]            = f;
                const ocean_outputs& o = outs[(size_t)t * b->S + s];
                ocean::ColUnit       c;
                c.dx     = o.dx;
                c.dy     = o.dy;
                c.dz     = o.dz;
                c.nj     = reinterpret_cast<float4*>(o.normal_j);
                c.scale  = (float)(0.5 / ((double)g.N * g.N));
                c.lambda = p.choppiness;
                c.inv2d  = (float)((double)g.N / (2.0 * (double)p.L));
                c.pad_   = 0.0f;
                cu[u]    = c;
            }
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((e = cudaGraphLaunch(b->exec, s)) != cudaSuccess) return cuda_fail(e, "batch graph launch");
    if ((e = cudaEventRecord(b->done, s)) != cudaSuccess) return cuda_fail(e, "batch event");
    b->launched = true;
    return OCEAN_OK;
}

int ocean_batch_device_status(ocean_batch_t* b, void* stream)
{
    if (!b) return fail(OCEAN_ERR_INVALID, "batch is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned     h = 0;
    cudaError_t  e;
    if ((e = cudaMemcpyAsync(&h, b->status, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(b->status, 0, sizeof(unsigned), s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "device status");
    if (h) return fail(OCEAN_ERR_TIMEOUT, "a kernel's bounded wait for its TMA copies timed out");
    return OCEAN_OK;
}

void ocean_batch_destroy(ocean_batch_t* b) { delete b; }

}  // extern "C"
