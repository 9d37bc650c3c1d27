// ocean_kernels.cu -- the per-frame Tessendorf ocean update on sm_103a.
//
// One frame is three kernels, chained by programmatic dependent launch (the
// reference dispatches 6*log2(N)+5 full-grid passes, main.cpp:240-244):
//
//   k_row_ws    spectrum evolution + choppy multiply (tilde_h0_t_cs.glsl:70-131)
//   k_row_pass  fused into the horizontal inverse FFT (butterfly_cs.glsl:54-91);
//               k_row_ws (N >= 512) splits each CTA into prepass and transform
//               warps, k_row_pass (below 512) runs both on every warp.
//               Only Re of the 2-D inverse transform is kept
//               (inversion_cs.glsl:35), so each field is first made Hermitian,
//               X_H(k) = (X(k) + conj X(-k))/2, which leaves Re unchanged and
//               makes the row-transformed rows y' and N-y' conjugates: only
//               rows 0..N/2 are transformed and stored.  Persistent CTAs walk
//               the row pairs (y', N-y'); the two spectrum rows of the next
//               pairs are fetched with 1-D bulk TMA copies into a two-stage
//               shared-memory ring while the current pair is transformed, and
//               the phase w*t is computed once per four modes for all three
//               fields.
//
//   k_col_fft   vertical inverse FFT (butterfly_cs.glsl:95-132) of a column
//               pair per line triple, two real results packed per complex
//               transform (one field of both columns per line), staged by
//               1-D bulk copies from the L2-resident intermediate,
//               fused with the (-1)^(x+y)/N^2 inversion (inversion_cs.glsl:29-41)
//               and the lambda scaling; writes the maps column-major.
//
//   k_col_out   32x32 output tiles: transposes the maps through shared memory,
//               adds the Sobel normal on Dy (normal_map_cs.glsl:37-53) and the
//               Jacobian, and writes dx, dy, dz and normal_j row-major with
//               full-line stores.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_line.cuh"
#include "launch_setup.cuh"
#include "ocean_device.cuh"
#include "ocean_internal.h"
#include "tma.cuh"

namespace ocean {

// ---------------------------------------------------------------------------
// h0 initialisation (tilde_h0_k_cs.glsl:35-93), one thread per mode.
// ---------------------------------------------------------------------------
__global__ void k_h0_init(H0Args a, const float* __restrict__ noise, float4* __restrict__ h0)
{
    const int N = a.N;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * N) return;
    const int    x = i % N, y = i / N;
    const size_t NN = (size_t)N * N;
    const int    ix = x - N / 2, iz = y - N / 2;
    float amp = 0.0f;                                     // DC pinned to 0 (normalize(0) is NaN)
    if (ix != 0 || iz != 0) {
        float kx = a.two_pi_over_L * (float)ix, kz = a.two_pi_over_L * (float)iz;
        float k2 = kx * kx + kz * kz;                     // |k| >= 2*pi/L > 1e-5: no floor needed
        float kd = (kx * a.wx + kz * a.wy) * rsqrtf(k2);  // dot(normalize(k), w)
        float P  = a.amplitude * expf(-a.inv_Lp2 / k2) * (kd * kd) * expf(-k2 * a.l2) / (k2 * k2);
        amp      = fminf(sqrtf(P) * 0.70710678118654752f, 4000.0f);
    }
    float n0 = fminf(fmaxf(noise[i], 0.001f), 1.0f);
    float n1 = fminf(fmaxf(noise[NN + i], 0.001f), 1.0f);
    float n2 = fminf(fmaxf(noise[2 * NN + i], 0.001f), 1.0f);
    float n3 = fminf(fmaxf(noise[3 * NN + i], 0.001f), 1.0f);
    float s0, c0, s1, c1;
    sincospif(2.0f * n0, &s0, &c0);                       // cos/sin(2*pi*n)
    sincospif(2.0f * n2, &s1, &c1);
    float v0 = sqrtf(-2.0f * logf(n1)) * amp, v1 = sqrtf(-2.0f * logf(n3)) * amp;
    h0[i] = make_float4(v0 * c0, v0 * s0, v1 * c1, v1 * s1);
}

// Dynamic shared memory, 128-byte aligned (TMA box destinations need it).
__device__ __forceinline__ float2* align_smem(unsigned char* raw)
{
    return reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(raw) + 127) & ~uintptr_t(127));
}

// ---------------------------------------------------------------------------
// Row pass.
// ---------------------------------------------------------------------------
// The spectrum the row pass reads.  With h(k,t) = h0(k) e^{iwt} +
// sigma(h0m(k)) e^{-iwt} (tilde_h0_t_cs.glsl:110; sigma = conj, or the
// identity for the shader's literal conjugate() :42-48) and the index mirror
// k' = (-k) mod N, the Hermitian line input of Dy is
//     h(k) + conj h(k') = e^{iwt} G(k) + e^{-iwt} conj G(k'),
//     G(k) = h0(k) + sigma(h0m(k')),
// and those of Dx and Dz are -i (kx/|k|) and -i (kz/|k|) times it, except on
// the Nyquist column (x = 0) for Dx and the Nyquist row (y = 0) for Dz, where
// k and k' carry the same kx (resp. kz) and the input is -i (k./|k|) times
//     h(k) - conj h(k') = e^{iwt} D(k) - e^{-iwt} conj D(k'),
//     D(k) = h0(k) - sigma(h0m(k')).
// k_spec_combine stores G, then D of column 0, then D of row 0: spec_len(N)
// complex values per tile.  The row pass then reads 8 bytes per mode instead of
// h0's 16.
__global__ void k_spec_combine(int N, const float4* __restrict__ h0, int literal_conj, float2* __restrict__ spec)
{
    const size_t NN = (size_t)N * N;
    const float4* h = h0 + (size_t)blockIdx.y * NN;
    float2*       o = spec + (size_t)blockIdx.y * spec_len(N);
    const int     i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * N + 2 * N) return;
    const float sg = literal_conj ? -1.0f : 1.0f;   // sigma(z) = (z.x, sg * z.y)
    int x, y, sign;
    size_t at;
    if (i < N * N) {
        x = i % N, y = i / N, sign = 1, at = i;
    } else if (i < N * N + N) {
        x = 0, y = i - N * N, sign = -1, at = i;
    } else {
        x = i - N * N - N, y = 0, sign = -1, at = i;
    }
    const int    xm = (N - x) & (N - 1), ym = (N - y) & (N - 1);
    const float4 a  = h[(size_t)y * N + x];
    const float4 b  = h[(size_t)ym * N + xm];
    o[at] = make_float2(a.x + sign * b.z, a.y + sign * sg * b.w);
}

// e^{iwt} g + e^{-iwt} conj(g2), with e^{iwt} = (c, s)
__device__ __forceinline__ float2 herm_sum(float2 g, float2 g2, float c, float s)
{
    return make_float2(c * (g.x + g2.x) - s * (g.y + g2.y), c * (g.y - g2.y) + s * (g.x - g2.x));
}
// e^{iwt} d - e^{-iwt} conj(d2)
__device__ __forceinline__ float2 herm_diff(float2 d, float2 d2, float c, float s)
{
    return make_float2(c * (d.x - d2.x) - s * (d.y - d2.y), c * (d.y + d2.y) + s * (d.x + d2.x));
}
// -i * f * z
__device__ __forceinline__ float2 mul_mi(float f, float2 z) { return make_float2(f * z.y, -f * z.x); }

// Row-line decompositions of the row passes: V = 0 the
// 16-point-first LineFor lines; V = 2 8-point-first lines (one more exchange,
// half the values per thread, twice the threads per line), whose twiddle plan
// follows the row and column plans in the table (k_twiddles); V = 3 (N = 1024)
// the column lines, 32 x 32 (one warp per line, one exchange), which use the
// column plan.  The every-warp row pass uses V = 0 or 3.
template <int N> struct ColLineFor;   // the column decompositions (below), whose plan precedes this one
template <int N, int V> struct RowLine { using type = typename LineFor<N>::type; };
template <> struct RowLine<1024, 3> { using type = LineCfg<1024, 32, 32>; };
template <> struct RowLine<1024, 5> { using type = LineCfg<1024, 32, 32>; };
template <> struct RowLine<512, 2> { using type = LineCfg<512, 8, 8, 8>; };
template <> struct RowLine<1024, 2> { using type = LineCfg<1024, 8, 8, 4, 4>; };
template <> struct RowLine<2048, 2> { using type = LineCfg<2048, 8, 8, 8, 4>; };

template <int N, bool FROM_H0, int V = 0>
struct RowCfg {
    using L = typename RowLine<N, V>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;  // row pairs per work item
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int ITEMS   = (N / 2 + 1 + PAIRS - 1) / PAIRS;  // work items per tile
    // One ring stage: with MINB CTAs resident per SM a tile's row pairs are
    // spread over (almost) every CTA slot at once, and the other resident
    // CTAs hide a CTA's wait for its rows.
    static constexpr int STAGES  = 1;
    // resident CTAs per SM the register budget is set for: <= 80 registers,
    // 128 for the 32 x 32 lines (32 values per thread)
    static constexpr int REGS    = V == 3 ? 128 : 80;
    static constexpr int MINB    = 65536 / (THREADS * REGS) < 1 ? 1 : (65536 / (THREADS * REGS) > 8 ? 8 : 65536 / (THREADS * REGS));
    static constexpr int EW      = FROM_H0 ? 2 : 1;   // float2 per staged mode (h0: float4, G: float2)
    // shared memory (float2 units): tw[N] | ring [STAGES][PAIRS][2 rows][N modes] |
    // line buffers [LINES][NPAD] (line inputs in natural order, then the FFT's exchanges)
    static constexpr size_t RING  = (size_t)STAGES * PAIRS * 2 * N * EW;
    static constexpr size_t WORK  = (size_t)LINES * L::NPAD;
    static constexpr int    TW    = TwPlan<L>::LEN;
    static constexpr size_t SMEM  = sizeof(float2) * (TW + RING + WORK) + 128;   // + base alignment slack
    static constexpr uint32_t ROW_BYTES = (uint32_t)(N * EW * sizeof(float2));
    // offset of the line decomposition's twiddle plan in the table (float2
    // units): the 32 x 32 lines use the column plan, which follows the row plan
    static constexpr int TWOFF = V == 3 ? TwPlan<typename LineFor<N>::type>::LEN : 0;
    static_assert(TWOFF % 2 == 0 && TW % 2 == 0, "16-byte twiddle copies");
};

// Fetch the spectrum rows of work item `item` (tile item/ITEMS, row pairs
// (item%ITEMS)*PAIRS ...) into a ring stage with 1-D bulk copies.
template <int N, bool FROM_H0>
__device__ __forceinline__ void row_issue(const RowArgs& a, float2* ring_stage, uint64_t* bar, int item,
                                          uint32_t extra_bytes = 0)
{
    using RC = RowCfg<N, FROM_H0>;
    const int    tile = item / RC::ITEMS, pi = item % RC::ITEMS;
    const float2* src = FROM_H0 ? reinterpret_cast<const float2*>(a.h0 + (size_t)tile * N * N)
                                : a.spec + (size_t)tile * spec_len(N);
    uint32_t bytes = extra_bytes;
#pragma unroll
    for (int pl = 0; pl < RC::PAIRS; ++pl)
        if (pi * RC::PAIRS + pl <= N / 2) bytes += 2 * RC::ROW_BYTES;
    mbar_arrive_expect_tx(bar, bytes);
#pragma unroll
    for (int pl = 0; pl < RC::PAIRS; ++pl) {
        const int yp = pi * RC::PAIRS + pl;
        if (yp > N / 2) break;
        const int yq = (N - yp) & (N - 1);
        bulk_g2s(ring_stage + (pl * 2 + 0) * N * RC::EW, src + (size_t)yp * N * RC::EW, RC::ROW_BYTES, bar);
        bulk_g2s(ring_stage + (pl * 2 + 1) * N * RC::EW, src + (size_t)yq * N * RC::EW, RC::ROW_BYTES, bar);
    }
}

// The four combined-spectrum values of one position pair (x, xm = N-x) of row
// pair (yp, yq = N-yp): g0 = G(x,yp), g1 = G(xm,yq), g2 = G(xm,yp),
// g3 = G(x,yq), and the D values at the same places where a Nyquist line needs
// them (d0..d3, valid when x == 0 or yp == 0).
template <int N, bool FROM_H0>
__device__ __forceinline__ void row_modes(const RowArgs& a, const float2* rA, const float2* rB, int tile, int x,
                                          int xm, int yp, int yq, int literal, float2 (&g)[4], float2 (&d)[4])
{
    if constexpr (FROM_H0) {
        // G and D from h0 = (h0k, h0m): G(k) = h0k(k) + sigma h0m(k'), k' the mirror
        const float4 a0 = reinterpret_cast<const float4*>(rA)[x], a1 = reinterpret_cast<const float4*>(rA)[xm];
        const float4 b0 = reinterpret_cast<const float4*>(rB)[xm], b1 = reinterpret_cast<const float4*>(rB)[x];
        const float  sg = literal ? -1.0f : 1.0f;
        g[0] = make_float2(a0.x + b0.z, a0.y + sg * b0.w);
        g[1] = make_float2(b0.x + a0.z, b0.y + sg * a0.w);
        g[2] = make_float2(a1.x + b1.z, a1.y + sg * b1.w);
        g[3] = make_float2(b1.x + a1.z, b1.y + sg * a1.w);
        d[0] = make_float2(a0.x - b0.z, a0.y - sg * b0.w);
        d[1] = make_float2(b0.x - a0.z, b0.y - sg * a0.w);
        d[2] = make_float2(a1.x - b1.z, a1.y - sg * b1.w);
        d[3] = make_float2(b1.x - a1.z, b1.y - sg * a1.w);
    } else {
        g[0] = rA[x];
        g[1] = rB[xm];
        g[2] = rA[xm];
        g[3] = rB[x];
        // L2 loads (ld.global.cg), not the read-only path: the row pass runs
        // as a programmatic dependent and may start before the kernel that
        // last wrote the spectrum has finished
        const float2* sp = a.spec + (size_t)tile * spec_len(N);
        if (x == 0) {                                   // column 0: D(0, yp), D(0, yq)
            d[0] = __ldcg(sp + (size_t)N * N + yp);
            d[1] = __ldcg(sp + (size_t)N * N + yq);
        }
        if (yp == 0) {                                  // row 0: D(x, 0), D(xm, 0)
            d[0] = __ldcg(sp + (size_t)N * N + N + x);
            d[1] = __ldcg(sp + (size_t)N * N + N + xm);
            d[2] = d[1];
            d[3] = d[0];
        }
    }
}

// Line inputs of row yp at the position pair (x, N-x) for the three fields:
// the modes (x, yp), (N-x, yp), (N-x, N-yp), (x, N-yp) share |k| (ix^2 and iz^2
// are even) and so the phase.  rows: the pair's two staged rows (yp, then
// N-yp); lines: the three line buffers (Dx, Dy, Dz, NPAD apart).
// The phase part (c, sn = cos, sin of the phase; r = 1/|k| in mode units)
// depends on the position and the time only, not on the staged rows.
template <int N>
__device__ __forceinline__ void row_phase(int x, int yp, const FrameConsts& fc, float& c, float& sn, float& r)
{
    const int ix = x - N / 2, iz = yp - N / 2;
    mode_phase_r(ix * ix + iz * iz, fc, c, sn, r);
}

template <int N, bool FROM_H0, int NPAD>
__device__ __forceinline__ void row_position(const RowArgs& a, const float2* rows, float2* lines, int tile, int x,
                                             int yp, const FrameConsts& fc, float c, float sn, float r)
{
    constexpr int EW = FROM_H0 ? 2 : 1;
    const int yq = (N - yp) & (N - 1), xm = (N - x) & (N - 1);
    const int ix = x - N / 2, iz = yp - N / 2;
    float2 g[4], d[4];
    row_modes<N, FROM_H0>(a, rows, rows + N * EW, tile, x, xm, yp, yq, fc.literal_conj, g, d);
    const float2 y0 = herm_sum(g[0], g[1], c, sn);
    const float2 y1 = herm_sum(g[2], g[3], c, sn);
    float2 ux0 = y0, uz0 = y0, uz1 = y1;
    if (x == 0) ux0 = herm_diff(d[0], d[1], c, sn);
    if (yp == 0) {
        uz0 = herm_diff(d[0], d[1], c, sn);
        uz1 = herm_diff(d[2], d[3], c, sn);
    }
    const float sx = (float)ix * r, sz = (float)iz * r;
    float2* bx = lines;
    float2* by = bx + NPAD;
    float2* bz = by + NPAD;
    bx[x] = mul_mi(sx, ux0);
    by[x] = y0;
    bz[x] = mul_mi(sz, uz0);
    if (xm != x) {                        // ix(xm) = -ix for x != 0
        bx[xm] = mul_mi(-sx, y1);
        by[xm] = y1;
        bz[xm] = mul_mi(sz, uz1);
    }
}

template <int N, bool FROM_H0, int NPAD>
__device__ __forceinline__ void row_position(const RowArgs& a, const float2* rows, float2* lines, int tile, int x,
                                             int yp, const FrameConsts& fc)
{
    float c, sn, r;
    row_phase<N>(x, yp, fc, c, sn, r);
    row_position<N, FROM_H0, NPAD>(a, rows, lines, tile, x, yp, fc, c, sn, r);
}

// MULTI: more than one (tile, sample) unit per launch (batches).  The single
// unit instantiation keeps the per-element constants out of a runtime sample
// loop, which the compiler would otherwise hoist into registers.  FROM_H0: the
// ring holds h0 rows and G, D are formed on the fly (ocean_update_noalloc).
template <int N, bool MULTI, bool FROM_H0, int V>
__device__ __forceinline__ void row_pass_body(const RowArgs& a)
{
    using RC = RowCfg<N, FROM_H0, V>;
    using L  = typename RC::L;
    static_assert(RC::PAIRS == RowCfg<N, FROM_H0>::PAIRS, "row_issue's item layout");
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* ring = smem + RC::TW;                                    // [STAGES][PAIRS][2][N*EW]
    float2* work = ring + RC::RING;                                  // line buffers
    __shared__ __align__(8) uint64_t bars[RC::STAGES];
    __shared__ int wait_ok;

    const int tid = threadIdx.x;
    const int n_items = a.tiles * RC::ITEMS;
    // Thread 0 starts every copy at once: the twiddle table rides on the first
    // stage's barrier (the first item waits for it before its transform).
    if (tid == 0) {
        for (int s = 0; s < RC::STAGES; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
        for (int s = 0; s < RC::STAGES; ++s) {
            const int item = blockIdx.x + s * gridDim.x;
            if (item >= n_items) break;
            const uint32_t twb = s == 0 ? (uint32_t)(RC::TW * sizeof(float2)) : 0u;
            row_issue<N, FROM_H0>(a, ring + (size_t)s * RC::PAIRS * 2 * N * RC::EW, &bars[s], item, twb);
            if (twb) bulk_g2s(tw_s, a.tw + RC::TWOFF, twb, &bars[0]);
        }
    }
    __syncthreads();
    // The column pass may start its set-up now; it waits for this grid to finish
    // before it reads the intermediate.
    pdl_launch_dependents();
    // the early CTAs ask L2 for the late CTAs' spectrum rows (as k_row_ws;
    // prefetch_ctas is 0 unless the launcher set it)
    if (!MULTI && !FROM_H0 && RC::PAIRS == 1 && (int)blockIdx.x < a.prefetch_ctas) {
        const int E = a.prefetch_ctas;
        for (int i = E + (int)blockIdx.x + E * (tid >> 1); i < n_items; i += E * (RC::THREADS >> 1)) {
            const int row = (tid & 1) ? (N - i) & (N - 1) : i;
            l2_prefetch(a.spec + (size_t)row * N, N * sizeof(float2), 0, 1);
        }
    }

    const int li = tid / L::G, t = tid % L::G;
    const int f  = li % 3;                                           // 0: Dx, 1: Dy, 2: Dz
    const int pl_line = li / 3;
    uint32_t phase_bits = 0;

    // 32 x 32 lines (one row pair per item, 128 registers): the first item's
    // phases, which do not depend on its rows, are computed while its rows
    // arrive.  (Under the 80-register budget of the other lines they would
    // spill.)
    constexpr bool PRE = V == 3 && RC::PAIRS == 1;
    constexpr int  PP  = PRE ? (N / 2 + RC::THREADS) / RC::THREADS : 1;   // positions per thread
    float pc[PP], ps[PP], pr[PP];
    if (PRE) {
        const int item = blockIdx.x, tile = item / RC::ITEMS, yp = item % RC::ITEMS;
        const FrameConsts fc = MULTI ? a.fcs[tile * a.S] : a.fc0;
#pragma unroll
        for (int k = 0; k < PP; ++k) {
            const int x = tid + k * RC::THREADS;
            if (x <= N / 2) row_phase<N>(x, yp, fc, pc[k], ps[k], pr[k]);
        }
    }

    for (int k = 0, item = blockIdx.x; item < n_items; ++k, item += gridDim.x) {
        const int s = k % RC::STAGES;
        float2* stage = ring + (size_t)s * RC::PAIRS * 2 * N * RC::EW;
        if (!block_wait(&bars[s], (phase_bits >> s) & 1u, &wait_ok, a.status)) return;
        phase_bits ^= 1u << s;
        const int tile = item / RC::ITEMS, pi = item % RC::ITEMS;

        // The staged rows serve every time sample of the tile.
        const int nsmp = MULTI ? a.S : 1;
        for (int smp = 0; smp < nsmp; ++smp) {
            const int         unit = MULTI ? tile * a.S + smp : 0;
            const FrameConsts fc   = MULTI ? a.fcs[unit] : a.fc0;
            // Line inputs of the pair's row yp for the three fields, position
            // pairs (x, N-x): the modes (x, yp), (N-x, yp), (N-x, N-yp), (x, N-yp)
            // share |k| (ix^2 and iz^2 are even) and so the phase.
            constexpr int HX = N / 2 + 1;
            if (PRE && k == 0 && smp == 0) {
#pragma unroll
                for (int kk = 0; kk < PP; ++kk) {
                    const int x = tid + kk * RC::THREADS;
                    if (x <= N / 2)
                        row_position<N, FROM_H0, L::NPAD>(a, stage, work, tile, x, pi, fc, pc[kk], ps[kk], pr[kk]);
                }
            } else {
                for (int i = tid; i < RC::PAIRS * HX; i += RC::THREADS) {
                    const int pl = RC::PAIRS == 1 ? 0 : i / HX, x = i - pl * HX;
                    const int yp = pi * RC::PAIRS + pl;
                    if (RC::PAIRS > 1 && yp > N / 2) continue;
                    row_position<N, FROM_H0, L::NPAD>(a, stage + (pl * 2) * N * RC::EW, work + (pl * 3) * L::NPAD,
                                                      tile, x, yp, fc);
                }
            }
            __syncthreads();                               // line inputs complete
            if (smp == nsmp - 1 && tid == 0) {             // ring stage consumed: refill it
                const int next = item + RC::STAGES * gridDim.x;
                if (next < n_items) {
                    fence_proxy_async_smem();
                    row_issue<N, FROM_H0>(a, stage, &bars[s], next);
                }
            }

            const int  yp     = pi * RC::PAIRS + pl_line;
            const bool active = yp <= N / 2;
            float2*    buf    = work + li * L::NPAD;
            float2     v[L::E];
#pragma unroll
            for (int r = 0; r < L::E; ++r) v[r] = buf[t + r * L::G];
            line_sync<L, true>(li);                        // the line's inputs are in registers
            line_fft<L, +1, true, true, true>(v, buf, tw_s, t, li);   // paired butterfly adds: faster here
            if (active) {
                // column-pair blocked: x and x+1 of a row are adjacent.  pos(t, e)
                // is t plus an even constant, so the parity is t's.
                static_assert(L::G % 2 == 0 && LineOut<L>::NS % 2 == 0, "even output offsets");
                float2* out = a.inter + (size_t)unit * inter_len(N) + inter_index(N, f, t, yp);
#pragma unroll
                for (int e = 0; e < L::E; ++e)
                    out[(size_t)(LineOut<L>::pos(0, e) >> 1) * (2 * inter_rows(N))] = v[e];
            }
            // the next inputs overwrite the line buffers: every line has
            // finished reading its own
            __syncthreads();
        }
    }
}

// The row pass is launched as a programmatic dependent of the stream's
// previous kernel, so that it can run while that kernel (normally the previous
// frame's output stage) is still writing.  It reads only the spectrum and the
// twiddle plans and writes only the intermediate, none of which that kernel
// touches once it has passed its own griddepcontrol.wait; so it waits for that
// kernel only at its end -- the grid completes, and the kernels that depend on
// it start, only after the previous kernel has completed, which keeps stream
// order for everything downstream.  wait_first: wait before reading too (the
// spectrum or h0 was just written by the previous kernel).
template <int N, bool MULTI, bool FROM_H0, int V = 0>
__global__ void __launch_bounds__(RowCfg<N, FROM_H0, V>::THREADS, RowCfg<N, FROM_H0, V>::MINB) k_row_pass(RowArgs a)
{
    if (a.wait_first) pdl_wait_prior();
    row_pass_body<N, MULTI, FROM_H0, V>(a);
    pdl_wait_prior();
}

// ---------------------------------------------------------------------------
// Warp-specialised row pass (lines of whole warps, N >= 512).  The three
// line FFTs of a job (row pair x time sample) run on 3*G "transform" threads
// while 128 "prepass" threads compute the next job's line inputs into the
// other of two line-buffer sets; each set is the inputs, then the FFT's
// exchange space.  Hand-off by named barriers: FULL[b] (prepass arrives,
// transform waits) and EMPTY[b] (transform arrives, prepass waits before
// refilling set b).  The first job's inputs are computed by every warp
// before the split (its phases while its rows are still arriving), so the
// transform warps start on job 0 without a FULL wait and the prepass warps
// start at job 1.  Both sides walk the same job sequence and execute matching
// barrier operations whatever happens, so a timed-out copy wait (flagged in
// the status word) never leaves a warp waiting.
// ---------------------------------------------------------------------------

template <int N, bool FROM_H0, int V = 0>
struct RowWsCfg {
    using L = typename RowLine<N, V>::type;
    static_assert(L::G >= 32 && L::G % 32 == 0, "lines of whole warps");
    static constexpr int FFT_THREADS = 3 * L::G;
    static constexpr int PRE_THREADS = N >= 2048 ? 256 : 128;
    static constexpr int THREADS     = FFT_THREADS + PRE_THREADS;
    static_assert(THREADS <= 1024, "one CTA");
    static constexpr int ITEMS       = N / 2 + 1;   // row pairs per tile
    // V = 5 (32 x 32 lines, three CTAs per SM): one ring stage and one
    // line-buffer set, so that three CTAs fit in shared memory; the prepass
    // of job j + 1 then waits for job j's transforms
    static constexpr int STAGES      = V == 5 ? 1 : 2;
    static constexpr int SETS        = V == 5 ? 1 : 2;
    static constexpr int EW          = FROM_H0 ? 2 : 1;
    static constexpr size_t RING     = (size_t)STAGES * 2 * N * EW;
    static constexpr size_t BUF      = (size_t)3 * L::NPAD;   // one job's three line buffers
    static constexpr int    TW       = TwPlan<L>::LEN;
    static constexpr size_t SMEM     = sizeof(float2) * (TW + RING + SETS * BUF) + 128;
    // register budget per thread the residency is set for: 96 for the
    // 16-point-first lines, 64 for the 8-point-first ones (8 values per
    // thread), 128 for the 32 x 32 lines (96 with three CTAs per SM)
    static constexpr int REGS        = V == 2 ? 64 : (V == 3 ? 128 : 96);
    static constexpr int MINB        = 65536 / (THREADS * REGS) < 1 ? 1 : 65536 / (THREADS * REGS);
    // offset of this decomposition's twiddle plan in the table (float2 units)
    static constexpr int TWOFF = V == 2   ? TwPlan<typename LineFor<N>::type>::LEN +
                                                TwPlan<typename ColLineFor<N>::type>::LEN
                                 : (V == 3 || V == 5) ? TwPlan<typename LineFor<N>::type>::LEN   // the column plan
                                          : 0;
    static_assert(TWOFF % 2 == 0 && TW % 2 == 0, "16-byte twiddle copies");
    static constexpr int BAR_FULL = 4, BAR_EMPTY = 6, BAR_PRE = 8, BAR_TW = 9;   // named barriers (lines use 1..3)
};

__device__ __forceinline__ void named_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

template <int N, bool MULTI, bool FROM_H0, int V>
__device__ __forceinline__ void row_ws_body(const RowArgs& a)
{
    using WC = RowWsCfg<N, FROM_H0, V>;
    using L  = typename WC::L;
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* ring = smem + WC::TW;                            // [STAGES][2 rows][N*EW]
    float2* bufs = ring + WC::RING;                          // [SETS][3 lines][NPAD]
    __shared__ __align__(8) uint64_t bars[WC::STAGES], bar_tw;
    __shared__ int wait_ok;

    const int tid     = threadIdx.x;
    const int n_items = a.tiles * WC::ITEMS;
    const int nsmp    = MULTI ? a.S : 1;
    const int n_jobs  = (n_items - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x * nsmp;
    if (tid == 0) {
        // issue order = need order: the first rows (prepass), the twiddles
        // (transforms), the next rows
        for (int s = 0; s < WC::STAGES; ++s) mbar_init(&bars[s], 1);
        mbar_init(&bar_tw, 1);
        fence_mbar_init();
        for (int s = 0; s < WC::STAGES; ++s) {
            const int item = blockIdx.x + s * gridDim.x;
            if (item >= n_items) break;
            row_issue<N, FROM_H0>(a, ring + (size_t)s * 2 * N * WC::EW, &bars[s], item);
            if (s == 0) {
                mbar_arrive_expect_tx(&bar_tw, WC::TW * sizeof(float2));
                bulk_g2s(tw_s, a.tw + WC::TWOFF, WC::TW * sizeof(float2), &bar_tw);
            }
        }
        wait_ok = 1;
    }
    __syncthreads();
    pdl_launch_dependents();
    // The first prefetch_ctas CTAs start on the SMs that the previous frame's
    // column stage leaves free, the others only when it ends: the early ones
    // ask L2 for the late ones' spectrum rows (item i >= E by CTA (i - E) % E,
    // one row per thread), so that those find their rows there instead of in
    // HBM.  A hint only; nothing waits for it.
    if (!MULTI && !FROM_H0 && (int)blockIdx.x < a.prefetch_ctas) {
        const int E = a.prefetch_ctas, i = E + (int)blockIdx.x + E * (tid >> 1);
        if (i < n_items) {
            const int yp = i, row = (tid & 1) ? (N - yp) & (N - 1) : yp;
            l2_prefetch(a.spec + (size_t)row * N, N * sizeof(float2), 0, 1);
        }
    }

    // The first job's line inputs are computed by every warp: until they
    // exist the transform warps have nothing to do.  (Every CTA has a job:
    // the grid is at most the number of items.)
    {
        const int item = blockIdx.x, tile = item / WC::ITEMS, yp = item % WC::ITEMS;
        const FrameConsts fc = MULTI ? a.fcs[tile * a.S] : a.fc0;
        // the phases do not depend on the rows: computed while they arrive
        constexpr int PP = (N / 2 + WC::THREADS) / WC::THREADS;   // positions per thread
        float c[PP], sn[PP], r[PP];
#pragma unroll
        for (int k = 0; k < PP; ++k) {
            const int x = tid + k * WC::THREADS;
            if (x <= N / 2) row_phase<N>(x, yp, fc, c[k], sn[k], r[k]);
        }
        if (tid == 0 && !mbar_wait_bounded(&bars[0], 0)) {
            atomicOr(a.status, kDeviceTimeout);
            (void)mbar_wait_bounded(&bars[0], 0);
            wait_ok = 0;
        }
        __syncthreads();                                     // the rows are in (or the wait gave up)
#pragma unroll
        for (int k = 0; k < PP; ++k) {
            const int x = tid + k * WC::THREADS;
            if (x <= N / 2) row_position<N, FROM_H0, L::NPAD>(a, ring, bufs, tile, x, yp, fc, c[k], sn[k], r[k]);
        }
        __syncthreads();                                     // job 0's inputs are complete
        if (nsmp == 1 && tid == 0 && wait_ok) {              // stage 0 is consumed: refill it
            const int next = item + WC::STAGES * gridDim.x;
            if (next < n_items) {
                fence_proxy_async_smem();
                row_issue<N, FROM_H0>(a, ring, &bars[0], next);
            }
        }
    }

    if (tid < WC::FFT_THREADS) {
        const int li = tid / L::G, t = tid % L::G;           // line = field 0: Dx, 1: Dy, 2: Dz
        if (tid == 0 && !mbar_wait_bounded(&bar_tw, 0)) {
            atomicOr(a.status, kDeviceTimeout);
            (void)mbar_wait_bounded(&bar_tw, 0);
        }
        named_sync(WC::BAR_TW, WC::FFT_THREADS);             // the twiddle plan is in
        for (int j = 0; j < n_jobs; ++j) {
            const int b = j % WC::SETS, ki = j / nsmp, smp = j - ki * nsmp;
            const int item = blockIdx.x + ki * gridDim.x, tile = item / WC::ITEMS, yp = item % WC::ITEMS;
            const int unit = MULTI ? tile * a.S + smp : 0;
            if (j > 0) named_sync(WC::BAR_FULL + b, WC::THREADS);   // the job's line inputs are complete
            float2* buf = bufs + b * WC::BUF + li * L::NPAD;
            float2  v[L::E];
#pragma unroll
            for (int r = 0; r < L::E; ++r) v[r] = buf[t + r * L::G];
            line_sync<L, true>(li);
            // no final line barrier: the prepass refills buf only after every
            // transform thread has arrived on EMPTY, each after its own reads
            line_fft<L, +1, true, false>(v, buf, tw_s, t, li);
            named_arrive(WC::BAR_EMPTY + b, WC::THREADS);    // this thread is done with buf
            static_assert(L::G % 2 == 0 && LineOut<L>::NS % 2 == 0, "even output offsets");
            float2* out = a.inter + (size_t)unit * inter_len(N) + inter_index(N, li, t, yp);
#pragma unroll
            for (int e = 0; e < L::E; ++e) out[(size_t)(LineOut<L>::pos(0, e) >> 1) * (2 * inter_rows(N))] = v[e];
        }
    } else {
        const int pt = tid - WC::FFT_THREADS;
        uint32_t  phase_bits = 1u;                            // stage 0's first phase went to job 0
        bool      gave_up    = wait_ok == 0;                  // a copy wait timed out: issue no more copies
        for (int j = 1; j < n_jobs; ++j) {
            const int b = j % WC::SETS, ki = j / nsmp, smp = j - ki * nsmp;
            const int item = blockIdx.x + ki * gridDim.x, tile = item / WC::ITEMS, yp = item % WC::ITEMS;
            const int st = ki % WC::STAGES;
            float2* stage = ring + (size_t)st * 2 * N * WC::EW;
            if (smp == 0) {                                  // the item's rows
                // every issued copy is waited for (bounded), so none is in
                // flight when the block exits
                if (pt == 0) {
                    if (!mbar_wait_bounded(&bars[st], (phase_bits >> st) & 1u)) {
                        atomicOr(a.status, kDeviceTimeout);
                        (void)mbar_wait_bounded(&bars[st], (phase_bits >> st) & 1u);
                        wait_ok = 0;
                    }
                }
                phase_bits ^= 1u << st;
                named_sync(WC::BAR_PRE, WC::PRE_THREADS);
                gave_up = wait_ok == 0;
            }
            if (j >= WC::SETS) named_sync(WC::BAR_EMPTY + b, WC::THREADS);   // set b's previous job is transformed
            const FrameConsts fc = MULTI ? a.fcs[tile * a.S + smp] : a.fc0;
#pragma unroll 4
            for (int x = pt; x <= N / 2; x += WC::PRE_THREADS)
                row_position<N, FROM_H0, L::NPAD>(a, stage, bufs + b * WC::BUF, tile, x, yp, fc);
            named_arrive(WC::BAR_FULL + b, WC::THREADS);
            if (smp == nsmp - 1) {                           // every prepass thread is done with the stage
                named_sync(WC::BAR_PRE, WC::PRE_THREADS);
                if (pt == 0 && !gave_up) {
                    const int next = item + WC::STAGES * gridDim.x;
                    if (next < n_items) {
                        fence_proxy_async_smem();
                        row_issue<N, FROM_H0>(a, stage, &bars[st], next);
                    }
                }
            }
        }
        // the transform side's last arrivals on EMPTY
        for (int j = n_jobs - WC::SETS > 0 ? n_jobs - WC::SETS : 0; j < n_jobs; ++j)
            named_sync(WC::BAR_EMPTY + j % WC::SETS, WC::THREADS);
    }
}

// Launched as k_row_pass is (see there): waits for the stream's previous
// kernel at its end, or first with wait_first.
template <int N, bool MULTI, bool FROM_H0, int V = 0>
__global__ void __launch_bounds__(RowWsCfg<N, FROM_H0, V>::THREADS, RowWsCfg<N, FROM_H0, V>::MINB) k_row_ws(RowArgs a)
{
    if (a.wait_first) pdl_wait_prior();
    row_ws_body<N, MULTI, FROM_H0, V>(a);
    pdl_wait_prior();
}

// ---------------------------------------------------------------------------
// Column transforms.
// ---------------------------------------------------------------------------
// Column line decomposition: 32-point first passes at N = 1024 (one warp per
// line, 32 x 32: one exchange instead of two) and N = 2048 (64 threads per
// line, 32 x 8 x 8, 168 registers: two CTAs per SM); else as LineFor.
template <int N> struct ColLineFor { using type = typename LineFor<N>::type; };
template <> struct ColLineFor<1024> { using type = LineCfg<1024, 32, 32>; };
template <> struct ColLineFor<2048> { using type = LineCfg<2048, 32, 8, 8>; };

template <int N>
struct ColCfg {
    using L = typename ColLineFor<N>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;   // column pairs per CTA
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int CTAS    = N / 2 / PAIRS;               // per unit
    static constexpr int H       = inter_rows(N);
    // the staged intermediate [3][PAIRS][H][2] shares the line buffers
    static constexpr size_t TILE = (size_t)3 * PAIRS * H * 2;
    static constexpr size_t WORK = (size_t)LINES * L::NPAD > TILE ? (size_t)LINES * L::NPAD : TILE;
    static constexpr int    TW   = TwPlan<L>::LEN;
    static constexpr int    TW0  = TwPlan<typename LineFor<N>::type>::LEN;   // the row plan precedes it
    static constexpr size_t SMEM = sizeof(float2) * (TW + WORK) + 128;
    static constexpr uint32_t FIELD_BYTES = (uint32_t)(sizeof(float2) * PAIRS * H * 2);
    static_assert((N / 2) % PAIRS == 0, "column pairs per CTA");
    static_assert(FIELD_BYTES % 16 == 0, "bulk copy size");
};

// Line triple of column pair (x0, x0+1): line f = field f of column x0 + i *
// field f of column x0+1 (f = 0: Dx, 1: Dy, 2: Dz).  Rows y > N/2 are the
// conjugates of rows N-y (the row-transformed spectra are Hermitian in y), so
// the inputs come from rows 0..N/2 of the intermediate, whose column pairs are
// contiguous: one 1-D bulk copy per field stages them.
template <int N>
__global__ void __launch_bounds__(ColCfg<N>::THREADS) k_col_fft(const __grid_constant__ ColArgs a)
{
    using CF = ColCfg<N>;
    using L  = typename CF::L;
    constexpr int H = CF::H;
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* work = smem + CF::TW;                            // staged tile, then line buffers
    __shared__ __align__(8) uint64_t bar, bar_tw;
    __shared__ int wait_ok;
    const int      tid  = threadIdx.x;
    const int      unit = blockIdx.y;
    const ColUnit* cu   = a.units ? a.units + unit : &a.u0;
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init(&bar_tw, 1);
        fence_mbar_init();
        // the twiddle plan does not depend on the row pass: fetch it now
        mbar_arrive_expect_tx(&bar_tw, CF::TW * sizeof(float2));
        bulk_g2s(tw_s, a.tw + CF::TW0, CF::TW * sizeof(float2), &bar_tw);
    }
    pdl_wait_prior();                                        // the row pass has finished
    __syncthreads();
    const int pair0 = blockIdx.x * CF::PAIRS;
    if (tid == 0) {
        mbar_arrive_expect_tx(&bar, 3 * CF::FIELD_BYTES);
        const float2* in = a.inter + (size_t)unit * inter_len(N);
#pragma unroll
        for (int f = 0; f < 3; ++f)
            bulk_g2s(work + (size_t)f * CF::PAIRS * H * 2, in + inter_index(N, f, 2 * pair0, 0), CF::FIELD_BYTES, &bar);
    }
    if (!block_wait(&bar, 0, &wait_ok, a.status)) {
        // the twiddle copy may still be in flight: let it land (bounded) before
        // the block's shared memory is released
        if (tid == 0) (void)mbar_wait_bounded(&bar_tw, 0);
        __syncthreads();
        return;
    }
    // The staged blocks are this CTA's alone and the next write of the
    // intermediate is the next frame's row pass: drop their L2 lines instead
    // of letting them be written back to HBM.
    {
        const float2* in = a.inter + (size_t)unit * inter_len(N);
#pragma unroll
        for (int f = 0; f < 3; ++f)
            l2_discard(in + inter_index(N, f, 2 * pair0, 0), CF::FIELD_BYTES, tid, CF::THREADS);
    }

    // Line li of pair pl holds field f = li % 3 (0: Dx, 1: Dy, 2: Dz) of both
    // columns, f(x0) + i*f(x0+1): the row-transformed spectra are Hermitian in
    // y, so the transform's real and imaginary parts are the two columns.
    const int li = tid / L::G, t = tid % L::G;
    const int f  = li % 3, pl = li / 3;
    const int x0 = 2 * (pair0 + pl);
    // Input r of thread t is row y = t + r*G (G = N/R1, t < G): rows below
    // N/2 for r < R1/2, the conjugate of row N - y for r > R1/2, and for
    // r = R1/2 row N/2 - t, conjugated unless t = 0 (y = N/2).  So every
    // shared-memory offset is a per-thread base plus a constant, and each read
    // is the 16-byte (column x0, column x0+1) pair of one row.
    constexpr int G = L::G;
    const float2* fp = work + ((size_t)(f * CF::PAIRS + pl) * H) * 2;
    float2 v[L::E];
#pragma unroll
    for (int r = 0; r < L::E; ++r) {
        const int    ys = r < L::R1 / 2 ? t + r * G : (r == L::R1 / 2 ? N / 2 - t : N - t - r * G);
        const bool   cj = r > L::R1 / 2 || (r == L::R1 / 2 && t != 0);
        const float4 z  = *reinterpret_cast<const float4*>(fp + 2 * ys);
        float2       p  = make_float2(z.x, z.y);                          // column x0
        float2       q  = make_float2(z.z, z.w);                          // column x0+1
        if (cj) { p.y = -p.y; q.y = -q.y; }
        v[r] = make_float2(p.x - q.y, p.y + q.x);                          // p + i*q
    }
    if (!block_wait(&bar_tw, 0, &wait_ok, a.status)) return;   // also: the tile is consumed
    pdl_launch_dependents();                                 // k_col_out may start its set-up
    // no final barrier (work is not reused); paired butterfly adds: faster here
    line_fft<L, +1, true, false, true>(v, work + li * L::NPAD, tw_s, t, li);

    // output y = pos(t, e) is t plus an even constant: the (-1)^(x+y) sign is
    // the thread's, and the two columns' signs are opposite.  Dy is scaled by
    // 1/(2N^2) (the 1/N^2 inversion and the Hermitian half), Dx and Dz also by
    // lambda.
    static_assert(L::G % 2 == 0 && LineOut<L>::NS % 2 == 0, "even output offsets");
    float* const tm = a.tmap + (size_t)unit * tmap_len(N);
    const float  sg = ((x0 + t) & 1) ? -1.0f : 1.0f;
    const float  k  = sg * (f == 1 ? cu->scale : cu->scale * cu->lambda);
    float* const o  = tm + ((size_t)f * N + x0) * N + t;     // field f, columns x0 and x0+1
#pragma unroll
    for (int e = 0; e < L::E; ++e) {
        o[LineOut<L>::pos(0, e)]     = k * v[e].x;
        o[N + LineOut<L>::pos(0, e)] = -k * v[e].y;
    }
}

// ---------------------------------------------------------------------------
// Output tiles: 32 x 32 texels per CTA, with a one-texel periodic halo.
// ---------------------------------------------------------------------------
constexpr int kOutT  = 32;             // tile edge
constexpr int kOutW  = kOutT + 2;      // with halo
constexpr int kOutP  = kOutT + 3;      // shared pitch: odd, so column-wise reads are conflict-free
constexpr int kOutTh = 256;
constexpr int kOutRows = kOutT * kOutT / kOutTh;   // rows per thread (one column, consecutive rows)

template <int N>
__global__ void __launch_bounds__(kOutTh, 5) k_col_out(const __grid_constant__ ColArgs a)
{
    __shared__ float S[3][kOutW][kOutP];                     // [field][x][y]: Dx, Dy, Dz; index = coordinate - origin + 1
    const int      unit = blockIdx.z;
    const int      x0 = blockIdx.x * kOutT, y0 = blockIdx.y * kOutT;
    const ColUnit* cu = a.units ? a.units + unit : &a.u0;
    const float*   tm = a.tmap + (size_t)unit * tmap_len(N);
    const int      tid = threadIdx.x;
    pdl_wait_prior();                                        // the column transforms have finished
    // The next frame's row pass may start now: the intermediate it writes has
    // been read (k_col_fft has completed), and it completes only after this
    // grid has.  Only when that row pass overlaps (tuning): otherwise its CTAs
    // would only wait on the SMs.
    if (a.trigger_next) pdl_launch_dependents();

    // Stage the maps: each of the 3 x 34 columns (field f, x = x0-1 .. x0+32)
    // is rows y0 .. y0+31 (eight aligned 16-byte pieces) plus the halo rows
    // y0-1 and y0+32.  All loads of a thread are issued before its stores.
    constexpr int NCOL = 3 * kOutW, NPC = NCOL * 8, NV = (NPC + kOutTh - 1) / kOutTh;
    float4 body[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int i = tid + j * kOutTh;                      // piece i: column i/8, rows y0 + 4*(i%8) ..
        if (i < NPC) {
            const int c = i >> 3, f = c / kOutW, xx = c - f * kOutW;
            body[j] = *reinterpret_cast<const float4*>(tm + ((size_t)f * N + ((x0 - 1 + xx) & (N - 1))) * N + y0 +
                                                       4 * (i & 7));
        }
    }
    float edge[(2 * NCOL + kOutTh - 1) / kOutTh];
#pragma unroll
    for (int j = 0; j < (2 * NCOL + kOutTh - 1) / kOutTh; ++j) {
        const int i = tid + j * kOutTh;                      // halo value i: column i/2, row y0-1 or y0+32
        if (i < 2 * NCOL) {
            const int c = i >> 1, f = c / kOutW, xx = c - f * kOutW;
            const int y = (i & 1) ? (y0 + kOutT) & (N - 1) : (y0 - 1) & (N - 1);
            edge[j] = tm[((size_t)f * N + ((x0 - 1 + xx) & (N - 1))) * N + y];
        }
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int i = tid + j * kOutTh;
        if (i < NPC) {
            const int c = i >> 3, f = c / kOutW, xx = c - f * kOutW, yy = 1 + 4 * (i & 7);
            S[f][xx][yy]     = body[j].x;
            S[f][xx][yy + 1] = body[j].y;
            S[f][xx][yy + 2] = body[j].z;
            S[f][xx][yy + 3] = body[j].w;
        }
    }
#pragma unroll
    for (int j = 0; j < (2 * NCOL + kOutTh - 1) / kOutTh; ++j) {
        const int i = tid + j * kOutTh;
        if (i < 2 * NCOL) {
            const int c = i >> 1, f = c / kOutW, xx = c - f * kOutW;
            S[f][xx][(i & 1) ? kOutT + 1 : 0] = edge[j];
        }
    }
    __syncthreads();

    // Four consecutive rows of one column per thread; a warp covers 32
    // consecutive columns, so every store is a full line.  Rows yy-1 .. yy+4
    // of the three columns around xx are read once and shared by the four
    // texels.
    const int xx = tid % kOutT + 1;                          // staged column of output x0 + xx - 1
    const int yb = (tid / kOutT) * kOutRows;                 // first output row - y0
    float C0[kOutRows + 2], C1[kOutRows + 2], C2[kOutRows + 2];   // Dy at xx-1, xx, xx+1
    float Xm[kOutRows], Xp[kOutRows], Zm[kOutRows], Zp[kOutRows];  // Dx, Dz at xx-1 and xx+1
    float Xc[kOutRows + 2], Zc[kOutRows + 2];                       // Dx, Dz at xx
#pragma unroll
    for (int k = 0; k < kOutRows + 2; ++k) {
        C0[k] = S[1][xx - 1][yb + k];
        C1[k] = S[1][xx][yb + k];
        C2[k] = S[1][xx + 1][yb + k];
        Xc[k] = S[0][xx][yb + k];
        Zc[k] = S[2][xx][yb + k];
    }
#pragma unroll
    for (int k = 0; k < kOutRows; ++k) {
        Xm[k] = S[0][xx - 1][yb + k + 1];
        Xp[k] = S[0][xx + 1][yb + k + 1];
        Zm[k] = S[2][xx - 1][yb + k + 1];
        Zp[k] = S[2][xx + 1][yb + k + 1];
    }
    float* const  odx = cu->dx;
    float* const  ody = cu->dy;
    float* const  odz = cu->dz;
    float4* const onj = cu->nj;
    const float   inv2d = cu->inv2d;
    const size_t  o0 = (size_t)(y0 + yb) * N + x0 + xx - 1;
#pragma unroll
    for (int k = 0; k < kOutRows; ++k) {
        // taps z0..z7 (normal_map_cs.glsl:37-44): z0 = (x-1, y-1), z1 = (x, y-1),
        // z2 = (x+1, y-1), z3 = (x-1, y), z4 = (x+1, y), z5..z7 the row below
        const float z0 = C0[k], z1 = C1[k], z2 = C2[k], z3 = C0[k + 1], z4 = C2[k + 1];
        const float z5 = C0[k + 2], z6 = C1[k + 2], z7 = C2[k + 2];
        const float nz = z0 + 2.0f * z1 + z2 - z5 - 2.0f * z6 - z7;
        const float nx = z0 + 2.0f * z3 + z5 - z2 - 2.0f * z4 - z7;
        const float rn = rsqrtf(nx * nx + 1.0f + nz * nz);
        const float dxx = (Xp[k] - Xm[k]) * inv2d;
        const float dxz = (Xc[k + 2] - Xc[k]) * inv2d;
        const float dzx = (Zp[k] - Zm[k]) * inv2d;
        const float dzz = (Zc[k + 2] - Zc[k]) * inv2d;
        // J = (1 - dxx)(1 - dzz) - dxz*dzx, formed as 1 + deviation so that the
        // only rounding at the scale of 1 is the final add
        const float  dJ = (dxx * dzz - dxz * dzx) - dxx - dzz;
        const size_t o  = o0 + (size_t)k * N;
        // streaming stores (evict first): the maps leave L2 before the
        // frame's scratch does
        __stcs(odx + o, Xc[k + 1]);
        __stcs(ody + o, C1[k + 1]);
        __stcs(odz + o, Zc[k + 1]);
        __stcs(onj + o, make_float4(nx * rn, rn, nz * rn, 1.0f + dJ));
    }
}

// ---------------------------------------------------------------------------
// Fused column side (N = 512, 1024; the tuning's col_fused): the column
// transforms with the inversion and lambda (k_col_fft) and the Sobel normal
// and Jacobian (k_col_out) in one kernel, so that the column-major maps never
// leave the SM (inversion_cs.glsl:25-43, normal_map_cs.glsl:24-54).
//
// A CTA owns P column pairs -- output columns x0 .. x0+2P-1 -- and also
// transforms its two halo columns x0-1 and x0+2P, packed into one complex line
// per field: any two real columns can share a transform, because the
// row-transformed spectra are Hermitian in y.  One warp per line, lines read
// straight from the L2-resident intermediate.  After the transforms the real
// columns are staged in shared memory (the exchange buffers, reused) and the
// CTA computes its 2P x N output texels from there, the lanes of a warp on 2P
// adjacent columns of 32/(2P) rows.
// ---------------------------------------------------------------------------
template <int N, int P>
struct FusedCfg {
    using L = typename ColLineFor<N>::type;
    static_assert(L::G == 32, "one warp per line");
    static constexpr int LINES    = 3 * (P + 1);           // P pairs and one halo line per field
    static constexpr int THREADS  = LINES * 32;
    static constexpr int CTAS     = N / (2 * P);           // per unit
    static constexpr int COLS     = 2 * P + 2;             // staged columns x0-1 .. x0+2P
    // staged column pitch (floats): the 2P columns a warp reads are 32/(2P)
    // banks apart, and its 32/(2P) rows fill the banks in between
    static constexpr int CP       = N + 16 / P;
    static constexpr int ETHREADS = THREADS;               // epilogue threads: all of them
    static constexpr int EROWS    = ETHREADS / (2 * P);    // rows per epilogue step (need not divide N)
    static constexpr size_t XBUF  = (size_t)LINES * L::NPAD;               // float2
    static constexpr size_t EBUF  = ((size_t)3 * COLS * CP + 1) / 2;       // float2
    static constexpr size_t WORK  = XBUF > EBUF ? XBUF : EBUF;
    static constexpr int    TW    = TwPlan<L>::LEN;
    static constexpr int    TW0   = TwPlan<typename LineFor<N>::type>::LEN;   // the row plan precedes it
    static constexpr size_t SMEM  = sizeof(float2) * (TW + WORK) + 128;
    static_assert(N % (2 * P) == 0 && THREADS % (2 * P) == 0, "fused column layout");
    static_assert((16 / P) * 2 * P == 32 && 32 % (2 * P) == 0, "conflict-free staging pitch");
};

template <int N, int P>
__global__ void __launch_bounds__(FusedCfg<N, P>::THREADS, P == 2 ? 2 : 1) k_col_fused(const __grid_constant__ ColArgs a)
{
    using FC = FusedCfg<N, P>;
    using L  = typename FC::L;
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* work = smem + FC::TW;                            // exchange buffers, then the staged columns
    __shared__ __align__(8) uint64_t bar_tw;
    __shared__ unsigned loaded_warps;
    const int      tid  = threadIdx.x;
    const int      unit = blockIdx.y;
    const ColUnit* cu   = a.units ? a.units + unit : &a.u0;
    if (tid == 0) {
        mbar_init(&bar_tw, 1);
        fence_mbar_init();
        loaded_warps = 0;
        // the twiddle plan does not depend on the row pass: fetch it now
        mbar_arrive_expect_tx(&bar_tw, FC::TW * sizeof(float2));
        bulk_g2s(tw_s, a.tw + FC::TW0, FC::TW * sizeof(float2), &bar_tw);
    }
    __syncthreads();                                         // the barrier and the counter are set up
    pdl_wait_prior();                                        // the row pass has finished

    // Line li: field f = li % 3 of columns ca (real part) and cb (imaginary
    // part); kind < P: the pair x0 + 2 kind, x0 + 2 kind + 1; kind == P: the
    // halo columns x0 - 1 and x0 + 2P (periodic).
    const int li = tid >> 5, t = tid & 31;
    const int f = li % 3, kind = li / 3;
    const int x0 = 2 * P * (int)blockIdx.x;
    const int ca = kind < P ? x0 + 2 * kind : (x0 - 1) & (N - 1);
    const int cb = kind < P ? ca + 1 : (x0 + 2 * P) & (N - 1);
    const float2* in = a.inter + (size_t)unit * inter_len(N);
    constexpr int G = L::G, R1 = L::R1, HR = L::R1 / 2;
    static_assert(G == 32 && L::E == R1, "one warp per line, one value per first-pass input");
    // Register r holds row y = t + r*G.  Rows up to N/2 are loaded: registers
    // r < R1/2 (rows t + r*G) and register R1/2 (row N/2 - t, the conjugate of
    // row N/2 + t for t > 0).  A row y > N/2 is the conjugate of row N - y
    // (the row-transformed spectra are Hermitian in y), which another lane has
    // loaded: N - t - r*G = (32 - t) + (R1 - 1 - r)*G, register R1 - 1 - r of
    // lane 32 - t (lane 0: its own register R1 - r).  L2 loads
    // (ld.global.cg): the read-only (non-coherent) path may keep lines of the
    // previous frame's intermediate, which the row pass rewrites while this
    // grid is already resident (it is launched as a programmatic dependent).
    float4 z[HR + 1];                                        // (column ca, column cb) of the row
#pragma unroll
    for (int r = 0; r <= HR; ++r) {
        const int ys = r < HR ? t + r * G : N / 2 - t;
        if (kind < P) {                                      // one 16-byte (ca, cb) pair of the row
            z[r] = __ldcg(reinterpret_cast<const float4*>(in + inter_index(N, f, ca, ys)));
        } else {
            const float2 p = __ldcg(in + inter_index(N, f, ca, ys));
            const float2 q = __ldcg(in + inter_index(N, f, cb, ys));
            z[r] = make_float4(p.x, p.y, q.x, q.y);
        }
    }
    float2 v[L::E];
    const int src = (32 - t) & 31;
#pragma unroll
    for (int r = HR + 1; r < R1; ++r) {
        const float4 w = z[R1 - 1 - r];
        float4 m = make_float4(__shfl_sync(0xffffffffu, w.x, src), __shfl_sync(0xffffffffu, w.y, src),
                               __shfl_sync(0xffffffffu, w.z, src), __shfl_sync(0xffffffffu, w.w, src));
        if (t == 0) m = z[R1 - r];
        v[r] = make_float2(m.x + m.w, m.z - m.y);            // conj(p) + i*conj(q)
    }
#pragma unroll
    for (int r = 0; r <= HR; ++r) {
        float4 m = z[r];
        if (r == HR && t != 0) { m.y = -m.y; m.w = -m.w; }
        v[r] = make_float2(m.x - m.w, m.y + m.z);            // p + i*q
    }
    // The next frame's row pass may overwrite the intermediate once every
    // thread's loads have returned (a CTA may count as triggered as soon as any
    // of its threads triggers).  Each warp reduces a word that depends on all
    // of its lanes' loaded values, so its lane 0 passes the reduction only
    // after the warp's loads have returned; it then counts the warp in, and
    // the lane that counts the last warp triggers.  The row pass then runs on
    // the SMs this grid leaves free and completes only after this grid.  No
    // block barrier: a warp goes on to its transform as soon as its own line
    // is loaded.
    {
        unsigned dep = 0;
#pragma unroll
        for (int r = 0; r < L::E; ++r) dep |= __float_as_uint(v[r].x) ^ __float_as_uint(v[r].y);
        dep = __reduce_or_sync(0xffffffffu, dep);
        asm volatile("" ::"r"(dep) : "memory");             // the reduction stays, before the count
        if (t == 0 && atomicAdd(&loaded_warps, 1u) == FC::LINES - 1 && a.trigger_next) pdl_launch_dependents();
    }
    // the twiddle plan, waited for per warp (bounded; a time-out is flagged,
    // and the warp goes on so that every block barrier below is reached)
    if (t == 0 && !mbar_wait_bounded(&bar_tw, 0)) {
        atomicOr(a.status, kDeviceTimeout);
        (void)mbar_wait_bounded(&bar_tw, 0);
    }
    __syncwarp();
    line_fft<L, +1, true, false>(v, work + li * L::NPAD, tw_s, t, li);
    __syncthreads();                                         // the exchange buffers are free

    // Stage the real columns: (-1)^(x+y) * 1/(2N^2) (* lambda for Dx, Dz).
    // y = pos(t, e) is t plus an even constant, so the sign is per thread.
    float* const E = reinterpret_cast<float*>(work);
    {
        const float sc = f == 1 ? cu->scale : cu->scale * cu->lambda;
        const float sA = ((ca + t) & 1) ? -sc : sc;
        const float sB = ((cb + t) & 1) ? -sc : sc;
        const int   cA = kind < P ? 1 + 2 * kind : 0;
        const int   cB = kind < P ? 2 + 2 * kind : 2 * P + 1;
        float* const ea = E + (size_t)(f * FC::COLS + cA) * FC::CP;
        float* const eb = E + (size_t)(f * FC::COLS + cB) * FC::CP;
        static_assert(L::G % 2 == 0 && LineOut<L>::NS % 2 == 0, "even output offsets");
#pragma unroll
        for (int e = 0; e < L::E; ++e) {
            const int y = LineOut<L>::pos(t, e);
            ea[y] = sA * v[e].x;
            eb[y] = sB * v[e].y;
        }
    }
    __syncthreads();

    const float* EX    = E;                                  // Dx columns
    const float* EY    = E + (size_t)FC::COLS * FC::CP;      // Dy
    const float* EZ    = E + (size_t)2 * FC::COLS * FC::CP;  // Dz
    const int    c     = tid % (2 * P) + 1;                  // staged column of the texel
    const int    cm    = (c - 1) * FC::CP, c0 = c * FC::CP, cp = (c + 1) * FC::CP;
    float* const  odx  = cu->dx;
    float* const  ody  = cu->dy;
    float* const  odz  = cu->dz;
    float4* const onj  = cu->nj;
    const float   inv2d = cu->inv2d;
    const int     x    = x0 + c - 1;
    if constexpr (P == 4) {
        // Epilogue, 4 pairs: thread (c, q), q = tid / 2P, walks its block of
        // rows [q*N/EBLK, (q+1)*N/EBLK) top to bottom with the 3 x 3
        // neighbourhood in registers: each row loads 9 staged values (row y+1
        // of Dy's three columns, of Dx's and Dz's own column, row y of their
        // side columns) instead of 19.  A warp covers 2P columns of 32/(2P)
        // row blocks, so its stores are 32/(2P) row pieces, as below.  (With
        // 2 pairs the independent rows below measured faster.)
        constexpr int EBLK = FC::THREADS / (2 * P);
        const int q  = tid / (2 * P);
        const int ya = q * N / EBLK, yb = (q + 1) * N / EBLK;
        // rows y-1 and y of the window (taps z0..z7, normal_map_cs.glsl:37-44)
        const int ym = (ya - 1) & (N - 1);
        float a0 = EY[cm + ym], a1 = EY[c0 + ym], a2 = EY[cp + ym];   // Dy, row y-1
        float b0 = EY[cm + ya], b1 = EY[c0 + ya], b2 = EY[cp + ya];   // Dy, row y
        float xu = EX[c0 + ym], xc = EX[c0 + ya];                      // Dx column, rows y-1, y
        float zu = EZ[c0 + ym], zc = EZ[c0 + ya];                      // Dz column, rows y-1, y
        for (int y = ya; y < yb; ++y) {
            const int   yq = (y + 1) & (N - 1);
            const float d0 = EY[cm + yq], d1 = EY[c0 + yq], d2 = EY[cp + yq];   // Dy, row y+1
            const float xd = EX[c0 + yq], zd = EZ[c0 + yq];
            const float nz = a0 + 2.0f * a1 + a2 - d0 - 2.0f * d1 - d2;
            const float nx = a0 + 2.0f * b0 + d0 - a2 - 2.0f * b2 - d2;
            const float rn = rsqrtf(nx * nx + 1.0f + nz * nz);
            const float dxx = (EX[cp + y] - EX[cm + y]) * inv2d;
            const float dxz = (xd - xu) * inv2d;
            const float dzx = (EZ[cp + y] - EZ[cm + y]) * inv2d;
            const float dzz = (zd - zu) * inv2d;
            const float dJ  = (dxx * dzz - dxz * dzx) - dxx - dzz;
            const size_t o  = (size_t)y * N + x;
            __stcs(odx + o, xc);
            __stcs(ody + o, b1);
            __stcs(odz + o, zc);
            __stcs(onj + o, make_float4(nx * rn, rn, nz * rn, 1.0f + dJ));
            a0 = b0; a1 = b1; a2 = b2;
            b0 = d0; b1 = d1; b2 = d2;
            xu = xc; xc = xd;
            zu = zc; zc = zd;
        }
    } else {
        // Epilogue: texel (x0 + c - 1, y), y = tid / 2P + EROWS * k.
        const int r0 = tid / (2 * P);
#pragma unroll 2
        for (int y = r0; y < N; y += FC::EROWS) {
            const int ym = (y - 1) & (N - 1), yq = (y + 1) & (N - 1);
            // taps z0..z7 (normal_map_cs.glsl:37-44) around (x, y)
            const float z0 = EY[cm + ym], z1 = EY[c0 + ym], z2 = EY[cp + ym];
            const float z3 = EY[cm + y], z4 = EY[cp + y];
            const float z5 = EY[cm + yq], z6 = EY[c0 + yq], z7 = EY[cp + yq];
            const float nz = z0 + 2.0f * z1 + z2 - z5 - 2.0f * z6 - z7;
            const float nx = z0 + 2.0f * z3 + z5 - z2 - 2.0f * z4 - z7;
            const float rn = rsqrtf(nx * nx + 1.0f + nz * nz);
            const float dxx = (EX[cp + y] - EX[cm + y]) * inv2d;
            const float dxz = (EX[c0 + yq] - EX[c0 + ym]) * inv2d;
            const float dzx = (EZ[cp + y] - EZ[cm + y]) * inv2d;
            const float dzz = (EZ[c0 + yq] - EZ[c0 + ym]) * inv2d;
            const float dJ  = (dxx * dzz - dxz * dzx) - dxx - dzz;
            const size_t o  = (size_t)y * N + x;
            __stcs(odx + o, EX[c0 + y]);
            __stcs(ody + o, EY[c0 + y]);
            __stcs(odz + o, EZ[c0 + y]);
            __stcs(onj + o, make_float4(nx * rn, rn, nz * rn, 1.0f + dJ));
        }
    }
}

// ---------------------------------------------------------------------------
// Twiddle plans: the row decomposition's, then the column decomposition's.
// ---------------------------------------------------------------------------
template <class C>
__device__ float2 plan_entry(int i)
{
    // segment of entry i (TwPlan): pass 2, 3 or 4 with butterfly stride NS and radix R
    using TP = TwPlan<C>;
    int ns, r;
    if (i < TP::P2) {
        ns = C::R1, r = C::R2;
    } else if (i < TP::P2 + TP::P3) {
        i -= TP::P2, ns = C::R1 * C::R2, r = C::R3;
    } else {
        i -= TP::P2 + TP::P3, ns = C::R1 * C::R2 * C::R3, r = C::R4;
    }
    const long e = (long)(i % ns) * (i / ns) * (C::N / (ns * r));   // exponent of W_N
    double sn, cs;
    sincospi(2.0 * (double)(e % C::N) / (double)C::N, &sn, &cs);
    return make_float2((float)cs, (float)sn);
}

template <int N>
__global__ void k_twiddles(float2* __restrict__ tw)
{
    using LR = typename LineFor<N>::type;
    using LC = typename ColLineFor<N>::type;
    using LV = typename RowLine<N, 2>::type;
    constexpr int A = TwPlan<LR>::LEN, B = A + TwPlan<LC>::LEN, C = B + TwPlan<LV>::LEN;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A) tw[i] = plan_entry<LR>(i);
    else if (i < B) tw[i] = plan_entry<LC>(i - A);
    else if (i < C) tw[i] = plan_entry<LV>(i - B);
}

template <int N>
static size_t twiddle_len_n()
{
    return (size_t)TwPlan<typename LineFor<N>::type>::LEN + TwPlan<typename ColLineFor<N>::type>::LEN +
           TwPlan<typename RowLine<N, 2>::type>::LEN;
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
cudaError_t launch_h0(const H0Args& a, const float* noise, float4* h0, cudaStream_t s)
{
    const int n = a.N * a.N;
    k_h0_init<<<(n + 255) / 256, 256, 0, s>>>(a, noise, h0);
    return cudaGetLastError();
}

cudaError_t launch_spec_combine(int N, int tiles, const float4* h0, int literal_conj, float2* spec, cudaStream_t s)
{
    const int n = N * N + 2 * N;
    k_spec_combine<<<dim3((n + 255) / 256, tiles), 256, 0, s>>>(N, h0, literal_conj, spec);
    return cudaGetLastError();
}

static cudaLaunchAttribute pdl_attr()
{
    cudaLaunchAttribute at;
    at.id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    return at;
}

// Launch `kernel`, as a programmatic dependent of the stream's previous kernel
// when `pdl` (the kernel itself then waits for that kernel with
// griddepcontrol.wait before touching memory).
template <class Args>
static cudaError_t launch_pdl(void (*kernel)(Args), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                              const Args& a)
{
    cudaLaunchAttribute at[1] = {pdl_attr()};
    cudaLaunchConfig_t  cfg   = {};
    cfg.gridDim               = grid;
    cfg.blockDim              = block;
    cfg.dynamicSmemBytes      = smem;
    cfg.stream                = s;
    cfg.attrs                 = at;
    cfg.numAttrs              = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

template <int N, bool MULTI, bool FROM_H0, int V = 0>
static cudaError_t row_pass_nm(const RowArgs& a, cudaStream_t s)
{
    using RC = RowCfg<N, FROM_H0, V>;
    static PerDevice cache;   // resident CTAs per SM on each device, found on its first launch
    int per_sm = 0, grid = 0;
    cudaError_t e = persistent_setup(cache, k_row_pass<N, MULTI, FROM_H0, V>, RC::THREADS, RC::SMEM, &per_sm);
    if (e != cudaSuccess || (e = persistent_grid(per_sm, tuning_for(N).row_ctas_per_sm, &grid)) != cudaSuccess)
        return e;
    const int items = a.tiles * RC::ITEMS;
    if (grid > items) grid = items;
    // one row pair per item, overlapping a fused column stage of the same N:
    // the CTAs on the SMs that stage leaves free prefetch the others' rows
    RowArgs b = a;
    b.prefetch_ctas = 0;
    const Tuning tu = tuning_for(N);
    int sms = 0;
    if (!MULTI && !FROM_H0 && RC::PAIRS == 1 && tu.row_overlap && tu.col_fused && device_sms(&sms) == cudaSuccess) {
        const int free_sms = sms - N / (2 * tu.col_fused);
        if (free_sms > 0) b.prefetch_ctas = free_sms * per_sm < grid ? free_sms * per_sm : grid;
    }
    return launch_pdl(k_row_pass<N, MULTI, FROM_H0, V>, dim3(grid), dim3(RC::THREADS), RC::SMEM, s, true, b);
}

template <int N, bool MULTI, bool FROM_H0, int V = 0>
static cudaError_t row_ws_nm(const RowArgs& a, cudaStream_t s)
{
    using WC = RowWsCfg<N, FROM_H0, V>;
    static PerDevice cache;   // resident CTAs per SM on each device, found on its first launch
    int per_sm = 0, grid = 0;
    cudaError_t e = persistent_setup(cache, k_row_ws<N, MULTI, FROM_H0, V>, WC::THREADS, WC::SMEM, &per_sm);
    if (e != cudaSuccess || (e = persistent_grid(per_sm, tuning_for(N).row_ctas_per_sm, &grid)) != cudaSuccess)
        return e;
    const int items = a.tiles * WC::ITEMS;
    if (grid > items) grid = items;
    // Overlapping a fused column stage of the same N (the previous frame's),
    // the CTAs on the SMs that stage leaves free start first and prefetch the
    // others' rows.
    RowArgs b = a;
    b.prefetch_ctas = 0;
    const Tuning tu = tuning_for(N);
    int sms = 0;
    if (!MULTI && !FROM_H0 && tu.row_overlap && tu.col_fused && device_sms(&sms) == cudaSuccess) {
        const int free_sms = sms - N / (2 * tu.col_fused);
        if (free_sms > 0) b.prefetch_ctas = free_sms * per_sm < grid ? free_sms * per_sm : grid;
    }
    return launch_pdl(k_row_ws<N, MULTI, FROM_H0, V>, dim3(grid), dim3(WC::THREADS), WC::SMEM, s, true, b);
}

template <int N>
static cudaError_t row_pass_n(const RowArgs& a, cudaStream_t s)
{
    const bool single = a.tiles == 1 && a.S == 1 && !a.fcs;
    if (!a.spec && !single) return cudaErrorInvalidValue;    // h0 input: single unit only
    if constexpr (LineFor<N>::type::G >= 32) {                // lines of whole warps: warp-specialised
        if (!a.spec) {
            if constexpr (N <= 1024) return row_ws_nm<N, false, true>(a, s);
            else return cudaErrorInvalidValue;                // its staged h0 rows would not fit
        }
        const int variant = tuning_for(N).row_variant;
        if (variant == 1)                                     // every warp runs the prepass and its line
            return single ? row_pass_nm<N, false, false>(a, s) : row_pass_nm<N, true, false>(a, s);
        if (variant == 2)                                     // warp-specialised, 8-point-first lines
            return single ? row_ws_nm<N, false, false, 2>(a, s) : row_ws_nm<N, true, false, 2>(a, s);
        if constexpr (N == 1024) {
            if (variant == 3)                                 // warp-specialised, 32 x 32 lines
                return single ? row_ws_nm<N, false, false, 3>(a, s) : row_ws_nm<N, true, false, 3>(a, s);
            if (variant == 5)                                 // the same, three CTAs per SM
                return single ? row_ws_nm<N, false, false, 5>(a, s) : row_ws_nm<N, true, false, 5>(a, s);
            if (variant == 4)                                 // every warp, 32 x 32 lines
                return single ? row_pass_nm<N, false, false, 3>(a, s) : row_pass_nm<N, true, false, 3>(a, s);
        }
        return single ? row_ws_nm<N, false, false>(a, s) : row_ws_nm<N, true, false>(a, s);
    } else {
        if (!a.spec) return row_pass_nm<N, false, true>(a, s);
        return single ? row_pass_nm<N, false, false>(a, s) : row_pass_nm<N, true, false>(a, s);
    }
}

template <int N>
static cudaError_t col_fft_n(int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    using CF = ColCfg<N>;
    static PerDevice attr;
    cudaError_t e = smem_setup(attr, k_col_fft<N>, CF::SMEM);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute at[1] = {pdl_attr()};
    cudaLaunchConfig_t  cfg   = {};
    cfg.gridDim               = dim3(CF::CTAS, units);
    cfg.blockDim              = dim3(CF::THREADS);
    cfg.dynamicSmemBytes      = CF::SMEM;
    cfg.stream                = s;
    cfg.attrs                 = at;
    cfg.numAttrs              = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_col_fft<N>, a);
}

template <int N>
static cudaError_t col_out_n(int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    cudaLaunchAttribute at[1] = {pdl_attr()};
    cudaLaunchConfig_t  cfg   = {};
    cfg.gridDim               = dim3(N / kOutT, N / kOutT, units);
    cfg.blockDim              = dim3(kOutTh);
    cfg.stream                = s;
    cfg.attrs                 = at;
    cfg.numAttrs              = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_col_out<N>, a);
}

// The fused column kernel with P column pairs per CTA.
template <int N, int P>
static cudaError_t col_fused_np(int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    using FC = FusedCfg<N, P>;
    static PerDevice attr;
    cudaError_t e = smem_setup(attr, k_col_fused<N, P>, FC::SMEM);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_col_fused<N, P>, dim3(FC::CTAS, units), dim3(FC::THREADS), FC::SMEM, s, pdl, a);
}

template <int N>
static cudaError_t col_fused_n(int pairs, int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    if constexpr (ColLineFor<N>::type::G == 32) {
        if (pairs == 2) return col_fused_np<N, 2>(units, a, s, pdl);
        if (pairs == 4) return col_fused_np<N, 4>(units, a, s, pdl);
    }
    return cudaErrorInvalidValue;                            // lines of more than one warp, or no such shape
}

#define OCEAN_FOR_EACH_N(M) M(32) M(64) M(128) M(256) M(512) M(1024) M(2048)

bool col_fused_available(int N) { return N == 512 || N == 1024; }

cudaError_t launch_col_fused(int N, int pairs, int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    switch (N) {
    case 512: return col_fused_n<512>(pairs, units, a, s, pdl);
    case 1024: return col_fused_n<1024>(pairs, units, a, s, pdl);
    default: return cudaErrorInvalidValue;
    }
}

size_t twiddle_len(int N)
{
    switch (N) {
#define CASE(n) case n: return twiddle_len_n<n>();
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return 0;
    }
}

cudaError_t launch_twiddles(int N, float2* tw, cudaStream_t s)
{
    const size_t n = twiddle_len(N);
    if (!n) return cudaErrorInvalidValue;
    switch (N) {
#define CASE(n_) case n_: k_twiddles<n_><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tw); break;
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s)
{
    switch (N) {
#define CASE(n) case n: return row_pass_n<n>(a, s);
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_col_fft(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    switch (N) {
#define CASE(n) case n: return col_fft_n<n>(units, a, s, pdl);
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_col_out(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    switch (N) {
#define CASE(n) case n: return col_out_n<n>(units, a, s, pdl);
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ocean
