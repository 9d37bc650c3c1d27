// ocean_kernels.cu -- the per-frame Tessendorf ocean update on sm_103a.
//
// One frame is two kernels and two HBM round trips (the reference dispatches
// 6*log2(N)+5 full-grid passes, main.cpp:240-244):
//
//   k_row_pass  spectrum evolution + choppy multiply (tilde_h0_t_cs.glsl:70-131)
//               fused into the horizontal inverse FFT (butterfly_cs.glsl:54-91).
//               Only Re of the 2-D inverse transform is kept
//               (inversion_cs.glsl:35), so each field is first made Hermitian,
//               X_H(k) = (X(k) + conj X(-k))/2, which leaves Re unchanged and
//               makes the row-transformed rows y' and N-y' conjugates: only
//               rows 0..N/2 are transformed and stored.  Persistent CTAs walk
//               the row pairs (y', N-y'); the two h0 rows of the next pairs are
//               fetched with 1-D bulk TMA copies into a two-stage shared-memory
//               ring while the current pair is transformed, and the phase w*t
//               is computed once per mode pair for all three fields.
//
//   k_col_pass  vertical inverse FFT (butterfly_cs.glsl:95-132) on column
//               tiles fetched by 2-D tensor TMA (tile + one neighbour column on
//               each side, thanks to the periodic padding of the
//               intermediate), with two real results packed per complex
//               transform (Dy + i*Dx per column, Dz of two columns), fused with
//               the (-1)^(x+y)/N^2 inversion (inversion_cs.glsl:29-41), lambda
//               scaling, the Sobel normal (normal_map_cs.glsl:37-53) and the
//               Jacobian.  Launched as a programmatic dependent of the row pass
//               so its set-up overlaps the row pass's tail.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_line.cuh"
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

template <int N, bool FROM_H0>
struct RowCfg {
    using L = typename LineFor<N>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;  // row pairs per work item
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int ITEMS   = (N / 2 + 1 + PAIRS - 1) / PAIRS;  // work items per tile
    static constexpr int STAGES  = 2;
    static constexpr int EW      = FROM_H0 ? 2 : 1;   // float2 per staged mode (h0: float4, G: float2)
    // shared memory (float2 units): tw[N] | ring [STAGES][PAIRS][2 rows][N modes] |
    // line buffers [LINES][NPAD] (line inputs in natural order, then the FFT's exchanges)
    static constexpr size_t RING  = (size_t)STAGES * PAIRS * 2 * N * EW;
    static constexpr size_t WORK  = (size_t)LINES * L::NPAD;
    static constexpr size_t SMEM  = sizeof(float2) * (N + RING + WORK) + 128;   // + base alignment slack
    static constexpr uint32_t ROW_BYTES = (uint32_t)(N * EW * sizeof(float2));
};

// Fetch the spectrum rows of work item `item` (tile item/ITEMS, row pairs
// (item%ITEMS)*PAIRS ...) into a ring stage with 1-D bulk copies.
template <int N, bool FROM_H0>
__device__ __forceinline__ void row_issue(const RowArgs& a, float2* ring_stage, uint64_t* bar, int item)
{
    using RC = RowCfg<N, FROM_H0>;
    const int    tile = item / RC::ITEMS, pi = item % RC::ITEMS;
    const float2* src = FROM_H0 ? reinterpret_cast<const float2*>(a.h0 + (size_t)tile * N * N)
                                : a.spec + (size_t)tile * spec_len(N);
    uint32_t bytes = 0;
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
        const float2* sp = a.spec + (size_t)tile * spec_len(N);
        if (x == 0) {                                   // column 0: D(0, yp), D(0, yq)
            d[0] = __ldg(sp + (size_t)N * N + yp);
            d[1] = __ldg(sp + (size_t)N * N + yq);
        }
        if (yp == 0) {                                  // row 0: D(x, 0), D(xm, 0)
            d[0] = __ldg(sp + (size_t)N * N + N + x);
            d[1] = __ldg(sp + (size_t)N * N + N + xm);
            d[2] = d[1];
            d[3] = d[0];
        }
    }
}

// MULTI: more than one (tile, sample) unit per launch (batches).  The single
// unit instantiation keeps the per-element constants out of a runtime sample
// loop, which the compiler would otherwise hoist into registers.  FROM_H0: the
// ring holds h0 rows and G, D are formed on the fly (ocean_update_noalloc).
template <int N, bool MULTI, bool FROM_H0>
__global__ void __launch_bounds__(RowCfg<N, FROM_H0>::THREADS) k_row_pass(RowArgs a)
{
    using RC = RowCfg<N, FROM_H0>;
    using L  = typename RC::L;
    constexpr int NP = inter_pitch(N), H = inter_rows(N);
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* ring = smem + N;                                         // [STAGES][PAIRS][2][N*EW]
    float2* work = smem + N + RC::RING;                              // line buffers
    __shared__ __align__(8) uint64_t bars[RC::STAGES];
    __shared__ int wait_ok;

    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < RC::STAGES; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    for (int i = tid; i < N; i += RC::THREADS) tw_s[i] = a.tw[i];
    __syncthreads();
    const int n_items = a.tiles * RC::ITEMS;
    if (tid == 0)
        for (int s = 0; s < RC::STAGES; ++s) {
            const int item = blockIdx.x + s * gridDim.x;
            if (item < n_items) row_issue<N, FROM_H0>(a, ring + (size_t)s * RC::PAIRS * 2 * N * RC::EW, &bars[s], item);
        }
    // The column pass may start its set-up now; it waits for this grid to finish
    // before it reads the intermediate.
    pdl_launch_dependents();

    const int li = tid / L::G, t = tid % L::G;
    const int f  = li % 3;                                           // 0: Dx, 1: Dy, 2: Dz
    const int pl_line = li / 3;
    uint32_t phase_bits = 0;

    for (int k = 0, item = blockIdx.x; item < n_items; ++k, item += gridDim.x) {
        const int s = k & 1;
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
            for (int i = tid; i < RC::PAIRS * HX; i += RC::THREADS) {
                const int pl = i / HX, x = i - pl * HX;
                const int yp = pi * RC::PAIRS + pl;
                if (yp > N / 2) continue;
                const int yq = (N - yp) & (N - 1), xm = (N - x) & (N - 1);
                const int ix = x - N / 2, iz = yp - N / 2;
                float c, sn, r;
                mode_phase_r(ix * ix + iz * iz, fc, c, sn, r);
                float2 g[4], d[4];
                const float2* rA = stage + (pl * 2 + 0) * N * RC::EW;
                const float2* rB = stage + (pl * 2 + 1) * N * RC::EW;
                row_modes<N, FROM_H0>(a, rA, rB, tile, x, xm, yp, yq, fc.literal_conj, g, d);
                const float2 y0 = herm_sum(g[0], g[1], c, sn);
                const float2 y1 = herm_sum(g[2], g[3], c, sn);
                float2 ux0 = y0, uz0 = y0, uz1 = y1;
                if (x == 0) ux0 = herm_diff(d[0], d[1], c, sn);
                if (yp == 0) {
                    uz0 = herm_diff(d[0], d[1], c, sn);
                    uz1 = herm_diff(d[2], d[3], c, sn);
                }
                const float sx = (float)ix * r, sz = (float)iz * r;
                float2* bx = work + (pl * 3 + 0) * L::NPAD;
                float2* by = bx + L::NPAD;
                float2* bz = by + L::NPAD;
                bx[x] = mul_mi(sx, ux0);
                by[x] = y0;
                bz[x] = mul_mi(sz, uz0);
                if (xm != x) {                        // ix(xm) = -ix for x != 0
                    bx[xm] = mul_mi(-sx, y1);
                    by[xm] = y1;
                    bz[xm] = mul_mi(sz, uz1);
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
            line_fft<L, +1>(v, buf, tw_s, t, li);
            if (active) {
                float2* out = a.inter + (((size_t)unit * 3 + f) * H + yp) * NP;
#pragma unroll
                for (int e = 0; e < L::E; ++e) out[LineOut<L>::pos(t, e) + 1] = v[e];
                // periodic pad columns: x = 0 is thread 0's first output and
                // x = N-1 the last thread's last one
                static_assert(LineOut<L>::pos(0, 0) == 0 && LineOut<L>::pos(L::G - 1, L::E - 1) == N - 1, "pad");
                if (t == 0) out[N + 1] = v[0];
                if (t == L::G - 1) out[0] = v[L::E - 1];
            }
            // the next inputs overwrite the line buffers: every line has
            // finished reading its own
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Column pass.
// ---------------------------------------------------------------------------
constexpr int ceil8(int x) { return (x + 7) / 8 * 8; }
constexpr int imax(int a, int b) { return a > b ? a : b; }

// Column-pass line decomposition: as LineFor except at N = 2048, where the
// column CTA's 6 lines x 64 threads (32-point first pass) keep 168 registers
// per thread without spilling (16-point lines would need 768 threads).
template <int N> struct ColLineFor { using type = typename LineFor<N>::type; };
template <> struct ColLineFor<2048> { using type = LineCfg<2048, 32, 8, 8>; };

template <int N>
struct ColCfg {
    using L = typename ColLineFor<N>::type;
    static constexpr int C       = N >= 2048 ? 4 : 8;   // output columns per CTA
    static constexpr int CC      = C + 2;               // + one neighbour column each side
    static constexpr int WL      = CC;                  // round 1: Dy + i*Dx lines, one per column
    static constexpr int ZL      = CC / 2;              // round 2: Dz(c) + i*Dz(c+1) lines
    static constexpr int THREADS = WL * L::G;
    static constexpr int H       = inter_rows(N);
    // Staged rows per field: at least H, and at least half a line buffer so
    // that a round's exchange buffers fit in the tile fields it has consumed.
    static constexpr int HP0     = imax(H, (L::NPAD + 1) / 2);
    static constexpr int NCHUNK  = (HP0 + 255) / 256;   // TMA boxes per field (<= 256 rows)
    static constexpr int BR      = ceil8((HP0 + NCHUNK - 1) / NCHUNK);   // 128-byte aligned boxes
    static constexpr int HP      = NCHUNK * BR;
    static constexpr int OS      = N + 4;               // staging column stride (floats)
    static constexpr size_t FIELD = (size_t)HP * CC;    // float2 per tile field
    static constexpr size_t SMEM = sizeof(float2) * (N + 3 * FIELD) + 128;   // + base alignment slack
    static constexpr int GRID    = N / C;
    static constexpr uint32_t TILE_BYTES = (uint32_t)(sizeof(float2) * 3 * FIELD);
    static_assert((size_t)WL * L::NPAD <= 2 * FIELD && (size_t)ZL * L::NPAD <= FIELD, "exchange buffers");
    static_assert((size_t)CC * OS <= 2 * FIELD, "staging");
};

template <int N>
__global__ void __launch_bounds__(ColCfg<N>::THREADS) k_col_pass(const __grid_constant__ ColArgs a)
{
    using CF = ColCfg<N>;
    using L  = typename CF::L;
    constexpr int C = CF::C, CC = CF::CC, H = CF::H, OS = CF::OS, ZL = CF::ZL;
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float2* tile = smem + N;                                 // [3][HP][CC]: Dx, Dy, Dz (TMA boxes)
    // round buffers and staging alias the tile fields once they are consumed
    float2* xbuf1 = tile;                                    // round 1 exchange: fields Dx, Dy
    float2* xbuf2 = tile + 2 * CF::FIELD;                    // round 2 exchange: field Dz
    float*  sx = reinterpret_cast<float*>(tile);             // staged Dx [CC][OS]
    float*  sy = reinterpret_cast<float*>(tile + CF::FIELD); // staged Dy
    float*  sz = reinterpret_cast<float*>(tile + 2 * CF::FIELD);
    __shared__ __align__(8) uint64_t bar;
    __shared__ int wait_ok;
    const int x0   = blockIdx.x * C;
    const int unit = blockIdx.y;
    const int tid  = threadIdx.x;
    // read the unit's fields where they are used (a struct copy would stay
    // live in registers across the FFTs)
    const ColUnit* cu = a.units ? a.units + unit : &a.u0;

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        asm volatile("prefetch.tensormap [%0];" ::"l"(&a.map) : "memory");
    }
    for (int i = tid; i < N; i += CF::THREADS) tw_s[i] = a.tw[i];
    pdl_wait_prior();                                        // the row pass has finished
    __syncthreads();
    if (tid == 0) {
        // Columns x0-1 .. x0+C are padded columns x0 .. x0+C+1 of the intermediate.
        mbar_arrive_expect_tx(&bar, CF::TILE_BYTES);
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int q = 0; q < CF::NCHUNK; ++q)
                tma_load_2d(tile + f * CF::FIELD + (size_t)q * CF::BR * CC, &a.map, 2 * x0,
                            (unit * 3 + f) * H + q * CF::BR, &bar);
    }
    if (!block_wait(&bar, 0, &wait_ok, a.status)) return;

    float2 v[L::E];
    // ---- round 1: column lines Dy + i*Dx, one line per G consecutive threads
    // (a warp never spans two lines' exchange buffers).
    {
        const int cc = tid / L::G, t = tid % L::G;
#pragma unroll
        for (int r = 0; r < L::E; ++r) {
            const int  y  = t + r * (N / L::R1);
            const bool lo = y <= N / 2;
            const int  ys = lo ? y : N - y;                  // rows N-y are conjugates of rows y
            float2 p = tile[CF::FIELD + ys * CC + cc];       // Dy
            float2 q = tile[ys * CC + cc];                   // Dx
            if (!lo) { p.y = -p.y; q.y = -q.y; }
            v[r] = make_float2(p.x - q.y, p.y + q.x);        // p + i*q
        }
        __syncthreads();                                     // fields Dx, Dy consumed
        line_fft<L, +1>(v, xbuf1 + cc * L::NPAD, tw_s, t, cc);
        __syncthreads();                                     // every line done with xbuf1
        const int   xa = x0 - 1 + cc;                        // parity is all that matters
        const float sa = cu->scale, sb = cu->scale * cu->lambda;
#pragma unroll
        for (int e = 0; e < L::E; ++e) {
            const int   y  = LineOut<L>::pos(t, e);
            const float sg = ((xa + y) & 1) ? -1.0f : 1.0f;
            sy[cc * OS + y] = sg * sa * v[e].x;
            sx[cc * OS + y] = sg * sb * v[e].y;
        }
    }
    // ---- round 2: Dz(c) + i*Dz(c+1) lines on the first ZL*G threads.
    {
        const bool zact = tid < ZL * L::G;
        const int  p2 = tid / L::G, t = tid % L::G;
        if (zact) {
#pragma unroll
            for (int r = 0; r < L::E; ++r) {
                const int  y  = t + r * (N / L::R1);
                const bool lo = y <= N / 2;
                const int  ys = lo ? y : N - y;
                const float4 z2 = *reinterpret_cast<const float4*>(tile + 2 * CF::FIELD + ys * CC + 2 * p2);
                float2 p = make_float2(z2.x, z2.y), q = make_float2(z2.z, z2.w);
                if (!lo) { p.y = -p.y; q.y = -q.y; }
                v[r] = make_float2(p.x - q.y, p.y + q.x);
            }
        }
        __syncthreads();                                     // field Dz consumed
        if (zact || L::G < 32) line_fft<L, +1>(v, xbuf2 + (zact ? p2 : 0) * L::NPAD, tw_s, t, zact ? p2 : 0, zact);
        __syncthreads();                                     // every line done with xbuf2
        if (zact) {
            const int   xa = x0 - 1 + 2 * p2;
            const float sb = cu->scale * cu->lambda;
#pragma unroll
            for (int e = 0; e < L::E; ++e) {
                const int   y  = LineOut<L>::pos(t, e);
                const float sg = ((xa + y) & 1) ? -1.0f : 1.0f;
                sz[(2 * p2) * OS + y]     = sg * sb * v[e].x;
                sz[(2 * p2 + 1) * OS + y] = -sg * sb * v[e].y;
            }
        }
    }
    __syncthreads();

    // Epilogue: a 4-row x 2-column block per thread (float4 shared reads down
    // the staged columns, float2 global stores across them); Sobel normal on Dy
    // and the Jacobian of x - (Dx, Dz).
    float* const  odx = cu->dx;
    float* const  ody = cu->dy;
    float* const  odz = cu->dz;
    float4* const onj = cu->nj;
    const float   inv2d = cu->inv2d;
    for (int i = tid; i < (C / 2) * (N / 4); i += CF::THREADS) {
        const int cp = i % (C / 2), y0 = 4 * (i / (C / 2));
        const int cb = 2 * cp + 1;                                // staged column of output column 2cp
        const int ym = (y0 - 1) & (N - 1), yn = (y0 + 4) & (N - 1);
        // Y[d][k]: Dy at staged column cb-1+d, rows y0-1+k (d < 4, k < 6)
        float Y[4][6], X[2][6], Z[2][6], XS[2][4], ZS[2][4];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const float* col = sy + (cb - 1 + d) * OS;
            const float4 m4 = *reinterpret_cast<const float4*>(col + y0);
            Y[d][0] = col[ym]; Y[d][1] = m4.x; Y[d][2] = m4.y; Y[d][3] = m4.z; Y[d][4] = m4.w; Y[d][5] = col[yn];
        }
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            const float* cx = sx + (cb + d) * OS;
            const float4 mx = *reinterpret_cast<const float4*>(cx + y0);
            X[d][0] = cx[ym]; X[d][1] = mx.x; X[d][2] = mx.y; X[d][3] = mx.z; X[d][4] = mx.w; X[d][5] = cx[yn];
            const float* cz = sz + (cb + d) * OS;
            const float4 mz = *reinterpret_cast<const float4*>(cz + y0);
            Z[d][0] = cz[ym]; Z[d][1] = mz.x; Z[d][2] = mz.y; Z[d][3] = mz.z; Z[d][4] = mz.w; Z[d][5] = cz[yn];
            // the outer x-neighbours: staged columns cb-1 (d = 0) and cb+2 (d = 1)
            const float4 ox = *reinterpret_cast<const float4*>(sx + (cb - 1 + 3 * d) * OS + y0);
            const float4 oz = *reinterpret_cast<const float4*>(sz + (cb - 1 + 3 * d) * OS + y0);
            XS[d][0] = ox.x; XS[d][1] = ox.y; XS[d][2] = ox.z; XS[d][3] = ox.w;
            ZS[d][0] = oz.x; ZS[d][1] = oz.y; ZS[d][2] = oz.z; ZS[d][3] = oz.w;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float4 njv[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                // taps z0..z7 (normal_map_cs.glsl:37-44) around (column d, row k+1)
                const float z0 = Y[d][k], z1 = Y[d + 1][k], z2 = Y[d + 2][k];
                const float z3 = Y[d][k + 1], z4 = Y[d + 2][k + 1];
                const float z5 = Y[d][k + 2], z6 = Y[d + 1][k + 2], z7 = Y[d + 2][k + 2];
                const float nz = z0 + 2.0f * z1 + z2 - z5 - 2.0f * z6 - z7;
                const float nx = z0 + 2.0f * z3 + z5 - z2 - 2.0f * z4 - z7;
                const float rn = rsqrtf(nx * nx + 1.0f + nz * nz);
                const float xl = d == 0 ? XS[0][k] : X[0][k + 1], xr = d == 0 ? X[1][k + 1] : XS[1][k];
                const float zl = d == 0 ? ZS[0][k] : Z[0][k + 1], zr = d == 0 ? Z[1][k + 1] : ZS[1][k];
                const float dxx = (xr - xl) * inv2d;
                const float dxz = (X[d][k + 2] - X[d][k]) * inv2d;
                const float dzx = (zr - zl) * inv2d;
                const float dzz = (Z[d][k + 2] - Z[d][k]) * inv2d;
                // J = (1 - dxx)(1 - dzz) - dxz*dzx, formed as 1 + deviation so that
                // the only rounding at the scale of 1 is the final add
                const float dJ = (dxx * dzz - dxz * dzx) - dxx - dzz;
                njv[d] = make_float4(nx * rn, rn, nz * rn, 1.0f + dJ);
            }
            const size_t o = (size_t)(y0 + k) * N + x0 + 2 * cp;
            *reinterpret_cast<float2*>(odx + o) = make_float2(X[0][k + 1], X[1][k + 1]);
            *reinterpret_cast<float2*>(ody + o) = make_float2(Y[1][k + 1], Y[2][k + 1]);
            *reinterpret_cast<float2*>(odz + o) = make_float2(Z[0][k + 1], Z[1][k + 1]);
            onj[o]     = njv[0];
            onj[o + 1] = njv[1];
        }
    }
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

template <int N, bool MULTI, bool FROM_H0>
static cudaError_t row_pass_nm(const RowArgs& a, cudaStream_t s)
{
    using RC = RowCfg<N, FROM_H0>;
    static int grid = 0;   // persistent grid: resident CTAs per SM x SMs
    if (!grid) {
        cudaError_t e = cudaFuncSetAttribute(k_row_pass<N, MULTI, FROM_H0>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RC::SMEM);
        if (e != cudaSuccess) return e;
        int per_sm = 0, dev = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_pass<N, MULTI, FROM_H0>, RC::THREADS,
                                                                RC::SMEM)) != cudaSuccess)
            return e;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        grid = per_sm * sms;
    }
    const int items = a.tiles * RC::ITEMS;
    k_row_pass<N, MULTI, FROM_H0><<<grid < items ? grid : items, RC::THREADS, RC::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N>
static cudaError_t row_pass_n(const RowArgs& a, cudaStream_t s)
{
    if (!a.spec) {   // h0 input: single unit only
        if (a.tiles != 1 || a.S != 1 || a.fcs) return cudaErrorInvalidValue;
        return row_pass_nm<N, false, true>(a, s);
    }
    return (a.tiles == 1 && a.S == 1 && !a.fcs) ? row_pass_nm<N, false, false>(a, s)
                                                : row_pass_nm<N, true, false>(a, s);
}

template <int N>
static cudaError_t col_pass_n(int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    using CF = ColCfg<N>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_col_pass<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim          = dim3(CF::GRID, units);
    cfg.blockDim         = dim3(CF::THREADS);
    cfg.dynamicSmemBytes = CF::SMEM;
    cfg.stream           = s;
    cudaLaunchAttribute at[1];
    at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs    = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_col_pass<N>, a);
}

template <int N>
static void col_box_n(unsigned box[2])
{
    box[0] = 2 * ColCfg<N>::CC;
    box[1] = ColCfg<N>::BR;
}

#define OCEAN_FOR_EACH_N(M) M(32) M(64) M(128) M(256) M(512) M(1024) M(2048)

cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s)
{
    switch (N) {
#define CASE(n) case n: return row_pass_n<n>(a, s);
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_col_pass(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl)
{
    switch (N) {
#define CASE(n) case n: return col_pass_n<n>(units, a, s, pdl);
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
    }
}

void col_pass_box(int N, unsigned box[2])
{
    box[0] = box[1] = 0;
    switch (N) {
#define CASE(n) case n: col_box_n<n>(box); break;
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: break;
    }
}

size_t row_pass_smem(int N)
{
    switch (N) {
#define CASE(n) case n: return RowCfg<n, true>::SMEM;
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return 0;
    }
}

size_t col_pass_smem(int N)
{
    switch (N) {
#define CASE(n) case n: return ColCfg<n>::SMEM;
        OCEAN_FOR_EACH_N(CASE)
#undef CASE
    default: return 0;
    }
}

}  // namespace ocean
