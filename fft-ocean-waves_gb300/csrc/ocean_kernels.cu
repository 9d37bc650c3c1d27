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
template <int N>
struct RowCfg {
    using L = typename LineFor<N>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;  // row pairs per work item
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int ITEMS   = (N / 2 + 1 + PAIRS - 1) / PAIRS;  // work items per tile
    static constexpr int STAGES  = 2;
    // shared memory (float2 units): tw[N] | h0 ring [STAGES][PAIRS][2][N] float4 |
    // work area = max(hy [PAIRS][2][N], line buffers [LINES][NPAD])
    static constexpr size_t RING  = (size_t)STAGES * PAIRS * 2 * N * 2;
    static constexpr size_t HY    = (size_t)PAIRS * 2 * N;
    static constexpr size_t XB    = (size_t)LINES * L::NPAD;
    static constexpr size_t WORK  = HY > XB ? HY : XB;
    static constexpr size_t SMEM  = sizeof(float2) * (N + RING + WORK) + 128;   // + base alignment slack
    static constexpr uint32_t ROW_BYTES = N * sizeof(float4);
};

// Fetch the h0 rows of work item `item` (tile item/ITEMS, row pairs
// (item%ITEMS)*PAIRS ...) into a ring stage with 1-D bulk copies.
template <int N>
__device__ __forceinline__ void row_issue(const RowArgs& a, float4* ring_stage, uint64_t* bar, int item)
{
    using RC = RowCfg<N>;
    const int     tile = item / RC::ITEMS, pi = item % RC::ITEMS;
    const float4* h0t  = a.h0 + (size_t)tile * N * N;
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
        bulk_g2s(ring_stage + (pl * 2 + 0) * N, h0t + (size_t)yp * N, RC::ROW_BYTES, bar);
        bulk_g2s(ring_stage + (pl * 2 + 1) * N, h0t + (size_t)yq * N, RC::ROW_BYTES, bar);
    }
}

// MULTI: more than one (tile, sample) unit per launch (batches).  The single
// unit instantiation keeps the per-element choppy factors out of a runtime
// sample loop, which the compiler would otherwise hoist into registers.
template <int N, bool MULTI>
__global__ void __launch_bounds__(RowCfg<N>::THREADS) k_row_pass(RowArgs a)
{
    using RC = RowCfg<N>;
    using L  = typename RC::L;
    constexpr int NP = inter_pitch(N), H = inter_rows(N);
    extern __shared__ unsigned char smem_raw[];
    float2* smem = align_smem(smem_raw);
    float2* tw_s = smem;
    float4* ring = reinterpret_cast<float4*>(smem + N);              // [STAGES][PAIRS][2][N]
    float2* work = smem + N + RC::RING;                              // hy, then line buffers
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
            if (item < n_items) row_issue<N>(a, ring + (size_t)s * RC::PAIRS * 2 * N, &bars[s], item);
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
        float4* stage = ring + (size_t)s * RC::PAIRS * 2 * N;
        if (!block_wait(&bars[s], (phase_bits >> s) & 1u, &wait_ok, a.status)) return;
        phase_bits ^= 1u << s;
        const int tile = item / RC::ITEMS, pi = item % RC::ITEMS;

        // The staged rows serve every time sample of the tile.
        const int nsmp = MULTI ? a.S : 1;
        for (int smp = 0; smp < nsmp; ++smp) {
            const int         unit = MULTI ? tile * a.S + smp : 0;
            const FrameConsts fc   = MULTI ? a.fcs[unit] : a.fc0;
            // Prepass: h(k,t) for the pair's two rows.  hy[pl][0][x] is the mode
            // (x, y'), hy[pl][1][x] the mode (N-x, N-y').  The four modes (x, y'),
            // (N-x, y'), (N-x, N-y'), (x, N-y') share |k| (ix^2 and iz^2 are
            // even) and so the phase, which is computed once for all four.
            float2* hy = work;
            constexpr int HX = N / 2 + 1;
            for (int i = tid; i < RC::PAIRS * HX; i += RC::THREADS) {
                const int pl = i / HX, x = i % HX;
                const int yp = pi * RC::PAIRS + pl;
                if (yp > N / 2) continue;
                const int xm = (N - x) & (N - 1);
                const int ix = x - N / 2, iz = yp - N / 2;
                float c, sn;
                mode_phase(ix * ix + iz * iz, fc, c, sn);
                const float4* r0  = stage + (pl * 2 + 0) * N;
                const float4* r1  = stage + (pl * 2 + 1) * N;
                float2*       h0r = hy + (pl * 2 + 0) * N;
                float2*       h1r = hy + (pl * 2 + 1) * N;
                h0r[x] = evolve(r0[x], c, sn, fc.literal_conj);
                h1r[x] = evolve(r1[xm], c, sn, fc.literal_conj);
                if (xm != x) {
                    h0r[xm] = evolve(r0[xm], c, sn, fc.literal_conj);
                    h1r[xm] = evolve(r1[x], c, sn, fc.literal_conj);
                }
            }
            __syncthreads();                               // hy complete
            if (smp == nsmp - 1 && tid == 0) {             // ring stage consumed: refill it
                const int next = item + RC::STAGES * gridDim.x;
                if (next < n_items) {
                    fence_proxy_async_smem();
                    row_issue<N>(a, stage, &bars[s], next);
                }
            }

            // Gather the line inputs: 2 * X_H,f(x) = X_f(x) + conj X_f(-x).
            const int  yp     = pi * RC::PAIRS + pl_line;
            const bool active = yp <= N / 2;
            const int  iz = yp - N / 2, izq = ((N - yp) & (N - 1)) - N / 2;
            float2 v[L::E];
#pragma unroll
            for (int r = 0; r < L::E; ++r) {
                const int x = t + r * (N / L::R1);
                float2 hk = active ? hy[(pl_line * 2 + 0) * N + x] : make_float2(0.f, 0.f);
                float2 hq = active ? hy[(pl_line * 2 + 1) * N + x] : make_float2(0.f, 0.f);
                if (f != 1) {
                    // -i (k/|k|) h (tilde_h0_t_cs.glsl:113-126); the DC mode gets 0
                    const int   ix  = x - N / 2;
                    const int   m   = ix * ix + iz * iz;
                    const float rs  = m ? __frsqrt_rn((float)m) : 0.0f;
                    const float fk  = -(float)(f == 0 ? ix : iz) * rs;
                    const float fkq = -(float)(f == 0 ? (((N - x) & (N - 1)) - N / 2) : izq) * rs;
                    hk = make_float2(-fk * hk.y, fk * hk.x);
                    hq = make_float2(-fkq * hq.y, fkq * hq.x);
                }
                v[r] = make_float2(hk.x + hq.x, hk.y - hq.y);
            }
            __syncthreads();                               // hy is read; the line buffers reuse it
            line_fft<L, +1>(v, work + li * L::NPAD, tw_s, t, li);
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
            // the next prepass overwrites `work`: every line has finished
            // reading its buffer
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

template <int N, bool MULTI>
static cudaError_t row_pass_nm(const RowArgs& a, cudaStream_t s)
{
    using RC = RowCfg<N>;
    static int grid = 0;   // persistent grid: resident CTAs per SM x SMs
    if (!grid) {
        cudaError_t e =
            cudaFuncSetAttribute(k_row_pass<N, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RC::SMEM);
        if (e != cudaSuccess) return e;
        int per_sm = 0, dev = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_pass<N, MULTI>, RC::THREADS, RC::SMEM)) !=
            cudaSuccess)
            return e;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        grid = per_sm * sms;
    }
    const int items = a.tiles * RC::ITEMS;
    k_row_pass<N, MULTI><<<grid < items ? grid : items, RC::THREADS, RC::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N>
static cudaError_t row_pass_n(const RowArgs& a, cudaStream_t s)
{
    return (a.tiles == 1 && a.S == 1 && !a.fcs) ? row_pass_nm<N, false>(a, s) : row_pass_nm<N, true>(a, s);
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
#define CASE(n) case n: return RowCfg<n>::SMEM;
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
