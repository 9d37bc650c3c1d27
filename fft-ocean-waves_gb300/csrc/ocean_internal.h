// ocean_internal.h -- kernel launch interface shared by the host code and the
// CUDA translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ocean {

// Per-frame constants of one (tile, time sample), computed on the host in
// double precision.
struct FrameConsts {
    float kt_hi, kt_lo;  // K*t as a double-float, K = sqrt(g/(2*pi*L)): phase in cycles = K*t*m^(1/4)
    float dc_cycles;     // reduced phase (cycles) of the DC mode, whose |k| is floored at 1e-5
    int   literal_conj;  // the tile's OCEAN_FLAG_LITERAL_CONJ
};

// Column-pass epilogue parameters and outputs of one (tile, time sample).
struct ColUnit {
    float*  dx;
    float*  dy;
    float*  dz;
    float4* nj;
    float   scale;   // 0.5/N^2: Hermitian average and inversion_cs.glsl's 1/N^2
    float   lambda;
    float   inv2d;   // N/(2L): central-difference factor
    float   pad_;
};

struct H0Args {
    int N;
    float two_pi_over_L;  // 2*pi/L
    float amplitude;
    float inv_Lp2;        // 1/Lw^2, Lw = V^2/g
    float l2;             // suppression^2
    float wx, wy;         // normalised wind direction
};

// Row-pass output ("intermediate"): three fields (Dx, Dy, Dz) of rows
// y' = 0..N/2 of the row-transformed Hermitian spectra, blocked by column pair
// so that the column transforms of a pair read one contiguous run:
// [3 fields][N/2 column pairs][N/2+1 rows][2 columns] complex.
__host__ __device__ constexpr int inter_rows(int N) { return N / 2 + 1; }
__host__ __device__ constexpr size_t inter_len(int N) { return 3 * (size_t)inter_rows(N) * N; }
__host__ __device__ constexpr size_t inter_index(int N, int f, int x, int y)
{
    return (((size_t)f * (N / 2) + (x >> 1)) * inter_rows(N) + y) * 2 + (x & 1);
}
// Column-FFT output ("transposed maps"): the final Dx, Dy, Dz of one unit,
// [3][N (x)][N (y)] floats, column-major so that each column transform writes
// one contiguous run; the output kernel transposes them.
__host__ __device__ constexpr size_t tmap_len(int N) { return 3 * (size_t)N * N; }

// Combined spectrum read by the row pass, per tile: G[N][N] (G(k) = h0k(k) +
// sigma(h0m(-k))), then D of column 0 [N], then D of row 0 [N]
// (D(k) = h0k(k) - sigma(h0m(-k))); sigma = conj, or the identity under
// OCEAN_FLAG_LITERAL_CONJ.
__host__ __device__ constexpr size_t spec_len(int N) { return (size_t)N * N + 2 * (size_t)N; }

// A launch covers `tiles` tiles of the same N, each advanced to S time
// samples: unit u = tile*S + s.  The spectrum of tile t is spec + t*spec_len(N)
// or, with spec NULL (single unit only), it is formed on the fly from h0
// ([N][N] float4 (h0k, h0m)).  The intermediate of unit u starts at
// inter + u*inter_len(N).  Per-unit constants come from `fcs` (device,
// [tiles*S]) or, for a single unit, from `fc0`.  The row pass is launched as
// a programmatic dependent of the stream's previous kernel (wait_first).
struct RowArgs {
    const float2*      spec;
    const float4*      h0;
    float2*            inter;
    const float2*      tw;      // twiddle plans (launch_twiddles)
    unsigned*          status;  // device status word (bounded-wait time-outs)
    const FrameConsts* fcs;
    FrameConsts        fc0;
    int                tiles, S;
    // 1: wait for the stream's previous kernel before reading anything (it
    // may have written the spectrum, h0 or the twiddle plans); 0: the row pass
    // may overlap that kernel and waits for it only at its end.
    int                wait_first;
    // single unit, warp-specialised pass: CTAs 0..prefetch_ctas-1 prefetch the
    // other CTAs' spectrum rows into L2 (0: none); set by the launcher
    int                prefetch_ctas;
};

// Column side of a frame: k_col_fft (column transforms, intermediate ->
// transposed maps) then k_col_out (transpose, Sobel normal, Jacobian ->
// caller's outputs).  Unit u reads inter + u*inter_len(N) and uses
// tmap + u*tmap_len(N).
struct ColArgs {
    const float2*  inter;
    float*         tmap;
    unsigned*      status;
    const float2*  tw;
    const ColUnit* units;   // device [units], or NULL: u0 for the single unit
    ColUnit        u0;
    // k_col_out lets the stream's next kernel (the next frame's row pass,
    // when it overlaps) launch as soon as it has started
    int            trigger_next;
};

// ---------------------------------------------------------------------------
// Adjoint (ocean_backward)
// ---------------------------------------------------------------------------
constexpr int kMaxChunkFrames = 64;   // frames per adjoint launch pair

struct AdjColArgs {
    const float* gx;  // upstream dL/dDx of the chunk's first frame, [T][N][N]; NULL = 0
    const float* gy;
    const float* gz;
    float2*      inter;  // [T][3][N/2+1][N]: column-transformed gradients, rows 0..N/2
    const float2* tw;
    float        scale;  // 0.5/N^2: (-1)^(x+y)/N^2 of the inversion and the unpacking 1/2
};

struct AdjRowArgs {
    const float2* inter;
    const float4* h0;
    const float2* tw;
    float4*       dh0;   // dL/dh0 accumulator [N][N] (added to); NULL = not wanted
    double*       sums;  // [4]: dA, dV, dtheta, dlambda (atomically added to)
    int           T;
    int           literal_conj;
    float         lambda;
    float         two_pi_over_L, amplitude, inv_Lp2, l2, wx, wy;  // to re-derive a(k) and its clamp
    float         wA;    // 1/(2A)
    float         wV;    // 2V/(g Lw^3); dV weight is wV/|k|^2
    FrameConsts   fc[kMaxChunkFrames];
};

// Launch configuration of size N (ocean_tuning of include/ocean.h): the
// compiled-in table (tuning_table.inc, written by tune.py) unless
// ocean_set_tuning replaced it.
struct Tuning {
    int row_overlap;       // the row pass overlaps the stream's previous kernel
    int row_ctas_per_sm;   // persistent row-pass CTAs per SM, 0 = as many as fit
    int wave_mib;          // batch wave scratch budget, MiB
    int col_fused;         // 0, or the fused column kernel's column pairs per CTA (2, 4)
    int row_variant;       // N >= 512: 0 k_row_ws, 1 every warp (k_row_pass), 2 k_row_ws with 8-point-first
                           // lines, 3 (N = 1024) k_row_ws with 32 x 32 lines, 4 (N = 1024) k_row_pass
                           // with 32 x 32 lines, 5 (N = 1024) k_row_ws with 32 x 32 lines, one stage
                           // and one buffer set, three CTAs per SM
};
Tuning tuning_for(int N);

cudaError_t launch_adj_col(int N, int T, const AdjColArgs& a, cudaStream_t s);
cudaError_t launch_adj_row(int N, const AdjRowArgs& a, cudaStream_t s);

cudaError_t launch_h0(const H0Args& a, const float* noise, float4* h0, cudaStream_t s);
// The twiddle plans of size N (row decomposition, then column decomposition;
// TwPlan in fft_line.cuh): twiddle_len(N) complex values.
size_t      twiddle_len(int N);
cudaError_t launch_twiddles(int N, float2* tw, cudaStream_t s);
cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s);
// spec[t] from h0[t] for `tiles` consecutive tiles of size N.
cudaError_t launch_spec_combine(int N, int tiles, const float4* h0, int literal_conj, float2* spec, cudaStream_t s);
// k_col_fft / k_col_out for `units` units; pdl: launch as a programmatic
// dependent of the preceding kernel in `s`.
cudaError_t launch_col_fft(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl);
cudaError_t launch_col_out(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl);
// k_col_fused (both column stages in one kernel; no column maps) with `pairs`
// (2 or 4) column pairs per CTA: sizes whose column lines are one warp
// (N = 512, 1024).
bool        col_fused_available(int N);
cudaError_t launch_col_fused(int N, int pairs, int units, const ColArgs& a, cudaStream_t s, bool pdl);

}  // namespace ocean
