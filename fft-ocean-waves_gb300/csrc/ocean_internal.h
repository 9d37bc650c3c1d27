// ocean_internal.h -- kernel launch interface shared by the host code and the
// CUDA translation units.  Not part of the public ABI.
#pragma once
#include <cuda.h>
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
// y' = 0..N/2 of the row-transformed Hermitian spectra.  Each row holds N+2
// complex values: padded column p = x + 1 for x = -1..N, with x = -1 and x = N
// the periodic copies of x = N-1 and x = 0, so that any column tile together
// with its two neighbour columns is one contiguous 16-byte-aligned box.
__host__ __device__ constexpr int inter_pitch(int N) { return N + 2; }
__host__ __device__ constexpr int inter_rows(int N) { return N / 2 + 1; }

// Combined spectrum read by the row pass, per tile: G[N][N] (G(k) = h0k(k) +
// sigma(h0m(-k))), then D of column 0 [N], then D of row 0 [N]
// (D(k) = h0k(k) - sigma(h0m(-k))); sigma = conj, or the identity under
// OCEAN_FLAG_LITERAL_CONJ.
__host__ __device__ constexpr size_t spec_len(int N) { return (size_t)N * N + 2 * (size_t)N; }

// A launch covers `tiles` tiles of the same N, each advanced to S time
// samples: unit u = tile*S + s.  The spectrum of tile t is spec + t*spec_len(N)
// or, with spec NULL (single unit only), it is formed on the fly from h0
// ([N][N] float4 (h0k, h0m)).  The intermediate of unit u starts at
// inter + u*3*(N/2+1)*(N+2).  Per-unit constants come from `fcs` (device,
// [tiles*S]) or, for a single unit, from `fc0`.
struct RowArgs {
    const float2*      spec;
    const float4*      h0;
    float2*            inter;
    const float2*      tw;      // [N] exp(+2*pi*i*k/N)
    unsigned*          status;  // device status word (bounded-wait time-outs)
    const FrameConsts* fcs;
    FrameConsts        fc0;
    int                tiles, S;
};

struct ColArgs {
    CUtensorMap    map;     // 2-D tensor map over inter: floats [units*3*(N/2+1)][2*(N+2)]
    unsigned*      status;
    const float2*  tw;
    const ColUnit* units;   // device [units], or NULL: u0 for the single unit
    ColUnit        u0;
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

cudaError_t launch_adj_col(int N, int T, const AdjColArgs& a, cudaStream_t s);
cudaError_t launch_adj_row(int N, const AdjRowArgs& a, cudaStream_t s);

cudaError_t launch_h0(const H0Args& a, const float* noise, float4* h0, cudaStream_t s);
cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s);
// spec[t] from h0[t] for `tiles` consecutive tiles of size N.
cudaError_t launch_spec_combine(int N, int tiles, const float4* h0, int literal_conj, float2* spec, cudaStream_t s);
// pdl: launch as a programmatic dependent of the preceding kernel in `s`.
cudaError_t launch_col_pass(int N, int units, const ColArgs& a, cudaStream_t s, bool pdl);
// Box of the column-pass tensor map at size N: {inner floats, rows}.
void col_pass_box(int N, unsigned box[2]);
// Shared memory the two passes need at size N (bytes), for validation.
size_t row_pass_smem(int N);
size_t col_pass_smem(int N);

}  // namespace ocean
