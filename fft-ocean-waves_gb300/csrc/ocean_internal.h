// ocean_internal.h -- kernel launch interface shared by the host code and the
// CUDA translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ocean {

// Per-frame constants computed on the host in double precision.
struct FrameConsts {
    float kt_hi, kt_lo;  // K*t as a double-float, K = sqrt(g/(2*pi*L)): phase in cycles = K*t*m^(1/4)
    float dc_cycles;     // reduced phase (cycles) of the DC mode, whose |k| is floored at 1e-5
};

struct H0Args {
    int N;
    float two_pi_over_L;  // 2*pi/L
    float amplitude;
    float inv_Lp2;        // 1/Lw^2, Lw = V^2/g
    float l2;             // suppression^2
    float wx, wy;         // normalised wind direction
};

struct RowArgs {
    const float4* h0;     // [N][N]
    float2*       inter;  // [3][N/2+1][N]   (Dx, Dy, Dz) half spectra after the row pass
    const float2* tw;     // [N] exp(+2*pi*i*k/N)
    FrameConsts   fc;
    int           literal_conj;
};

struct ColArgs {
    const float2* inter;
    const float2* tw;
    float*        dx;
    float*        dy;
    float*        dz;
    float4*       nj;
    float         scale;   // 0.5/N^2: Hermitian average and inversion_cs.glsl's 1/N^2
    float         lambda;
    float         inv2d;   // N/(2L): central-difference factor
};

cudaError_t launch_h0(const H0Args& a, const float* noise, float4* h0, cudaStream_t s);
cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s);
cudaError_t launch_col_pass(int N, const ColArgs& a, cudaStream_t s);
// Shared memory the two passes need at size N (bytes), for validation.
size_t row_pass_smem(int N);
size_t col_pass_smem(int N);

}  // namespace ocean
