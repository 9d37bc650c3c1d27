// ocean_adjoint.cu -- hand-written adjoint of the per-frame ocean update.
//
// Forward (per frame t, field f in {x, y, z}):
//   X_y(k) = h0k(k) e^{iwt} + C(h0minusk(k)) e^{-iwt}     (C = conj, or identity
//   X_x = -i (kx/|k|) X_y,  X_z = -i (kz/|k|) X_y          in literal mode)
//   D_f(x,y) = lambda_f (-1)^(x+y)/N^2 Re sum_k X_f(k) e^{+2 pi i k.x/N}
// For upstream gradients g_f = dL/dD_f (complex convention dL/dRe + i dL/dIm):
//   G_f(k)   = sum_x (-1)^(x+y)/N^2 g_f(x) e^{-2 pi i k.x/N}   forward 2-D DFT:
//              the transpose of the inverse butterfly network and the inversion
//   G_tot(k) = G_y + lambda (i kx/|k| G_x + i kz/|k| G_z)     transpose of the
//              choppy multiply
//   dh0k    += e^{-iwt} G_tot,   dh0minusk += conj(G_tot) e^{-iwt}
//              (literal mode: e^{+iwt} G_tot)                  conjugate phase
//   dlambda += Re(conj(G_x) X_x + conj(G_z) X_z)
// and through the Phillips amplitude a(k) (h0 = xi * a with fixed noise xi):
//   a dL/da = Re(conj(dh0k) h0k + conj(dh0minusk) h0minusk) =: Q(k)
//   dL/dA = sum Q / (2A),  dL/dV = sum Q 2V/(g |k|^2 Lw^3),
//   dL/dtheta = sum Q (k^.w_perp)/(k^.w)          (clamped and DC modes excluded)
//
// Two kernels per chunk of <= 64 frames:
//   k_adj_col_pass  column DFTs of (-1)^(x+y) g / N^2, two real fields packed per
//                   complex transform (gy + i gx per column, gz of two columns),
//                   unpacked with the Hermitian symmetry of real-input DFTs; only
//                   rows ky = 0..N/2 are kept (the rest are conjugates).
//   k_adj_row_pass  one CTA per row pair (ky, N-ky): row DFTs of the three
//                   fields for every frame of the chunk, then the per-mode chain
//                   above for both rows, dh0 accumulated in shared memory across
//                   frames and written (added) once; parameter sums reduced per
//                   CTA and added to four doubles.
// No frame of the forward is stored: only h0 is read.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_line.cuh"
#include "launch_setup.cuh"
#include "ocean_device.cuh"
#include "ocean_internal.h"

namespace ocean {

// ---------------------------------------------------------------------------
// Column pass of the adjoint.
// ---------------------------------------------------------------------------
template <int N>
struct AdjColCfg {
    using L = typename LineFor<N>::type;
    static constexpr int C       = N >= 2048 ? 4 : 8;   // columns per CTA
    static constexpr int WL      = C;                   // gy + i*gx lines
    static constexpr int ZL      = C / 2;               // gz(c) + i*gz(c+1) lines
    static constexpr int LINES   = WL + ZL;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int H       = N / 2 + 1;
    static constexpr int LS      = L::NPAD + 1;         // odd line stride: lines hit distinct banks
    static constexpr int TW      = TwPlan<L>::LEN;
    static constexpr size_t SMEM = sizeof(float2) * (TW + (size_t)LINES * LS);
};

template <int N>
__global__ void __launch_bounds__(AdjColCfg<N>::THREADS) k_adj_col_pass(AdjColArgs a)
{
    using CF = AdjColCfg<N>;
    using L  = typename CF::L;
    constexpr int C = CF::C, H = CF::H, LS = CF::LS, WL = CF::WL, ZL = CF::ZL;
    extern __shared__ float2 smem[];
    float2* tw_s = smem;
    float2* buf  = smem + CF::TW;
    for (int i = threadIdx.x; i < CF::TW; i += CF::THREADS) tw_s[i] = a.tw[i];

    const int    x0 = blockIdx.x * C;
    const size_t NN = (size_t)N * N;
    const size_t fo = (size_t)blockIdx.y * NN;            // this frame's gradients
    // Thread -> (line, t): columns vary fastest across lanes so that each
    // load instruction reads whole 32-byte row segments.
    const int  tid   = threadIdx.x;
    const bool wline = tid < WL * L::G;
    const int  u     = wline ? tid : tid - WL * L::G;
    const int  lane  = wline ? u % WL : u % ZL;
    const int  t     = wline ? u / WL : u / ZL;
    const int  li    = wline ? lane : WL + lane;
    float2 v[L::E];
#pragma unroll
    for (int r = 0; r < L::E; ++r) {
        const int    y   = t + r * (N / L::R1);
        const size_t row = fo + (size_t)y * N;
        if (wline) {
            const int   x  = x0 + lane;
            const float s  = ((x + y) & 1) ? -a.scale : a.scale;
            const float gy = a.gy ? __ldg(a.gy + row + x) : 0.0f;
            const float gx = a.gx ? __ldg(a.gx + row + x) : 0.0f;
            v[r] = make_float2(s * gy, s * gx);
        } else {
            const int   x  = x0 + 2 * lane;                   // even: x and x+1 differ in sign
            const float s  = ((x + y) & 1) ? -a.scale : a.scale;
            float2      gz = a.gz ? __ldg(reinterpret_cast<const float2*>(a.gz + row + x)) : make_float2(0.0f, 0.0f);
            v[r] = make_float2(s * gz.x, -s * gz.y);
        }
    }
    __syncthreads();
    float2* lb = buf + li * LS;
    // columns-fastest lanes put several lines in one warp: block barriers
    line_fft<L, -1, false>(v, lb, tw_s, t, li);
#pragma unroll
    for (int e = 0; e < L::E; ++e) lb[L::pad(LineOut<L>::pos(t, e))] = v[e];
    __syncthreads();

    // Unpack the two real-field spectra of each line: A = Z + conj Z(-k),
    // B = -i (Z - conj Z(-k))  (the 1/2 is in `scale`); keep ky <= N/2.
    float2* out = a.inter + (size_t)blockIdx.y * 3 * H * N;
    for (int i = tid; i < H * WL; i += CF::THREADS) {
        const int c = i % WL, ky = i / WL;
        const float2 z  = buf[c * LS + L::pad(ky)];
        const float2 zm = buf[c * LS + L::pad((N - ky) & (N - 1))];
        out[((size_t)1 * H + ky) * N + x0 + c] = make_float2(z.x + zm.x, z.y - zm.y);   // Dy
        out[((size_t)0 * H + ky) * N + x0 + c] = make_float2(z.y + zm.y, zm.x - z.x);   // Dx
    }
    for (int i = tid; i < H * ZL; i += CF::THREADS) {
        const int p = i % ZL, ky = i / ZL;
        const float2 z  = buf[(WL + p) * LS + L::pad(ky)];
        const float2 zm = buf[(WL + p) * LS + L::pad((N - ky) & (N - 1))];
        *reinterpret_cast<float4*>(out + ((size_t)2 * H + ky) * N + x0 + 2 * p) =
            make_float4(z.x + zm.x, z.y - zm.y, z.y + zm.y, zm.x - z.x);
    }
}

// ---------------------------------------------------------------------------
// Row pass of the adjoint.
// ---------------------------------------------------------------------------
template <int N>
struct AdjRowCfg {
    using L = typename LineFor<N>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int H       = N / 2 + 1;
    static constexpr int LS      = L::NPAD + 1;
    static constexpr int TW      = TwPlan<L>::LEN;
    // twiddle plan | line buffers | h0 rows [PAIRS][2][N] | accumulators [PAIRS][2][N];
    // the float4 arrays start on a 128-byte boundary (LS is odd, LINES may be)
    static constexpr size_t F4OFF = ((size_t)(TW + LINES * LS) + 15) / 16 * 16;   // in float2
    static constexpr size_t SMEM  = sizeof(float2) * F4OFF + sizeof(float4) * 4 * (size_t)PAIRS * N + 128;
    static constexpr int GRID     = (H + PAIRS - 1) / PAIRS;
};

__device__ __forceinline__ double block_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x / 32, nw = (blockDim.x + 31) / 32;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < nw; ++i) s += red[i];
    return s;  // valid in thread 0
}

template <int N>
__global__ void __launch_bounds__(AdjRowCfg<N>::THREADS) k_adj_row_pass(AdjRowArgs a)
{
    using CF = AdjRowCfg<N>;
    using L  = typename CF::L;
    constexpr int H = CF::H, LS = CF::LS, PAIRS = CF::PAIRS;
    extern __shared__ unsigned char smem_raw[];
    float2* smem = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float2* tw_s = smem;
    float2* buf  = smem + CF::TW;
    float4* h0s  = reinterpret_cast<float4*>(smem + CF::F4OFF);          // [PAIRS][2][N], 128-byte aligned
    float4* acc  = h0s + 2 * PAIRS * N;                                // [PAIRS][2][N]
    __shared__ double red[32];

    const int tid = threadIdx.x;
    for (int i = tid; i < CF::TW; i += CF::THREADS) tw_s[i] = a.tw[i];
    for (int i = tid; i < 2 * PAIRS * N; i += CF::THREADS) {
        const int pl = i / (2 * N), side = (i / N) & 1, x = i % N;
        const int yp = blockIdx.x * PAIRS + pl;
        const int y  = side ? ((N - yp) & (N - 1)) : yp;
        h0s[i] = yp < H ? __ldg(a.h0 + (size_t)y * N + x) : make_float4(0.f, 0.f, 0.f, 0.f);
        acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    const int  li = tid / L::G, t = tid % L::G;
    const int  f  = li % 3;
    const int  ypl = blockIdx.x * PAIRS + li / 3;
    const bool lactive = ypl < H;
    double dlam = 0.0;

    for (int j = 0; j < a.T; ++j) {
        float2 v[L::E];
        const float2* in = a.inter + (((size_t)j * 3 + f) * H + (lactive ? ypl : 0)) * N;
#pragma unroll
        for (int r = 0; r < L::E; ++r)
            v[r] = lactive ? __ldg(in + t + r * (N / L::R1)) : make_float2(0.f, 0.f);
        __syncthreads();                                   // previous frame's mode loop is done with buf
        float2* lb = buf + li * LS;
        line_fft<L, -1>(v, lb, tw_s, t, li);
#pragma unroll
        for (int e = 0; e < L::E; ++e) lb[L::pad(LineOut<L>::pos(t, e))] = v[e];
        __syncthreads();

        const FrameConsts fc = a.fc[j];
        for (int i = tid; i < PAIRS * N; i += CF::THREADS) {
            const int pl = i / N, kx = i % N;
            const int yp = blockIdx.x * PAIRS + pl;
            if (yp >= H) continue;
            const int  yq   = (N - yp) & (N - 1);
            const bool self = yq == yp;
            const int  kxq  = (N - kx) & (N - 1);
            const float2 Gx = buf[(3 * pl + 0) * LS + L::pad(kx)];
            const float2 Gy = buf[(3 * pl + 1) * LS + L::pad(kx)];
            const float2 Gz = buf[(3 * pl + 2) * LS + L::pad(kx)];
            const int ix = kx - N / 2, iz = yp - N / 2;
            const int m  = ix * ix + iz * iz;
            float c, s;
            mode_phase(m, fc, c, s);
            const float rs = m ? __frsqrt_rn((float)m) : 0.0f;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                if (side && self) break;
                // mode (kx, yp) or its mirror (kxq, yq), where G(-k) = conj G(k)
                const float  sg  = side ? -1.0f : 1.0f;
                const float2 gx  = make_float2(Gx.x, sg * Gx.y);
                const float2 gy  = make_float2(Gy.x, sg * Gy.y);
                const float2 gz  = make_float2(Gz.x, sg * Gz.y);
                const int    mx  = side ? kxq : kx;
                const float  ux  = (float)(mx - N / 2) * rs;
                const float  uz  = (float)((side ? yq : yp) - N / 2) * rs;
                // G_tot = G_y + lambda (i ux G_x + i uz G_z)
                const float tr = gy.x - a.lambda * (ux * gx.y + uz * gz.y);
                const float ti = gy.y + a.lambda * (ux * gx.x + uz * gz.x);
                float4* ac = acc + (pl * 2 + side) * N + mx;
                float4  A  = *ac;
                A.x += tr * c + ti * s;                      // e^{-iwt} G_tot
                A.y += ti * c - tr * s;
                if (a.literal_conj) {                        // e^{+iwt} G_tot
                    A.z += tr * c - ti * s;
                    A.w += ti * c + tr * s;
                } else {                                     // conj(G_tot) e^{-iwt}
                    A.z += tr * c - ti * s;
                    A.w += -ti * c - tr * s;
                }
                *ac = A;
                // dlambda: Re(conj G_x X_x + conj G_z X_z), X_x = -i ux X_y
                const float2 xy = evolve(h0s[(pl * 2 + side) * N + mx], c, s, a.literal_conj);
                dlam += (double)(gx.x * ux * xy.y - gx.y * ux * xy.x + gz.x * uz * xy.y - gz.y * uz * xy.x);
            }
        }
    }
    __syncthreads();

    // Epilogue: dh0 out, and the chain through a(k) to A, V, theta.
    double dA = 0.0, dV = 0.0, dth = 0.0;
    for (int i = tid; i < 2 * PAIRS * N; i += CF::THREADS) {
        const int pl = i / (2 * N), side = (i / N) & 1, x = i % N;
        const int yp = blockIdx.x * PAIRS + pl;
        if (yp >= H) continue;
        const int y = side ? ((N - yp) & (N - 1)) : yp;
        if (side && y == yp) continue;
        const float4 g = acc[i];
        if (a.dh0) {
            float4* d = a.dh0 + (size_t)y * N + x;
            float4  o = *d;
            *d        = make_float4(o.x + g.x, o.y + g.y, o.z + g.z, o.w + g.w);
        }
        const int ix = x - N / 2, iz = y - N / 2;
        if (ix == 0 && iz == 0) continue;
        const float4 h  = h0s[i];
        const float  Q  = g.x * h.x + g.y * h.y + g.z * h.z + g.w * h.w;   // a dL/da
        const float  kx = a.two_pi_over_L * (float)ix, kz = a.two_pi_over_L * (float)iz;
        const float  k2 = kx * kx + kz * kz;
        const float  rk = rsqrtf(k2);
        const float  cd = (kx * a.wx + kz * a.wy) * rk;
        const float  cp = (-kx * a.wy + kz * a.wx) * rk;
        const float  P  = a.amplitude * expf(-a.inv_Lp2 / k2) * (cd * cd) * expf(-k2 * a.l2) / (k2 * k2);
        const float  amp = sqrtf(P) * 0.70710678118654752f;
        if (!(amp < 4000.0f) || amp == 0.0f) continue;        // clamped, or no dependence
        dA  += (double)Q * a.wA;
        dV  += (double)Q * a.wV / k2;
        dth += (double)Q * cp / cd;
    }
    const double sA = block_sum(dA, red);
    const double sV = block_sum(dV, red);
    const double sT = block_sum(dth, red);
    const double sL = block_sum(dlam, red);
    if (tid == 0) {
        atomicAdd(a.sums + 0, sA);
        atomicAdd(a.sums + 1, sV);
        atomicAdd(a.sums + 2, sT);
        atomicAdd(a.sums + 3, sL);
    }
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int N>
static cudaError_t adj_col_n(int T, const AdjColArgs& a, cudaStream_t s)
{
    using CF = AdjColCfg<N>;
    static PerDevice attr;
    cudaError_t e = smem_setup(attr, k_adj_col_pass<N>, CF::SMEM);
    if (e != cudaSuccess) return e;
    k_adj_col_pass<N><<<dim3(N / CF::C, T), CF::THREADS, CF::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N>
static cudaError_t adj_row_n(const AdjRowArgs& a, cudaStream_t s)
{
    using CF = AdjRowCfg<N>;
    static PerDevice attr;
    cudaError_t e = smem_setup(attr, k_adj_row_pass<N>, CF::SMEM);
    if (e != cudaSuccess) return e;
    k_adj_row_pass<N><<<CF::GRID, CF::THREADS, CF::SMEM, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_adj_col(int N, int T, const AdjColArgs& a, cudaStream_t s)
{
    switch (N) {
    case 32: return adj_col_n<32>(T, a, s);
    case 64: return adj_col_n<64>(T, a, s);
    case 128: return adj_col_n<128>(T, a, s);
    case 256: return adj_col_n<256>(T, a, s);
    case 512: return adj_col_n<512>(T, a, s);
    case 1024: return adj_col_n<1024>(T, a, s);
    case 2048: return adj_col_n<2048>(T, a, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_adj_row(int N, const AdjRowArgs& a, cudaStream_t s)
{
    switch (N) {
    case 32: return adj_row_n<32>(a, s);
    case 64: return adj_row_n<64>(a, s);
    case 128: return adj_row_n<128>(a, s);
    case 256: return adj_row_n<256>(a, s);
    case 512: return adj_row_n<512>(a, s);
    case 1024: return adj_row_n<1024>(a, s);
    case 2048: return adj_row_n<2048>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ocean
