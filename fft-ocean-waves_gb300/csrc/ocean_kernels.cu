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
//               rows 0..N/2 are transformed and stored.  A CTA owns the row
//               pair (y', N-y'), reads each h0 mode once and shares one phase
//               w*t per mode pair.
//
//   k_col_pass  vertical inverse FFT (butterfly_cs.glsl:95-132) on column
//               tiles staged in shared memory, with two real results packed
//               per complex transform (Dy + i*Dx per column, Dz of two
//               columns), fused with the (-1)^(x+y)/N^2 inversion
//               (inversion_cs.glsl:29-41), lambda scaling, the Sobel normal
//               (normal_map_cs.glsl:37-53) and the Jacobian.  Each tile also
//               transforms the two neighbouring columns it needs for the
//               stencils.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_line.cuh"
#include "ocean_internal.h"

namespace ocean {

// ---------------------------------------------------------------------------
// Phase w*t in double-float arithmetic.
// w = sqrt(g*|k|), |k| = (2*pi/L)*sqrt(m), m = ix^2 + iz^2 (exact integer), so
// w*t/(2*pi) = K*t*m^(1/4) with K = sqrt(g/(2*pi*L)).  K*t comes from the host
// as a double-float; m^(1/4) is formed by two double-float square roots
// (Dekker 1971: one Newton correction on the FP32 root with an exact FMA
// residual) and the product by Dekker's two-product via FMA.  The integer
// number of cycles is dropped before sincospi, so the reduced phase keeps
// ~1e-7 absolute accuracy at any t the double can carry.
// ---------------------------------------------------------------------------
struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl df_sqrt_int(float a)  // a >= 1, an exact integer
{
    float s = __fsqrt_rn(a);
    float e = __fmaf_rn(-s, s, a);
    return {s, __fmul_rn(e, 0.5f * __frcp_rn(s))};
}

__device__ __forceinline__ dfl df_sqrt(dfl a)
{
    float s = __fsqrt_rn(a.hi);
    float e = __fadd_rn(__fmaf_rn(-s, s, a.hi), a.lo);
    float c = __fmul_rn(e, 0.5f * __frcp_rn(s));
    float r = __fadd_rn(s, c);
    return {r, __fadd_rn(c, -__fadd_rn(r, -s))};
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e       = __fmaf_rn(a.hi, b.lo, e);
    e       = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
}

// cos/sin of the phase of mode m (m = ix^2 + iz^2) at the frame's time.
__device__ __forceinline__ void mode_phase(int m, const FrameConsts& fc, float& c, float& s)
{
    float f;
    if (m == 0) {
        f = fc.dc_cycles;
    } else {
        dfl q   = df_sqrt(df_sqrt_int((float)m));
        dfl cyc = df_mul(dfl{fc.kt_hi, fc.kt_lo}, q);
        float n = rintf(cyc.hi);
        f       = __fadd_rn(__fadd_rn(cyc.hi, -n), cyc.lo);
        f       = __fadd_rn(f, -rintf(f));
    }
    sincospif(2.0f * f, &s, &c);
}

// h(k,t) = h0(k) e^{iwt} + conj(h0(-k)) e^{-iwt} (tilde_h0_t_cs.glsl:110);
// literal_conj reproduces the shader's no-op conjugate() (:42-48).
__device__ __forceinline__ float2 evolve(float4 h, float c, float s, int literal_conj)
{
    float bi = literal_conj ? h.w : -h.w;
    return make_float2(h.x * c - h.y * s + h.z * c + bi * s, h.x * s + h.y * c - h.z * s + bi * c);
}

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

// ---------------------------------------------------------------------------
// Row pass.
// ---------------------------------------------------------------------------
template <int N>
struct RowCfg {
    using L = typename LineFor<N>::type;
    static constexpr int PAIRS   = L::G >= 32 ? 1 : 32 / L::G;  // row pairs per CTA
    static constexpr int LINES   = 3 * PAIRS;
    static constexpr int THREADS = LINES * L::G;
    static constexpr size_t SMEM = sizeof(float2) * (N + (size_t)LINES * L::NPAD);
    static constexpr int GRID    = (N / 2 + 1 + PAIRS - 1) / PAIRS;
};

template <int N>
__global__ void __launch_bounds__(RowCfg<N>::THREADS) k_row_pass(RowArgs a)
{
    using RC = RowCfg<N>;
    using L  = typename RC::L;
    extern __shared__ float2 smem[];
    float2* tw_s = smem;
    for (int i = threadIdx.x; i < N; i += RC::THREADS) tw_s[i] = a.tw[i];

    const int li = threadIdx.x / L::G, t = threadIdx.x % L::G;
    const int f  = li % 3;                               // 0: Dx, 1: Dy, 2: Dz
    const int yp = blockIdx.x * RC::PAIRS + li / 3;      // row y' in [0, N/2]
    const bool active = yp <= N / 2;
    const int yq = (N - yp) & (N - 1);                   // row of -k
    float2 v[L::E];
#pragma unroll
    for (int r = 0; r < L::E; ++r) v[r] = make_float2(0.0f, 0.0f);
    if (active) {
        const int iz = yp - N / 2, izq = yq - N / 2;
        const float4* rowp = a.h0 + (size_t)yp * N;
        const float4* rowq = a.h0 + (size_t)yq * N;
#pragma unroll
        for (int r = 0; r < L::E; ++r) {
            const int x  = t + r * (N / L::R1);
            const int xq = (N - x) & (N - 1);
            const int ix = x - N / 2;
            const int m  = ix * ix + iz * iz;
            float c, s;
            mode_phase(m, a.fc, c, s);
            float2 hk = evolve(__ldg(rowp + x), c, s, a.literal_conj);
            float2 hq = evolve(__ldg(rowq + xq), c, s, a.literal_conj);
            float2 X, Xq;
            if (f == 1) {
                X = hk; Xq = hq;
            } else {
                // -i (k/|k|) h (tilde_h0_t_cs.glsl:113-126); the DC mode gets 0
                const float rs  = m ? __frsqrt_rn((float)m) : 0.0f;
                const float fk  = -(float)(f == 0 ? ix : iz) * rs;
                const float fkq = -(float)(f == 0 ? (xq - N / 2) : izq) * rs;
                X  = make_float2(-fk * hk.y, fk * hk.x);
                Xq = make_float2(-fkq * hq.y, fkq * hq.x);
            }
            v[r] = make_float2(X.x + Xq.x, X.y - Xq.y);  // 2 * X_H
        }
    }
    __syncthreads();
    line_fft<L, +1>(v, smem + N + li * L::NPAD, tw_s, t);
    if (active) {
        float2* out = a.inter + ((size_t)f * (N / 2 + 1) + yp) * N;
#pragma unroll
        for (int e = 0; e < L::E; ++e) out[LineOut<L>::pos(t, e)] = v[e];
    }
}

// ---------------------------------------------------------------------------
// Column pass.
// ---------------------------------------------------------------------------
template <int N>
struct ColCfg {
    using L = typename LineFor<N>::type;
    static constexpr int C       = N >= 2048 ? 4 : 8;   // output columns per CTA
    static constexpr int CC      = C + 2;               // + one neighbour column each side
    static constexpr int WL      = CC;                  // Dy + i*Dx lines
    static constexpr int ZL      = CC / 2;              // Dz(c) + i*Dz(c+1) lines
    static constexpr int LINES   = WL + ZL;
    static constexpr int THREADS = LINES * L::G;
    static constexpr int H       = N / 2 + 1;           // stored half-spectrum rows
    static constexpr int TS      = CC + 1;              // tile row stride (odd: bank-free)
    static constexpr int OS      = N + 32 / C;          // output-staging column stride
    static constexpr size_t TILE = sizeof(float2) * 3 * (size_t)H * TS;
    static constexpr size_t XBUF = sizeof(float2) * (size_t)LINES * L::NPAD;
    static constexpr size_t OBUF = sizeof(float) * 3 * (size_t)CC * OS;
    static constexpr size_t AREG = TILE > XBUF ? (TILE > OBUF ? TILE : OBUF) : (XBUF > OBUF ? XBUF : OBUF);
    static constexpr size_t SMEM = sizeof(float2) * N + AREG;
    static constexpr int GRID    = N / C;
};

template <int N>
__global__ void __launch_bounds__(ColCfg<N>::THREADS) k_col_pass(ColArgs a)
{
    using CC_ = ColCfg<N>;
    using L   = typename CC_::L;
    constexpr int C = CC_::C, CC = CC_::CC, H = CC_::H, TS = CC_::TS, OS = CC_::OS;
    extern __shared__ float2 smem[];
    float2* tw_s = smem;
    float2* tile = smem + N;                                 // [3][H][TS]
    float2* xbuf = smem + N;                                 // aliases the tile after the gather
    float*  obuf = reinterpret_cast<float*>(smem + N);       // [3][CC][OS], aliases again
    const int x0 = blockIdx.x * C;

    for (int i = threadIdx.x; i < N; i += CC_::THREADS) tw_s[i] = a.tw[i];
    // Stage columns x0-1 .. x0+C (periodic) of rows 0..N/2 of the three fields.
    for (int i = threadIdx.x; i < 3 * H * CC; i += CC_::THREADS) {
        const int cc = i % CC, row = i / CC;                 // row = f*H + y'
        const int x  = (x0 - 1 + cc + N) & (N - 1);
        tile[row * TS + cc] = a.inter[(size_t)row * N + x];
    }
    __syncthreads();

    const int li = threadIdx.x / L::G, t = threadIdx.x % L::G;
    const bool wline = li < CC_::WL;
    const int  c1 = wline ? li : 2 * (li - CC_::WL);         // tile columns of the two packed reals
    const int  c2 = wline ? li : c1 + 1;
    const int  fa = wline ? 1 : 2, fb = wline ? 0 : 2;       // real part: Dy or Dz(c1); imag: Dx or Dz(c2)
    float2 v[L::E];
#pragma unroll
    for (int r = 0; r < L::E; ++r) {
        const int y = t + r * (N / L::R1);
        const bool lo = y <= N / 2;
        const int  ys = lo ? y : N - y;                      // rows N-y are conjugates of rows y
        float2 p = tile[(fa * H + ys) * TS + c1];
        float2 q = tile[(fb * H + ys) * TS + c2];
        if (!lo) { p.y = -p.y; q.y = -q.y; }
        v[r] = make_float2(p.x - q.y, p.y + q.x);            // p + i*q
    }
    __syncthreads();                                         // tile dead; xbuf reuses it
    line_fft<L, +1>(v, xbuf + li * L::NPAD, tw_s, t);        // ends with a block barrier

    // Unpack, apply (-1)^(x+y) * scale (* lambda for Dx, Dz) and stage per column.
    {
        const int xa = x0 - 1 + c1, xb = x0 - 1 + c2;        // parity is all that matters
        const float sa = wline ? a.scale : a.scale * a.lambda;
        const float sb = a.scale * a.lambda;
        float* oa = obuf + (fa * CC + c1) * OS;
        float* ob = obuf + (fb * CC + c2) * OS;
#pragma unroll
        for (int e = 0; e < L::E; ++e) {
            const int y = LineOut<L>::pos(t, e);
            oa[y] = ((xa + y) & 1) ? -sa * v[e].x : sa * v[e].x;
            ob[y] = ((xb + y) & 1) ? -sb * v[e].y : sb * v[e].y;
        }
    }
    __syncthreads();

    // Epilogue: outputs, Sobel normal on Dy, Jacobian of x - (Dx, Dz).
    const float* sx = obuf;
    const float* sy = obuf + CC * OS;
    const float* sz = obuf + 2 * CC * OS;
    for (int i = threadIdx.x; i < C * N; i += CC_::THREADS) {
        const int c = i % C, y = i / C;
        const int cc = c + 1;
        const int ym = (y - 1) & (N - 1), yn = (y + 1) & (N - 1);
        const float z0 = sy[(cc - 1) * OS + ym], z1 = sy[cc * OS + ym], z2 = sy[(cc + 1) * OS + ym];
        const float z3 = sy[(cc - 1) * OS + y], zc = sy[cc * OS + y], z4 = sy[(cc + 1) * OS + y];
        const float z5 = sy[(cc - 1) * OS + yn], z6 = sy[cc * OS + yn], z7 = sy[(cc + 1) * OS + yn];
        const float nz = z0 + 2.0f * z1 + z2 - z5 - 2.0f * z6 - z7;
        const float nx = z0 + 2.0f * z3 + z5 - z2 - 2.0f * z4 - z7;
        const float rn = rsqrtf(nx * nx + 1.0f + nz * nz);
        const float vx = sx[cc * OS + y], vz = sz[cc * OS + y];
        const float dxx = (sx[(cc + 1) * OS + y] - sx[(cc - 1) * OS + y]) * a.inv2d;
        const float dxz = (sx[cc * OS + yn] - sx[cc * OS + ym]) * a.inv2d;
        const float dzx = (sz[(cc + 1) * OS + y] - sz[(cc - 1) * OS + y]) * a.inv2d;
        const float dzz = (sz[cc * OS + yn] - sz[cc * OS + ym]) * a.inv2d;
        const size_t o = (size_t)y * N + x0 + c;
        a.dx[o] = vx;
        a.dy[o] = zc;
        a.dz[o] = vz;
        // J = (1 - dxx)(1 - dzz) - dxz*dzx, formed as 1 + deviation so that the
        // only rounding at the scale of 1 is the final add
        const float dJ = (dxx * dzz - dxz * dzx) - dxx - dzz;
        a.nj[o] = make_float4(nx * rn, rn, nz * rn, 1.0f + dJ);
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

template <int N>
static cudaError_t row_pass_n(const RowArgs& a, cudaStream_t s)
{
    using RC = RowCfg<N>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_row_pass<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RC::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_row_pass<N><<<RC::GRID, RC::THREADS, RC::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N>
static cudaError_t col_pass_n(const ColArgs& a, cudaStream_t s)
{
    using CC = ColCfg<N>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_col_pass<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CC::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_col_pass<N><<<CC::GRID, CC::THREADS, CC::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N> struct RowSmem { static constexpr size_t v = RowCfg<N>::SMEM; };
template <int N> struct ColSmem { static constexpr size_t v = ColCfg<N>::SMEM; };

cudaError_t launch_row_pass(int N, const RowArgs& a, cudaStream_t s)
{
#define ROWCALL(n) row_pass_n<n>(a, s)
    switch (N) {
    case 32: return ROWCALL(32);
    case 64: return ROWCALL(64);
    case 128: return ROWCALL(128);
    case 256: return ROWCALL(256);
    case 512: return ROWCALL(512);
    case 1024: return ROWCALL(1024);
    case 2048: return ROWCALL(2048);
    default: return cudaErrorInvalidValue;
    }
#undef ROWCALL
}

cudaError_t launch_col_pass(int N, const ColArgs& a, cudaStream_t s)
{
#define COLCALL(n) col_pass_n<n>(a, s)
    switch (N) {
    case 32: return COLCALL(32);
    case 64: return COLCALL(64);
    case 128: return COLCALL(128);
    case 256: return COLCALL(256);
    case 512: return COLCALL(512);
    case 1024: return COLCALL(1024);
    case 2048: return COLCALL(2048);
    default: return cudaErrorInvalidValue;
    }
#undef COLCALL
}

size_t row_pass_smem(int N)
{
    switch (N) {
    case 32: return RowSmem<32>::v;
    case 64: return RowSmem<64>::v;
    case 128: return RowSmem<128>::v;
    case 256: return RowSmem<256>::v;
    case 512: return RowSmem<512>::v;
    case 1024: return RowSmem<1024>::v;
    case 2048: return RowSmem<2048>::v;
    default: return 0;
    }
}

size_t col_pass_smem(int N)
{
    switch (N) {
    case 32: return ColSmem<32>::v;
    case 64: return ColSmem<64>::v;
    case 128: return ColSmem<128>::v;
    case 256: return ColSmem<256>::v;
    case 512: return ColSmem<512>::v;
    case 1024: return ColSmem<1024>::v;
    case 2048: return ColSmem<2048>::v;
    default: return 0;
    }
}

}  // namespace ocean
