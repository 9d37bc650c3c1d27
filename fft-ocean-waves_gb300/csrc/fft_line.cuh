// fft_line.cuh -- complex FP32 FFT building blocks for the ocean kernels.
//
// A "line" is one N-point transform (one row or one column of a spectrum).
// It is computed by G = N/R1 cooperating threads, each holding R1 complex
// values in registers, as a Stockham auto-sort FFT of 2 to 4 passes
// (radices R1, R2[, R3[, R4]]; every radix <= 32 and dividing R1):
//
//   pass 1 (radix R1, Ns = 1):   thread t owns inputs x[t + r*N/R1], r < R1,
//                                so a line is loaded with unit stride across
//                                threads (coalesced rows / bank-free columns).
//   pass p (radix R, Ns = prod of earlier radices): butterfly j reads
//                                x[j + r*N/R] from shared memory, multiplies
//                                by W_{Ns*R}^{(j mod Ns)*r}, does an R-point
//                                DFT in registers and writes outputs to
//                                ((j/Ns)*Ns*R + j mod Ns) + r*Ns.
//   after the last pass         butterfly j holds X[j + r*N/R_last], again
//                                unit stride across threads (coalesced store).
//
// The unnormalised inverse transform (SIGN = +1, exponent +2*pi*i*n*k/N) is
// what the reference's butterfly passes compute (butterfly_cs.glsl:54-132,
// twiddles exp(+2*pi*i*k/N) twiddle_factors_cs.glsl:37-38).  SIGN = -1 gives
// the forward transform used by the adjoint.
//
// Shared-memory exchange buffers are padded by one complex per R1 entries:
// the pass-1 writes (stride R1 across threads) and the later unit-stride
// reads are then free of bank conflicts for 8-byte accesses.
#pragma once
#include <cuda_runtime.h>

namespace ocean {

__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// Complex add and subtract as one paired FP32 instruction each (add.rn.f32x2 /
// sub.rn.f32x2, sm_100 and later): the two lanes round exactly as two scalar
// adds.  With them the butterflies of an in-register DFT issue half the adds;
// whether that shortens a kernel depends on the kernel (the line transforms
// take them through their PAIRED parameter).
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    float2 r;
    asm("{.reg .b64 a, b, r;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tadd.rn.f32x2 r, a, b;\n\t"
        "mov.b64 {%0, %1}, r;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    float2 r;
    asm("{.reg .b64 a, b, r;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tsub.rn.f32x2 r, a, b;\n\t"
        "mov.b64 {%0, %1}, r;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// cos(2*pi*k/32) and sin(2*pi*k/32), rounded to float.  Plain switches (no
// recursion) so that, with k a constant after unrolling, they fold to
// immediates instead of becoming called functions.
__host__ __device__ __forceinline__ constexpr float cos32(int k)
{
    switch (k & 31) {
    case 0: return 1.0f;
    case 1: return 0.980785251f;
    case 2: return 0.923879504f;
    case 3: return 0.831469595f;
    case 4: return 0.707106769f;
    case 5: return 0.555570245f;
    case 6: return 0.382683426f;
    case 7: return 0.195090324f;
    case 8: return 0.0f;
    case 9: return -0.195090324f;
    case 10: return -0.382683426f;
    case 11: return -0.555570245f;
    case 12: return -0.707106769f;
    case 13: return -0.831469595f;
    case 14: return -0.923879504f;
    case 15: return -0.980785251f;
    case 16: return -1.0f;
    case 17: return -0.980785251f;
    case 18: return -0.923879504f;
    case 19: return -0.831469595f;
    case 20: return -0.707106769f;
    case 21: return -0.555570245f;
    case 22: return -0.382683426f;
    case 23: return -0.195090324f;
    case 24: return 0.0f;
    case 25: return 0.195090324f;
    case 26: return 0.382683426f;
    case 27: return 0.555570245f;
    case 28: return 0.707106769f;
    case 29: return 0.831469595f;
    case 30: return 0.923879504f;
    case 31: return 0.980785251f;
    default: return 0.0f;
    }
}
__host__ __device__ __forceinline__ constexpr float sin32(int k) { return cos32((k + 24) & 31); }

// x * W_32^idx with W = exp(SIGN * 2*pi*i/32); idx is a compile-time constant
// after unrolling, so the branches fold away.
template <int SIGN>
__device__ __forceinline__ float2 mul_w32(float2 x, int idx)
{
    if (idx == 0) return x;
    if (idx == 8) return SIGN > 0 ? make_float2(-x.y, x.x) : make_float2(x.y, -x.x);
    const float c = cos32(idx), s = SIGN > 0 ? sin32(idx) : -sin32(idx);
    return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
}

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Bit reversal of i over `bits` bits (linear loop: fully unrolled and folded
// when i and bits are compile-time constants).
__host__ __device__ constexpr int bitrev_bits(int i, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}

// In-register R-point DFT (R = 1..32, power of two), natural order in and out.
// Radix-2 decimation in time on bit-reversed input.  Every loop has a linear
// induction variable so that it unrolls completely and all register indices
// are compile-time constants.
template <int R, int SIGN, bool PAIRED = false>
__device__ __forceinline__ void dft(float2* v)
{
    constexpr int LG = ilog2c(R);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j = bitrev_bits(i, LG);
        if (j > i) {
            float2 t = v[i];
            v[i]     = v[j];
            v[j]     = t;
        }
    }
#pragma unroll
    for (int s = 0; s < LG; ++s) {
        const int h = 1 << s;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const int idx = k * (16 >> s);  // W_{2h}^k == W_32^{16k/h}
#pragma unroll
            for (int g = 0; g < R / (2 * h); ++g) {
                const int i = k + g * 2 * h;
                float2 b = mul_w32<SIGN>(v[i + h], idx);
                float2 a = v[i];
                v[i]     = PAIRED ? add2(a, b) : a + b;
                v[i + h] = PAIRED ? sub2(a, b) : a - b;
            }
        }
    }
}

template <int N_, int R1_, int R2_, int R3_ = 1, int R4_ = 1>
struct LineCfg {
    static constexpr int N    = N_;
    static constexpr int R1   = R1_;
    static constexpr int R2   = R2_;
    static constexpr int R3   = R3_;
    static constexpr int R4   = R4_;
    static constexpr int G    = N / R1;      // threads per line
    static constexpr int E    = R1;          // complex values per thread
    static constexpr int NPAD = N + N / R1;  // padded exchange-buffer length
    static_assert(R1 * R2 * R3 * R4 == N, "radices must multiply to N");
    static_assert(R1 <= 32 && R2 <= R1 && R3 <= R1 && R4 <= R1 && R1 % R2 == 0 && R1 % R3 == 0 && R1 % R4 == 0,
                  "bad radices");
    static_assert(R4 == 1 || R3 > 1, "a fourth pass needs a third");
    __device__ __forceinline__ static int pad(int i) { return i + i / R1; }
};

// Line-size -> decomposition used by every kernel.
template <int N> struct LineFor;
template <> struct LineFor<32>   { using type = LineCfg<32, 8, 4>; };
template <> struct LineFor<64>   { using type = LineCfg<64, 8, 8>; };
template <> struct LineFor<128>  { using type = LineCfg<128, 16, 8>; };
template <> struct LineFor<256>  { using type = LineCfg<256, 16, 16>; };
// 16-point first passes from N = 512 up: ~95 registers per thread instead of
// ~168 for 32-point ones, so twice the threads per line fit on an SM.
template <> struct LineFor<512>  { using type = LineCfg<512, 16, 16, 2>; };
template <> struct LineFor<1024> { using type = LineCfg<1024, 16, 16, 4>; };
template <> struct LineFor<2048> { using type = LineCfg<2048, 16, 16, 8>; };

// Inter-pass twiddles of a decomposition, laid out so that the threads of a
// warp read consecutive entries (no bank conflicts, no index arithmetic).
// Pass p (p = 2, 3, 4) has NS = R1 ... R(p-1) butterfly strides and radix R =
// Rp; its segment holds T[off + r*NS + k] = W_N^(k*r*N/(NS*R)), k < NS,
// r < R:
//   pass 2: off 0,        NS = R1;
//   pass 3: off P2,       NS = R1*R2;
//   pass 4: off P2 + P3,  NS = R1*R2*R3.
// W_N = exp(+2*pi*i/N), rounded from double (conjugated in the transform for
// SIGN < 0).  Built once per size by launch_twiddles().
template <class C>
struct TwPlan {
    static constexpr int P2  = C::R1 * C::R2;
    static constexpr int P3  = C::R3 > 1 ? C::R1 * C::R2 * C::R3 : 0;
    static constexpr int P4  = C::R4 > 1 ? C::R1 * C::R2 * C::R3 * C::R4 : 0;
    static constexpr int LEN = P2 + P3 + P4;
};

// Barrier among the threads of one line.  With NAMED, lines of >= 32 threads
// use named barrier 1 + li, so lines progress independently; this requires
// every warp to belong to a single line (threads of one warp must not wait on
// different barriers).  Smaller lines, or kernels whose warps mix lines, use
// the block barrier.
template <class C, bool NAMED>
__device__ __forceinline__ void line_sync(int li)
{
    if constexpr (NAMED && C::G >= 32)
        asm volatile("bar.sync %0, %1;" ::"r"(1 + li), "n"(C::G) : "memory");
    else
        __syncthreads();
}

// One exchange + pass: the registers hold the outputs of a pass of radix RP
// with stride NSP; they are written to `buf`, re-read as the inputs of a pass
// of radix RN (stride NSP*RP), twiddled (plan segment at TWOFF) and
// transformed.  Contains two line barriers (see line_sync); without TAIL_SYNC
// only the first, and a thread may then leave while others of its line still
// read `buf`.
template <class C, int RP, int NSP, int RN, int TWOFF, int SIGN, bool NAMED, bool TAIL_SYNC = true, bool PAIRED = false>
__device__ __forceinline__ void stockham_pass(float2* v, float2* buf, const float2* tw, int t, bool active, int li)
{
    constexpr int N   = C::N;
    constexpr int NSN = NSP * RP;
    if (active) {
#pragma unroll
        for (int b = 0; b < C::R1 / RP; ++b) {
            const int j    = t + b * C::G;
            const int idxD = (j / NSP) * NSP * RP + (j % NSP);
#pragma unroll
            for (int r = 0; r < RP; ++r) buf[C::pad(idxD + r * NSP)] = v[b * RP + r];
        }
    }
    line_sync<C, NAMED>(li);
    if (active) {
#pragma unroll
        for (int b = 0; b < C::R1 / RN; ++b) {
            const int j = t + b * C::G;
#pragma unroll
            for (int r = 0; r < RN; ++r) v[b * RN + r] = buf[C::pad(j + r * (N / RN))];
        }
    }
    if constexpr (TAIL_SYNC) line_sync<C, NAMED>(li);
    if (!active) return;
    // twiddle plan of this pass: entry r*NSN + k
    const float2* T = tw + TWOFF;
#pragma unroll
    for (int b = 0; b < C::R1 / RN; ++b) {
        const int j = t + b * C::G;
        const int k = j % NSN;
#pragma unroll
        for (int r = 1; r < RN; ++r) {
            float2 w = T[r * NSN + k];
            if (SIGN < 0) w.y = -w.y;
            v[b * RN + r] = cmul(v[b * RN + r], w);
        }
        dft<RN, SIGN, PAIRED>(v + b * RN);
    }
}

// Full line transform of line `li` (barrier id 1 + li, so li < 15; NAMED as
// in line_sync).  On entry
// v[r] = x[t + r*N/R1]; on exit v[b*RL + r] = X[(t + b*G) + r*(N/RL)] with RL
// the last radix.  tw: the decomposition's twiddle plan (TwPlan<C>).  With
// TAIL_SYNC, on return every thread of the line has finished reading `buf`.
// Without it the final line barrier is left out: for callers that do not
// write `buf` again, or that order the reuse by a barrier of their own.
// Threads with active == false do no work; for lines of >= 32 threads
// they may skip the call entirely, for smaller lines they must call it (the
// barrier is then the block's).  PAIRED: the DFT butterflies add and subtract
// with paired FP32 instructions (same results, bit for bit).
template <class C, int SIGN, bool NAMED = true, bool TAIL_SYNC = true, bool PAIRED = false>
__device__ __forceinline__ void line_fft(float2* v, float2* buf, const float2* tw, int t, int li, bool active = true)
{
    using TP = TwPlan<C>;
    if (active) dft<C::R1, SIGN, PAIRED>(v);
    stockham_pass<C, C::R1, 1, C::R2, 0, SIGN, NAMED, (C::R3 > 1) || TAIL_SYNC, PAIRED>(v, buf, tw, t, active, li);
    if constexpr (C::R3 > 1)
        stockham_pass<C, C::R2, C::R1, C::R3, TP::P2, SIGN, NAMED, (C::R4 > 1) || TAIL_SYNC, PAIRED>(v, buf, tw, t,
                                                                                                    active, li);
    if constexpr (C::R4 > 1)
        stockham_pass<C, C::R3, C::R1 * C::R2, C::R4, TP::P2 + TP::P3, SIGN, NAMED, TAIL_SYNC, PAIRED>(v, buf, tw, t,
                                                                                                     active, li);
}

template <class C>
struct LineOut {
    static constexpr int RL = C::R4 > 1 ? C::R4 : (C::R3 > 1 ? C::R3 : C::R2);
    static constexpr int B  = C::R1 / RL;          // butterflies per thread in the last pass
    static constexpr int NS = C::N / RL;           // output stride of the last pass
    // position of register e = b*RL + r after line_fft
    __host__ __device__ __forceinline__ static constexpr int pos(int t, int e)
    {
        return (t + (e / RL) * C::G) + (e % RL) * NS;
    }
};

}  // namespace ocean
