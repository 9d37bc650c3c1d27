// ocean_device.cuh -- device helpers shared by the forward and adjoint
// kernels: the double-float phase w*t and the spectrum evolution.
#pragma once
#include <cuda_runtime.h>

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

}  // namespace ocean
