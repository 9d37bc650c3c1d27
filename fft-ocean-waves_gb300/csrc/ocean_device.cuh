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
// as a double-float; m^(1/4) is formed by two double-float square roots, each
// a hardware reciprocal-square-root estimate refined by one Newton step on the
// exact FMA residual (Dekker 1971; Karp & Markstein 1997): relative error
// ~2^-44.  The product with K*t is Dekker's two-product via FMA.  The integer
// number of cycles is dropped before sincospi, so the reduced phase keeps
// ~1e-7 absolute accuracy while K*t*m^(1/4) stays below ~2^20 cycles.
// ---------------------------------------------------------------------------
// sin and cos of 2*pi*f for |f| <= 1/2: the quadrant q = rint(4f) is split
// off exactly (g = f - q/4, |g| <= 1/8), theta = 2*pi*g (|theta| <= pi/4), and
// sin/cos theta are their Taylor series to theta^9 / theta^10 (truncation
// below 2e-9 on the octant), Horner-evaluated with FMA; the quadrant rotates
// the result.  Max abs error ~8e-8 against double (FP32 rounding level).
__device__ __forceinline__ void sincos_2pi(float f, float& s, float& c)
{
    const float q  = rintf(4.0f * f);
    const float g  = __fmaf_rn(-0.25f, q, f);                 // exact
    const float th = 6.28318530717958648f * g;
    const float t2 = th * th;
    float ps = __fmaf_rn(t2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps       = __fmaf_rn(t2, ps, 1.0f / 120.0f);
    ps       = __fmaf_rn(t2, ps, -1.0f / 6.0f);
    const float sn = __fmaf_rn(th, t2 * ps, th);
    float pc = __fmaf_rn(t2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc       = __fmaf_rn(t2, pc, -1.0f / 720.0f);
    pc       = __fmaf_rn(t2, pc, 1.0f / 24.0f);
    pc       = __fmaf_rn(t2, pc, -0.5f);
    const float cs = __fmaf_rn(t2, pc, 1.0f);
    const int   qi = (int)q & 3;
    s = (qi & 1) ? cs : sn;
    c = (qi & 1) ? sn : cs;
    if (qi == 1 || qi == 2) c = -c;
    if (qi >= 2) s = -s;
}

// cos/sin of the phase of mode m at the frame's time, and r = 1/sqrt(m)
// (0 for m = 0) to the accuracy of rsqrtf.
__device__ __forceinline__ void mode_phase_r(int m, const FrameConsts& fc, float& c, float& s, float& r)
{
    float f;
    if (m == 0) {
        f = fc.dc_cycles;
        r = 0.0f;
    } else {
        const float mf  = (float)m;                            // exact: m < 2^24
        const float r1  = rsqrtf(mf);
        const float s1  = mf * r1;                             // sqrt(m), a few ulp
        const float s1l = __fmaf_rn(-s1, s1, mf) * (0.5f * r1);
        const float r2  = rsqrtf(s1);
        const float q   = s1 * r2;                             // m^(1/4), a few ulp
        const float ql  = __fadd_rn(__fmaf_rn(-q, q, s1), s1l) * (0.5f * r2);
        const float p   = __fmul_rn(fc.kt_hi, q);
        float       e   = __fmaf_rn(fc.kt_hi, q, -p);
        e               = __fmaf_rn(fc.kt_hi, ql, e);
        e               = __fmaf_rn(fc.kt_lo, q, e);
        f               = __fadd_rn(__fadd_rn(p, -rintf(p)), e);
        f               = __fadd_rn(f, -rintf(f));
        r               = r1;
    }
    sincos_2pi(f, s, c);
}

__device__ __forceinline__ void mode_phase(int m, const FrameConsts& fc, float& c, float& s)
{
    float r;
    mode_phase_r(m, fc, c, s, r);
}

// h(k,t) = h0(k) e^{iwt} + conj(h0(-k)) e^{-iwt} (tilde_h0_t_cs.glsl:110);
// literal_conj reproduces the shader's no-op conjugate() (:42-48).
__device__ __forceinline__ float2 evolve(float4 h, float c, float s, int literal_conj)
{
    float bi = literal_conj ? h.w : -h.w;
    return make_float2(h.x * c - h.y * s + h.z * c + bi * s, h.x * s + h.y * c - h.z * s + bi * c);
}

}  // namespace ocean
