// ocean_sky.cu -- the sky environment cube map (precomputed atmospheric
// scattering, Bruneton & Neyret 2008) as one CUDA kernel: per cube-map texel,
// the view direction through the texel centre, the sun disk attenuated by the
// transmittance, plus the single-lookup sky radiance of the 4-D inscatter
// table.  Follows sky_envmap_fs.glsl:25-38 and atmosphere.glsl:61-199 in FP32
// with the shader's operation order; this translation unit is compiled
// without FMA contraction so that its rounding is the plain FP32 one the CPU
// restatement of the oracle reproduces.  The tables are sampled as the
// reference's GL_LINEAR / CLAMP_TO_EDGE textures (main.cpp:168-184): texel
// coordinate u*W - 0.5, floor, FP32 weights, indices clamped to the edge.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "ocean.h"
#include "ocean_host.h"

namespace {

// atmosphere.glsl:43-50
constexpr float kPi   = 3.141592f;
constexpr float kRg   = 6360000.0f;
constexpr float kRt   = 6420000.0f;
constexpr float kResR = 32.0f, kResMu = 128.0f, kResMuS = 32.0f, kResNu = 8.0f;

struct SkyArgs {
    float3 cam, sun, earth, beta_r;
    float  mie_g, intensity;
    float  tan_mus;      // tan(1.26 * 1.1) (atmosphere.glsl:74)
    float  tan_mu;       // tan(1.5)        (atmosphere.glsl:108)
    float  cos_sun;      // cos(M_PI / 360) (sky_envmap_fs.glsl:29)
    int    S;
};

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float w)
{
    const float v = 1.0f - w;
    return make_float4(a.x * v + b.x * w, a.y * v + b.y * w, a.z * v + b.z * w, a.w * v + b.w * w);
}

// one axis of GL_LINEAR + CLAMP_TO_EDGE: the two texels and the weight of the second
__device__ __forceinline__ void lin_axis(float u, int W, int& i0, int& i1, float& w)
{
    const float t = u * (float)W - 0.5f;
    const float f = floorf(t);
    w             = t - f;
    const int i   = (int)f;
    i0            = min(max(i, 0), W - 1);
    i1            = min(max(i + 1, 0), W - 1);
}

__device__ float4 tex2d(const float4* __restrict__ T, int W, int H, float u, float v)
{
    int x0, x1, y0, y1;
    float wx, wy;
    lin_axis(u, W, x0, x1, wx);
    lin_axis(v, H, y0, y1, wy);
    const float4 a = lerp4(__ldg(T + (size_t)y0 * W + x0), __ldg(T + (size_t)y0 * W + x1), wx);
    const float4 b = lerp4(__ldg(T + (size_t)y1 * W + x0), __ldg(T + (size_t)y1 * W + x1), wx);
    return lerp4(a, b, wy);
}

__device__ float4 tex3d(const float4* __restrict__ T, int W, int H, int D, float u, float v, float q)
{
    int x0, x1, y0, y1, z0, z1;
    float wx, wy, wz;
    lin_axis(u, W, x0, x1, wx);
    lin_axis(v, H, y0, y1, wy);
    lin_axis(q, D, z0, z1, wz);
    auto plane = [&](int z) {
        const float4* P = T + (size_t)z * H * W;
        const float4  a = lerp4(__ldg(P + (size_t)y0 * W + x0), __ldg(P + (size_t)y0 * W + x1), wx);
        const float4  b = lerp4(__ldg(P + (size_t)y1 * W + x0), __ldg(P + (size_t)y1 * W + x1), wx);
        return lerp4(a, b, wy);
    };
    return lerp4(plane(z0), plane(z1), wz);
}

// atmosphere.glsl:61-81: the 4-D (r, mu, muS, nu) table packed in a 3-D texture
__device__ float4 texture4d(const float4* __restrict__ T, const SkyArgs& a, float r, float mu, float muS, float nu)
{
    const float H     = sqrtf(kRt * kRt - kRg * kRg);
    const float rho   = sqrtf(r * r - kRg * kRg);
    const float rmu   = r * mu;
    const float delta = rmu * rmu - r * r + kRg * kRg;
    const bool  below = rmu < 0.0f && delta > 0.0f;
    const float c0 = below ? 1.0f : -1.0f, c1 = below ? 0.0f : H * H, c2 = below ? 0.0f : H;
    const float c3 = below ? 0.5f - 0.5f / kResMu : 0.5f + 0.5f / kResMu;
    const float uR   = 0.5f / kResR + rho / H * (1.0f - 1.0f / kResR);
    const float uMu  = c3 + (rmu * c0 + sqrtf(delta + c1)) / (rho + c2) * (0.5f - 1.0f / kResMu);
    const float uMuS = 0.5f / kResMuS +
                       (atanf(fmaxf(muS, -0.1975f) * a.tan_mus) / 1.1f + (1.0f - 0.26f)) * 0.5f * (1.0f - 1.0f / kResMuS);
    float       lep  = (nu + 1.0f) / 2.0f * (kResNu - 1.0f);
    const float uNu  = floorf(lep);
    lep              = lep - uNu;
    const float4 t0 = tex3d(T, OCEAN_SKY_INSCATTER_W, OCEAN_SKY_INSCATTER_H, OCEAN_SKY_INSCATTER_D,
                            (uNu + uMuS) / kResNu, uMu, uR);
    const float4 t1 = tex3d(T, OCEAN_SKY_INSCATTER_W, OCEAN_SKY_INSCATTER_H, OCEAN_SKY_INSCATTER_D,
                            (uNu + uMuS + 1.0f) / kResNu, uMu, uR);
    const float m = 1.0f - lep;
    return make_float4(t0.x * m + t1.x * lep, t0.y * m + t1.y * lep, t0.z * m + t1.z * lep, t0.w * m + t1.w * lep);
}

// atmosphere.glsl:102-111
__device__ float3 transmittance(const float4* __restrict__ T, const SkyArgs& a, float r, float mu)
{
    const float uR  = sqrtf((r - kRg) / (kRt - kRg));
    const float uMu = atanf((mu + 0.15f) / (1.0f + 0.15f) * a.tan_mu) / 1.5f;
    const float4 t  = tex2d(T, OCEAN_SKY_TRANSMITTANCE_W, OCEAN_SKY_TRANSMITTANCE_H, uMu, uR);
    return make_float3(t.x, t.y, t.z);
}

// sky_envmap_fs.glsl:27 / the cube-map orientation: direction through the
// centre of texel (i, j) of `face`
__device__ float3 face_dir(int face, float sc, float tc)
{
    switch (face) {
    case 0: return make_float3(1.0f, -tc, -sc);
    case 1: return make_float3(-1.0f, -tc, sc);
    case 2: return make_float3(sc, 1.0f, tc);
    case 3: return make_float3(sc, -1.0f, -tc);
    case 4: return make_float3(sc, -tc, 1.0f);
    default: return make_float3(-sc, -tc, -1.0f);
    }
}

__global__ void k_sky_envmap(SkyArgs a, const float4* __restrict__ trans, const float4* __restrict__ insc,
                             float4* __restrict__ out)
{
    const int S = a.S;
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= 6LL * S * S) return;
    const int face = (int)(idx / ((long long)S * S));
    const int rem  = (int)(idx - (long long)face * S * S);
    const int j = rem / S, i = rem - j * S;
    const float3 d0  = face_dir(face, 2.0f * (((float)i + 0.5f) / (float)S) - 1.0f,
                                2.0f * (((float)j + 0.5f) / (float)S) - 1.0f);
    const float  len = sqrtf(d0.x * d0.x + d0.y * d0.y + d0.z * d0.z);
    const float3 v   = make_float3(d0.x / len, d0.y / len, d0.z / len);

    // sun disk (sky_envmap_fs.glsl:29-31)
    const float sun = (v.x * a.sun.x + v.y * a.sun.y + v.z * a.sun.z) < a.cos_sun ? 0.0f : 1.0f;
    const float sun_c = sun * a.intensity;

    // SkyRadiance (atmosphere.glsl:152-199)
    float3 cam = make_float3(a.cam.x + a.earth.x, a.cam.y + a.earth.y, a.cam.z + a.earth.z);
    float  r   = sqrtf(cam.x * cam.x + cam.y * cam.y + cam.z * cam.z);
    float  rMu = cam.x * v.x + cam.y * v.y + cam.z * v.z;
    float  mu  = rMu / r;
    const float deltaSq = sqrtf(rMu * rMu - r * r + kRt * kRt);
    const float din     = fmaxf(-rMu - deltaSq, 0.0f);
    if (din > 0.0f) {
        cam = make_float3(cam.x + din * v.x, cam.y + din * v.y, cam.z + din * v.z);
        rMu = rMu + din;
        mu  = rMu / kRt;
        r   = kRt;
    }
    const float nu  = v.x * a.sun.x + v.y * a.sun.y + v.z * a.sun.z;
    const float muS = (cam.x * a.sun.x + cam.y * a.sun.y + cam.z * a.sun.z) / r;
    const float4 is = texture4d(insc, a, r, rMu / r, muS, nu);
    float3 ext      = transmittance(trans, a, r, mu);
    float3 res      = make_float3(0.0f, 0.0f, 0.0f);
    if (r <= kRt) {
        // GetMie (atmosphere.glsl:83-88), phase functions (:90-100)
        const float  mx = fmaxf(is.x, 1e-4f);
        const float3 m  = make_float3(is.x * is.w / mx * (a.beta_r.x / a.beta_r.x), is.y * is.w / mx * (a.beta_r.x / a.beta_r.y),
                                      is.z * is.w / mx * (a.beta_r.x / a.beta_r.z));
        const float pr = (3.0f / (16.0f * kPi)) * (1.0f + nu * nu);
        const float g  = a.mie_g;
        const float pm = 1.5f * 1.0f / (4.0f * kPi) * (1.0f - g * g) * powf(1.0f + (g * g) - 2.0f * g * nu, -3.0f / 2.0f) *
                         (1.0f + nu * nu) / (2.0f + g * g);
        res = make_float3(is.x * pr + m.x * pm, is.y * pr + m.y * pm, is.z * pr + m.z * pm);
    } else {
        ext = make_float3(1.0f, 1.0f, 1.0f);
    }
    const float I = a.intensity;
    out[idx] = make_float4(sun_c * ext.x + res.x * I, sun_c * ext.y + res.y * I, sun_c * ext.z + res.z * I, 1.0f);
}

}  // namespace

extern "C" int ocean_sky_envmap(const ocean_sky_params* p, const float* transmittance_tab, const float* inscatter_tab,
                                float* cubemap, void* stream)
{
    using namespace ocean::host;
    if (!p || !transmittance_tab || !inscatter_tab || !cubemap) return fail(OCEAN_ERR_INVALID, "NULL pointer");
    if (p->size < 1 || p->size > 8192) return fail(OCEAN_ERR_INVALID, "size must be in [1, 8192]");
    if ((reinterpret_cast<uintptr_t>(transmittance_tab) | reinterpret_cast<uintptr_t>(inscatter_tab) |
         reinterpret_cast<uintptr_t>(cubemap)) % 16)
        return fail(OCEAN_ERR_INVALID, "tables and cubemap must be 16-byte aligned");
    const float v[] = {p->camera[0], p->camera[1], p->camera[2], p->sun_direction[0], p->sun_direction[1],
                       p->sun_direction[2], p->earth_pos[0], p->earth_pos[1], p->earth_pos[2], p->beta_r[0],
                       p->beta_r[1], p->beta_r[2], p->mie_g, p->sun_intensity};
    for (float x : v)
        if (!std::isfinite(x)) return fail(OCEAN_ERR_INVALID, "sky parameters must be finite");
    if (!(p->beta_r[0] > 0.0f && p->beta_r[1] > 0.0f && p->beta_r[2] > 0.0f))
        return fail(OCEAN_ERR_INVALID, "beta_r must be positive");
    SkyArgs a;
    a.cam       = make_float3(p->camera[0], p->camera[1], p->camera[2]);
    a.sun       = make_float3(p->sun_direction[0], p->sun_direction[1], p->sun_direction[2]);
    a.earth     = make_float3(p->earth_pos[0], p->earth_pos[1], p->earth_pos[2]);
    a.beta_r    = make_float3(p->beta_r[0], p->beta_r[1], p->beta_r[2]);
    a.mie_g     = p->mie_g;
    a.intensity = p->sun_intensity;
    a.tan_mus   = std::tan(1.26f * 1.1f);
    a.tan_mu    = std::tan(1.5f);
    a.cos_sun   = std::cos(kPi / 360.0f);
    a.S         = p->size;
    const long long n = 6LL * p->size * p->size;
    k_sky_envmap<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        a, reinterpret_cast<const float4*>(transmittance_tab), reinterpret_cast<const float4*>(inscatter_tab),
        reinterpret_cast<float4*>(cubemap));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "sky envmap launch");
    return OCEAN_OK;
}
