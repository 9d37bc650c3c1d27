// ocean_grid.cu -- the displaced grid: the consumer side of the maps.
//
// The reference renders a grid of GRID_SIZE = 1024 squares per side with a
// texture repeat of GRID_UV_SCALE = 64 (main.cpp:20-21, generate_grid
// main.cpp:748-824): (n+1)^2 vertices at (x, 0, z), x, z in [-n/2, n/2], two
// triangles per square.  Its tessellation control stage picks per-triangle
// levels from the eye distance (grid_tcs.glsl:27-59) and its evaluation stage
// displaces each vertex by the maps (grid_tes.glsl:55-66).  These kernels
// produce the same quantities into headless device buffers:
//
//   k_displace_grid   per grid vertex: y += Dy(uv) * displacement_scale,
//                     x -= Dx(uv), z -= Dz(uv) (Dx, Dz already carry lambda),
//                     normal = normal_map(uv).xyz, texcoord; the maps are
//                     sampled bilinearly with REPEAT wrap.
//   k_tess_levels     per triangle: outer levels from the mean eye distance of
//                     each edge's end points (20 / 10 / 5 / 1 up to 10 / 20 /
//                     30 / beyond), inner = outer[2].
//   k_shade           per displaced vertex: the ocean fragment shader
//                     (ocean_fs.glsl:11-37): Fresnel-Schlick mix of the sea
//                     colour and the sky cube map along the reflected view
//                     ray, N.L, Reinhard tonemap, gamma 1/2.2.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <utility>

#include "ocean.h"
#include "ocean_host.h"

namespace {

struct GridArgs {
    const float*  dx;
    const float*  dy;
    const float*  dz;
    const float4* nj;
    int           N;         // map size
    int           n;         // squares per side
    long long     step_int;  // integer part of texels per vertex step (uv_scale * N / n)
    float         step_frac; // its fraction
    float         uv_scale;
    float         disp;
};

// Texel coordinate of vertex index i along one axis, reduced into [0, N) before
// the half-texel shift so that large repeats keep sub-texel precision.
__device__ __forceinline__ float texel_coord(const GridArgs& a, int i)
{
    const long long ip = ((long long)i * a.step_int) % a.N;
    return (float)ip + (float)i * a.step_frac - 0.5f;
}

__device__ __forceinline__ void bilinear_taps(int N, float s, int& i0, int& i1, float& w)
{
    const float f = floorf(s);
    w             = s - f;
    int i         = (int)f % N;
    if (i < 0) i += N;
    i0 = i;
    i1 = i + 1 == N ? 0 : i + 1;
}

__global__ void k_displace_grid(GridArgs a, float* __restrict__ out)
{
    const int nv = a.n + 1;
    const int v  = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv * nv) return;
    const int zi = v / nv, xi = v - zi * nv;
    int   x0, x1, y0, y1;
    float wx, wy;
    bilinear_taps(a.N, texel_coord(a, xi), x0, x1, wx);
    bilinear_taps(a.N, texel_coord(a, zi), y0, y1, wy);
    const size_t o00 = (size_t)y0 * a.N + x0, o01 = (size_t)y0 * a.N + x1;
    const size_t o10 = (size_t)y1 * a.N + x0, o11 = (size_t)y1 * a.N + x1;
    auto lerp2 = [&](const float* m) {
        const float top = __ldg(m + o00) * (1.0f - wx) + __ldg(m + o01) * wx;
        const float bot = __ldg(m + o10) * (1.0f - wx) + __ldg(m + o11) * wx;
        return top * (1.0f - wy) + bot * wy;
    };
    const float4 n00 = __ldg(a.nj + o00), n01 = __ldg(a.nj + o01), n10 = __ldg(a.nj + o10), n11 = __ldg(a.nj + o11);
    const float  w00 = (1.0f - wx) * (1.0f - wy), w01 = wx * (1.0f - wy), w10 = (1.0f - wx) * wy, w11 = wx * wy;
    const int    h = a.n / 2;
    float4* o = reinterpret_cast<float4*>(out + 8 * (size_t)v);
    o[0] = make_float4((float)(xi - h) - lerp2(a.dx), lerp2(a.dy) * a.disp, (float)(zi - h) - lerp2(a.dz),
                       n00.x * w00 + n01.x * w01 + n10.x * w10 + n11.x * w11);
    o[1] = make_float4(n00.y * w00 + n01.y * w01 + n10.y * w10 + n11.y * w11,
                       n00.z * w00 + n01.z * w01 + n10.z * w10 + n11.z * w11, (float)xi / (float)a.n * a.uv_scale,
                       (float)zi / (float)a.n * a.uv_scale);
}

__device__ __forceinline__ float tess_level(float d0, float d1)
{
    const float avg = (d0 + d1) / 2.0f;
    return avg <= 10.0f ? 20.0f : avg <= 20.0f ? 10.0f : avg <= 30.0f ? 5.0f : 1.0f;
}

__global__ void k_tess_levels(int n, float cx, float cy, float cz, float4* __restrict__ out)
{
    const int sq = blockIdx.x * blockDim.x + threadIdx.x;
    if (sq >= n * n) return;
    const int   zi = sq / n, xi = sq - zi * n, h = n / 2;
    const float x0 = (float)(xi - h), x1 = x0 + 1.0f, z0 = (float)(zi - h), z1 = z0 + 1.0f;
    auto dist = [&](float x, float z) {
        const float ex = cx - x, ez = cz - z;
        return sqrtf(ex * ex + cy * cy + ez * ez);
    };
    // triangle A: (x, z), (x, z+1), (x+1, z); triangle B: (x+1, z), (x, z+1), (x+1, z+1)
    const float a0 = dist(x0, z0), a1 = dist(x0, z1), a2 = dist(x1, z0), b2 = dist(x1, z1);
    const float oa2 = tess_level(a0, a1), ob2 = tess_level(a2, a1);
    out[2 * (size_t)sq]     = make_float4(tess_level(a1, a2), tess_level(a2, a0), oa2, oa2);
    out[2 * (size_t)sq + 1] = make_float4(tess_level(a1, b2), tess_level(b2, a2), ob2, ob2);
}

// Cube-map lookup (faces +X, -X, +Y, -Y, +Z, -Z of S x S RGBA texels): face and
// face coordinates from the major axis of r as in the OpenGL specification's
// cube-map table (ties go to x, then y), bilinear within the face, clamp to
// edge.
__device__ __forceinline__ float3 cube_sample(const float4* __restrict__ sky, int S, float3 r)
{
    const float ax = fabsf(r.x), ay = fabsf(r.y), az = fabsf(r.z);
    int   face;
    float ma, sc, tc;
    if (ax >= ay && ax >= az) {
        face = r.x >= 0.0f ? 0 : 1; ma = ax; sc = r.x >= 0.0f ? -r.z : r.z; tc = -r.y;
    } else if (ay >= az) {
        face = r.y >= 0.0f ? 2 : 3; ma = ay; sc = r.x; tc = r.y >= 0.0f ? r.z : -r.z;
    } else {
        face = r.z >= 0.0f ? 4 : 5; ma = az; sc = r.z >= 0.0f ? r.x : -r.x; tc = -r.y;
    }
    const float s = 0.5f * (sc / ma + 1.0f) * S - 0.5f, t = 0.5f * (tc / ma + 1.0f) * S - 0.5f;
    const float fs = floorf(s), ft = floorf(t), ws = s - fs, wt = t - ft;
    const int   s0 = (int)fs, t0 = (int)ft;
    const int   sa = min(max(s0, 0), S - 1), sb = min(max(s0 + 1, 0), S - 1);
    const int   ta = min(max(t0, 0), S - 1), tb = min(max(t0 + 1, 0), S - 1);
    const float4* f = sky + (size_t)face * S * S;
    const float4 a = __ldg(f + (size_t)ta * S + sa), b = __ldg(f + (size_t)ta * S + sb);
    const float4 c = __ldg(f + (size_t)tb * S + sa), d = __ldg(f + (size_t)tb * S + sb);
    const float w00 = (1 - ws) * (1 - wt), w01 = ws * (1 - wt), w10 = (1 - ws) * wt, w11 = ws * wt;
    return make_float3(a.x * w00 + b.x * w01 + c.x * w10 + d.x * w11, a.y * w00 + b.y * w01 + c.y * w10 + d.y * w11,
                       a.z * w00 + b.z * w01 + c.z * w10 + d.z * w11);
}

// sky_vs.glsl + sky_fs.glsl: the far-plane point of each pixel centre
// through inverse(projection * mat4(mat3(view))) (column-major m), the cube
// map there, Reinhard and gamma.
struct SkyboxArgs {
    float m[16];
    int   S, W, H;
};

__global__ void k_skybox(SkyboxArgs a, const float4* __restrict__ sky, float4* __restrict__ img)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)a.W * a.H) return;
    const int   y = (int)(idx / a.W), x = (int)(idx - (long long)y * a.W);
    const float cx = 2.0f * ((float)x + 0.5f) / (float)a.W - 1.0f, cy = 2.0f * ((float)y + 0.5f) / (float)a.H - 1.0f;
    float d[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) d[i] = a.m[i] * cx + a.m[4 + i] * cy + a.m[8 + i] + a.m[12 + i];
    const float3 c = cube_sample(sky, a.S, make_float3(d[0] / d[3], d[1] / d[3], d[2] / d[3]));
    auto tone = [](float v) { return powf(v / (v + 1.0f), 1.0f / 2.2f); };
    img[idx] = make_float4(tone(c.x), tone(c.y), tone(c.z), 1.0f);
}

struct ShadeArgs {
    float3 cam, sun, sea;
    int    S;
};

__global__ void k_shade(const float4* __restrict__ vert, long long n, ShadeArgs a, const float4* __restrict__ sky,
                        float4* __restrict__ out)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p0 = __ldg(vert + 2 * i), p1 = __ldg(vert + 2 * i + 1);   // position xyz, normal x | normal yz, uv
    const float3 N  = make_float3(p0.w, p1.x, p1.y);
    float3       V  = make_float3(a.cam.x - p0.x, a.cam.y - p0.y, a.cam.z - p0.z);
    const float  iv = rsqrtf(V.x * V.x + V.y * V.y + V.z * V.z);
    V               = make_float3(V.x * iv, V.y * iv, V.z * iv);
    const float  nv = N.x * V.x + N.y * V.y + N.z * V.z;
    const float3 R  = make_float3(2.0f * nv * N.x - V.x, 2.0f * nv * N.y - V.y, 2.0f * nv * N.z - V.z);
    const float3 sk = cube_sample(sky, a.S, R);
    const float  om = 1.0f - fmaxf(nv, 0.0f);
    const float  F  = 0.04f + 0.96f * (om * om) * (om * om) * om;
    const float  nl = fmaxf(-(N.x * a.sun.x + N.y * a.sun.y + N.z * a.sun.z), 0.0f);
    auto tone = [&](float sea, float skyc) {
        const float c = nl * (sea * (1.0f - F) + skyc * F);
        return powf(c / (c + 1.0f), 1.0f / 2.2f);
    };
    out[i] = make_float4(tone(a.sea.x, sk.x), tone(a.sea.y, sk.y), tone(a.sea.z, sk.z), 1.0f);
}

int check_grid(const ocean_grid_params* g)
{
    using namespace ocean::host;
    if (!g) return fail(OCEAN_ERR_INVALID, "grid params are NULL");
    if (g->squares < 2 || g->squares > 16384 || (g->squares & 1))
        return fail(OCEAN_ERR_INVALID, "squares must be even and in [2, 16384]");
    if (!std::isfinite(g->texcoord_scale) || !std::isfinite(g->displacement_scale))
        return fail(OCEAN_ERR_INVALID, "grid scales must be finite");
    // bounds the texel step (scale * N / squares <= 3.3e10) so that it and its
    // per-vertex multiples stay exact integers (the reference uses 64)
    if (std::fabs(g->texcoord_scale) > 1.0e6f)
        return fail(OCEAN_ERR_INVALID, "texcoord_scale must be within +-1e6");
    return OCEAN_OK;
}

}  // namespace

extern "C" int ocean_displace_grid(const ocean_outputs* maps, int32_t N, const ocean_grid_params* g, float* vertices,
                                   void* stream)
{
    using namespace ocean::host;
    int rc = check_grid(g);
    if (rc) return rc;
    if (!maps || !maps->dx || !maps->dy || !maps->dz || !maps->normal_j || !vertices)
        return fail(OCEAN_ERR_INVALID, "NULL pointer");
    if (!is_pow2(N) || N < 2 || N > 65536) return fail(OCEAN_ERR_INVALID, "N must be a power of two");
    if ((reinterpret_cast<uintptr_t>(vertices) | reinterpret_cast<uintptr_t>(maps->normal_j)) % 16)
        return fail(OCEAN_ERR_INVALID, "vertices and normal_j must be 16-byte aligned");
    GridArgs a;
    a.dx = maps->dx;
    a.dy = maps->dy;
    a.dz = maps->dz;
    a.nj = reinterpret_cast<const float4*>(maps->normal_j);
    a.N  = N;
    a.n  = g->squares;
    const double step = (double)g->texcoord_scale * N / g->squares;   // texels per vertex
    const double fl   = std::floor(step);
    a.step_int  = (long long)fl;
    a.step_frac = (float)(step - fl);
    a.uv_scale  = g->texcoord_scale;
    a.disp      = g->displacement_scale;
    const long long nv = (long long)(g->squares + 1) * (g->squares + 1);
    k_displace_grid<<<(unsigned)((nv + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, vertices);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "displaced grid launch");
    return OCEAN_OK;
}

extern "C" int ocean_grid_tess_levels(const ocean_grid_params* g, float* levels, void* stream)
{
    using namespace ocean::host;
    int rc = check_grid(g);
    if (rc) return rc;
    if (!levels) return fail(OCEAN_ERR_INVALID, "levels is NULL");
    if (reinterpret_cast<uintptr_t>(levels) % 16) return fail(OCEAN_ERR_INVALID, "levels must be 16-byte aligned");
    const long long sq = (long long)g->squares * g->squares;
    k_tess_levels<<<(unsigned)((sq + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g->squares, g->camera[0], g->camera[1], g->camera[2], reinterpret_cast<float4*>(levels));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "tessellation level launch");
    return OCEAN_OK;
}

extern "C" int ocean_shade_grid(const float* vertices, int64_t n_vertices, const ocean_shade_params* p,
                                const float* sky_cubemap, float* colors, void* stream)
{
    using namespace ocean::host;
    if (!vertices || !p || !sky_cubemap || !colors) return fail(OCEAN_ERR_INVALID, "NULL pointer");
    if (n_vertices < 0 || n_vertices > (int64_t)0x7fffffff * 256)   // one launch of 256-thread blocks
        return fail(OCEAN_ERR_INVALID, "n_vertices must be in [0, 2^31 * 256)");
    if (p->sky_size < 1 || p->sky_size > 16384) return fail(OCEAN_ERR_INVALID, "sky_size must be in [1, 16384]");
    if ((reinterpret_cast<uintptr_t>(vertices) | reinterpret_cast<uintptr_t>(sky_cubemap) |
         reinterpret_cast<uintptr_t>(colors)) % 16)
        return fail(OCEAN_ERR_INVALID, "vertices, sky_cubemap and colors must be 16-byte aligned");
    for (int c = 0; c < 3; ++c)
        if (!std::isfinite(p->camera[c]) || !std::isfinite(p->sun_direction[c]) || !std::isfinite(p->sea_color[c]))
            return fail(OCEAN_ERR_INVALID, "shading parameters must be finite");
    if (!n_vertices) return OCEAN_OK;
    ShadeArgs a;
    a.cam = make_float3(p->camera[0], p->camera[1], p->camera[2]);
    a.sun = make_float3(p->sun_direction[0], p->sun_direction[1], p->sun_direction[2]);
    a.sea = make_float3(p->sea_color[0], p->sea_color[1], p->sea_color[2]);
    a.S   = p->sky_size;
    k_shade<<<(unsigned)((n_vertices + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(vertices), n_vertices, a, reinterpret_cast<const float4*>(sky_cubemap),
        reinterpret_cast<float4*>(colors));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "shading launch");
    return OCEAN_OK;
}

extern "C" int ocean_render_skybox(const float* sky_cubemap, int32_t sky_size, const float* view, const float* projection,
                                   int32_t width, int32_t height, float* image, void* stream)
{
    using namespace ocean::host;
    if (!sky_cubemap || !view || !projection || !image) return fail(OCEAN_ERR_INVALID, "NULL pointer");
    if (sky_size < 1 || sky_size > 16384) return fail(OCEAN_ERR_INVALID, "sky_size must be in [1, 16384]");
    if (width < 1 || height < 1 || width > 32768 || height > 32768)
        return fail(OCEAN_ERR_INVALID, "width and height must be in [1, 32768]");
    if ((reinterpret_cast<uintptr_t>(sky_cubemap) | reinterpret_cast<uintptr_t>(image)) % 16)
        return fail(OCEAN_ERR_INVALID, "sky_cubemap and image must be 16-byte aligned");
    // M = projection * mat4(mat3(view)), column-major, in double; then its inverse
    double R[16] = {0}, M[16], A[4][8];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) R[c * 4 + r] = view[c * 4 + r];
    R[15] = 1.0;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += (double)projection[k * 4 + r] * R[c * 4 + k];
            M[c * 4 + r] = s;
        }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) A[r][c] = c < 4 ? M[c * 4 + r] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; ++col) {   // Gauss-Jordan with partial pivoting
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
        if (!(std::fabs(A[piv][col]) > 1e-300)) return fail(OCEAN_ERR_INVALID, "projection * view is singular");
        for (int c = 0; c < 8; ++c) std::swap(A[col][c], A[piv][c]);
        const double p = A[col][col];
        for (int c = 0; c < 8; ++c) A[col][c] /= p;
        for (int r = 0; r < 4; ++r)
            if (r != col) {
                const double f = A[r][col];
                for (int c = 0; c < 8; ++c) A[r][c] -= f * A[col][c];
            }
    }
    SkyboxArgs a;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            a.m[c * 4 + r] = (float)A[r][4 + c];
            if (!std::isfinite(a.m[c * 4 + r])) return fail(OCEAN_ERR_INVALID, "view and projection must be finite");
        }
    a.S = sky_size;
    a.W = width;
    a.H = height;
    const long long n = (long long)width * height;
    k_skybox<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        a, reinterpret_cast<const float4*>(sky_cubemap), reinterpret_cast<float4*>(image));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "skybox launch");
    return OCEAN_OK;
}
