// ref_shaders.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own hot-path compute shaders (src/shader/*.glsl of
// diharaw/fft-ocean-waves, included unchanged from where they lie) and its
// reverse_bits() (src/main.cpp:29-64, extracted at build time) for the CPU,
// and restates the host orchestration of src/main.cpp that dispatches them:
//   tilde_h0_k()               main.cpp:553-583
//   generate_bit_reversed_indices() main.cpp:733-744
//   generate_twiddle_factors() main.cpp:711-729
//   tilde_h0_t()               main.cpp:587-608
//   butterfly_fft()            main.cpp:612-683
//   generate_normal_map()      main.cpp:687-707
// The outputs are the golden vectors the oracle is pinned to.  Built only where
// the reference sources exist (oracle/build_ref.py); output in oracle/_ref/.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "glsl_shim.hpp"

namespace ref_main {
#include "ref_reverse_bits.inc"
}

#define REF_SHADER_PROLOGUE                    \
    using namespace glsl;                      \
    static thread_local uvec3 gl_GlobalInvocationID;

namespace sh_h0k {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "tilde_h0_k_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_h0k

namespace sh_h0t {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "tilde_h0_t_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_h0t

namespace sh_twiddle {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "twiddle_factors_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_twiddle

namespace sh_butterfly {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "butterfly_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_butterfly

namespace sh_inversion {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "inversion_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_inversion

namespace sh_normal {
REF_SHADER_PROLOGUE
#include "glsl_begin.hpp"
#include "normal_map_cs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_normal

// The sky: sky_envmap_fs.glsl, which includes atmosphere.glsl.  The build
// recipe resolves that include to a copy in oracle/_ref/ whose `out vec3`
// parameters are C++ references (the one rewrite C++ needs); sky_envmap_fs.glsl
// itself is included unchanged.
namespace sh_sky {
using namespace glsl;
using glsl::abs;   // over the C library's ::abs overloads
#include "glsl_begin.hpp"
#include "sky_envmap_fs.glsl"
#include "glsl_end.hpp"
}  // namespace sh_sky

namespace {

int ilog2(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// glDispatchCompute(gx, gy, 1) with local size (lx, ly, 1).
template <class F>
void dispatch(int gx, int gy, int lx, int ly, F body)
{
    const int W = gx * lx, H = gy * ly;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) body((unsigned)x, (unsigned)y);
}

glsl::image2D img(float* p, int w, int h, int ch)
{
    glsl::image2D i;
    i.data = p;
    i.w    = w;
    i.h    = h;
    i.ch   = ch;
    return i;
}

}  // namespace

extern "C" {

// generate_bit_reversed_indices(): main.cpp:733-744.
void ref_bit_reversed(int N, int32_t* out)
{
    int32_t num_bits = ilog2(N);
    for (int i = 0; i < N; i++) out[i] = (int32_t)ref_main::reverse_bits(i, num_bits);
}

// generate_twiddle_factors(): main.cpp:711-729.  out: the RGBA32F image,
// width log2(N) x height N, row-major [y][stage][4].
void ref_twiddle(int N, const int32_t* bitrev, float* out)
{
    namespace S = sh_twiddle;
    const int lg = ilog2(N);
    S::u_N       = N;
    S::twiddle_factors       = img(out, lg, N, 4);
    S::ref_bit_reversed_ptr  = (S::indices_t*)malloc(sizeof(S::indices_t) + sizeof(int32_t) * (N + 1));
    memcpy(S::ref_bit_reversed_ptr->j, bitrev, sizeof(int32_t) * N);
    S::ref_bit_reversed_ptr->j[N] = 0;  // never read for a power-of-two N (top wing only below N-1)
    dispatch(lg, N / 32, 1, 32, [](unsigned x, unsigned y) {
        S::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
        S::main();
    });
    free(S::ref_bit_reversed_ptr);
    S::ref_bit_reversed_ptr = nullptr;
}

// tilde_h0_k(): main.cpp:553-583.  noise: four N x N R planes (the noise
// textures, CLAMP_TO_EDGE + NEAREST, main.cpp:1102-1116).  h0k, h0mk: RG32F.
void ref_h0(int N, int L, float A, float V, float wx, float wy, float l, const float* noise, float* h0k,
            float* h0mk)
{
    namespace S = sh_h0k;
    float n = __builtin_sqrtf(wx * wx + wy * wy);    // glm::normalize, main.cpp:555
    S::u_WindDirection = glsl::vec2(wx / n, wy / n);
    S::u_Amplitude     = A;
    S::u_WindSpeed     = V;
    S::u_SuppressFactor = l;
    S::u_N = N;
    S::u_L = L;
    glsl::sampler2D* s[4] = {&S::noise0, &S::noise1, &S::noise2, &S::noise3};
    for (int p = 0; p < 4; ++p) {
        s[p]->data   = noise + (size_t)p * N * N;
        s[p]->w      = N;
        s[p]->h      = N;
        s[p]->ch     = 1;
        s[p]->repeat = false;
    }
    S::tilde_h0k      = img(h0k, N, N, 2);
    S::tilde_h0minusk = img(h0mk, N, N, 2);
    dispatch(N / 32, N / 32, 32, 32, [](unsigned x, unsigned y) {
        S::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
        S::main();
    });
}

// tilde_h0_t(): main.cpp:587-608 with u_Time = t (FP32).  Outputs RGBA32F.
void ref_h0_t(int N, int L, float t, float* h0k, float* h0mk, float* dx, float* dy, float* dz)
{
    namespace S = sh_h0t;
    S::u_Time = t;
    S::u_N    = N;
    S::u_L    = L;
    S::tilde_h0k      = img(h0k, N, N, 2);
    S::tilde_h0minusk = img(h0mk, N, N, 2);
    S::tilde_hkt_dx   = img(dx, N, N, 4);
    S::tilde_hkt_dy   = img(dy, N, N, 4);
    S::tilde_hkt_dz   = img(dz, N, N, 4);
    dispatch(N / 32, N / 32, 32, 32, [](unsigned x, unsigned y) {
        S::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
        S::main();
    });
}

// butterfly_fft(src, dst): main.cpp:612-683.  spectrum (RGBA32F) is ping-pong
// slot 0 and is overwritten, pong is slot 1, dst is the R32F result.
void ref_butterfly_fft(int N, float* twiddle, float* spectrum, float* pong, float* dst)
{
    namespace B = sh_butterfly;
    namespace I = sh_inversion;
    const int lg = ilog2(N);
    B::twiddle_factors = img(twiddle, lg, N, 4);
    B::pingpong0       = img(spectrum, N, N, 4);
    B::pingpong1       = img(pong, N, N, 4);
    int pingpong = 0;
    for (int dir = 0; dir < 2; ++dir)
        for (int i = 0; i < lg; i++) {
            B::u_PingPong  = pingpong;
            B::u_Direction = dir;
            B::u_Stage     = i;
            dispatch(N / 32, N / 32, 32, 32, [](unsigned x, unsigned y) {
                B::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
                B::main();
            });
            pingpong++;
            pingpong %= 2;
        }
    I::u_PingPong   = pingpong;
    I::u_N          = N;
    I::displacement = img(dst, N, N, 1);
    I::pingpong0    = img(spectrum, N, N, 4);
    I::pingpong1    = img(pong, N, N, 4);
    dispatch(N / 32, N / 32, 32, 32, [](unsigned x, unsigned y) {
        I::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
        I::main();
    });
}

// generate_normal_map(): main.cpp:687-707, s_HeightMap = dy sampled with
// REPEAT + NEAREST (the pinned sampler state).  normal: RGBA32F.
void ref_normal_map(int N, const float* dy, float* normal)
{
    namespace S = sh_normal;
    S::u_N                = N;
    S::s_HeightMap.data   = dy;
    S::s_HeightMap.w      = N;
    S::s_HeightMap.h      = N;
    S::s_HeightMap.ch     = 1;
    S::s_HeightMap.repeat = true;
    S::normal_map         = img(normal, N, N, 4);
    dispatch(N / 32, N / 32, 32, 32, [](unsigned x, unsigned y) {
        S::gl_GlobalInvocationID = glsl::uvec3(x, y, 0);
        S::main();
    });
}

// render_envmap(): main.cpp:500-523 with SkyModel::set_render_uniforms()
// (:149-158).  The rasteriser's part is restated: the fragment of texel
// (i, j) of face f of the capture views (:1463-1470) sees the cube-surface
// point through the texel centre, so PS_IN_WorldPos is that point.
// prm: camera[3], sun_direction[3], earth_pos[3], beta_r[3], mie_g,
// sun_intensity.  out [6][S][S][4].
void ref_sky_envmap(const float* prm, int S, const float* trans, const float* insc, float* out)
{
    namespace K = sh_sky;
    K::u_CameraPos             = glsl::vec3(prm[0], prm[1], prm[2]);
    K::SUN_DIR                 = glsl::vec3(prm[3], prm[4], prm[5]);
    K::EARTH_POS               = glsl::vec3(prm[6], prm[7], prm[8]);
    K::betaR                   = glsl::vec3(prm[9], prm[10], prm[11]);
    K::mieG                    = prm[12];
    K::SUN_INTENSITY           = prm[13];
    K::s_Transmittance.data    = trans;
    K::s_Transmittance.w       = 256;
    K::s_Transmittance.h       = 64;
    K::s_Transmittance.ch      = 4;
    K::s_Transmittance.linear  = true;
    K::s_Inscatter.data        = insc;
    K::s_Inscatter.w           = 256;
    K::s_Inscatter.h           = 128;
    K::s_Inscatter.d           = 32;
    for (int f = 0; f < 6; ++f)
        for (int j = 0; j < S; ++j)
            for (int i = 0; i < S; ++i) {
                const float sc = 2.0f * (((float)i + 0.5f) / (float)S) - 1.0f;
                const float tc = 2.0f * (((float)j + 0.5f) / (float)S) - 1.0f;
                glsl::vec3  p;
                switch (f) {
                case 0: p = glsl::vec3(1.0f, -tc, -sc); break;
                case 1: p = glsl::vec3(-1.0f, -tc, sc); break;
                case 2: p = glsl::vec3(sc, 1.0f, tc); break;
                case 3: p = glsl::vec3(sc, -1.0f, -tc); break;
                case 4: p = glsl::vec3(sc, -tc, 1.0f); break;
                default: p = glsl::vec3(-sc, -tc, -1.0f); break;
                }
                K::PS_IN_WorldPos = p;
                K::main();
                float* o = out + 4 * (((size_t)f * S + j) * S + i);
                o[0]     = K::PS_OUT_Color.x;
                o[1]     = K::PS_OUT_Color.y;
                o[2]     = K::PS_OUT_Color.z;
                o[3]     = K::PS_OUT_Color.w;
            }
}

}  // extern "C"
