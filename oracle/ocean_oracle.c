/*
 * ocean_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of diharaw/fft-ocean-waves' per-frame ocean path, used as the
 * checker for the CUDA library and as the timed CPU baseline.  Nothing in the
 * product links this file: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.
 *
 * Two restatements live here:
 *
 *   orc_*   FP64 oracle.  Follows the shader arithmetic with every quantity in
 *           double, the phase w*t included, and the 2-D inverse transform done
 *           by an FP64 radix-2 FFT.  This is the reference the GPU results are
 *           graded against (relative L2 <= 1e-5 per field).
 *
 *   port_*  FP32 port of the reference's *algorithm*: the same passes the GL
 *           demo dispatches per frame (spectrum pass, 2*log2(N) table-driven
 *           radix-2 ping-pong passes per field, inversion, Sobel normal map),
 *           each pass a full-grid sweep parallelised with OpenMP.  It is the
 *           CPU baseline bench.py times, and a second parity point.
 *
 * Pinned semantics (the reference leaves these undefined or quirky):
 *   Q1  tilde_h0_t_cs.glsl:42-48 `conjugate()` returns its argument unchanged.
 *       Default here is the textbook conj(h0(-k)); literal_conj=1 reproduces
 *       the shader (no conjugation).
 *   Q3  tilde_h0_k_cs.glsl:76-77,44: normalize(k) at k=0 is NaN.  The DC mode
 *       is pinned to h0 = 0.
 *   Q4  pow(x, 2.0) with x<0 is undefined in GLSL (tilde_h0_k_cs.glsl:44);
 *       (k^.w^)^2 is used.
 *   Q7  normal_map_cs.glsl:37-44 samples the height map through a sampler
 *       whose filter/wrap are left to the GL framework.  Pinned: integer texel
 *       taps with periodic wrap.
 *   Q8  Outputs are Dx*lambda, Dy, Dz*lambda (grid_tes.glsl:60-62 applies
 *       lambda with a minus sign at render time; the renderer subtracts), and
 *       the Jacobian of p = x - (Dx, Dz) with periodic central differences of
 *       spacing L/N goes in normal.w (a build addition; the reference's
 *       normal.w is 1).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

typedef struct orc_params {
    int32_t N;
    int32_t literal_conj;
    double L;           /* patch length in metres (the shader's u_L, an int there) */
    double amplitude;   /* u_Amplitude */
    double wind_speed;  /* u_WindSpeed */
    double wind_x;      /* u_WindDirection, normalised here as main.cpp:555 does */
    double wind_y;
    double choppiness;  /* lambda (grid_tes.glsl:61-62 u_Choppiness) */
    double suppression; /* u_SuppressFactor, small-wave cutoff l in metres */
    double gravity;     /* g = 9.81 in the shaders */
} orc_params;

static int ilog2i(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

/* ------------------------------------------------------------------------- */
/* FP64 oracle                                                               */
/* ------------------------------------------------------------------------- */

/* Phillips amplitude a(k) = clamp(sqrt(P(k))/sqrt(2), -4000, 4000) of
 * tilde_h0_k_cs.glsl:35-45,76-88, in double.  P(-k) == P(k) with (k^.w^)^2,
 * so h0minusk uses the same amplitude (tilde_h0_k_cs.glsl:88). */
static double orc_amp(const orc_params* p, double kx, double kz, double wx, double wy, int* clamped)
{
    double kl  = sqrt(kx * kx + kz * kz);
    double km  = kl < 0.00001 ? 0.00001 : kl;           /* :81-82 */
    double k2  = km * km;                               /* :84 */
    double Lp  = p->wind_speed * p->wind_speed / p->gravity; /* :78 */
    double sup = exp(-k2 * p->suppression * p->suppression); /* :35-38 */
    double kd  = (kx * wx + kz * wy) / kl;              /* dot(normalize(k), w) */
    double P   = p->amplitude * exp(-1.0 / (k2 * Lp * Lp)) * (kd * kd) * sup / (k2 * k2); /* :42-45 */
    double a   = sqrt(P) / sqrt(2.0);                   /* :87 */
    if (clamped) *clamped = a > 4000.0;
    return a > 4000.0 ? 4000.0 : a;                     /* clamp(.., -4000, 4000); a >= 0 */
}

/* Number of modes the +-4000 clamp is active on (diagnostic for tests). */
int orc_count_clamped(const orc_params* p)
{
    int N = p->N, n = 0;
    double wn = sqrt(p->wind_x * p->wind_x + p->wind_y * p->wind_y);
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            double ix = x - N / 2.0, iz = y - N / 2.0;
            if (ix == 0.0 && iz == 0.0) continue;
            int c = 0;
            orc_amp(p, 2.0 * ORC_PI * ix / p->L, 2.0 * ORC_PI * iz / p->L, p->wind_x / wn, p->wind_y / wn, &c);
            n += c;
        }
    return n;
}

/* h0 initialisation: tilde_h0_k_cs.glsl:51-68 (Box-Muller) and :74-93.
 * noise: four N*N planes [plane][y][x] of U(0,1] values (the four noise
 * textures sampled at texel (x, y)).  h0: N*N*4 doubles per mode
 * (h0k.re, h0k.im, h0minusk.re, h0minusk.im), row-major [y][x]. */
void orc_h0(const orc_params* p, const float* noise, double* h0)
{
    int    N  = p->N;
    size_t NN = (size_t)N * N;
    double wn = sqrt(p->wind_x * p->wind_x + p->wind_y * p->wind_y);
    double wx = p->wind_x / wn, wy = p->wind_y / wn;    /* main.cpp:555 */
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            size_t i  = (size_t)y * N + x;
            double ix = x - N / 2.0, iz = y - N / 2.0;  /* :76 */
            double kx = 2.0 * ORC_PI * ix / p->L, kz = 2.0 * ORC_PI * iz / p->L; /* :77 */
            double a  = (ix == 0.0 && iz == 0.0) ? 0.0 : orc_amp(p, kx, kz, wx, wy, NULL); /* Q3 */
            double n[4];
            for (int q = 0; q < 4; ++q) {
                double v = noise[q * NN + i];
                n[q]     = v < 0.001 ? 0.001 : (v > 1.0 ? 1.0 : v); /* :55-58 */
            }
            double u0 = 2.0 * ORC_PI * n[0], v0 = sqrt(-2.0 * log(n[1])); /* :60-61 */
            double u1 = 2.0 * ORC_PI * n[2], v1 = sqrt(-2.0 * log(n[3])); /* :62-63 */
            h0[4 * i + 0] = v0 * cos(u0) * a;            /* :92 rnd.xy * h0k */
            h0[4 * i + 1] = v0 * sin(u0) * a;
            h0[4 * i + 2] = v1 * cos(u1) * a;            /* :93 rnd.zw * h0minusk */
            h0[4 * i + 3] = v1 * sin(u1) * a;
        }
}

/* Per-frame spectra: tilde_h0_t_cs.glsl:70-131 in double.
 * spec: 3 fields [f][y][x][re,im], f = 0 (Dx), 1 (Dy, height), 2 (Dz). */
void orc_spectrum(const orc_params* p, const double* h0, double t, double* spec)
{
    int    N  = p->N;
    size_t NN = (size_t)N * N;
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            size_t i  = (size_t)y * N + x;
            double ix = x - N / 2.0, iz = y - N / 2.0;  /* :72 */
            double kx = 2.0 * ORC_PI * ix / p->L, kz = 2.0 * ORC_PI * iz / p->L; /* :73 */
            double km = sqrt(kx * kx + kz * kz);
            if (km < 0.00001) km = 0.00001;             /* :76-77 */
            double w  = sqrt(p->gravity * km);          /* :79 */
            double c  = cos(w * t), s = sin(w * t);     /* :96-97 (FP64 phase) */
            double ar = h0[4 * i + 0], ai = h0[4 * i + 1];
            double br = h0[4 * i + 2], bi = h0[4 * i + 3];
            if (!p->literal_conj) bi = -bi;             /* Q1: conj(h0(-k)) */
            /* hy = a e^{iwt} + b e^{-iwt} (:110) */
            double hr = ar * c - ai * s + br * c + bi * s;
            double hi = ar * s + ai * c - br * s + bi * c;
            /* hx = (-i kx/|k|) hy (:113-118), hz = (-i kz/|k|) hy (:121-126) */
            double fx = -kx / km, fz = -kz / km;
            spec[2 * (0 * NN + i) + 0] = -fx * hi;
            spec[2 * (0 * NN + i) + 1] = fx * hr;
            spec[2 * (1 * NN + i) + 0] = hr;
            spec[2 * (1 * NN + i) + 1] = hi;
            spec[2 * (2 * NN + i) + 0] = -fz * hi;
            spec[2 * (2 * NN + i) + 1] = fz * hr;
        }
}

/* In-place radix-2 FFT of n complex doubles (interleaved), exponent sign `sg`.
 * Unnormalised. */
static void orc_fft1(double* a, int n, int stride, int sg)
{
    int lg = ilog2i(n);
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b) r |= ((i >> b) & 1) << (lg - 1 - b);
        if (r > i) {
            double* u = a + 2 * (size_t)i * stride;
            double* v = a + 2 * (size_t)r * stride;
            double  t0 = u[0], t1 = u[1];
            u[0] = v[0]; u[1] = v[1]; v[0] = t0; v[1] = t1;
        }
    }
    for (int h = 1; h < n; h <<= 1)
        for (int k = 0; k < h; ++k) {
            double ang = sg * ORC_PI * k / h;
            double wr = cos(ang), wi = sin(ang);
            for (int i = k; i < n; i += 2 * h) {
                double* u = a + 2 * (size_t)i * stride;
                double* v = a + 2 * (size_t)(i + h) * stride;
                double  br = v[0] * wr - v[1] * wi, bi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - br; v[1] = u[1] - bi;
                u[0] += br; u[1] += bi;
            }
        }
}

/* In-place 2-D FFT of an N x N complex field [y][x][2]: every row, then every
 * column.  Lines are independent and run in parallel; a column is gathered
 * into a contiguous buffer, transformed with the same arithmetic as in place,
 * and scattered back, so the result does not depend on the thread count. */
static void orc_fft2(double* a, int N, int sg)
{
#pragma omp parallel
    {
        double* col = (double*)malloc(2 * (size_t)N * sizeof(double));
#pragma omp for schedule(static)
        for (int y = 0; y < N; ++y) orc_fft1(a + 2 * (size_t)y * N, N, 1, sg);
#pragma omp for schedule(static)
        for (int x = 0; x < N; ++x) {
            for (int y = 0; y < N; ++y) {
                col[2 * y]     = a[2 * ((size_t)y * N + x)];
                col[2 * y + 1] = a[2 * ((size_t)y * N + x) + 1];
            }
            orc_fft1(col, N, 1, sg);
            for (int y = 0; y < N; ++y) {
                a[2 * ((size_t)y * N + x)]     = col[2 * y];
                a[2 * ((size_t)y * N + x) + 1] = col[2 * y + 1];
            }
        }
        free(col);
    }
}

/* Re of the unnormalised 2-D inverse DFT (positive exponent) that the
 * butterfly passes compute (butterfly_cs.glsl:54-132), followed by the
 * (-1)^(x+y)/N^2 of inversion_cs.glsl:29-41.  spec_f: one field [y][x][2]. */
void orc_ifft2_real(int N, const double* spec_f, double* d)
{
    size_t  NN = (size_t)N * N;
    double* a  = (double*)malloc(2 * NN * sizeof(double));
    memcpy(a, spec_f, 2 * NN * sizeof(double));
    orc_fft2(a, N, +1);
    double inv = 1.0 / ((double)N * N);
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            double perm = ((x + y) & 1) ? -1.0 : 1.0;
            d[(size_t)y * N + x] = perm * a[2 * ((size_t)y * N + x)] * inv;
        }
    free(a);
}

/* Output stage: lambda scaling (Q8), Sobel normal on Dy (normal_map_cs.glsl:
 * 37-53, Q7), Jacobian (Q8).  raw: 3 planes (Dx, Dy, Dz) before lambda.
 * nj: N*N*4 (nx, ny, nz, J). */
void orc_finish(const orc_params* p, const double* raw, double* dx, double* dy, double* dz, double* nj)
{
    int    N  = p->N;
    size_t NN = (size_t)N * N;
    double lam = p->choppiness;
    for (size_t i = 0; i < NN; ++i) {
        dx[i] = lam * raw[i];
        dy[i] = raw[NN + i];
        dz[i] = lam * raw[2 * NN + i];
    }
    double inv2d = (double)N / (2.0 * p->L);            /* 1 / (2 * L/N) */
#define AT(arr, xx, yy) arr[(size_t)(((yy) + N) % N) * N + (size_t)(((xx) + N) % N)]
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            double z0 = AT(dy, x - 1, y - 1), z1 = AT(dy, x, y - 1), z2 = AT(dy, x + 1, y - 1);
            double z3 = AT(dy, x - 1, y), z4 = AT(dy, x + 1, y);
            double z5 = AT(dy, x - 1, y + 1), z6 = AT(dy, x, y + 1), z7 = AT(dy, x + 1, y + 1);
            double nz = z0 + 2 * z1 + z2 - z5 - 2 * z6 - z7; /* :49 */
            double nx = z0 + 2 * z3 + z5 - z2 - 2 * z4 - z7; /* :50 */
            double ny = 1.0;
            double rn = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
            double dxx = (AT(dx, x + 1, y) - AT(dx, x - 1, y)) * inv2d;
            double dxz = (AT(dx, x, y + 1) - AT(dx, x, y - 1)) * inv2d;
            double dzx = (AT(dz, x + 1, y) - AT(dz, x - 1, y)) * inv2d;
            double dzz = (AT(dz, x, y + 1) - AT(dz, x, y - 1)) * inv2d;
            size_t i = (size_t)y * N + x;
            nj[4 * i + 0] = nx * rn;
            nj[4 * i + 1] = ny * rn;
            nj[4 * i + 2] = nz * rn;
            nj[4 * i + 3] = (1.0 - dxx) * (1.0 - dzz) - dxz * dzx;
        }
#undef AT
}

/* One full frame from h0 at time t (double). */
void orc_update(const orc_params* p, const double* h0, double t, double* dx, double* dy, double* dz, double* nj)
{
    size_t  NN   = (size_t)p->N * p->N;
    double* spec = (double*)malloc(6 * NN * sizeof(double));
    double* raw  = (double*)malloc(3 * NN * sizeof(double));
    orc_spectrum(p, h0, t, spec);
    for (int f = 0; f < 3; ++f) orc_ifft2_real(p->N, spec + 2 * f * NN, raw + f * NN);
    orc_finish(p, raw, dx, dy, dz, nj);
    free(spec);
    free(raw);
}

/* FP64 adjoint of orc_update's displacement outputs (Dx, Dy, Dz) over T
 * frames.  The loss gradient is given per frame as g_dx, g_dy, g_dz
 * (T*N*N each, NULL = zero).  Outputs:
 *   dh0    N*N*4: dL/dh0 per mode in the complex convention dL/dRe + i dL/dIm
 *          for (h0k, h0minusk), summed over the frames;
 *   grads  [0] dL/dA, [1] dL/dV, [2] dL/dtheta (wind direction angle),
 *          [3] dL/dlambda.  The suppression length l, L and g are constants;
 *          modes on the +-4000 clamp and the DC mode do not depend on A, V,
 *          theta.
 * Steps per frame: forward 2-D DFT of (-1)^(x+y)/N^2 * g (the transpose of
 * the inverse butterfly network + inversion), transpose of the choppy
 * multiply, conjugate phase rotation. */
void orc_backward(const orc_params* p, const double* h0, const double* times, int T, const double* g_dx,
                  const double* g_dy, const double* g_dz, double* dh0, double* grads)
{
    int     N  = p->N;
    size_t  NN = (size_t)N * N;
    double* G  = (double*)malloc(3 * 2 * NN * sizeof(double));
    double  lam = p->choppiness, dlam = 0.0;
    memset(dh0, 0, NN * 4 * sizeof(double));
    for (int j = 0; j < T; ++j) {
        const double* gs[3] = { g_dx ? g_dx + j * NN : NULL, g_dy ? g_dy + j * NN : NULL, g_dz ? g_dz + j * NN : NULL };
        for (int f = 0; f < 3; ++f) {
            double* a = G + f * 2 * NN;
            for (int y = 0; y < N; ++y)
                for (int x = 0; x < N; ++x) {
                    size_t i = (size_t)y * N + x;
                    double s = (((x + y) & 1) ? -1.0 : 1.0) / ((double)N * N);
                    a[2 * i]     = gs[f] ? s * gs[f][i] : 0.0;
                    a[2 * i + 1] = 0.0;
                }
            orc_fft2(a, N, -1);
        }
        double t = times[j];
#pragma omp parallel for schedule(static) reduction(+ : dlam)
        for (int y = 0; y < N; ++y)
            for (int x = 0; x < N; ++x) {
                size_t i  = (size_t)y * N + x;
                double kx = 2.0 * ORC_PI * (x - N / 2.0) / p->L, kz = 2.0 * ORC_PI * (y - N / 2.0) / p->L;
                double km = sqrt(kx * kx + kz * kz);
                if (km < 0.00001) km = 0.00001;
                double w = sqrt(p->gravity * km), c = cos(w * t), s = sin(w * t);
                double gxr = G[2 * i], gxi = G[2 * i + 1];
                double gyr = G[2 * (NN + i)], gyi = G[2 * (NN + i) + 1];
                double gzr = G[2 * (2 * NN + i)], gzi = G[2 * (2 * NN + i) + 1];
                double ux = kx / km, uz = kz / km;           /* conj(a_x) = +i ux, conj(a_z) = +i uz */
                double tr = gyr + lam * (-ux * gxi - uz * gzi);
                double ti = gyi + lam * (ux * gxr + uz * gzr);
                /* dh0k += e^{-iwt} Gtot */
                dh0[4 * i + 0] += tr * c + ti * s;
                dh0[4 * i + 1] += ti * c - tr * s;
                if (!p->literal_conj) { /* dh0mk += conj(Gtot) e^{-iwt} */
                    dh0[4 * i + 2] += tr * c - ti * s;
                    dh0[4 * i + 3] += -ti * c - tr * s;
                } else {                /* dh0mk += e^{+iwt} Gtot */
                    dh0[4 * i + 2] += tr * c - ti * s;
                    dh0[4 * i + 3] += ti * c + tr * s;
                }
                /* dlambda: Re(conj(Gx) Xx + conj(Gz) Xz), Xx = -i ux Xy, Xz = -i uz Xy */
                double ar = h0[4 * i], ai = h0[4 * i + 1], br = h0[4 * i + 2], bi = h0[4 * i + 3];
                if (!p->literal_conj) bi = -bi;
                double hr = ar * c - ai * s + br * c + bi * s;
                double hi = ar * s + ai * c - br * s + bi * c;
                double xxr = ux * hi, xxi = -ux * hr, xzr = uz * hi, xzi = -uz * hr;
                dlam += gxr * xxr + gxi * xxi + gzr * xzr + gzi * xzi;
            }
    }
    free(G);
    /* chain through a(k) = clamp(sqrt(P)/sqrt2): h0 = xi * a with fixed noise xi */
    double wn = sqrt(p->wind_x * p->wind_x + p->wind_y * p->wind_y);
    double wx = p->wind_x / wn, wy = p->wind_y / wn;
    double Lp = p->wind_speed * p->wind_speed / p->gravity;
    double dA = 0.0, dV = 0.0, dth = 0.0;
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            double ix = x - N / 2.0, iz = y - N / 2.0;
            if (ix == 0.0 && iz == 0.0) continue;
            size_t i  = (size_t)y * N + x;
            double kx = 2.0 * ORC_PI * ix / p->L, kz = 2.0 * ORC_PI * iz / p->L;
            int    cl = 0;
            double a  = orc_amp(p, kx, kz, wx, wy, &cl);
            if (cl || a == 0.0) continue;
            double Q = dh0[4 * i] * h0[4 * i] + dh0[4 * i + 1] * h0[4 * i + 1] + dh0[4 * i + 2] * h0[4 * i + 2] +
                       dh0[4 * i + 3] * h0[4 * i + 3];      /* a * dL/da */
            double kl = sqrt(kx * kx + kz * kz);
            double cdir = (kx * wx + kz * wy) / kl, cperp = (-kx * wy + kz * wx) / kl;
            dA  += Q / (2.0 * p->amplitude);
            dV  += Q * 2.0 * p->wind_speed / (p->gravity * kl * kl * Lp * Lp * Lp);
            dth += Q * cperp / cdir;
        }
    grads[0] = dA;
    grads[1] = dV;
    grads[2] = dth;
    grads[3] = dlam;
}

/* Displaced grid (the consumer of the maps).
 *
 * The grid of main.cpp:748-824 (generate_grid(GRID_SIZE = 1024, GRID_UV_SCALE
 * = 64), :20-21): n squares per side, (n+1)^2 vertices at (x, 0, z) for
 * integer x, z in [-n/2, n/2], texcoord ((x + n/2)/n, (z + n/2)/n) * scale,
 * two triangles per square with indices (i0, i1, i2), (i2, i1, i1 + 1),
 * i0 = (n+1) z' + x', i1 = i0 + n + 1, i2 = i0 + 1.
 *
 * orc_displace_grid: the tessellation evaluation stage at the grid's own
 * vertices (grid_tes.glsl:55-66): y += Dy(uv) * disp_scale, x -= Dx(uv),
 * z -= Dz(uv), normal = normal_map(uv).xyz, with the maps sampled bilinearly
 * with REPEAT wrap (texel centres at (i + 0.5)/N).  dx and dz are the build's
 * outputs, which already carry lambda (the shader's u_Choppiness factor).
 * out: (n+1)^2 * 8 = position xyz, normal xyz, texcoord uv.
 *
 * orc_tess_levels: the tessellation control stage (grid_tcs.glsl:27-59) per
 * triangle: outer[0] = level(d1, d2), outer[1] = level(d2, d0), outer[2] =
 * level(d0, d1), inner = outer[2], level of the mean eye distance: 20 up to
 * 10, 10 up to 20, 5 up to 30, else 1.  out: 2 n^2 * 4. */
static double orc_bilinear(const double* m, int N, int stride, int comp, double u, double v)
{
    double sx = u * N - 0.5, sy = v * N - 0.5;
    double fx = floor(sx), fy = floor(sy);
    double ax = sx - fx, ay = sy - fy;
    long   x0 = (long)fx, y0 = (long)fy;
    long   xa = ((x0 % N) + N) % N, xb = (xa + 1) % N;
    long   ya = ((y0 % N) + N) % N, yb = (ya + 1) % N;
#define M(yy, xx) m[((size_t)(yy) * N + (xx)) * stride + comp]
    double top = M(ya, xa) * (1.0 - ax) + M(ya, xb) * ax;
    double bot = M(yb, xa) * (1.0 - ax) + M(yb, xb) * ax;
#undef M
    return top * (1.0 - ay) + bot * ay;
}

void orc_displace_grid(int N, const double* dx, const double* dy, const double* dz, const double* nj, int n,
                       double uv_scale, double disp_scale, double* out)
{
    int h = n / 2;
    for (int zi = 0; zi <= n; ++zi)
        for (int xi = 0; xi <= n; ++xi) {
            double  u = (double)xi / n * uv_scale, v = (double)zi / n * uv_scale;
            double* o = out + 8 * ((size_t)zi * (n + 1) + xi);
            o[0] = (double)(xi - h) - orc_bilinear(dx, N, 1, 0, u, v);
            o[1] = orc_bilinear(dy, N, 1, 0, u, v) * disp_scale;
            o[2] = (double)(zi - h) - orc_bilinear(dz, N, 1, 0, u, v);
            for (int c = 0; c < 3; ++c) o[3 + c] = orc_bilinear(nj, N, 4, c, u, v);
            o[6] = u;
            o[7] = v;
        }
}

static double orc_level(double d0, double d1)
{
    double avg = (d0 + d1) / 2.0;
    return avg <= 10.0 ? 20.0 : avg <= 20.0 ? 10.0 : avg <= 30.0 ? 5.0 : 1.0;
}

void orc_tess_levels(int n, const double* cam, double* out)
{
    int h = n / 2;
    for (int zi = 0; zi < n; ++zi)
        for (int xi = 0; xi < n; ++xi) {
            /* triangle A: (x, z), (x, z+1), (x+1, z); triangle B: (x+1, z), (x, z+1), (x+1, z+1) */
            double px[2][3] = {{xi - h, xi - h, xi + 1 - h}, {xi + 1 - h, xi - h, xi + 1 - h}};
            double pz[2][3] = {{zi - h, zi + 1 - h, zi - h}, {zi - h, zi + 1 - h, zi + 1 - h}};
            for (int tr = 0; tr < 2; ++tr) {
                double d[3];
                for (int k = 0; k < 3; ++k) {
                    double ex = cam[0] - px[tr][k], ey = cam[1], ez = cam[2] - pz[tr][k];
                    d[k] = sqrt(ex * ex + ey * ey + ez * ez);
                }
                double* o = out + 4 * (2 * ((size_t)zi * n + xi) + tr);
                o[0] = orc_level(d[1], d[2]);
                o[1] = orc_level(d[2], d[0]);
                o[2] = orc_level(d[0], d[1]);
                o[3] = o[2];
            }
        }
}

/* Ocean shading (ocean_fs.glsl:11-37) at the displaced grid's vertices:
 * N = the vertex normal as given (not renormalised, as the shader uses the
 * interpolated FS_IN_Normal), V = normalize(camera - P), R = reflect(-V, N),
 * L = -sun_direction, F = F0 + (1 - F0)(1 - max(N.V, 0))^5 with F0 = 0.04,
 * albedo = mix(sea_color, sky(R), F), color = max(N.L, 0) * albedo, then the
 * Reinhard tonemap c / (c + 1) and gamma 1/2.2.  sky: a cube map of 6 faces
 * (+X, -X, +Y, -Y, +Z, -Z) of S x S RGBA texels, face and face coordinates
 * chosen by the major axis of R as in the OpenGL specification's cube-map
 * table, bilinear within the face with clamp to edge.
 * vert: n * 8 (position, normal, texcoord); out: n * 4 (RGB, 1). */
static void orc_cube_sample(const double* sky, int S, const double* r, double* rgb)
{
    double ax = fabs(r[0]), ay = fabs(r[1]), az = fabs(r[2]), ma, sc, tc;
    int    face;
    if (ax >= ay && ax >= az) {
        face = r[0] >= 0 ? 0 : 1; ma = ax; sc = r[0] >= 0 ? -r[2] : r[2]; tc = -r[1];
    } else if (ay >= az) {
        face = r[1] >= 0 ? 2 : 3; ma = ay; sc = r[0]; tc = r[1] >= 0 ? r[2] : -r[2];
    } else {
        face = r[2] >= 0 ? 4 : 5; ma = az; sc = r[2] >= 0 ? r[0] : -r[0]; tc = -r[1];
    }
    double s = 0.5 * (sc / ma + 1.0) * S - 0.5, t = 0.5 * (tc / ma + 1.0) * S - 0.5;
    double fs = floor(s), ft = floor(t), ws = s - fs, wt = t - ft;
    int    s0 = (int)fs, t0 = (int)ft;
    int    sa = s0 < 0 ? 0 : (s0 > S - 1 ? S - 1 : s0), sb = s0 + 1 < 0 ? 0 : (s0 + 1 > S - 1 ? S - 1 : s0 + 1);
    int    ta = t0 < 0 ? 0 : (t0 > S - 1 ? S - 1 : t0), tb = t0 + 1 < 0 ? 0 : (t0 + 1 > S - 1 ? S - 1 : t0 + 1);
    const double* f = sky + (size_t)face * S * S * 4;
    for (int c = 0; c < 3; ++c) {
        double top = f[((size_t)ta * S + sa) * 4 + c] * (1 - ws) + f[((size_t)ta * S + sb) * 4 + c] * ws;
        double bot = f[((size_t)tb * S + sa) * 4 + c] * (1 - ws) + f[((size_t)tb * S + sb) * 4 + c] * ws;
        rgb[c] = top * (1 - wt) + bot * wt;
    }
}

/* render_skybox(): sky_vs.glsl + sky_fs.glsl per pixel centre of a W x H
 * framebuffer (row 0 at the bottom): minv = inverse(projection *
 * mat4(mat3(view))) column-major; the far-plane point's direction; the cube
 * map there; c / (c + 1), gamma 1/2.2 (sky_fs.glsl:14-20). */
void orc_skybox(const double* sky, int S, const double* minv, int W, int H, double* out)
{
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double cx = 2.0 * (x + 0.5) / W - 1.0, cy = 2.0 * (y + 0.5) / H - 1.0, d[4], rgb[3];
            for (int i = 0; i < 4; ++i) d[i] = minv[i] * cx + minv[4 + i] * cy + minv[8 + i] + minv[12 + i];
            double r[3] = {d[0] / d[3], d[1] / d[3], d[2] / d[3]};
            orc_cube_sample(sky, S, r, rgb);
            double* o = out + 4 * ((size_t)y * W + x);
            for (int c = 0; c < 3; ++c) o[c] = pow(rgb[c] / (rgb[c] + 1.0), 1.0 / 2.2);
            o[3] = 1.0;
        }
}

void orc_shade(const double* vert, long n, const double* cam, const double* sun, const double* sea, const double* sky,
               int S, double* out)
{
    for (long i = 0; i < n; ++i) {
        const double* p = vert + 8 * i;
        const double* N = p + 3;
        double V[3] = {cam[0] - p[0], cam[1] - p[1], cam[2] - p[2]};
        double vl = sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
        for (int c = 0; c < 3; ++c) V[c] /= vl;
        double nv = N[0] * V[0] + N[1] * V[1] + N[2] * V[2];
        double R[3] = {2.0 * nv * N[0] - V[0], 2.0 * nv * N[1] - V[1], 2.0 * nv * N[2] - V[2]};
        double sky_rgb[3];
        orc_cube_sample(sky, S, R, sky_rgb);
        double F  = 0.04 + 0.96 * pow(1.0 - (nv > 0 ? nv : 0.0), 5.0);
        double nl = -(N[0] * sun[0] + N[1] * sun[1] + N[2] * sun[2]);
        if (nl < 0) nl = 0;
        for (int c = 0; c < 3; ++c) {
            double col = nl * (sea[c] * (1.0 - F) + sky_rgb[c] * F);
            col        = col / (col + 1.0);
            out[4 * i + c] = pow(col, 1.0 / 2.2);
        }
        out[4 * i + 3] = 1.0;
    }
}

/* FFT tables of the reference, restated in double.
 * Bit reversal over log2(N) bits: main.cpp:35-64 (reverse_bits) as used by
 * generate_bit_reversed_indices() main.cpp:733-744. */
void orc_bit_reversed(int N, int32_t* out)
{
    int lg = ilog2i(N);
    for (int i = 0; i < N; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b) r |= ((i >> b) & 1) << (lg - 1 - b);
        out[i] = r;
    }
}

/* Butterfly table twiddle_factors_cs.glsl:34-69: table[s][y] =
 * (Re w, Im w, index p, index q) for stage s < log2(N), row y < N,
 * w = exp(+2 pi i k / N), k = (y * N / 2^(s+1)) mod N.  out: log2N*N*4. */
void orc_twiddle_table(int N, double* out)
{
    int      lg = ilog2i(N);
    int32_t* br = (int32_t*)malloc(sizeof(int32_t) * N);
    orc_bit_reversed(N, br);
    for (int s = 0; s < lg; ++s)
        for (int y = 0; y < N; ++y) {
            long   span = 1L << s;
            double k    = fmod((double)y * ((double)N / (double)(2L << s)), (double)N); /* :37 */
            int    top  = (y % (2L << s)) < span;                                        /* :44 */
            double* o   = out + 4 * ((size_t)s * N + y);
            o[0] = cos(2.0 * ORC_PI * k / N);
            o[1] = sin(2.0 * ORC_PI * k / N);
            if (s == 0) {                                                                /* :50-58 */
                o[2] = top ? br[y] : br[y - 1];
                o[3] = top ? br[y + 1] : br[y];
            } else {                                                                     /* :60-68 */
                o[2] = top ? y : y - span;
                o[3] = top ? y + span : y;
            }
        }
    free(br);
}

/* ------------------------------------------------------------------------- */
/* FP32 port of the reference algorithm (CPU baseline)                        */
/* ------------------------------------------------------------------------- */

typedef struct port_state {
    orc_params p;
    int        N, lg;
    float*     h0;      /* N*N*4 */
    float*     tw;      /* lg*N*4 (w.re, w.im, p, q) */
    float*     spec;    /* 3 fields N*N*2 (the RGBA32F spectrum textures, .rg used) */
    float*     pong;    /* N*N*2 ping-pong texture */
    float*     raw;     /* 3 planes of inversion output */
} port_state;

/* tilde_h0_k_cs.glsl in FP32 (same pins as the oracle). */
static void port_h0(port_state* s, const float* noise)
{
    const orc_params* p = &s->p;
    int    N  = s->N;
    size_t NN = (size_t)N * N;
    float  wn = sqrtf((float)(p->wind_x * p->wind_x + p->wind_y * p->wind_y));
    float  wx = (float)p->wind_x / wn, wy = (float)p->wind_y / wn;
    float  Lp = (float)(p->wind_speed * p->wind_speed / p->gravity);
    float  A = (float)p->amplitude, l = (float)p->suppression, L = (float)p->L;
    const float PI = 3.14159265358979f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            size_t i  = (size_t)y * N + x;
            float  ix = (float)x - N / 2.0f, iz = (float)y - N / 2.0f;
            float  kx = 2.0f * PI * ix / L, kz = 2.0f * PI * iz / L;
            float  kl = sqrtf(kx * kx + kz * kz);
            float  km = kl < 0.00001f ? 0.00001f : kl;
            float  k2 = km * km;
            float  a  = 0.0f;
            if (!(ix == 0.0f && iz == 0.0f)) {
                float kd = (kx * wx + kz * wy) / kl;
                float P  = A * expf(-1.0f / (k2 * Lp * Lp)) * kd * kd * expf(-k2 * l * l) / (k2 * k2);
                a        = sqrtf(P) / sqrtf(2.0f);
                if (a > 4000.0f) a = 4000.0f;
            }
            float n[4];
            for (int q = 0; q < 4; ++q) {
                float v = noise[q * NN + i];
                n[q]    = v < 0.001f ? 0.001f : (v > 1.0f ? 1.0f : v);
            }
            float u0 = 2.0f * PI * n[0], v0 = sqrtf(-2.0f * logf(n[1]));
            float u1 = 2.0f * PI * n[2], v1 = sqrtf(-2.0f * logf(n[3]));
            s->h0[4 * i + 0] = v0 * cosf(u0) * a;
            s->h0[4 * i + 1] = v0 * sinf(u0) * a;
            s->h0[4 * i + 2] = v1 * cosf(u1) * a;
            s->h0[4 * i + 3] = v1 * sinf(u1) * a;
        }
}

port_state* port_create(const orc_params* p, const float* noise)
{
    port_state* s = (port_state*)calloc(1, sizeof(port_state));
    s->p  = *p;
    s->N  = p->N;
    s->lg = ilog2i(p->N);
    size_t NN = (size_t)s->N * s->N;
    s->h0   = (float*)malloc(NN * 4 * sizeof(float));
    s->tw   = (float*)malloc((size_t)s->lg * s->N * 4 * sizeof(float));
    s->spec = (float*)malloc(3 * NN * 2 * sizeof(float));
    s->pong = (float*)malloc(NN * 2 * sizeof(float));
    s->raw  = (float*)malloc(3 * NN * sizeof(float));
    port_h0(s, noise);
    /* twiddle texture, FP32 (twiddle_factors_cs.glsl is an FP32 shader) */
    double* t64 = (double*)malloc((size_t)s->lg * s->N * 4 * sizeof(double));
    orc_twiddle_table(s->N, t64);
    for (size_t i = 0; i < (size_t)s->lg * s->N * 4; ++i) s->tw[i] = (float)t64[i];
    free(t64);
    return s;
}

void port_destroy(port_state* s)
{
    if (!s) return;
    free(s->h0); free(s->tw); free(s->spec); free(s->pong); free(s->raw);
    free(s);
}

/* tilde_h0_t_cs.glsl:70-131 in FP32 with FP32 time (main.cpp:599). */
static void port_spectrum(port_state* s, float t)
{
    int    N  = s->N;
    size_t NN = (size_t)N * N;
    float  L = (float)s->p.L, g = (float)s->p.gravity;
    int    lit = s->p.literal_conj;
    const float PI = 3.14159265358979f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            size_t i  = (size_t)y * N + x;
            float  kx = 2.0f * PI * ((float)x - N / 2.0f) / L, kz = 2.0f * PI * ((float)y - N / 2.0f) / L;
            float  km = sqrtf(kx * kx + kz * kz);
            if (km < 0.00001f) km = 0.00001f;
            float w = sqrtf(g * km);
            float c = cosf(w * t), sn = sinf(w * t);
            float ar = s->h0[4 * i], ai = s->h0[4 * i + 1], br = s->h0[4 * i + 2], bi = s->h0[4 * i + 3];
            if (!lit) bi = -bi;
            float hr = ar * c - ai * sn + br * c + bi * sn;
            float hi = ar * sn + ai * c - br * sn + bi * c;
            float fx = -kx / km, fz = -kz / km;
            s->spec[2 * (0 * NN + i)] = -fx * hi; s->spec[2 * (0 * NN + i) + 1] = fx * hr;
            s->spec[2 * (1 * NN + i)] = hr;       s->spec[2 * (1 * NN + i) + 1] = hi;
            s->spec[2 * (2 * NN + i)] = -fz * hi; s->spec[2 * (2 * NN + i) + 1] = fz * hr;
        }
}

/* butterfly_fft() main.cpp:612-683: log2N horizontal then log2N vertical
 * radix-2 passes (butterfly_cs.glsl:54-132), ping-pong between the spectrum
 * texture and one scratch texture, then inversion_cs.glsl into `out`. */
static void port_butterfly_fft(port_state* s, float* tex, float* out)
{
    int    N = s->N;
    float* buf[2] = { tex, s->pong };
    int    pp = 0;
    for (int dir = 0; dir < 2; ++dir)
        for (int st = 0; st < s->lg; ++st) {
            const float* src = buf[pp];
            float*       dst = buf[pp ^ 1];
#pragma omp parallel for schedule(static)
            for (int y = 0; y < N; ++y)
                for (int x = 0; x < N; ++x) {
                    const float* d = s->tw + 4 * ((size_t)st * N + (dir == 0 ? x : y));
                    int ip = (int)d[2], iq = (int)d[3];
                    size_t a = dir == 0 ? (size_t)y * N + ip : (size_t)ip * N + x;
                    size_t b = dir == 0 ? (size_t)y * N + iq : (size_t)iq * N + x;
                    float pr = src[2 * a], pi = src[2 * a + 1], qr = src[2 * b], qi = src[2 * b + 1];
                    dst[2 * ((size_t)y * N + x)]     = pr + (d[0] * qr - d[1] * qi);
                    dst[2 * ((size_t)y * N + x) + 1] = pi + (d[0] * qi + d[1] * qr);
                }
            pp ^= 1;
        }
    const float* res = buf[pp];
    float        inv = 1.0f / (float)(N * N);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            float perm = ((x + y) & 1) ? -1.0f : 1.0f;          /* inversion_cs.glsl:29-31 */
            out[(size_t)y * N + x] = perm * (res[2 * ((size_t)y * N + x)] * inv);
        }
}

/* One frame of the reference algorithm (main.cpp:240-244) plus the lambda /
 * Jacobian additions, FP32.  Outputs as orc_finish. */
void port_frame(port_state* s, float t, float* dx, float* dy, float* dz, float* nj)
{
    int    N  = s->N;
    size_t NN = (size_t)N * N;
    port_spectrum(s, t);
    port_butterfly_fft(s, s->spec + 2 * NN, s->raw + NN);   /* dy */
    port_butterfly_fft(s, s->spec + 0, s->raw);             /* dx */
    port_butterfly_fft(s, s->spec + 4 * NN, s->raw + 2 * NN); /* dz */
    float lam = (float)s->p.choppiness, inv2d = (float)N / (2.0f * (float)s->p.L);
    const float* rx = s->raw;
    const float* ry = s->raw + NN;
    const float* rz = s->raw + 2 * NN;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y) {
        int ym = (y + N - 1) % N, yp = (y + 1) % N;
        for (int x = 0; x < N; ++x) {
            int    xm = (x + N - 1) % N, xp = (x + 1) % N;
            size_t i  = (size_t)y * N + x;
            float z0 = ry[ym * N + xm], z1 = ry[ym * N + x], z2 = ry[ym * N + xp];
            float z3 = ry[y * N + xm], z4 = ry[y * N + xp];
            float z5 = ry[yp * N + xm], z6 = ry[yp * N + x], z7 = ry[yp * N + xp];
            float nz = z0 + 2 * z1 + z2 - z5 - 2 * z6 - z7;
            float nx = z0 + 2 * z3 + z5 - z2 - 2 * z4 - z7;
            float rn = 1.0f / sqrtf(nx * nx + 1.0f + nz * nz);
            float dxx = lam * (rx[y * N + xp] - rx[y * N + xm]) * inv2d;
            float dxz = lam * (rx[yp * N + x] - rx[ym * N + x]) * inv2d;
            float dzx = lam * (rz[y * N + xp] - rz[y * N + xm]) * inv2d;
            float dzz = lam * (rz[yp * N + x] - rz[ym * N + x]) * inv2d;
            dx[i] = lam * rx[i];
            dy[i] = ry[i];
            dz[i] = lam * rz[i];
            nj[4 * i + 0] = nx * rn;
            nj[4 * i + 1] = rn;
            nj[4 * i + 2] = nz * rn;
            nj[4 * i + 3] = (1.0f - dxx) * (1.0f - dzz) - dxz * dzx;
        }
    }
}

const float* port_h0_ptr(const port_state* s) { return s->h0; }

int port_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void port_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------------------
 * Sky environment cube map (sky_envmap_fs.glsl:25-38 with SkyRadiance,
 * atmosphere.glsl:61-199).  Unlike the rest of the oracle this is FP32 in the
 * shader's operation order: the shader's float rounding is part of its result
 * (r*r - Rg*Rg cancels at the sea surface), so an FP64 restatement would not
 * be the reference.  Built with -ffp-contract=off; every literal is float.
 * Tables are sampled as GL_LINEAR + CLAMP_TO_EDGE textures with FP32 weights
 * (main.cpp:168-184).
 * params: camera[3], sun_direction[3], earth_pos[3], beta_r[3], mie_g,
 * sun_intensity; trans [64][256][4], insc [32][128][256][4];
 * out [6][S][S][4] (faces +X, -X, +Y, -Y, +Z, -Z, texel centres).
 * ------------------------------------------------------------------------- */
typedef struct { float x, y, z, w; } sky_f4;

static sky_f4 sky_lerp(sky_f4 a, sky_f4 b, float w)
{
    float  v = 1.0f - w;
    sky_f4 r = {a.x * v + b.x * w, a.y * v + b.y * w, a.z * v + b.z * w, a.w * v + b.w * w};
    return r;
}

static sky_f4 sky_at(const float* T, size_t i)
{
    sky_f4 r = {T[4 * i], T[4 * i + 1], T[4 * i + 2], T[4 * i + 3]};
    return r;
}

static void sky_axis(float u, int W, int* i0, int* i1, float* w)
{
    float t = u * (float)W - 0.5f;
    float f = floorf(t);
    int   i = (int)f;
    *w      = t - f;
    *i0     = i < 0 ? 0 : (i > W - 1 ? W - 1 : i);
    *i1     = i + 1 < 0 ? 0 : (i + 1 > W - 1 ? W - 1 : i + 1);
}

static sky_f4 sky_tex2d(const float* T, int W, int H, float u, float v)
{
    int   x0, x1, y0, y1;
    float wx, wy;
    sky_axis(u, W, &x0, &x1, &wx);
    sky_axis(v, H, &y0, &y1, &wy);
    sky_f4 a = sky_lerp(sky_at(T, (size_t)y0 * W + x0), sky_at(T, (size_t)y0 * W + x1), wx);
    sky_f4 b = sky_lerp(sky_at(T, (size_t)y1 * W + x0), sky_at(T, (size_t)y1 * W + x1), wx);
    return sky_lerp(a, b, wy);
}

static sky_f4 sky_tex3d(const float* T, int W, int H, int D, float u, float v, float q)
{
    int    x0, x1, y0, y1, z0, z1;
    float  wx, wy, wz;
    sky_f4 p[2];
    sky_axis(u, W, &x0, &x1, &wx);
    sky_axis(v, H, &y0, &y1, &wy);
    sky_axis(q, D, &z0, &z1, &wz);
    for (int k = 0; k < 2; ++k) {
        const float* P = T + (size_t)4 * (k ? z1 : z0) * H * W;
        sky_f4       a = sky_lerp(sky_at(P, (size_t)y0 * W + x0), sky_at(P, (size_t)y0 * W + x1), wx);
        sky_f4       b = sky_lerp(sky_at(P, (size_t)y1 * W + x0), sky_at(P, (size_t)y1 * W + x1), wx);
        p[k]           = sky_lerp(a, b, wy);
    }
    return sky_lerp(p[0], p[1], wz);
}

#define SKY_RG 6360000.0f
#define SKY_RT 6420000.0f

/* atmosphere.glsl:61-81 */
static sky_f4 sky_texture4d(const float* T, float r, float mu, float muS, float nu, float tan_mus)
{
    const float H     = sqrtf(SKY_RT * SKY_RT - SKY_RG * SKY_RG);
    const float rho   = sqrtf(r * r - SKY_RG * SKY_RG);
    const float rmu   = r * mu;
    const float delta = rmu * rmu - r * r + SKY_RG * SKY_RG;
    const int   below = rmu < 0.0f && delta > 0.0f;
    const float c0 = below ? 1.0f : -1.0f, c1 = below ? 0.0f : H * H, c2 = below ? 0.0f : H;
    const float c3   = below ? 0.5f - 0.5f / 128.0f : 0.5f + 0.5f / 128.0f;
    const float uR   = 0.5f / 32.0f + rho / H * (1.0f - 1.0f / 32.0f);
    const float uMu  = c3 + (rmu * c0 + sqrtf(delta + c1)) / (rho + c2) * (0.5f - 1.0f / 128.0f);
    const float mus  = muS > -0.1975f ? muS : -0.1975f;
    const float uMuS = 0.5f / 32.0f + (atanf(mus * tan_mus) / 1.1f + (1.0f - 0.26f)) * 0.5f * (1.0f - 1.0f / 32.0f);
    float       lep  = (nu + 1.0f) / 2.0f * (8.0f - 1.0f);
    const float uNu  = floorf(lep);
    lep              = lep - uNu;
    sky_f4 t0 = sky_tex3d(T, 256, 128, 32, (uNu + uMuS) / 8.0f, uMu, uR);
    sky_f4 t1 = sky_tex3d(T, 256, 128, 32, (uNu + uMuS + 1.0f) / 8.0f, uMu, uR);
    float  m  = 1.0f - lep;
    sky_f4 r4 = {t0.x * m + t1.x * lep, t0.y * m + t1.y * lep, t0.z * m + t1.z * lep, t0.w * m + t1.w * lep};
    return r4;
}

void orc_sky_envmap(const float* prm, int S, const float* trans, const float* insc, float* out)
{
    const float* cam0 = prm;
    const float* sun  = prm + 3;
    const float* ep   = prm + 6;
    const float* br   = prm + 9;
    const float  g = prm[12], I = prm[13];
    const float  tan_mus = tanf(1.26f * 1.1f), tan_mu = tanf(1.5f);
    const float  cos_sun = cosf(3.141592f / 360.0f);
    const float  pi      = 3.141592f;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < 6L * S * S; ++idx) {
        int   face = (int)(idx / ((long)S * S)), rem = (int)(idx - (long)face * S * S);
        int   j = rem / S, i = rem - j * S;
        float sc = 2.0f * (((float)i + 0.5f) / (float)S) - 1.0f, tc = 2.0f * (((float)j + 0.5f) / (float)S) - 1.0f;
        float d[3];
        switch (face) {   /* OpenGL cube-map orientation: the inverse of orc_cube_sample's table */
        case 0: d[0] = 1.0f; d[1] = -tc; d[2] = -sc; break;
        case 1: d[0] = -1.0f; d[1] = -tc; d[2] = sc; break;
        case 2: d[0] = sc; d[1] = 1.0f; d[2] = tc; break;
        case 3: d[0] = sc; d[1] = -1.0f; d[2] = -tc; break;
        case 4: d[0] = sc; d[1] = -tc; d[2] = 1.0f; break;
        default: d[0] = -sc; d[1] = -tc; d[2] = -1.0f; break;
        }
        float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        float v[3] = {d[0] / len, d[1] / len, d[2] / len};
        float sunv = (v[0] * sun[0] + v[1] * sun[1] + v[2] * sun[2]) < cos_sun ? 0.0f : 1.0f;
        float sun_c = sunv * I;
        float c[3] = {cam0[0] + ep[0], cam0[1] + ep[1], cam0[2] + ep[2]};
        float r   = sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        float rMu = c[0] * v[0] + c[1] * v[1] + c[2] * v[2];
        float mu  = rMu / r;
        float deltaSq = sqrtf(rMu * rMu - r * r + SKY_RT * SKY_RT);
        float din     = -rMu - deltaSq;
        if (din < 0.0f) din = 0.0f;
        if (din > 0.0f) {
            c[0] = c[0] + din * v[0];
            c[1] = c[1] + din * v[1];
            c[2] = c[2] + din * v[2];
            rMu  = rMu + din;
            mu   = rMu / SKY_RT;
            r    = SKY_RT;
        }
        float  nu  = v[0] * sun[0] + v[1] * sun[1] + v[2] * sun[2];
        float  muS = (c[0] * sun[0] + c[1] * sun[1] + c[2] * sun[2]) / r;
        sky_f4 is  = sky_texture4d(insc, r, rMu / r, muS, nu, tan_mus);
        /* Transmittance(r, mu), atmosphere.glsl:102-111 */
        float  tuR  = sqrtf((r - SKY_RG) / (SKY_RT - SKY_RG));
        float  tuMu = atanf((mu + 0.15f) / (1.0f + 0.15f) * tan_mu) / 1.5f;
        sky_f4 tr   = sky_tex2d(trans, 256, 64, tuMu, tuR);
        float  ext[3] = {tr.x, tr.y, tr.z}, res[3] = {0.0f, 0.0f, 0.0f};
        if (r <= SKY_RT) {
            float mx = is.x > 1e-4f ? is.x : 1e-4f;
            float m[3] = {is.x * is.w / mx * (br[0] / br[0]), is.y * is.w / mx * (br[0] / br[1]),
                          is.z * is.w / mx * (br[0] / br[2])};
            float pr = (3.0f / (16.0f * pi)) * (1.0f + nu * nu);
            float pm = 1.5f * 1.0f / (4.0f * pi) * (1.0f - g * g) * powf(1.0f + (g * g) - 2.0f * g * nu, -3.0f / 2.0f) *
                       (1.0f + nu * nu) / (2.0f + g * g);
            res[0] = is.x * pr + m[0] * pm;
            res[1] = is.y * pr + m[1] * pm;
            res[2] = is.z * pr + m[2] * pm;
        } else {
            ext[0] = ext[1] = ext[2] = 1.0f;
        }
        float* o = out + 4 * idx;
        o[0] = sun_c * ext[0] + res[0] * I;
        o[1] = sun_c * ext[1] + res[1] * I;
        o[2] = sun_c * ext[2] + res[2] * I;
        o[3] = 1.0f;
    }
}
