/*
 * ocean.h -- C ABI of the GB300 Tessendorf FFT ocean library.
 *
 * Drop-in for the per-frame compute-shader path of diharaw/fft-ocean-waves
 * (src/main.cpp, class FFTOceanWaves).  All file:line citations below are
 * paths inside that project.
 *
 * Conventions
 *   - Every int-returning call returns OCEAN_OK (0) or a negative OCEAN_ERR_*;
 *     ocean_last_error() then describes the failure (thread-local string).
 *     No C++ exception crosses this boundary.
 *   - Device buffers are row-major [y][x] with x the column (the reference's
 *     image coordinate gl_GlobalInvocationID.xy).  Mode (x, y) holds the wave
 *     vector k = 2*pi*(x - N/2, y - N/2)/L (tilde_h0_k_cs.glsl:76-77).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  Calls that take a stream are asynchronous and stream-ordered.
 *   - A handle is not thread-safe; distinct handles may be used concurrently.
 *   - Device output pointers must be 16-byte aligned.
 */
#ifndef OCEAN_GB300_H
#define OCEAN_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define OCEAN_API __attribute__((visibility("default")))
#else
#define OCEAN_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define OCEAN_OK 0
#define OCEAN_ERR_INVALID -1     /* bad argument (size, pointer, parameter) */
#define OCEAN_ERR_CUDA -2        /* a CUDA runtime call or launch failed   */
#define OCEAN_ERR_NOMEM -3       /* device or host allocation failed       */
#define OCEAN_ERR_UNSUPPORTED -4 /* no kernel for this device / size       */
#define OCEAN_ERR_TIMEOUT -5     /* a kernel's bounded wait timed out       */

#define OCEAN_MIN_N 32
#define OCEAN_MAX_N 2048

/* Flags for ocean_params.flags */
/* Reproduce tilde_h0_t_cs.glsl:42-48,94 literally: its conjugate() returns the
 * argument unchanged, so h0(-k) enters the evolution unconjugated.  Default
 * (flag clear) is the textbook conj(h0(-k)). */
#define OCEAN_FLAG_LITERAL_CONJ 1u

/* Spectrum parameters: the reference's uniforms u_N, u_L, u_Amplitude,
 * u_WindSpeed, u_WindDirection, u_SuppressFactor (tilde_h0_k_cs.glsl:19-24)
 * and u_Choppiness (grid_tes.glsl:33), with defaults main.cpp:1631-1646. */
typedef struct ocean_params {
    int32_t  N;           /* grid size: power of two, 32..2048 (main.cpp:17,1645)   */
    uint32_t flags;       /* OCEAN_FLAG_*                                           */
    float    L;           /* patch length, metres (reference: int u_L = 1000)       */
    float    amplitude;   /* Phillips A (2.0)                                       */
    float    wind_speed;  /* V, m/s (80.0)                                          */
    float    wind_dir_x;  /* wind direction, normalised internally (main.cpp:555)   */
    float    wind_dir_y;  /*   reference default (1, 1)                             */
    float    choppiness;  /* lambda applied to Dx, Dz (0.75)                         */
    float    suppression; /* small-wave cutoff l, metres (0.1)                      */
    float    gravity;     /* g (9.81, tilde_h0_k_cs.glsl:26); <= 0 selects 9.81      */
} ocean_params;

/* Per-frame outputs, device pointers, each N*N elements row-major.
 * dx, dy, dz: R32F displacement maps (the reference's m_dx, m_dy, m_dz,
 * main.cpp:1096-1098) with dx, dz already multiplied by lambda.
 * normal_j: RGBA32F (nx, ny, nz, J): the Sobel normal of dy
 * (normal_map_cs.glsl:24-54, periodic integer taps) and the Jacobian of the
 * rendered surface p = x - (dx, dz) (reference normal.w is 1). */
typedef struct ocean_outputs {
    float* dx;
    float* dy;
    float* dz;
    float* normal_j; /* N*N*4 floats */
} ocean_outputs;

typedef struct ocean_s ocean_t;

/* Create a tile: validates params, uploads the four U(0,1] noise planes
 * (host pointer, 4*N*N floats, [plane][y][x]; planes 0/1 feed h0(k), 2/3 feed
 * h0(-k)) and builds h0 on the device.
 * Replaces FFTOceanWaves::init's tilde_h0_k(), generate_bit_reversed_indices()
 * and generate_twiddle_factors() (main.cpp:217-220, :553-583, :711-744).
 * Synchronous. */
OCEAN_API int ocean_create(const ocean_params* params, const float* noise_host, ocean_t** out);

/* ocean_create with noise from ocean_fill_noise(seed, N). */
OCEAN_API int ocean_create_seeded(const ocean_params* params, uint64_t seed, ocean_t** out);

OCEAN_API void ocean_destroy(ocean_t* ocean);

/* One frame at time t (seconds, double; the phase omega*t is reduced in
 * double-float precision).  Replaces tilde_h0_t(); butterfly_fft(dy),
 * butterfly_fft(dx), butterfly_fft(dz); generate_normal_map()
 * (main.cpp:240-244).  out == NULL writes the handle-owned buffers returned
 * by ocean_get_outputs().  Three kernel launches on `stream`. */
OCEAN_API int ocean_update(ocean_t* ocean, double t, const ocean_outputs* out, void* stream);

/* ocean_update in its three stages, one kernel each, for callers that
 * interleave other work or time the kernels separately:
 *   rows     evolution + horizontal FFT (tilde_h0_t() and the horizontal
 *            butterfly passes, main.cpp:240, :626-640) into the handle's
 *            intermediate;
 *   columns  vertical FFT + inversion (the vertical butterfly passes and
 *            inversion_cs.glsl, main.cpp:647-682) into the handle's
 *            column-major maps;
 *   outputs  the maps written to dx, dy, dz, plus the normal map and
 *            Jacobian (generate_normal_map(), main.cpp:244, :687-707); out ==
 *            NULL writes the handle-owned buffers.
 * ocean_update == rows, columns, outputs on one stream (or rows and
 * ocean_update_columns_outputs, below). */
OCEAN_API int ocean_update_rows(ocean_t* ocean, double t, void* stream);
OCEAN_API int ocean_update_columns(ocean_t* ocean, void* stream);
OCEAN_API int ocean_update_outputs(ocean_t* ocean, const ocean_outputs* out, void* stream);

/* columns + outputs as one stage (the vertical butterfly passes, inversion_cs.glsl
 * and generate_normal_map(), main.cpp:647-707): one fused kernel where the
 * launch configuration says so (ocean_tuning.col_fused; the column-major maps
 * then stay on chip), else ocean_update_columns then ocean_update_outputs.
 * ocean_update == ocean_update_rows, ocean_update_columns_outputs. */
OCEAN_API int ocean_update_columns_outputs(ocean_t* ocean, const ocean_outputs* out, void* stream);

/* Synchronise `stream` and report (and clear) the handle's device status:
 * OCEAN_ERR_TIMEOUT if a kernel gave up a bounded wait for its TMA copies
 * (its outputs for that frame are incomplete), else OCEAN_OK.  The reference
 * never checks its dispatches. */
OCEAN_API int ocean_device_status(ocean_t* ocean, void* stream);

/* Test hook for failure paths: from now on the library's device and pinned
 * host allocations succeed `after` more times and then fail (the calling
 * function returns OCEAN_ERR_NOMEM and releases what it had allocated) until
 * the hook is set again; after < 0, the default, turns it off.  Process-wide. */
OCEAN_API void ocean_debug_fail_allocations(int32_t after);

/* Handle-owned output buffers (allocated on first use); the headless
 * stand-ins for the reference's GL textures m_dx/m_dy/m_dz/m_normal_map. */
OCEAN_API int ocean_get_outputs(ocean_t* ocean, ocean_outputs* out);

/* Replace the spectrum parameters (same N) and rebuild h0 from the stored
 * noise.  The reference reads GUI edits of wind speed and amplitude
 * (main.cpp:348-358) but never re-runs tilde_h0_k(), so they have no effect
 * there; here they do.  Synchronous: it first waits for all work on the
 * current device (frames of this handle in flight on any stream), then
 * rebuilds h0 and the combined spectrum and waits for that too. */
OCEAN_API int ocean_set_params(ocean_t* ocean, const ocean_params* params);
OCEAN_API int ocean_get_params(const ocean_t* ocean, ocean_params* params);

/* Checkpoint / restore of the spectrum state: N*N*4 floats
 * (h0k.re, h0k.im, h0minusk.re, h0minusk.im) per mode, host or device
 * pointer (unified addressing), stream-ordered. */
OCEAN_API int ocean_get_h0(const ocean_t* ocean, float* dst, void* stream);
OCEAN_API int ocean_set_h0(ocean_t* ocean, const float* src, void* stream);

/* Stateless h0 initialisation (tilde_h0_k_cs.glsl:35-93) into a caller
 * buffer: noise_dev (device, 4*N*N) -> h0_dev (device, N*N*4). */
OCEAN_API int ocean_compute_h0(const ocean_params* params, const float* noise_dev, float* h0_dev, void* stream);

/* Seeded uniform noise: splitmix64 -> 24-bit uniforms in (0, 1], 4*N*N
 * floats [plane][y][x] into a host buffer.  Stands in for the blue-noise
 * textures data/noise/LDR_LLL1_{0..3}.png (main.cpp:1085-1088). */
OCEAN_API int ocean_fill_noise(uint64_t seed, int32_t N, float* host_out);

/* The reference's FFT tables, host side, for callers that consumed them:
 * bit-reversed indices (main.cpp:29-64,733-744), N int32, and the butterfly
 * table (twiddle_factors_cs.glsl:34-69): log2(N) x N x 4 floats
 * (Re w, Im w, index p, index q).  The kernels use their own Stockham
 * twiddles and do not need either. */
OCEAN_API int ocean_bit_reversed_indices(int32_t N, int32_t* host_out);
OCEAN_API int ocean_butterfly_table(int32_t N, float* host_out);

/* ---- Batched tiles ---------------------------------------------------- */

typedef struct ocean_batch_s ocean_batch_t;

/* A batch of n_tiles independent tiles, each with its own parameters (any
 * supported N; tiles of equal N are grouped) and its own seeded noise
 * (ocean_fill_noise(seeds[i], N)), advanced `samples` time samples per
 * ocean_batch_update.  h0 is built at creation.  Synchronous. */
OCEAN_API int ocean_batch_create(const ocean_params* params, const uint64_t* seeds, int32_t n_tiles,
                                 int32_t samples, ocean_batch_t** out);

/* Advance every tile to its `samples` times: times[tile*samples + s] (host),
 * outputs into outs[tile*samples + s] (device pointers, 16-byte aligned).
 * All launches (per distinct N: one persistent row pass reading each h0 row
 * once for all samples, one column pass) replay as one CUDA graph on
 * `stream`.  The host-side constants go through a pinned staging buffer: a
 * call first waits for the previous call's graph to finish. */
OCEAN_API int ocean_batch_update(ocean_batch_t* batch, const double* times, const ocean_outputs* outs, void* stream);

/* As ocean_device_status, for the batch's kernels. */
OCEAN_API int ocean_batch_device_status(ocean_batch_t* batch, void* stream);

OCEAN_API void ocean_batch_destroy(ocean_batch_t* batch);

/* ---- Frame update without device allocation ------------------------ */

/* One frame, like ocean_update, for callers that cannot call cudaMalloc:
 * plug-in hosts that own the CUDA context and forbid allocation from plug-in
 * code, code running while the application's allocator is locked or its pool
 * exhausted, and callers held to a memory budget fixed at load time.  No
 * handle: the caller passes the parameters, the spectrum h0 (device,
 * N*N*4 floats, the layout of ocean_get_h0 / ocean_compute_h0) and the output
 * maps.  The frame's scratch (the row-pass intermediate and the column
 * transforms' maps, 25,190,400 bytes, plus a twiddle table and a status word)
 * lives in static device arrays
 * compiled into the library, sized for N <= 1024; every GPU that loads the
 * library holds them until the process exits.  N > 1024 is rejected with
 * OCEAN_ERR_INVALID.  The first call on a device resolves the arrays' addresses
 * (cudaGetSymbolAddress) and clears the status word, and the first call after
 * a change of N rebuilds the twiddle table: such a call made inside a stream
 * capture is refused with OCEAN_ERR_INVALID (make it before the capture).
 * Every call uses the same arrays, so calls whose work overlaps on the GPU
 * (other streams, other threads) race: serialise them.  Calls no
 * cudaMalloc/cudaFree.  No counterpart in the reference. */
OCEAN_API int ocean_update_noalloc(const ocean_params* params, const float* h0_dev, double t,
                                   const ocean_outputs* out, void* stream);

/* The device status of ocean_update_noalloc on the current device, as
 * ocean_device_status reports a handle's: synchronises `stream`, returns
 * OCEAN_ERR_TIMEOUT if a kernel of an earlier call gave up a bounded wait for
 * its TMA copies (that frame's outputs are incomplete), else OCEAN_OK, and
 * clears the status word.  OCEAN_OK when no call has run on the device.
 * Allocates nothing.  No counterpart in the reference. */
OCEAN_API int ocean_noalloc_device_status(void* stream);

/* ---- Displaced grid (the consumer of the maps) ------------------------ */

/* The render grid of main.cpp:748-824 (generate_grid(GRID_SIZE, GRID_UV_SCALE),
 * main.cpp:20-21): `squares` squares per side, (squares+1)^2 vertices at
 * (x, 0, z) with integer x, z in [-squares/2, squares/2], two triangles per
 * square (vertex indices i0, i0+squares+1, i0+1 and i0+1, i0+squares+1,
 * i0+squares+2). */
typedef struct ocean_grid_params {
    int32_t squares;            /* even, 2..16384; the reference uses 1024 */
    float   texcoord_scale;     /* texture repeats over the grid, |.| <= 1e6; the reference uses 64 */
    float   displacement_scale; /* vertical scale of Dy; the reference's default 0.5 (main.cpp:1632) */
    float   camera[3];          /* eye position for the tessellation levels */
} ocean_grid_params;

/* The tessellation evaluation stage at the grid's vertices
 * (grid_tes.glsl:55-66): position (x - Dx, Dy * displacement_scale, z - Dz),
 * normal = normal_map.xyz, texcoord, with the maps (one frame's outputs,
 * N x N, device) sampled bilinearly with REPEAT wrap.  dx and dz are
 * ocean_update's outputs, which already carry lambda (the shader's
 * u_Choppiness).  vertices: device, (squares+1)^2 * 8 floats (position xyz,
 * normal xyz, texcoord uv), 16-byte aligned. */
OCEAN_API int ocean_displace_grid(const ocean_outputs* maps, int32_t N, const ocean_grid_params* grid,
                                  float* vertices, void* stream);

/* The tessellation control stage (grid_tcs.glsl:27-59) per triangle:
 * outer[0..2] from the mean eye distance of edges (v1, v2), (v2, v0),
 * (v0, v1): 20 up to 10, 10 up to 20, 5 up to 30, else 1; inner = outer[2].
 * levels: device, 2 * squares^2 * 4 floats (triangle 2*(z*squares + x) + t),
 * 16-byte aligned. */
OCEAN_API int ocean_grid_tess_levels(const ocean_grid_params* grid, float* levels, void* stream);

/* The ocean fragment shader (ocean_fs.glsl:11-37) at the displaced grid's
 * vertices: N = the vertex normal as given, V = normalize(camera - P),
 * R = reflect(-V, N), F = 0.04 + 0.96 (1 - max(N.V, 0))^5,
 * color = max(-N.sun_direction, 0) * mix(sea_color, sky(R), F), then
 * c / (c + 1) and gamma 1/2.2.  sky_cubemap: device, 6 faces (+X, -X, +Y,
 * -Y, +Z, -Z) of sky_size^2 RGBA floats, looked up as the OpenGL cube-map
 * table specifies (bilinear within a face, clamp to edge).  vertices: as
 * ocean_displace_grid writes them (n_vertices * 8 floats, 0 <= n_vertices <
 * 2^31 * 256: one launch).  colors: device,
 * n_vertices * 4 floats (RGB, 1).  All three 16-byte aligned.  As in the
 * shader, the result is undefined (NaN) for normals longer than 1 with
 * N.V > 1, where the Fresnel term goes negative. */
typedef struct ocean_shade_params {
    float   camera[3];
    float   sun_direction[3];   /* direction the sunlight travels (the shader's u_SunDirection) */
    float   sea_color[3];       /* the shader's u_SeaColor */
    int32_t sky_size;           /* cube-map face edge in texels */
} ocean_shade_params;

OCEAN_API int ocean_shade_grid(const float* vertices, int64_t n_vertices, const ocean_shade_params* params,
                               const float* sky_cubemap, float* colors, void* stream);

/* ---- Sky environment cube map (precomputed atmospheric scattering) ----- */

/* Lookup-table sizes of the sky model (main.cpp:66-80): transmittance
 * [64][256] RGBA (x = view-zenith parameter, y = altitude), inscatter
 * [32][128][256] RGBA (x = sun-zenith x view-sun, 32 x 8; y = view zenith;
 * z = altitude).  Row-major float32, as the reference's .raw texture files. */
#define OCEAN_SKY_TRANSMITTANCE_W 256
#define OCEAN_SKY_TRANSMITTANCE_H 64
#define OCEAN_SKY_INSCATTER_W     256
#define OCEAN_SKY_INSCATTER_H     128
#define OCEAN_SKY_INSCATTER_D     32

/* Uniforms of the sky model (main.cpp:149-158, atmosphere.glsl:37-41); the
 * reference's values are earth_pos (0, 6360010, 0), sun_intensity 100,
 * beta_r (0.0058, 0.0135, 0.0331) / 1000, mie_g 0.75, and sun_direction =
 * -normalize(0, sin a, cos a) for the GUI sun angle a. */
typedef struct ocean_sky_params {
    float   camera[3];          /* u_CameraPos (world units, y up)                 */
    float   sun_direction[3];   /* SUN_DIR: unit vector the shader dots view rays with */
    float   earth_pos[3];       /* EARTH_POS                                       */
    float   beta_r[3];          /* betaR (Rayleigh scattering per unit length)     */
    float   mie_g;              /* mieG                                            */
    float   sun_intensity;      /* SUN_INTENSITY                                   */
    int32_t size;               /* cube-map face edge in texels (the reference: 512) */
} ocean_sky_params;

/* The sky environment cube map of render_envmap() (main.cpp:500-523,
 * sky_envmap_fs.glsl:25-38): per texel of the six faces, the sun disk times
 * the extinction plus SkyRadiance() (atmosphere.glsl:152-199), with the
 * tables sampled as the reference's GL_LINEAR / CLAMP_TO_EDGE textures.
 * Faces +X, -X, +Y, -Y, +Z, -Z in the OpenGL cube-map orientation (the
 * capture views of main.cpp:1463-1470), texel centres; output
 * [6][size][size] RGBA float32 (alpha 1), the layout ocean_shade_grid reads.
 * The reference stores the map as RGB16F; this writes float32.
 * transmittance and inscatter are device tables of the sizes above (the
 * reference ships transmittance.raw; its inscatter.raw is missing, so the
 * caller supplies one).  All pointers 16-byte aligned.  One launch. */
OCEAN_API int ocean_sky_envmap(const ocean_sky_params* params, const float* transmittance, const float* inscatter,
                               float* cubemap, void* stream);

/* The skybox of render_skybox() (main.cpp:527-547, sky_vs.glsl, sky_fs.glsl)
 * into a headless image: per pixel centre of a width x height framebuffer
 * (row 0 at the bottom, as GL's), the direction through the far plane of
 * projection * mat4(mat3(view)), the cube map sampled there (level 0,
 * bilinear within the face, as ocean_shade_grid), then c / (c + 1) and
 * gamma 1/2.2.  view and projection are 4x4 column-major (glm) host arrays;
 * sky_cubemap [6][sky_size][sky_size] RGBA as ocean_sky_envmap writes it;
 * image [height][width] RGBA float32 (alpha 1).  16-byte aligned. */
OCEAN_API int ocean_render_skybox(const float* sky_cubemap, int32_t sky_size, const float* view, const float* projection,
                                  int32_t width, int32_t height, float* image, void* stream);

/* ---- Adjoint --------------------------------------------------------- */

/* Flags for ocean_backward */
#define OCEAN_GRAD_ACCUMULATE 1u /* add into *grads and dh0 instead of overwriting */

/* Gradients of a scalar loss L with respect to the spectrum parameters and,
 * optionally, the per-mode spectrum state.  Complex gradients use the
 * convention dL/dRe + i dL/dIm. */
typedef struct ocean_grads {
    double dA;       /* dL/d amplitude                                            */
    double dV;       /* dL/d wind speed                                           */
    double dtheta;   /* dL/d wind direction angle (w = (cos theta, sin theta))    */
    double dlambda;  /* dL/d choppiness                                           */
    float* dh0;      /* optional device N*N*4 (layout of ocean_get_h0), or NULL   */
} ocean_grads;

/* Adjoint of ocean_update's displacement outputs over T frames: given
 * dL/d(dx, dy, dz) for frame times[j] (device, T*N*N floats each, frame-major;
 * NULL = zero gradient for that field), compute the gradients above.  The
 * frames are not stored or recomputed: the adjoint reads only h0 (forward
 * DFT as the transpose of the inverse butterfly network, conjugate phase
 * rotation, transpose of the choppy multiply, chain through the Phillips
 * amplitude).  Parameter gradients hold l, L and g fixed, exclude modes on the
 * +-4000 clamp and assume h0 was built from the current parameters (not set
 * with ocean_set_h0).  The normal/Jacobian map carries no gradient.
 * Two kernel launches per chunk of <= 64 frames; scratch is allocated on
 * first use (at most 512 MiB).  Returns after the scalar gradients are on the
 * host (synchronises `stream`). No counterpart in the reference. */
OCEAN_API int ocean_backward(ocean_t* ocean, const double* times, int32_t T, const float* g_dx, const float* g_dy,
                             const float* g_dz, uint32_t flags, ocean_grads* grads, void* stream);

/* ---- Launch configuration per N ---------------------------------------- */

/* How the kernels of size N are launched.  The defaults are a table compiled
 * into the library (written by the project's tuner from GB300 measurements);
 * ocean_set_tuning replaces the entry of one N for the rest of the process
 * (all handles; a batch reads wave_mib when it is created).  No counterpart in
 * the reference, which dispatches every shader in one fixed shape. */
typedef struct ocean_tuning {
    int32_t row_overlap;      /* 1: a frame's row pass starts while the stream's previous kernel (the previous
                                 frame's output stage) still runs, and waits for it only at its end; 0: it waits
                                 before starting.  Stream order is kept either way.                            */
    int32_t row_ctas_per_sm;  /* persistent row-pass CTAs per SM, 0 = as many as fit                            */
    int32_t wave_mib;         /* batches: scratch (intermediate + column maps) of one wave of units, MiB        */
    int32_t col_fused;        /* 2 or 4: ocean_update, batches and ocean_update_noalloc run the column
                                 transforms and the normal/Jacobian stage as one kernel with that many column
                                 pairs per CTA (N = 512 and 1024; reads 0 elsewhere); 0: as two kernels through
                                 column-major maps, as ocean_update_columns and ocean_update_outputs do        */
    int32_t row_variant;      /* N >= 512: 0 = warp-specialised row pass (prepass warps feed transform warps),
                                 1 = every warp runs the prepass and then its line FFT (one row pair per CTA
                                 at N = 1024), 2 = warp-specialised with 8-point-first lines (half the
                                 registers per thread, one more exchange), 3 = warp-specialised with 32 x 32
                                 lines (N = 1024 only; reads 0 elsewhere), 4 = every warp with 32 x 32 lines
                                 (N = 1024 only; reads 1 elsewhere), 5 = as 3 with one ring stage and one
                                 line-buffer set, three CTAs per SM (N = 1024 only; reads 0 elsewhere);
                                 below 512 only 1 exists and this reads 1                                    */
} ocean_tuning;

OCEAN_API int ocean_get_tuning(int32_t N, ocean_tuning* out);
OCEAN_API int ocean_set_tuning(int32_t N, const ocean_tuning* cfg);

OCEAN_API const char* ocean_last_error(void);
OCEAN_API int ocean_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OCEAN_GB300_H */
