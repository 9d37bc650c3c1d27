"""Python face of the oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/libocean_oracle.so (built by oracle/build_oracle.py) and
exposes the FP64 restatement of the reference ocean path (``h0``,
``spectrum``, ``update``, FFT tables) and the FP32 port of the reference
algorithm (``Port``), plus the seeded noise generator shared with the CUDA
library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import os

import numpy as np

from . import build_oracle

_LIB = None


class _OrcParams(C.Structure):
    _fields_ = [("N", C.c_int32), ("literal_conj", C.c_int32), ("L", C.c_double),
                ("amplitude", C.c_double), ("wind_speed", C.c_double),
                ("wind_x", C.c_double), ("wind_y", C.c_double),
                ("choppiness", C.c_double), ("suppression", C.c_double),
                ("gravity", C.c_double)]


@dataclasses.dataclass
class Params:
    """Spectrum parameters of one ocean tile (the reference's uniforms,
    main.cpp:1631-1646 and tilde_h0_k_cs.glsl:19-24)."""
    N: int = 256
    L: float = 1000.0
    amplitude: float = 2.0
    wind_speed: float = 80.0
    wind_x: float = 1.0
    wind_y: float = 1.0
    choppiness: float = 0.75
    suppression: float = 0.1
    gravity: float = 9.81
    literal_conj: bool = False

    @staticmethod
    def from_angle(N, L, amplitude, wind_speed, angle_deg, choppiness, suppression=0.1, **kw):
        a = math.radians(angle_deg)
        return Params(N=N, L=L, amplitude=amplitude, wind_speed=wind_speed,
                      wind_x=math.cos(a), wind_y=math.sin(a), choppiness=choppiness,
                      suppression=suppression, **kw)

    def _c(self) -> _OrcParams:
        return _OrcParams(self.N, int(self.literal_conj), self.L, self.amplitude, self.wind_speed,
                          self.wind_x, self.wind_y, self.choppiness, self.suppression, self.gravity)


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        pp = C.POINTER(_OrcParams)
        L.orc_h0.argtypes = [pp, fp, dp]
        L.orc_spectrum.argtypes = [pp, dp, C.c_double, dp]
        L.orc_ifft2_real.argtypes = [C.c_int, dp, dp]
        L.orc_finish.argtypes = [pp, dp, dp, dp, dp, dp]
        L.orc_update.argtypes = [pp, dp, C.c_double, dp, dp, dp, dp]
        L.orc_backward.argtypes = [pp, dp, dp, C.c_int, dp, dp, dp, dp, dp]
        L.orc_bit_reversed.argtypes = [C.c_int, C.POINTER(C.c_int32)]
        L.orc_twiddle_table.argtypes = [C.c_int, dp]
        L.orc_displace_grid.argtypes = [C.c_int, dp, dp, dp, dp, C.c_int, C.c_double, C.c_double, dp]
        L.orc_tess_levels.argtypes = [C.c_int, dp, dp]
        L.orc_shade.argtypes = [dp, C.c_long, dp, dp, dp, dp, C.c_int, dp]
        L.orc_sky_envmap.argtypes = [fp, C.c_int, fp, fp, fp]
        L.orc_skybox.argtypes = [dp, C.c_int, dp, C.c_int, C.c_int, dp]
        L.orc_count_clamped.argtypes = [pp]
        L.orc_count_clamped.restype = C.c_int
        L.port_create.argtypes = [pp, fp]
        L.port_create.restype = C.c_void_p
        L.port_destroy.argtypes = [C.c_void_p]
        L.port_frame.argtypes = [C.c_void_p, C.c_float, fp, fp, fp, fp]
        L.port_h0_ptr.argtypes = [C.c_void_p]
        L.port_h0_ptr.restype = fp
        L.port_max_threads.restype = C.c_int
        L.port_set_threads.argtypes = [C.c_int]
        _LIB = L
    return _LIB


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


# ---------------------------------------------------------------------------
# Seeded noise: splitmix64 (Steele, Lea & Flood 2014) -> 24-bit uniforms in
# (0, 1].  The i-th draw of a stream seeded with s uses state s + (i+1)*gamma.
# Plane order [4][N][N]; planes 0/1 feed h0k, 2/3 feed h0minusk.
# ---------------------------------------------------------------------------
_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, count: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def noise(seed: int, N: int) -> np.ndarray:
    """Four N x N planes of U(0,1] float32 noise for tile seed `seed`."""
    z = splitmix64(seed, 4 * N * N)
    u = ((z >> np.uint64(40)).astype(np.float64) + 1.0) * (2.0 ** -24)
    return u.astype(np.float32).reshape(4, N, N)


# ---------------------------------------------------------------------------
# FP64 oracle
# ---------------------------------------------------------------------------

def h0(p: Params, nz: np.ndarray) -> np.ndarray:
    nz = np.ascontiguousarray(nz, dtype=np.float32)
    assert nz.shape == (4, p.N, p.N)
    out = np.empty((p.N, p.N, 4), dtype=np.float64)
    cp = p._c()
    lib().orc_h0(C.byref(cp), _p(nz, C.c_float), _p(out, C.c_double))
    return out


def count_clamped(p: Params) -> int:
    cp = p._c()
    return lib().orc_count_clamped(C.byref(cp))


def spectrum(p: Params, h0a: np.ndarray, t: float) -> np.ndarray:
    """(3, N, N) complex128 spectra (Dx, Dy, Dz) at time t."""
    h0a = np.ascontiguousarray(h0a, dtype=np.float64)
    out = np.empty((3, p.N, p.N, 2), dtype=np.float64)
    cp = p._c()
    lib().orc_spectrum(C.byref(cp), _p(h0a, C.c_double), float(t), _p(out, C.c_double))
    return out[..., 0] + 1j * out[..., 1]


def update(p: Params, h0a: np.ndarray, t: float) -> dict:
    """One frame: dict of dx, dy, dz (N, N) and nj (N, N, 4), float64."""
    h0a = np.ascontiguousarray(h0a, dtype=np.float64)
    N = p.N
    dx, dy, dz = (np.empty((N, N)) for _ in range(3))
    nj = np.empty((N, N, 4))
    cp = p._c()
    lib().orc_update(C.byref(cp), _p(h0a, C.c_double), float(t), _p(dx, C.c_double),
                     _p(dy, C.c_double), _p(dz, C.c_double), _p(nj, C.c_double))
    return {"dx": dx, "dy": dy, "dz": dz, "nj": nj}


def finish(p: Params, raw: np.ndarray) -> dict:
    """Output stage (lambda, Sobel normal, Jacobian) from raw (3, N, N)."""
    raw = np.ascontiguousarray(raw, dtype=np.float64)
    N = p.N
    dx, dy, dz = (np.empty((N, N)) for _ in range(3))
    nj = np.empty((N, N, 4))
    cp = p._c()
    lib().orc_finish(C.byref(cp), _p(raw, C.c_double), _p(dx, C.c_double), _p(dy, C.c_double),
                     _p(dz, C.c_double), _p(nj, C.c_double))
    return {"dx": dx, "dy": dy, "dz": dz, "nj": nj}


def ifft2_real(spec_f: np.ndarray) -> np.ndarray:
    N = spec_f.shape[0]
    a = np.ascontiguousarray(np.stack([spec_f.real, spec_f.imag], -1), dtype=np.float64)
    out = np.empty((N, N))
    lib().orc_ifft2_real(N, _p(a, C.c_double), _p(out, C.c_double))
    return out


def backward(p: Params, h0a: np.ndarray, times, g_dx=None, g_dy=None, g_dz=None):
    """FP64 adjoint: returns (dh0 (N, N, 4), dict(dA, dV, dtheta, dlambda)) for
    upstream gradients g_* of shape (T, N, N) (None = zero)."""
    h0a = np.ascontiguousarray(h0a, dtype=np.float64)
    ts = np.ascontiguousarray(np.atleast_1d(times), dtype=np.float64)
    T = len(ts)
    gs = [None if g is None else np.ascontiguousarray(np.reshape(g, (T, p.N, p.N)), dtype=np.float64)
          for g in (g_dx, g_dy, g_dz)]
    dh0 = np.empty((p.N, p.N, 4))
    gr = np.empty(4)
    cp = p._c()
    lib().orc_backward(C.byref(cp), _p(h0a, C.c_double), _p(ts, C.c_double), T,
                       *[(_p(g, C.c_double) if g is not None else None) for g in gs],
                       _p(dh0, C.c_double), _p(gr, C.c_double))
    return dh0, {"dA": gr[0], "dV": gr[1], "dtheta": gr[2], "dlambda": gr[3]}


def displace_grid(frame: dict, n: int, uv_scale: float = 64.0, disp_scale: float = 0.5) -> np.ndarray:
    """Displaced grid vertices (n+1)^2 x 8 (position, normal, texcoord) from
    one frame's maps (dx, dy, dz (N, N), nj (N, N, 4)): orc_displace_grid."""
    N = frame["dy"].shape[0]
    m = [np.ascontiguousarray(frame[k], dtype=np.float64) for k in ("dx", "dy", "dz", "nj")]
    out = np.empty(((n + 1) * (n + 1), 8))
    lib().orc_displace_grid(N, *[_p(x, C.c_double) for x in m], n, float(uv_scale), float(disp_scale),
                            _p(out, C.c_double))
    return out


def tess_levels(n: int, camera) -> np.ndarray:
    """Per-triangle tessellation levels 2n^2 x 4 (outer 0..2, inner): orc_tess_levels."""
    cam = np.asarray(camera, dtype=np.float64)
    out = np.empty((2 * n * n, 4))
    lib().orc_tess_levels(n, _p(cam, C.c_double), _p(out, C.c_double))
    return out


def shade(vertices: np.ndarray, camera, sun_direction, sea_color, sky: np.ndarray) -> np.ndarray:
    """ocean_fs.glsl's colour at each vertex (n x 8 -> n x 4): orc_shade.  sky:
    (6, S, S, 4) cube map, faces +X, -X, +Y, -Y, +Z, -Z."""
    v = np.ascontiguousarray(vertices, dtype=np.float64)
    sk = np.ascontiguousarray(sky, dtype=np.float64)
    vec = [np.asarray(x, dtype=np.float64) for x in (camera, sun_direction, sea_color)]
    out = np.empty((v.shape[0], 4))
    lib().orc_shade(_p(v, C.c_double), v.shape[0], *[_p(x, C.c_double) for x in vec], _p(sk, C.c_double),
                    sk.shape[1], _p(out, C.c_double))
    return out


SKY_DEFAULTS = dict(earth_pos=(0.0, 6360010.0, 0.0), beta_r=(0.0058 / 1000, 0.0135 / 1000, 0.0331 / 1000),
                    mie_g=0.75, sun_intensity=100.0)


def sky_sun_direction(angle: float) -> np.ndarray:
    """SUN_DIR of the reference for its GUI sun angle (main.cpp:151,157):
    -normalize(0, sin a, cos a) in FP32."""
    v = np.array([0.0, np.sin(np.float32(angle)), np.cos(np.float32(angle))], dtype=np.float32)
    return -(v * (np.float32(1.0) / np.sqrt(np.float32(v @ v)))).astype(np.float32)


def sky_envmap(camera, sun_direction, transmittance: np.ndarray, inscatter: np.ndarray, S: int,
               earth_pos=SKY_DEFAULTS["earth_pos"], beta_r=SKY_DEFAULTS["beta_r"], mie_g=SKY_DEFAULTS["mie_g"],
               sun_intensity=SKY_DEFAULTS["sun_intensity"]) -> np.ndarray:
    """The sky cube map (6, S, S, 4) of sky_envmap_fs.glsl: orc_sky_envmap
    (FP32, the shader's operation order).  transmittance (64, 256, 4),
    inscatter (32, 128, 256, 4), float32."""
    prm = np.array([*camera, *sun_direction, *earth_pos, *beta_r, mie_g, sun_intensity], dtype=np.float32)
    tr = np.ascontiguousarray(transmittance, dtype=np.float32)
    ins = np.ascontiguousarray(inscatter, dtype=np.float32)
    assert tr.shape == (64, 256, 4) and ins.shape == (32, 128, 256, 4)
    out = np.empty((6, S, S, 4), dtype=np.float32)
    lib().orc_sky_envmap(_p(prm, C.c_float), S, _p(tr, C.c_float), _p(ins, C.c_float), _p(out, C.c_float))
    return out


def skybox_matrix(view, projection) -> np.ndarray:
    """inverse(projection * mat4(mat3(view))) for 4x4 column-major (glm)
    matrices given as (4, 4) arrays indexed [column][row]; returned the same
    way, float64."""
    V = np.asarray(view, np.float64).T          # [row][column]
    P = np.asarray(projection, np.float64).T
    R = np.eye(4)
    R[:3, :3] = V[:3, :3]
    return np.linalg.inv(P @ R).T


def skybox(sky: np.ndarray, view, projection, W: int, H: int) -> np.ndarray:
    """sky_fs.glsl's colour per pixel (H, W, 4): orc_skybox on a (6, S, S, 4)
    cube map."""
    sk = np.ascontiguousarray(sky, dtype=np.float64)
    m = np.ascontiguousarray(skybox_matrix(view, projection).reshape(16))
    out = np.empty((H, W, 4))
    lib().orc_skybox(_p(sk, C.c_double), sk.shape[1], _p(m, C.c_double), W, H, _p(out, C.c_double))
    return out


def bit_reversed(N: int) -> np.ndarray:
    out = np.empty(N, dtype=np.int32)
    lib().orc_bit_reversed(N, _p(out, C.c_int32))
    return out


def twiddle_table(N: int) -> np.ndarray:
    lg = N.bit_length() - 1
    out = np.empty((lg, N, 4))
    lib().orc_twiddle_table(N, _p(out, C.c_double))
    return out


# ---------------------------------------------------------------------------
# FP32 port of the reference algorithm (CPU baseline)
# ---------------------------------------------------------------------------

class Port:
    """The reference's per-frame algorithm in FP32 C with OpenMP: spectrum
    pass, 2*log2(N) table-driven radix-2 ping-pong passes per field,
    inversion, Sobel normal map (main.cpp:240-244)."""

    def __init__(self, p: Params, nz: np.ndarray):
        self.p = p
        nz = np.ascontiguousarray(nz, dtype=np.float32)
        cp = p._c()
        self._s = lib().port_create(C.byref(cp), _p(nz, C.c_float))
        N = p.N
        self.dx, self.dy, self.dz = (np.empty((N, N), np.float32) for _ in range(3))
        self.nj = np.empty((N, N, 4), np.float32)

    def h0(self) -> np.ndarray:
        N = self.p.N
        ptr = lib().port_h0_ptr(self._s)
        return np.ctypeslib.as_array(ptr, shape=(N, N, 4)).copy()

    def frame(self, t: float) -> dict:
        lib().port_frame(self._s, float(t), _p(self.dx, C.c_float), _p(self.dy, C.c_float),
                         _p(self.dz, C.c_float), _p(self.nj, C.c_float))
        return {"dx": self.dx, "dy": self.dy, "dz": self.dz, "nj": self.nj}

    def close(self):
        if self._s:
            lib().port_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def max_threads() -> int:
    return lib().port_max_threads()


def set_threads(n: int) -> None:
    lib().port_set_threads(int(n))


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
