"""Python face of oracle/_ref/libref_glsl.so -- TEST INFRASTRUCTURE ONLY.

Runs the reference's own compute shaders (compiled for the CPU by
oracle/build_ref.py) in the order src/main.cpp dispatches them.  Only the
golden-fixture generator (tests/golden/make_golden.py) and CPU tests that skip
when the library is absent use this module.
"""
import ctypes as C
import os

import numpy as np

from . import build_ref

_LIB = None


def available() -> bool:
    return os.path.exists(build_ref.LIB) or build_ref.available()


def lib():
    global _LIB
    if _LIB is None:
        path = build_ref.LIB if os.path.exists(build_ref.LIB) and not build_ref.available() else build_ref.build()
        L = C.CDLL(path)
        fp, ip = C.POINTER(C.c_float), C.POINTER(C.c_int32)
        L.ref_bit_reversed.argtypes = [C.c_int, ip]
        L.ref_twiddle.argtypes = [C.c_int, ip, fp]
        L.ref_h0.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp, fp]
        L.ref_h0_t.argtypes = [C.c_int, C.c_int, C.c_float, fp, fp, fp, fp, fp]
        L.ref_butterfly_fft.argtypes = [C.c_int, fp, fp, fp, fp]
        L.ref_normal_map.argtypes = [C.c_int, fp, fp]
        L.ref_sky_envmap.argtypes = [fp, C.c_int, fp, fp, fp]
        for n in ("ref_bit_reversed", "ref_twiddle", "ref_h0", "ref_h0_t", "ref_butterfly_fft", "ref_normal_map",
                  "ref_sky_envmap"):
            getattr(L, n).restype = None
        _LIB = L
    return _LIB


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def bit_reversed(N):
    out = np.empty(N, np.int32)
    lib().ref_bit_reversed(N, out.ctypes.data_as(C.POINTER(C.c_int32)))
    return out


def twiddle_image(N):
    """The RGBA32F twiddle texture, [y][stage][4]."""
    br = bit_reversed(N)
    lg = N.bit_length() - 1
    out = np.zeros((N, lg, 4), np.float32)
    lib().ref_twiddle(N, br.ctypes.data_as(C.POINTER(C.c_int32)), _f(out))
    return out


def h0(N, L, A, V, wx, wy, l, noise):
    noise = np.ascontiguousarray(noise, np.float32)
    h0k = np.zeros((N, N, 2), np.float32)
    h0mk = np.zeros((N, N, 2), np.float32)
    lib().ref_h0(N, int(L), A, V, wx, wy, l, _f(noise), _f(h0k), _f(h0mk))
    return h0k, h0mk


def frame(N, L, t, h0k, h0mk):
    """tilde_h0_t + butterfly_fft(dy), (dx), (dz) + generate_normal_map
    (main.cpp:240-244).  Returns raw dx, dy, dz (R32F) and normal (RGBA32F)."""
    h0k = np.ascontiguousarray(h0k, np.float32).copy()
    h0mk = np.ascontiguousarray(h0mk, np.float32).copy()
    spec = {k: np.zeros((N, N, 4), np.float32) for k in ("dx", "dy", "dz")}
    lib().ref_h0_t(N, int(L), float(t), _f(h0k), _f(h0mk), _f(spec["dx"]), _f(spec["dy"]), _f(spec["dz"]))
    tw = twiddle_image(N)
    pong = np.zeros((N, N, 4), np.float32)
    out = {}
    for k in ("dy", "dx", "dz"):
        dst = np.zeros((N, N), np.float32)
        lib().ref_butterfly_fft(N, _f(tw), _f(spec[k]), _f(pong), _f(dst))
        out[k] = dst
    normal = np.zeros((N, N, 4), np.float32)
    lib().ref_normal_map(N, _f(out["dy"]), _f(normal))
    out["normal"] = normal
    return out


def sky_envmap(prm, S, transmittance, inscatter):
    """sky_envmap_fs.glsl (with atmosphere.glsl) over the six capture faces:
    (6, S, S, 4).  prm: camera[3], sun_direction[3], earth_pos[3], beta_r[3],
    mie_g, sun_intensity."""
    p = np.ascontiguousarray(prm, dtype=np.float32)
    tr = np.ascontiguousarray(transmittance, dtype=np.float32)
    ins = np.ascontiguousarray(inscatter, dtype=np.float32)
    assert tr.shape == (64, 256, 4) and ins.shape == (32, 128, 256, 4)
    out = np.empty((6, S, S, 4), np.float32)
    lib().ref_sky_envmap(_f(p), S, _f(tr), _f(ins), _f(out))
    return out
