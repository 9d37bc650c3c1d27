"""The smallest ctypes binding of the per-frame path: what a Python host of
the reference's ocean would add to call the library instead of dispatching the
compute shaders of FFTOceanWaves::update() (src/main.cpp:240-244).

ocean_gb300.py is the complete binding; this stub is the part a maintainer
copies.  Its structures must stay identical to include/ocean.h (checked by the
CPU tests against the full binding and the header).

    import ctypes_stub as cs
    lib = cs.load("fft-ocean-waves_gb300/libocean_gb300.so")
    h = C.c_void_p()
    p = cs.ocean_params(1024, 0, 2000.0, 2.0, 30.0, 0.866, 0.5, 1.3, 0.1, 9.81)
    assert lib.ocean_create_seeded(C.byref(p), 1, C.byref(h)) == 0, lib.ocean_last_error()
    outs = cs.ocean_outputs(dx_ptr, dy_ptr, dz_ptr, nj_ptr)   # device addresses, 16-byte aligned
    assert lib.ocean_update(h, t, C.byref(outs), stream_ptr) == 0, lib.ocean_last_error()
    lib.ocean_destroy(h)
"""
import ctypes as C


class ocean_params(C.Structure):
    _fields_ = [("N", C.c_int32), ("flags", C.c_uint32), ("L", C.c_float), ("amplitude", C.c_float),
                ("wind_speed", C.c_float), ("wind_dir_x", C.c_float), ("wind_dir_y", C.c_float),
                ("choppiness", C.c_float), ("suppression", C.c_float), ("gravity", C.c_float)]


class ocean_outputs(C.Structure):
    _fields_ = [("dx", C.c_void_p), ("dy", C.c_void_p), ("dz", C.c_void_p), ("normal_j", C.c_void_p)]


def load(path: str) -> C.CDLL:
    lib = C.CDLL(path)
    lib.ocean_create_seeded.argtypes = [C.POINTER(ocean_params), C.c_uint64, C.POINTER(C.c_void_p)]
    lib.ocean_create_seeded.restype = C.c_int
    lib.ocean_update.argtypes = [C.c_void_p, C.c_double, C.POINTER(ocean_outputs), C.c_void_p]
    lib.ocean_update.restype = C.c_int
    lib.ocean_destroy.argtypes = [C.c_void_p]
    lib.ocean_destroy.restype = None
    lib.ocean_last_error.restype = C.c_char_p
    return lib
