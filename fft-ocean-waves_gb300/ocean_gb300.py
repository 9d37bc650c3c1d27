"""ctypes binding of include/ocean.h (libocean_gb300.so).

This is the binding a Python caller of the library uses; it mirrors the
reference's per-frame interface (FFTOceanWaves::init / update, main.cpp:199-255):
``Ocean(params, noise)`` runs the init-time h0 and table set-up and
``Ocean.update(t)`` runs one frame of the hot path on the GPU.

The library must have been built (``python fft-ocean-waves_gb300/build.py``
or ``__graft_entry__.build()``); there is no CPU fallback and loading fails
loudly when it is missing.  Device buffers are passed as integer addresses;
torch tensors are accepted where convenient (``data_ptr()``).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libocean_gb300.so")

OCEAN_OK = 0
OCEAN_ERR_INVALID = -1
OCEAN_ERR_CUDA = -2
OCEAN_ERR_NOMEM = -3
OCEAN_ERR_UNSUPPORTED = -4
OCEAN_ERR_TIMEOUT = -5
OCEAN_FLAG_LITERAL_CONJ = 1

# Every entry point include/ocean.h declares (checked by the CPU tests).
EXPORTS = [
    "ocean_create", "ocean_create_seeded", "ocean_destroy", "ocean_update", "ocean_update_rows",
    "ocean_update_columns", "ocean_update_outputs", "ocean_update_columns_outputs", "ocean_get_outputs",
    "ocean_set_params", "ocean_get_params", "ocean_get_h0", "ocean_set_h0", "ocean_compute_h0",
    "ocean_fill_noise", "ocean_bit_reversed_indices", "ocean_butterfly_table", "ocean_last_error",
    "ocean_version", "ocean_backward", "ocean_device_status", "ocean_batch_create", "ocean_batch_update",
    "ocean_batch_device_status", "ocean_batch_destroy", "ocean_update_noalloc", "ocean_displace_grid",
    "ocean_grid_tess_levels", "ocean_shade_grid", "ocean_sky_envmap", "ocean_render_skybox",
    "ocean_debug_fail_allocations", "ocean_noalloc_device_status", "ocean_get_tuning", "ocean_set_tuning",
]
OCEAN_GRAD_ACCUMULATE = 1


class OceanError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ocean error {code}: {msg}")
        self.code = code


class ocean_params(C.Structure):
    _fields_ = [("N", C.c_int32), ("flags", C.c_uint32), ("L", C.c_float), ("amplitude", C.c_float),
                ("wind_speed", C.c_float), ("wind_dir_x", C.c_float), ("wind_dir_y", C.c_float),
                ("choppiness", C.c_float), ("suppression", C.c_float), ("gravity", C.c_float)]


class ocean_outputs(C.Structure):
    _fields_ = [("dx", C.c_void_p), ("dy", C.c_void_p), ("dz", C.c_void_p), ("normal_j", C.c_void_p)]


class ocean_tuning(C.Structure):
    _fields_ = [("row_overlap", C.c_int32), ("row_ctas_per_sm", C.c_int32), ("wave_mib", C.c_int32),
                ("col_fused", C.c_int32), ("row_variant", C.c_int32)]


class ocean_grads(C.Structure):
    _fields_ = [("dA", C.c_double), ("dV", C.c_double), ("dtheta", C.c_double), ("dlambda", C.c_double),
                ("dh0", C.c_void_p)]


@dataclasses.dataclass
class Params:
    """Tile parameters (defaults: the reference's main.cpp:1631-1646)."""
    N: int = 256
    L: float = 1000.0
    amplitude: float = 2.0
    wind_speed: float = 80.0
    wind_dir_x: float = 1.0
    wind_dir_y: float = 1.0
    choppiness: float = 0.75
    suppression: float = 0.1
    gravity: float = 9.81
    literal_conj: bool = False

    @staticmethod
    def from_angle(N, L, amplitude, wind_speed, angle_deg, choppiness, suppression=0.1, **kw):
        a = math.radians(angle_deg)
        return Params(N=N, L=L, amplitude=amplitude, wind_speed=wind_speed, wind_dir_x=math.cos(a),
                      wind_dir_y=math.sin(a), choppiness=choppiness, suppression=suppression, **kw)

    def c(self) -> ocean_params:
        return ocean_params(self.N, OCEAN_FLAG_LITERAL_CONJ if self.literal_conj else 0, self.L,
                            self.amplitude, self.wind_speed, self.wind_dir_x, self.wind_dir_y,
                            self.choppiness, self.suppression, self.gravity)


_lib = None


def load() -> C.CDLL:
    """Load libocean_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OceanError(OCEAN_ERR_UNSUPPORTED,
                         f"{LIB_PATH} is missing: build it with fft-ocean-waves_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp, P = C.c_void_p, C.POINTER
    L.ocean_create.argtypes = [P(ocean_params), P(C.c_float), P(vp)]
    L.ocean_create_seeded.argtypes = [P(ocean_params), C.c_uint64, P(vp)]
    L.ocean_destroy.argtypes = [vp]
    L.ocean_destroy.restype = None
    L.ocean_update.argtypes = [vp, C.c_double, P(ocean_outputs), vp]
    L.ocean_update_rows.argtypes = [vp, C.c_double, vp]
    L.ocean_update_columns.argtypes = [vp, vp]
    L.ocean_update_outputs.argtypes = [vp, P(ocean_outputs), vp]
    L.ocean_update_columns_outputs.argtypes = [vp, P(ocean_outputs), vp]
    L.ocean_get_outputs.argtypes = [vp, P(ocean_outputs)]
    L.ocean_set_params.argtypes = [vp, P(ocean_params)]
    L.ocean_get_params.argtypes = [vp, P(ocean_params)]
    L.ocean_get_h0.argtypes = [vp, vp, vp]
    L.ocean_set_h0.argtypes = [vp, vp, vp]
    L.ocean_compute_h0.argtypes = [P(ocean_params), vp, vp, vp]
    L.ocean_fill_noise.argtypes = [C.c_uint64, C.c_int32, P(C.c_float)]
    L.ocean_bit_reversed_indices.argtypes = [C.c_int32, P(C.c_int32)]
    L.ocean_butterfly_table.argtypes = [C.c_int32, P(C.c_float)]
    L.ocean_backward.argtypes = [vp, P(C.c_double), C.c_int32, vp, vp, vp, C.c_uint32, P(ocean_grads), vp]
    L.ocean_device_status.argtypes = [vp, vp]
    L.ocean_batch_create.argtypes = [P(ocean_params), P(C.c_uint64), C.c_int32, C.c_int32, P(vp)]
    L.ocean_batch_update.argtypes = [vp, P(C.c_double), P(ocean_outputs), vp]
    L.ocean_batch_device_status.argtypes = [vp, vp]
    L.ocean_batch_destroy.argtypes = [vp]
    L.ocean_batch_destroy.restype = None
    L.ocean_update_noalloc.argtypes = [P(ocean_params), vp, C.c_double, P(ocean_outputs), vp]
    L.ocean_noalloc_device_status.argtypes = [vp]
    L.ocean_get_tuning.argtypes = [C.c_int32, P(ocean_tuning)]
    L.ocean_set_tuning.argtypes = [C.c_int32, P(ocean_tuning)]
    L.ocean_displace_grid.argtypes = [P(ocean_outputs), C.c_int32, P(ocean_grid_params), vp, vp]
    L.ocean_grid_tess_levels.argtypes = [P(ocean_grid_params), vp, vp]
    L.ocean_shade_grid.argtypes = [vp, C.c_int64, P(ocean_shade_params), vp, vp, vp]
    L.ocean_sky_envmap.argtypes = [P(ocean_sky_params), vp, vp, vp, vp]
    L.ocean_render_skybox.argtypes = [vp, C.c_int32, P(C.c_float), P(C.c_float), C.c_int32, C.c_int32, vp, vp]
    L.ocean_last_error.restype = C.c_char_p
    L.ocean_debug_fail_allocations.argtypes = [C.c_int32]
    L.ocean_debug_fail_allocations.restype = None
    not_int = ("ocean_destroy", "ocean_batch_destroy", "ocean_debug_fail_allocations",   # void
               "ocean_last_error")                                                      # const char*
    for name in EXPORTS:
        if name not in not_int:
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OCEAN_OK:
        raise OceanError(rc, load().ocean_last_error().decode())


def _addr(x) -> int | None:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_contiguous") and not x.is_contiguous():
            raise ValueError("device buffers passed to the C ABI must be contiguous")
        return x.data_ptr()
    raise TypeError(f"cannot take a device address of {type(x)}")


def _stream(s) -> int | None:
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream  # torch.cuda.Stream


def fill_noise(seed: int, N: int):
    import numpy as np
    out = np.empty((4, N, N), dtype=np.float32)
    check(load().ocean_fill_noise(seed, N, out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def bit_reversed_indices(N: int):
    import numpy as np
    out = np.empty(N, dtype=np.int32)
    check(load().ocean_bit_reversed_indices(N, out.ctypes.data_as(C.POINTER(C.c_int32))))
    return out


def butterfly_table(N: int):
    import numpy as np
    lg = N.bit_length() - 1
    out = np.empty((lg, N, 4), dtype=np.float32)
    check(load().ocean_butterfly_table(N, out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def update_noalloc(params: Params, h0_dev, t: float, dx, dy, dz, normal_j, stream=None) -> None:
    """One frame from a caller-held h0 without any device allocation
    (ocean_update_noalloc: static scratch, N <= 1024)."""
    cp = params.c()
    o = ocean_outputs(_addr(dx), _addr(dy), _addr(dz), _addr(normal_j))
    check(load().ocean_update_noalloc(C.byref(cp), _addr(h0_dev), float(t), C.byref(o), _stream(stream)))


def get_tuning(N: int) -> dict:
    """The launch configuration of size N (ocean_get_tuning)."""
    t = ocean_tuning()
    check(load().ocean_get_tuning(int(N), C.byref(t)))
    return {"row_overlap": t.row_overlap, "row_ctas_per_sm": t.row_ctas_per_sm, "wave_mib": t.wave_mib,
            "col_fused": t.col_fused, "row_variant": t.row_variant}


def set_tuning(N: int, row_overlap=None, row_ctas_per_sm=None, wave_mib=None, col_fused=None,
               row_variant=None) -> dict:
    """Replace fields of size N's launch configuration for this process
    (ocean_set_tuning); returns the previous configuration."""
    old = get_tuning(N)
    new = dict(old)
    for k, v in (("row_overlap", row_overlap), ("row_ctas_per_sm", row_ctas_per_sm), ("wave_mib", wave_mib),
                 ("col_fused", col_fused), ("row_variant", row_variant)):
        if v is not None:
            new[k] = int(v)
    t = ocean_tuning(new["row_overlap"], new["row_ctas_per_sm"], new["wave_mib"], new["col_fused"],
                     new["row_variant"])
    check(load().ocean_set_tuning(int(N), C.byref(t)))
    return old


def noalloc_device_status(stream=None) -> None:
    """Raise OceanError (OCEAN_ERR_TIMEOUT) if a kernel of ocean_update_noalloc
    on the current device gave up a bounded wait; clears the status."""
    check(load().ocean_noalloc_device_status(_stream(stream)))


class ocean_grid_params(C.Structure):
    _fields_ = [("squares", C.c_int32), ("texcoord_scale", C.c_float), ("displacement_scale", C.c_float),
                ("camera", C.c_float * 3)]


def grid_params(squares=1024, texcoord_scale=64.0, displacement_scale=0.5, camera=(0.0, 10.0, 0.0)):
    """The reference's render grid (GRID_SIZE 1024, GRID_UV_SCALE 64, displacement 0.5) by default."""
    return ocean_grid_params(int(squares), float(texcoord_scale), float(displacement_scale),
                             (C.c_float * 3)(*[float(c) for c in camera]))


def displace_grid(dx, dy, dz, normal_j, grid: "ocean_grid_params", vertices, stream=None) -> None:
    """Displaced grid vertices ((squares+1)^2, 8) from one frame's maps (device)."""
    N = int(dy.shape[0])
    o = ocean_outputs(_addr(dx), _addr(dy), _addr(dz), _addr(normal_j))
    check(load().ocean_displace_grid(C.byref(o), N, C.byref(grid), _addr(vertices), _stream(stream)))


def grid_tess_levels(grid: "ocean_grid_params", levels, stream=None) -> None:
    """Per-triangle tessellation levels (2*squares^2, 4) into `levels` (device)."""
    check(load().ocean_grid_tess_levels(C.byref(grid), _addr(levels), _stream(stream)))


class ocean_shade_params(C.Structure):
    _fields_ = [("camera", C.c_float * 3), ("sun_direction", C.c_float * 3), ("sea_color", C.c_float * 3),
                ("sky_size", C.c_int32)]


def shade_grid(vertices, camera, sun_direction, sea_color, sky, colors, stream=None) -> None:
    """ocean_fs.glsl's colour at each displaced vertex: vertices (n, 8), sky
    (6, S, S, 4) cube map, colors (n, 4); device tensors."""
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])
    p = ocean_shade_params(f3(camera), f3(sun_direction), f3(sea_color), int(sky.shape[1]))
    check(load().ocean_shade_grid(_addr(vertices), int(vertices.shape[0]), C.byref(p), _addr(sky), _addr(colors),
                                  _stream(stream)))


class ocean_sky_params(C.Structure):
    _fields_ = [("camera", C.c_float * 3), ("sun_direction", C.c_float * 3), ("earth_pos", C.c_float * 3),
                ("beta_r", C.c_float * 3), ("mie_g", C.c_float), ("sun_intensity", C.c_float), ("size", C.c_int32)]


# The reference's sky uniforms (main.cpp:80-84,149-158).
SKY_EARTH_POS = (0.0, 6360010.0, 0.0)
SKY_BETA_R = (0.0058 / 1000.0, 0.0135 / 1000.0, 0.0331 / 1000.0)
SKY_MIE_G = 0.75
SKY_SUN_INTENSITY = 100.0


def sky_sun_direction(angle: float):
    """SUN_DIR for the reference's GUI sun angle (main.cpp:151,157):
    -normalize(0, sin a, cos a), in FP32 as glm computes it."""
    import numpy as np
    v = np.array([0.0, np.sin(np.float32(angle)), np.cos(np.float32(angle))], dtype=np.float32)
    return tuple(float(x) for x in -(v * (np.float32(1.0) / np.sqrt(np.float32(v @ v)))))


def sky_envmap(camera, sun_direction, transmittance, inscatter, cubemap, earth_pos=SKY_EARTH_POS, beta_r=SKY_BETA_R,
               mie_g=SKY_MIE_G, sun_intensity=SKY_SUN_INTENSITY, stream=None) -> None:
    """The sky environment cube map of render_envmap(): transmittance (64,
    256, 4), inscatter (32, 128, 256, 4), cubemap (6, S, S, 4) output; device
    tensors (float32)."""
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])
    p = ocean_sky_params(f3(camera), f3(sun_direction), f3(earth_pos), f3(beta_r), float(mie_g), float(sun_intensity),
                         int(cubemap.shape[1]))
    check(load().ocean_sky_envmap(C.byref(p), _addr(transmittance), _addr(inscatter), _addr(cubemap),
                                  _stream(stream)))


def render_skybox(sky, view, projection, image, stream=None) -> None:
    """sky_fs.glsl into a headless image: sky (6, S, S, 4) cube map, view and
    projection 4x4 column-major (glm; (4, 4) arrays indexed [column][row] or
    16 floats), image (H, W, 4); device tensors for sky and image."""
    import numpy as np
    v = (C.c_float * 16)(*[float(x) for x in np.asarray(view, dtype=np.float32).reshape(16)])
    p = (C.c_float * 16)(*[float(x) for x in np.asarray(projection, dtype=np.float32).reshape(16)])
    check(load().ocean_render_skybox(_addr(sky), int(sky.shape[1]), v, p, int(image.shape[1]), int(image.shape[0]),
                                     _addr(image), _stream(stream)))


def debug_fail_allocations(after: int) -> None:
    """Test hook: the library's allocations succeed `after` more times, then
    fail with OCEAN_ERR_NOMEM; after < 0 turns it off."""
    load().ocean_debug_fail_allocations(int(after))


def load_sky_tables(texture_dir: str):
    """The reference's sky tables from its data/texture directory (the .raw
    files main.cpp:89-143 reads): transmittance (64, 256, 4), irradiance (16,
    64, 4) and inscatter (32, 128, 256, 4) as float32 arrays, None for a file
    that is absent (the reference ships without inscatter.raw)."""
    import os
    import numpy as np
    shapes = {"transmittance": (64, 256, 4), "irradiance": (16, 64, 4), "inscatter": (32, 128, 256, 4)}
    out = {}
    for name, shape in shapes.items():
        path = os.path.join(texture_dir, name + ".raw")
        if not os.path.exists(path):
            out[name] = None
            continue
        a = np.fromfile(path, dtype="<f4")
        if a.size != int(np.prod(shape)):
            raise ValueError(f"{path}: {a.size} floats, expected {int(np.prod(shape))}")
        out[name] = a.reshape(shape)
    return out


def _png_channel0(path: str):
    """Channel 0 of an 8-bit, non-interlaced PNG (gray, gray+alpha, RGB or
    RGBA) as a uint8 array (height, width): chunk walk, zlib inflate, per-row
    filter reversal (filter types 0-4 of the PNG specification)."""
    import struct
    import zlib
    import numpy as np
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
        pos += 12 + ln
    if hdr is None:
        raise ValueError(f"{path}: no IHDR chunk")
    w, h, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth != 8 or chans is None or interlace:
        raise ValueError(f"{path}: only 8-bit non-interlaced gray/RGB(A) PNGs are supported")
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    stride = w * chans
    raw = raw.reshape(h, stride + 1)
    img = np.zeros((h, stride), dtype=np.int32)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        out = np.empty(stride, dtype=np.int32)
        if f == 0:
            out[:] = line
        elif f == 2:
            out[:] = (line + prev) & 255
        else:
            for i in range(stride):
                left = out[i - chans] if i >= chans else 0
                up, ul = prev[i], (prev[i - chans] if i >= chans else 0)
                if f == 1:
                    pr = left
                elif f == 3:
                    pr = (left + up) >> 1
                elif f == 4:
                    p_ = left + up - ul
                    pa, pb, pc = abs(p_ - left), abs(p_ - up), abs(p_ - ul)
                    pr = left if (pa <= pb and pa <= pc) else (up if pb <= pc else ul)
                else:
                    raise ValueError(f"{path}: bad filter type {f}")
                out[i] = (line[i] + pr) & 255
        img[y] = out
        prev = out
    return img[:, ::chans].astype(np.uint8)


def noise_from_pngs(paths, N: int | None = None):
    """The reference's noise textures (data/noise/LDR_LLL1_{0..3}.png,
    main.cpp:1085-1088) as ocean_create's noise: 4 planes of N x N floats,
    channel 0 / 255 (the shaders read .r of an unsigned-normalised texture;
    tilde_h0_k_cs.glsl clamps to [0.001, 1]).  N defaults to the texture size;
    another N samples texel floor(x * size / N) (nearest)."""
    import numpy as np
    planes = [_png_channel0(p) for p in paths]
    if len(planes) != 4:
        raise ValueError("four noise textures are needed")
    H, W = planes[0].shape
    if any(p.shape != (H, W) for p in planes):
        raise ValueError("the noise textures differ in size")
    N = N or W
    ys, xs = (np.arange(N) * H) // N, (np.arange(N) * W) // N
    return np.stack([p[np.ix_(ys, xs)] for p in planes]).astype(np.float32) / np.float32(255.0)


def compute_h0(params: Params, noise_dev, h0_dev, stream=None) -> None:
    cp = params.c()
    check(load().ocean_compute_h0(C.byref(cp), _addr(noise_dev), _addr(h0_dev), _stream(stream)))


class Ocean:
    """One ocean tile on the GPU (handle of include/ocean.h)."""

    def __init__(self, params: Params, noise=None, seed: int | None = None):
        L = load()
        self.params = params
        self._h = C.c_void_p()
        cp = params.c()
        if noise is not None:
            import numpy as np
            nz = np.ascontiguousarray(noise, dtype=np.float32)
            if nz.size != 4 * params.N * params.N:
                raise ValueError("noise must hold 4*N*N floats")
            check(L.ocean_create(C.byref(cp), nz.ctypes.data_as(C.POINTER(C.c_float)), C.byref(self._h)))
        else:
            check(L.ocean_create_seeded(C.byref(cp), int(seed or 0), C.byref(self._h)))

    @property
    def handle(self) -> int:
        return self._h.value

    def update(self, t: float, dx=None, dy=None, dz=None, normal_j=None, stream=None) -> None:
        """One frame at time t.  Without output buffers, the handle's own
        buffers (``outputs()``) are written."""
        if dx is None:
            check(load().ocean_update(self._h, float(t), None, _stream(stream)))
            return
        o = ocean_outputs(_addr(dx), _addr(dy), _addr(dz), _addr(normal_j))
        check(load().ocean_update(self._h, float(t), C.byref(o), _stream(stream)))

    def update_rows(self, t: float, stream=None) -> None:
        check(load().ocean_update_rows(self._h, float(t), _stream(stream)))

    def update_columns(self, stream=None) -> None:
        check(load().ocean_update_columns(self._h, _stream(stream)))

    def update_outputs(self, dx=None, dy=None, dz=None, normal_j=None, stream=None) -> None:
        if dx is None:
            check(load().ocean_update_outputs(self._h, None, _stream(stream)))
            return
        o = ocean_outputs(_addr(dx), _addr(dy), _addr(dz), _addr(normal_j))
        check(load().ocean_update_outputs(self._h, C.byref(o), _stream(stream)))

    def update_columns_outputs(self, dx=None, dy=None, dz=None, normal_j=None, stream=None) -> None:
        """Columns and outputs as one stage (one fused kernel where the tuning
        says so)."""
        if dx is None:
            check(load().ocean_update_columns_outputs(self._h, None, _stream(stream)))
            return
        o = ocean_outputs(_addr(dx), _addr(dy), _addr(dz), _addr(normal_j))
        check(load().ocean_update_columns_outputs(self._h, C.byref(o), _stream(stream)))

    def backward(self, times, g_dx=None, g_dy=None, g_dz=None, dh0=None, accumulate=False, stream=None) -> dict:
        """Gradients for upstream dL/d(dx, dy, dz) of shape (T, N, N) (device
        tensors or addresses; None = zero).  dh0 (device N*N*4) receives
        dL/dh0 when given.  Returns dA, dV, dtheta, dlambda."""
        ts = (C.c_double * len(times))(*[float(t) for t in times])
        g = ocean_grads(0.0, 0.0, 0.0, 0.0, _addr(dh0))
        check(load().ocean_backward(self._h, ts, len(times), _addr(g_dx), _addr(g_dy), _addr(g_dz),
                                    OCEAN_GRAD_ACCUMULATE if accumulate else 0, C.byref(g), _stream(stream)))
        return {"dA": g.dA, "dV": g.dV, "dtheta": g.dtheta, "dlambda": g.dlambda}

    def device_status(self, stream=None) -> None:
        """Synchronise and raise if a kernel reported a bounded-wait time-out."""
        check(load().ocean_device_status(self._h, _stream(stream)))

    def outputs(self) -> dict:
        o = ocean_outputs()
        check(load().ocean_get_outputs(self._h, C.byref(o)))
        return {"dx": o.dx, "dy": o.dy, "dz": o.dz, "normal_j": o.normal_j}

    def set_params(self, params: Params) -> None:
        cp = params.c()
        check(load().ocean_set_params(self._h, C.byref(cp)))
        self.params = params

    def get_h0(self, dst, stream=None) -> None:
        check(load().ocean_get_h0(self._h, _addr(dst), _stream(stream)))

    def set_h0(self, src, stream=None) -> None:
        check(load().ocean_set_h0(self._h, _addr(src), _stream(stream)))

    def close(self) -> None:
        if self._h and self._h.value:
            load().ocean_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OceanBatch:
    """Independent tiles (any mix of N) advanced `samples` time samples per
    update in one CUDA-graph replay (ocean_batch_* of include/ocean.h)."""

    def __init__(self, params_list, seeds, samples: int):
        L = load()
        n = len(params_list)
        if len(seeds) != n:
            raise ValueError("one seed per tile")
        self.params = list(params_list)
        self.samples = int(samples)
        ps = (ocean_params * n)(*[p.c() for p in params_list])
        ss = (C.c_uint64 * n)(*[int(x) for x in seeds])
        self._h = C.c_void_p()
        check(L.ocean_batch_create(ps, ss, n, self.samples, C.byref(self._h)))

    def update(self, times, outputs, stream=None) -> None:
        """times: n_tiles*samples values (tile-major); outputs: as many
        (dx, dy, dz, normal_j) tuples of device buffers."""
        n = len(self.params) * self.samples
        if len(times) != n or len(outputs) != n:
            raise ValueError(f"need {n} times and output sets")
        ts = (C.c_double * n)(*[float(t) for t in times])
        os_ = (ocean_outputs * n)(*[ocean_outputs(*[_addr(b) for b in o]) for o in outputs])
        check(load().ocean_batch_update(self._h, ts, os_, _stream(stream)))

    def device_status(self, stream=None) -> None:
        check(load().ocean_batch_device_status(self._h, _stream(stream)))

    def close(self) -> None:
        if self._h and self._h.value:
            load().ocean_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
