"""The oracle's displaced grid and tessellation levels against an independent
numpy restatement of grid_tes.glsl:55-66 / grid_tcs.glsl:27-59 and of the
grid of main.cpp:748-824 (bilinear REPEAT sampling, texel centres at
(i + 0.5)/N)."""
import numpy as np


def _bilinear(m, u, v):
    N = m.shape[0]
    sx, sy = u * N - 0.5, v * N - 0.5
    fx, fy = np.floor(sx), np.floor(sy)
    ax, ay = sx - fx, sy - fy
    x0, y0 = fx.astype(np.int64) % N, fy.astype(np.int64) % N
    x1, y1 = (x0 + 1) % N, (y0 + 1) % N
    if m.ndim == 3:
        ax, ay = ax[..., None], ay[..., None]
    top = m[y0, x0] * (1 - ax) + m[y0, x1] * ax
    bot = m[y1, x0] * (1 - ax) + m[y1, x1] * ax
    return top * (1 - ay) + bot * ay


def _grid_np(frame, n, uv_scale, disp):
    h = n // 2
    zi, xi = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    u, v = xi / n * uv_scale, zi / n * uv_scale
    out = np.empty((n + 1, n + 1, 8))
    out[..., 0] = (xi - h) - _bilinear(frame["dx"], u, v)
    out[..., 1] = _bilinear(frame["dy"], u, v) * disp
    out[..., 2] = (zi - h) - _bilinear(frame["dz"], u, v)
    out[..., 3:6] = _bilinear(frame["nj"], u, v)[..., :3]
    out[..., 6], out[..., 7] = u, v
    return out.reshape(-1, 8)


def _levels_np(n, cam):
    h = n // 2
    lv = lambda a, b: np.select([(a + b) / 2 <= 10, (a + b) / 2 <= 20, (a + b) / 2 <= 30], [20.0, 10.0, 5.0], 1.0)
    zi, xi = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    d = lambda x, z: np.sqrt((cam[0] - (x - h)) ** 2 + cam[1] ** 2 + (cam[2] - (z - h)) ** 2)
    a0, a1, a2, b2 = d(xi, zi), d(xi, zi + 1), d(xi + 1, zi), d(xi + 1, zi + 1)
    A = np.stack([lv(a1, a2), lv(a2, a0), lv(a0, a1), lv(a0, a1)], -1)
    B = np.stack([lv(a1, b2), lv(b2, a2), lv(a2, a1), lv(a2, a1)], -1)
    return np.stack([A, B], 2).reshape(-1, 4)


def test_displace_grid_matches_numpy(oracle_mod):
    rng = np.random.default_rng(4)
    N, n = 32, 20
    frame = {k: rng.standard_normal((N, N)) for k in ("dx", "dy", "dz")}
    frame["nj"] = rng.standard_normal((N, N, 4))
    for uv, disp in ((64.0, 0.5), (3.25, 1.7), (1.0, -0.3)):
        got = oracle_mod.displace_grid(frame, n, uv, disp)
        want = _grid_np(frame, n, uv, disp)
        assert np.abs(got - want).max() < 1e-12


def test_tess_levels_match_numpy(oracle_mod):
    for n, cam in ((16, (0.0, 5.0, 0.0)), (40, (3.3, 2.0, -7.1)), (64, (100.0, 1.0, 0.0))):
        got = oracle_mod.tess_levels(n, cam)
        assert np.array_equal(got, _levels_np(n, cam))
        assert set(np.unique(got)) <= {1.0, 5.0, 10.0, 20.0}
