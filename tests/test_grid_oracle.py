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


def _cube_np(sky, r):
    S = sky.shape[1]
    ax, ay, az = np.abs(r[:, 0]), np.abs(r[:, 1]), np.abs(r[:, 2])
    xm = (ax >= ay) & (ax >= az)
    ym = ~xm & (ay >= az)
    zm = ~xm & ~ym
    face = np.where(xm, np.where(r[:, 0] >= 0, 0, 1), np.where(ym, np.where(r[:, 1] >= 0, 2, 3),
                                                                np.where(r[:, 2] >= 0, 4, 5)))
    ma = np.where(xm, ax, np.where(ym, ay, az))
    sc = np.select([face == 0, face == 1, face == 2, face == 3, face == 4], [-r[:, 2], r[:, 2], r[:, 0], r[:, 0], r[:, 0]],
                   -r[:, 0])
    tc = np.select([face == 2, face == 3], [r[:, 2], -r[:, 2]], -r[:, 1])
    s = 0.5 * (sc / ma + 1) * S - 0.5
    t = 0.5 * (tc / ma + 1) * S - 0.5
    s0, t0 = np.floor(s), np.floor(t)
    ws, wt = (s - s0)[:, None], (t - t0)[:, None]
    cl = lambda i: np.clip(i.astype(np.int64), 0, S - 1)
    sa, sb, ta, tb = cl(s0), cl(s0 + 1), cl(t0), cl(t0 + 1)
    f = sky[face]
    g = lambda tt, ss: f[np.arange(len(r)), tt, ss, :3]
    return (g(ta, sa) * (1 - ws) + g(ta, sb) * ws) * (1 - wt) + (g(tb, sa) * (1 - ws) + g(tb, sb) * ws) * wt


def test_shade_matches_numpy(oracle_mod):
    rng = np.random.default_rng(8)
    n = 4000
    v = np.zeros((n, 8))
    v[:, :3] = rng.uniform(-50, 50, (n, 3))
    nrm = rng.standard_normal((n, 3)) * 0.4 + np.array([0, 1, 0])
    v[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1)[:, None]      # unit normals, as the normal map holds
    sky = rng.uniform(0, 3, (6, 7, 7, 4))
    cam, sun, sea = np.array([1.0, 20.0, -3.0]), np.array([0.2, -0.9, 0.3]), np.array([0.0, 0.1, 0.3])
    got = oracle_mod.shade(v, cam, sun, sea, sky)
    V = cam - v[:, :3]
    V /= np.linalg.norm(V, axis=1)[:, None]
    N = v[:, 3:6]
    nv = np.sum(N * V, 1)
    R = 2 * nv[:, None] * N - V
    F = 0.04 + 0.96 * (1 - np.maximum(nv, 0)) ** 5
    nl = np.maximum(-(N @ sun), 0)
    col = nl[:, None] * (sea * (1 - F[:, None]) + _cube_np(sky, R) * F[:, None])
    want = (col / (col + 1)) ** (1 / 2.2)
    assert np.abs(got[:, :3] - want).max() < 1e-12
    assert np.all(got[:, 3] == 1.0)
