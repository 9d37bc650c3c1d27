"""Displaced grid and tessellation levels on the GPU (ocean_displace_grid,
ocean_grid_tess_levels through the C ABI) against the FP64 oracle.

Tolerances (FP32 texel coordinates and bilinear weights against FP64): vertex
positions within 2e-5 absolute per unit of map amplitude plus the FP32
rounding of the grid coordinate (|x| <= squares/2); normals and texcoords
within 1e-5 per unit of their magnitude; tessellation levels equal except where
the FP64 mean distance lies within 1e-4 of a level threshold (10, 20, 30)."""
import numpy as np
import pytest

import params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _to_dev(torch, frame):
    dev = torch.device("cuda")
    return [torch.tensor(np.ascontiguousarray(frame[k], dtype=np.float32), device=dev) for k in ("dx", "dy", "dz", "nj")]


def _check_vertices(got, want, n, amp):
    assert got.shape == want.shape
    assert np.abs(got[:, :3] - want[:, :3]).max() < 2e-5 * max(1.0, amp) + 1e-7 * n
    assert np.abs(got[:, 3:6] - want[:, 3:6]).max() < 1e-5 * max(1.0, float(np.abs(want[:, 3:6]).max()))
    assert np.abs(got[:, 6:] - want[:, 6:]).max() < 1e-5 * max(1.0, float(want[:, 6:].max()))


@pytest.mark.parametrize("N,n,uv,disp", [(64, 48, 3.25, 1.7), (32, 2, 1.0, 0.5), (256, 1024, 64.0, 0.5)])
def test_displace_grid_random_maps(torch_cuda, ocean_lib, oracle_mod, N, n, uv, disp):
    torch = torch_cuda
    rng = np.random.default_rng(N + n)
    frame = {k: rng.standard_normal((N, N)) for k in ("dx", "dy", "dz")}
    frame["nj"] = rng.standard_normal((N, N, 4))
    maps = _to_dev(torch, frame)
    g = ocean_lib.grid_params(n, uv, disp, (0.0, 10.0, 0.0))
    out = torch.empty(((n + 1) * (n + 1), 8), device=torch.device("cuda"))
    ocean_lib.displace_grid(*maps, g, out)
    torch.cuda.synchronize()
    want = oracle_mod.displace_grid({k: v.astype(np.float32).astype(np.float64) for k, v in frame.items()}, n, uv, disp)
    _check_vertices(out.cpu().numpy().astype(np.float64), want, n, max(float(np.abs(frame[k]).max()) for k in frame))


def test_displace_grid_of_a_frame(torch_cuda, ocean_lib, oracle_mod):
    """The reference's grid (1024 squares, UV repeat 64, displacement 0.5) over
    a frame of the reference's default-size map (N = 256) from ocean_update."""
    torch = torch_cuda
    d = P.c1()
    N = d["N"]
    dev = torch.device("cuda")
    bufs = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        oc.update(1.0, *bufs)
    torch.cuda.synchronize()
    frame = {k: b.cpu().numpy().astype(np.float64) for k, b in zip(("dx", "dy", "dz", "nj"), bufs)}
    g = ocean_lib.grid_params()
    out = torch.empty((1025 * 1025, 8), device=dev)
    ocean_lib.displace_grid(*bufs, g, out)
    torch.cuda.synchronize()
    _check_vertices(out.cpu().numpy().astype(np.float64), oracle_mod.displace_grid(frame, 1024, 64.0, 0.5), 1024,
                    max(float(np.abs(frame[k]).max()) for k in frame))


@pytest.mark.parametrize("n,cam", [(1024, (0.0, 10.0, 0.0)), (64, (3.3, 2.0, -7.1)), (256, (-100.0, 4.0, 60.0))])
def test_tess_levels(torch_cuda, ocean_lib, oracle_mod, n, cam):
    torch = torch_cuda
    out = torch.empty((2 * n * n, 4), device=torch.device("cuda"))
    ocean_lib.grid_tess_levels(ocean_lib.grid_params(n, 64.0, 0.5, cam), out)
    torch.cuda.synchronize()
    got, want = out.cpu().numpy().astype(np.float64), oracle_mod.tess_levels(n, cam)
    bad = np.nonzero(got != want)[0]
    if bad.size:
        # only triangles whose FP64 edge means sit on a threshold may differ
        h = n // 2
        sq, t = bad // 2, bad % 2
        zi, xi = sq // n, sq % n
        d = lambda x, z: np.sqrt((cam[0] - (x - h)) ** 2 + cam[1] ** 2 + (cam[2] - (z - h)) ** 2)
        pts = [(d(xi, zi), d(xi, zi + 1), d(xi + 1, zi)), (d(xi + 1, zi), d(xi, zi + 1), d(xi + 1, zi + 1))]
        for j, (s, tt) in enumerate(zip(sq, t)):
            v0, v1, v2 = [p[j] for p in pts[tt]]
            means = np.array([(v1 + v2) / 2, (v2 + v0) / 2, (v0 + v1) / 2])
            assert np.min(np.abs(means[:, None] - np.array([10.0, 20.0, 30.0])[None, :])) < 1e-4
    assert bad.size <= 1e-4 * got.shape[0]


def test_grid_argument_errors(torch_cuda, ocean_lib):
    torch = torch_cuda
    dev = torch.device("cuda")
    maps = [torch.zeros((32, 32), device=dev) for _ in range(3)] + [torch.zeros((32, 32, 4), device=dev)]
    out = torch.empty((4 * 4, 8), device=dev)
    for bad in (ocean_lib.grid_params(3), ocean_lib.grid_params(0), ocean_lib.grid_params(2, float("nan"))):
        with pytest.raises(ocean_lib.OceanError):
            ocean_lib.displace_grid(*maps, bad, out)


def test_shade_grid(torch_cuda, ocean_lib, oracle_mod):
    """ocean_fs.glsl at displaced vertices against the FP64 oracle: random
    vertices and cube map (1e-5 absolute on the 0..1 colours, 1e-3 where the
    reflected ray lies within 1e-4 of a cube-map face edge, where the face choice
    may differ between FP32 and FP64)."""
    torch = torch_cuda
    rng = np.random.default_rng(12)
    n = 20000
    v = np.zeros((n, 8), dtype=np.float32)
    v[:, :3] = rng.uniform(-60, 60, (n, 3))
    nrm = rng.standard_normal((n, 3)) * 0.4 + np.array([0, 1, 0])
    v[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1)[:, None]      # unit normals, as the normal map holds
    sky = rng.uniform(0, 3, (6, 16, 16, 4)).astype(np.float32)
    cam, sun, sea = (2.0, 25.0, -7.0), (0.3, -0.85, 0.2), (0.0, 0.12, 0.3)
    dev = torch.device("cuda")
    vt, skt = torch.tensor(v, device=dev), torch.tensor(sky, device=dev)
    out = torch.empty((n, 4), device=dev)
    ocean_lib.shade_grid(vt, cam, sun, sea, skt, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    want = oracle_mod.shade(v.astype(np.float64), cam, sun, sea, sky.astype(np.float64))
    err = np.abs(got - want).max(1)
    Vv = np.asarray(cam) - v[:, :3].astype(np.float64)
    Vv /= np.linalg.norm(Vv, axis=1)[:, None]
    N = v[:, 3:6].astype(np.float64)
    R = 2 * np.sum(N * Vv, 1)[:, None] * N - Vv
    a = np.sort(np.abs(R), 1)
    near_edge = (a[:, 2] - a[:, 1]) < 1e-4 * a[:, 2]
    assert np.isfinite(got).all()
    assert err[~near_edge].max() < 1e-5


def test_frame_grid_shade_pipeline(torch_cuda, ocean_lib, oracle_mod):
    """frame -> displaced grid -> shaded vertices, end to end on the device."""
    torch = torch_cuda
    d = P.c1()
    N = d["N"]
    dev = torch.device("cuda")
    bufs = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        oc.update(2.5, *bufs)
    g = ocean_lib.grid_params(256, 16.0, 0.5, (0.0, 12.0, 0.0))
    verts = torch.empty((257 * 257, 8), device=dev)
    ocean_lib.displace_grid(*bufs, g, verts)
    sky = torch.ones((6, 4, 4, 4), device=dev) * 0.5
    cols = torch.empty((257 * 257, 4), device=dev)
    ocean_lib.shade_grid(verts, (0.0, 12.0, 0.0), (0.0, -0.7071, 0.7071), (0.0, 0.1, 0.2), sky, cols)
    torch.cuda.synchronize()
    want = oracle_mod.shade(verts.cpu().numpy().astype(np.float64), (0.0, 12.0, 0.0), (0.0, -0.7071, 0.7071),
                            (0.0, 0.1, 0.2), sky.cpu().numpy().astype(np.float64))
    assert np.abs(cols.cpu().numpy() - want).max() < 1e-5
    assert np.isfinite(cols.cpu().numpy()).all()
