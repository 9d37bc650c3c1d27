"""GPU adjoint (ocean_backward through the C ABI) against the FP64 oracle's
adjoint and against central finite differences of the FP64 forward.

Tolerances: per-mode dL/dh0 relative L2 <= 1e-5 against the FP64 adjoint;
parameter gradients within 1e-4 relative of finite differences (h = 1e-3
relative, FP64 forward) and of the FP64 adjoint."""
import math

import numpy as np
import pytest

from conftest import rel_l2
import params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _setup(N, literal=False, seed=3):
    d = dict(N=N, L=1500.0, amplitude=3.0, wind_speed=22.0, wind_x=P.f32(math.cos(math.radians(50))),
             wind_y=P.f32(math.sin(math.radians(50))), choppiness=P.f32(1.1), suppression=P.f32(0.1), seed=seed)
    return d, P.oracle_params(d, literal_conj=literal), P.lib_params(d, literal_conj=literal)


def _gpu_backward(torch, ocean_lib, lp, seed, times, g, want_dh0=True, accumulate_split=None):
    dev = torch.device("cuda")
    N = lp.N
    gt = [torch.tensor(np.asarray(x, np.float32), device=dev) for x in g]
    dh0 = torch.zeros((N, N, 4), dtype=torch.float32, device=dev) if want_dh0 else None
    with ocean_lib.Ocean(lp, seed=seed) as oc:
        if accumulate_split is None:
            r = oc.backward(times, gt[0], gt[1], gt[2], dh0=dh0)
        else:
            k = accumulate_split
            r1 = oc.backward(times[:k], gt[0][:k], gt[1][:k], gt[2][:k], dh0=dh0)
            r2 = oc.backward(times[k:], gt[0][k:], gt[1][k:], gt[2][k:], dh0=dh0, accumulate=True)
            r = {key: r1[key] + r2[key] for key in r1}
        torch.cuda.synchronize()
    return r, (dh0.cpu().numpy() if want_dh0 else None)


def _check_params(r, ref, tol):
    for k in ("dA", "dV", "dtheta", "dlambda"):
        assert abs(r[k] - ref[k]) <= tol * max(abs(ref[k]), 1e-30), (k, r[k], ref[k])


@pytest.mark.parametrize("N,literal", [(32, False), (64, True), (256, False), (512, False), (1024, False),
                                       (2048, False)])
def test_backward_matches_fp64_adjoint(torch_cuda, ocean_lib, oracle_mod, N, literal):
    d, op, lp = _setup(N, literal)
    times = [0.0, 0.7, 3.1] if N <= 1024 else [0.7]
    T = len(times)
    rng = np.random.default_rng(N)
    g = [rng.standard_normal((T, N, N)).astype(np.float32) for _ in range(3)]
    h = oracle_mod.h0(op, oracle_mod.noise(d["seed"], N))
    dh0_ref, ref = oracle_mod.backward(op, h, times, *[x.astype(np.float64) for x in g])
    r, dh0 = _gpu_backward(torch_cuda, ocean_lib, lp, d["seed"], times, g)
    assert rel_l2(dh0, dh0_ref) < 1e-5
    _check_params(r, ref, 1e-4)


def test_backward_chunks_and_accumulates(torch_cuda, ocean_lib, oracle_mod):
    """T above one chunk (64 frames) and OCEAN_GRAD_ACCUMULATE split calls give
    the one-call result."""
    N = 64
    d, op, lp = _setup(N)
    times = [0.05 * j for j in range(70)]
    rng = np.random.default_rng(1)
    g = [rng.standard_normal((70, N, N)).astype(np.float32) for _ in range(3)]
    h = oracle_mod.h0(op, oracle_mod.noise(d["seed"], N))
    dh0_ref, ref = oracle_mod.backward(op, h, times, *[x.astype(np.float64) for x in g])
    r, dh0 = _gpu_backward(torch_cuda, ocean_lib, lp, d["seed"], times, g)
    assert rel_l2(dh0, dh0_ref) < 1e-5
    _check_params(r, ref, 1e-4)
    r2, dh02 = _gpu_backward(torch_cuda, ocean_lib, lp, d["seed"], times, g, accumulate_split=23)
    assert rel_l2(dh02, dh0) < 1e-6
    _check_params(r2, r, 1e-6)


def test_backward_null_fields(torch_cuda, ocean_lib, oracle_mod):
    """NULL upstream gradients count as zero (here only Dy carries a loss)."""
    N = 128
    d, op, lp = _setup(N)
    times = [1.25]
    rng = np.random.default_rng(5)
    gy = rng.standard_normal((1, N, N)).astype(np.float32)
    h = oracle_mod.h0(op, oracle_mod.noise(d["seed"], N))
    dh0_ref, ref = oracle_mod.backward(op, h, times, None, gy.astype(np.float64), None)
    dev = torch_cuda.device("cuda")
    dh0 = torch_cuda.zeros((N, N, 4), dtype=torch_cuda.float32, device=dev)
    with ocean_lib.Ocean(lp, seed=d["seed"]) as oc:
        r = oc.backward(times, None, torch_cuda.tensor(gy, device=dev), None, dh0=dh0)
    assert rel_l2(dh0.cpu().numpy(), dh0_ref) < 1e-5
    # no Dx/Dz loss: dlambda is zero up to the FP32 residue of unpacking two
    # real fields from one complex transform
    assert abs(r["dlambda"]) < 1e-5 * max(abs(ref["dA"]), abs(ref["dV"]), abs(ref["dtheta"]))
    _check_params({k: r[k] for k in ("dA", "dV", "dtheta")} | {"dlambda": 0.0}, ref | {"dlambda": 0.0}, 1e-4)


def test_parameter_gradients_vs_finite_differences(torch_cuda, ocean_lib, oracle_mod):
    """Central differences (h = 1e-3 relative for A, V, lambda) of
    L = sum_t <g_t, D_t> with the FP64 forward, against the GPU adjoint: 1e-4
    relative.  theta uses an absolute step of 1e-5 rad: the amplitude goes
    as |k^.w|, which has a kink where k^.w = 0, and a larger step straddles
    the kinks of the modes near it."""
    N = 128
    d, op, lp = _setup(N)
    times = [0.4, 2.2]
    rng = np.random.default_rng(9)
    g = [rng.standard_normal((2, N, N)) for _ in range(3)]
    nz = oracle_mod.noise(d["seed"], N)
    base = dict(N=N, L=d["L"], amplitude=d["amplitude"], wind_speed=d["wind_speed"], wind_x=d["wind_x"],
                wind_y=d["wind_y"], choppiness=d["choppiness"], suppression=d["suppression"], gravity=P.f32(9.81))

    def loss(prm):
        p = oracle_mod.Params(**prm)
        hh = oracle_mod.h0(p, nz)
        s = 0.0
        for j, t in enumerate(times):
            o = oracle_mod.update(p, hh, t)
            s += np.sum(g[0][j] * o["dx"]) + np.sum(g[1][j] * o["dy"]) + np.sum(g[2][j] * o["dz"])
        return s

    r, _ = _gpu_backward(torch_cuda, ocean_lib, lp, d["seed"], times, [x.astype(np.float32) for x in g],
                         want_dh0=False)
    fd = {}
    for name, key in (("dA", "amplitude"), ("dV", "wind_speed"), ("dlambda", "choppiness")):
        e = 1e-3 * base[key]
        a, b = dict(base), dict(base)
        a[key] += e
        b[key] -= e
        fd[name] = (loss(a) - loss(b)) / (2 * e)
    th = math.atan2(base["wind_y"], base["wind_x"])
    e = 1e-5
    a, b = dict(base), dict(base)
    a["wind_x"], a["wind_y"] = math.cos(th + e), math.sin(th + e)
    b["wind_x"], b["wind_y"] = math.cos(th - e), math.sin(th - e)
    fd["dtheta"] = (loss(a) - loss(b)) / (2 * e)
    _check_params(r, fd, 1e-4)
