"""Parity at the full sizes of the batched and full-spectrum adjoint workloads
(fft-ocean-waves_gb300/workloads.py), and ocean_set_params against a fresh
handle.

Batched: the 64-tile, 8-sample launch the benchmark times (N uniform in
{128..2048}, numpy seed 2).  Every (tile, sample) is compared on the device
with the single-tile ocean_update of the same tile and time (relative L2
<= 1e-6 per map), and one tile of every N -- among them an N = 2048 tile whose
samples run as separate waves -- with the FP64 oracle (1e-5).

Full-spectrum adjoint: N = 2048, T = 65 frames at dt = 0.05 s (one frame past
the 64-frame chunk of ocean_backward), two of the sixteen parameter sets.  The
upstream gradient is the MSE residual against the target sequence of the
5 %-perturbed h0, formed on the device; dL/dh0 must be within 1e-5 relative
L2 of the FP64 adjoint (the oracle runs over the 65 frames in groups, which
is exact: the adjoint is linear in the upstream gradient), and the parameter
gradients within 1e-4."""
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


def _bufs(torch, N, lead=()):
    dev = torch.device("cuda")
    return (torch.empty((*lead, N, N), device=dev), torch.empty((*lead, N, N), device=dev),
            torch.empty((*lead, N, N), device=dev), torch.empty((*lead, N, N, 4), device=dev))


def _rel_l2_dev(torch, a, b):
    a, b = a.double(), b.double()
    den = torch.linalg.vector_norm(b).item()
    return torch.linalg.vector_norm(a - b).item() / (den if den > 0 else 1.0)


def test_batched_workload_full_size(torch_cuda, ocean_lib, oracle_mod):
    import workloads as W
    torch = torch_cuda
    S = 8
    tiles, seeds, times = W.batched_tiles(samples=S)
    outs = [[_bufs(torch, p.N) for _ in range(S)] for p in tiles]
    with ocean_lib.OceanBatch(tiles, seeds, S) as b:
        b.update(times, [o for row in outs for o in row])
        torch.cuda.synchronize()
        b.device_status()
    ref = {}
    worst = 0.0
    for i, (p, sd) in enumerate(zip(tiles, seeds)):
        if p.N not in ref:
            ref[p.N] = _bufs(torch, p.N)
        r = ref[p.N]
        with ocean_lib.Ocean(p, seed=sd) as oc:
            for s in range(S):
                oc.update(times[i * S + s], *r)
                for k in range(4):
                    e = _rel_l2_dev(torch, outs[i][s][k], r[k])
                    worst = max(worst, e)
                    assert e < 1e-6, (i, p.N, s, k, e)
            oc.device_status()
    # one tile of every N against the FP64 oracle; the N = 2048 tile's first
    # and last samples (separate waves)
    picked = {}
    for i, p in enumerate(tiles):
        picked.setdefault(p.N, i)
    assert sorted(picked) == [128, 256, 512, 1024, 2048]
    checks = [(i, 0) for i in picked.values()] + [(picked[2048], S - 1)]
    for i, s in checks:
        p = tiles[i]
        op = P.oracle_from_lib(p)
        h = oracle_mod.h0(op, oracle_mod.noise(seeds[i], p.N))
        want = oracle_mod.update(op, h, times[i * S + s])
        got = [x.cpu().numpy() for x in outs[i][s]]
        for k, name in enumerate(("dx", "dy", "dz")):
            assert rel_l2(got[k], want[name]) < 1e-5, (i, p.N, s, name)
        assert rel_l2(got[3][..., :3], want["nj"][..., :3]) < 1e-5
        assert rel_l2(got[3][..., 3], want["nj"][..., 3]) < 1e-5


@pytest.mark.parametrize("set_index", [0, 9])
def test_full_spectrum_adjoint_crosses_a_chunk(torch_cuda, ocean_lib, oracle_mod, set_index):
    import workloads as W
    torch = torch_cuda
    dev = torch.device("cuda")
    N, T, dt = W.ADJ_N, 65, W.ADJ_DT
    p, seed = W.adjoint_sets()[set_index]
    times = [dt * j for j in range(T)]
    G = torch.empty((3, T, N, N), device=dev)
    nj = torch.empty((N, N, 4), device=dev)
    with ocean_lib.Ocean(p, seed=seed) as oc, ocean_lib.Ocean(p, seed=seed) as target:
        h0 = torch.empty((N, N, 4), device=dev)
        oc.get_h0(h0)
        gen = torch.Generator(device=dev).manual_seed(W.perturb_seed(set_index))
        h0_target = h0 * (1.0 + 0.05 * torch.randn(h0.shape, device=dev, generator=gen))
        target.set_h0(h0_target)
        tb = _bufs(torch, N)
        M = 3.0 * T * N * N
        for j, t in enumerate(times):                 # residual D(h0) - D(h0'), scaled: dMSE/dD
            oc.update(t, G[0, j], G[1, j], G[2, j], nj)
            target.update(t, *tb)
            for f in range(3):
                G[f, j].sub_(tb[f]).mul_(2.0 / M)
        dh0 = torch.zeros((N, N, 4), device=dev)
        r = oc.backward(times, G[0], G[1], G[2], dh0=dh0)
        torch.cuda.synchronize()
        oc.device_status()
    op = P.oracle_from_lib(p)
    h = oracle_mod.h0(op, oracle_mod.noise(seed, N))
    want = np.zeros((N, N, 4))
    wg = {"dA": 0.0, "dV": 0.0, "dtheta": 0.0, "dlambda": 0.0}
    for j0 in range(0, T, 8):                           # the FP64 adjoint, eight frames at a time
        j1 = min(T, j0 + 8)
        g = [G[f, j0:j1].double().cpu().numpy() for f in range(3)]
        d, gr = oracle_mod.backward(op, h, times[j0:j1], *g)
        want += d
        for k in wg:
            wg[k] += gr[k]
    assert rel_l2(dh0.cpu().numpy(), want) < 1e-5
    for k in ("dA", "dV", "dtheta", "dlambda"):
        assert abs(r[k] - wg[k]) <= 1e-4 * abs(wg[k]), (k, r[k], wg[k])


@pytest.mark.parametrize("N", [256, 1024])
def test_set_params_equals_a_fresh_handle(torch_cuda, ocean_lib, N):
    """After ocean_set_params the handle's frames are bit for bit those of a
    handle created with the new parameters and the same noise (including a
    switch of the conjugation flag)."""
    import workloads as W
    torch = torch_cuda
    p1 = W.plain(N)
    p2 = W.fit_params()
    p2.N = N
    p3 = W.fit_params(A=1.0, V=10.0, theta_deg=0.0, lam=0.5)
    p3.N, p3.literal_conj = N, True
    with ocean_lib.Ocean(p1, seed=7) as oc:
        for p in (p2, p3):
            oc.set_params(p)
            with ocean_lib.Ocean(p, seed=7) as fresh:
                for t in (0.0, 3.5, 1.0e5):
                    a, b = _bufs(torch, N), _bufs(torch, N)
                    oc.update(t, *a)
                    fresh.update(t, *b)
                    torch.cuda.synchronize()
                    for x, y in zip(a, b):
                        assert torch.equal(x, y), (p, t)
