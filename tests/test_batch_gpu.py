"""Batched tiles (ocean_batch_* through the C ABI): every (tile, sample)
output against the single-tile update of the same tile and time, and a few
against the FP64 oracle; CUDA-graph replays with new times; argument errors."""
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


def _tiles(sizes, rng):
    out = []
    for N in sizes:
        th = rng.uniform(0, 2 * math.pi)
        out.append(dict(N=N, L=P.f32(rng.uniform(100, 4000)), amplitude=P.f32(rng.uniform(0.5, 8)),
                        wind_speed=P.f32(rng.uniform(5, 40)), wind_x=P.f32(math.cos(th)), wind_y=P.f32(math.sin(th)),
                        choppiness=P.f32(rng.uniform(0, 2)), suppression=P.f32(0.1),
                        seed=int(rng.integers(0, 2 ** 31))))
    return out


def _alloc(torch, N):
    dev = torch.device("cuda")
    return (torch.empty((N, N), device=dev), torch.empty((N, N), device=dev), torch.empty((N, N), device=dev),
            torch.empty((N, N, 4), device=dev))


def _frame(bufs):
    return {"dx": bufs[0].cpu().numpy(), "dy": bufs[1].cpu().numpy(), "dz": bufs[2].cpu().numpy(),
            "nj": bufs[3].cpu().numpy()}


def test_batch_matches_single_tiles(torch_cuda, ocean_lib, oracle_mod):
    torch = torch_cuda
    rng = np.random.default_rng(2)
    sizes = [1024, 32, 256, 64, 512, 128, 256, 2048, 32]
    tiles = _tiles(sizes, rng)
    tiles[2]["literal"] = True
    S = 3
    times = rng.uniform(0, 600, size=(len(tiles), S))
    lps = [P.lib_params(d, literal_conj=d.get("literal", False)) for d in tiles]
    outs = [[_alloc(torch, d["N"]) for _ in range(S)] for d in tiles]
    with ocean_lib.OceanBatch(lps, [d["seed"] for d in tiles], S) as b:
        for rep in range(2):                                     # the graph replays with new times
            tt = times + 17.0 * rep
            b.update(tt.ravel().tolist(), [o for row in outs for o in row])
            torch.cuda.synchronize()
            b.device_status()
            for i, d in enumerate(tiles):
                with ocean_lib.Ocean(lps[i], seed=d["seed"]) as oc:
                    ref = _alloc(torch, d["N"])
                    for s in range(S):
                        oc.update(float(tt[i, s]), *ref)
                        torch.cuda.synchronize()
                        got, want = _frame(outs[i][s]), _frame(ref)
                        for k in ("dx", "dy", "dz", "nj"):
                            assert rel_l2(got[k], want[k]) < 1e-6, (i, s, k)
    # two tiles against the FP64 oracle
    for i in (1, 4):
        d = tiles[i]
        op = P.oracle_params(d, literal_conj=d.get("literal", False))
        h = oracle_mod.h0(op, oracle_mod.noise(d["seed"], d["N"]))
        ref = oracle_mod.update(op, h, float(times[i, 0] + 17.0))
        got = _frame(outs[i][0])
        for k in ("dx", "dy", "dz"):
            assert rel_l2(got[k], ref[k]) < 1e-5
        assert rel_l2(got["nj"][..., :3], ref["nj"][..., :3]) < 1e-5


def test_batch_argument_errors(torch_cuda, ocean_lib):
    torch = torch_cuda
    good = P.lib_params(dict(N=64, L=500.0, amplitude=2.0, wind_speed=20.0, wind_x=1.0, wind_y=0.0,
                             choppiness=1.0, suppression=P.f32(0.1), seed=1))
    bad = P.lib_params(dict(N=48, L=500.0, amplitude=2.0, wind_speed=20.0, wind_x=1.0, wind_y=0.0,
                            choppiness=1.0, suppression=P.f32(0.1), seed=1))
    with pytest.raises(ocean_lib.OceanError) as e:
        ocean_lib.OceanBatch([good, bad], [1, 2], 2)
    assert e.value.code == ocean_lib.OCEAN_ERR_INVALID and "tile 1" in str(e.value)
    with ocean_lib.OceanBatch([good], [1], 2) as b:
        with pytest.raises(ValueError):
            b.update([0.0], [_alloc(torch, 64)])
        o = _alloc(torch, 64)
        with pytest.raises(ocean_lib.OceanError):
            b.update([0.0, float("nan")], [o, o])
