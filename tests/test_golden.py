"""Pins the oracle (and the library's host-side tables) to golden vectors that
the reference's own shader code produced (tests/golden/make_golden.py runs the
reference compute shaders compiled for the CPU).

The reference computes in FP32 with FP32 time and a no-op conjugate(); the
oracle is compared in its literal-conjugate mode with lambda = 1 (the compute
shaders never apply lambda) at FP32 tolerances.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

GOLD = os.path.join(ROOT, "tests", "golden")


def _load(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    return z, json.loads(str(z["meta"]))


def _oracle_params(oracle_mod, meta):
    f = lambda v: float(np.float32(v))
    return oracle_mod.Params(N=meta["N"], L=float(meta["L"]), amplitude=meta["A"], wind_speed=meta["V"],
                             wind_x=meta["wx"], wind_y=meta["wy"], choppiness=1.0, suppression=meta["l"],
                             gravity=f(9.81), literal_conj=True)


def test_bit_reversal_matches_reference(oracle_mod, ocean_lib):
    z, _ = _load("ref_tables")
    for N in (32, 64, 128, 256, 512, 1024, 2048):
        g = z[f"bitrev_{N}"]
        assert np.array_equal(oracle_mod.bit_reversed(N), g)
        assert np.array_equal(ocean_lib.bit_reversed_indices(N), g)


def test_twiddle_table_matches_reference(oracle_mod, ocean_lib):
    z, _ = _load("ref_tables")
    for N in (32, 64, 256):
        g = z[f"twiddle_{N}"].transpose(1, 0, 2)          # [stage][y][4]
        o = oracle_mod.twiddle_table(N)
        lib = ocean_lib.butterfly_table(N)
        assert np.array_equal(o[..., 2:], g[..., 2:])
        assert np.array_equal(lib[..., 2:], g[..., 2:])
        assert np.abs(o[..., :2] - g[..., :2]).max() < 1e-6
        assert np.abs(lib[..., :2] - g[..., :2]).max() < 1e-6


@pytest.mark.parametrize("name", ["ref_frame_N32", "ref_frame_N64"])
def test_h0_matches_reference(oracle_mod, name):
    z, meta = _load(name)
    N = meta["N"]
    g = np.concatenate([z["h0k"], z["h0minusk"]], -1).astype(np.float64)
    # the reference's DC mode is NaN (normalize(0)); the oracle pins it to 0
    assert np.isnan(g[N // 2, N // 2]).all()
    g[N // 2, N // 2] = 0.0
    o = oracle_mod.h0(_oracle_params(oracle_mod, meta), oracle_mod.noise(meta["seed"], N))
    assert rel_l2(o, g) < 2e-6


@pytest.mark.parametrize("name", ["ref_frame_N32", "ref_frame_N64"])
def test_frames_match_reference(oracle_mod, name):
    z, meta = _load(name)
    N = meta["N"]
    p = _oracle_params(oracle_mod, meta)
    h = oracle_mod.h0(p, oracle_mod.noise(meta["seed"], N))
    for i, t in enumerate(z["times"]):
        o = oracle_mod.update(p, h, float(t))
        for k in ("dx", "dy", "dz"):
            assert rel_l2(o[k], z[f"{k}_{i}"]) < 1e-5, (k, t)
        n = z[f"normal_{i}"]
        assert rel_l2(o["nj"][..., :3], n[..., :3]) < 1e-5
        assert np.all(n[..., 3] == 1.0)                    # the reference's normal.w


def test_fp32_port_matches_reference(oracle_mod):
    """The FP32 port (CPU baseline) runs the same algorithm as the shaders."""
    z, meta = _load("ref_frame_N64")
    N = meta["N"]
    p = _oracle_params(oracle_mod, meta)
    port = oracle_mod.Port(p, oracle_mod.noise(meta["seed"], N))
    for i, t in enumerate(z["times"]):
        o = port.frame(float(t))
        for k in ("dx", "dy", "dz"):
            assert rel_l2(o[k], z[f"{k}_{i}"]) < 1e-5, (k, t)
    port.close()
