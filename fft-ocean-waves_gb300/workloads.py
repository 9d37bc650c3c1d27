"""Seeded synthetic workloads of the benchmark configurations, shared by the
benchmark and the tests so that both run exactly the same tiles.

The reference publishes no benchmark; these are the configurations its
per-frame path is measured on here (seeded uniform noise, float32 parameters):

  plain(N)        the drop-in tile: L=2000 m, A=2, wind 30 m/s at 30 deg,
                  lambda=1.3, l=0.1, seed 1 (N=512 and N=1024 are timed).
  batched_tiles() 64 tiles, N uniform in {128..2048}, L~U(100,4000),
                  A~U(0.5,8), V~U(5,40), theta~U(0,2pi), lambda~U(0,2), own
                  noise; numpy seed 2; 8 time samples t~U(0,600) s each.
  fit_params()    the parameter-fit tile, N=512: A=3, V=22 m/s at 50 deg,
                  lambda=1.1, L=1500 m, seed 3.
  adjoint_sets()  16 full-spectrum adjoint sets at N=2048: L=3000, A~U(1,6),
                  V~U(10,35), theta~U(0,2pi), lambda~U(0.5,1.5), seeds 10..25;
                  the target of set s comes from h0 * (1 + 0.05 xi), xi
                  standard normal per component (perturb_seed(s)).
"""
from __future__ import annotations

import math

import numpy as np

import ocean_gb300 as og


def f32(v) -> float:
    return float(np.float32(v))


def plain(N: int = 1024) -> og.Params:
    a = math.radians(30.0)
    return og.Params(N=N, L=2000.0, amplitude=2.0, wind_speed=30.0, wind_dir_x=f32(math.cos(a)),
                     wind_dir_y=f32(math.sin(a)), choppiness=f32(1.3), suppression=f32(0.1), gravity=f32(9.81))


PLAIN_SEED = 1


def batched_tiles(n_tiles: int = 64, seed: int = 2, samples: int = 8):
    """(tile params, noise seeds, times [n_tiles * samples], tile-major)."""
    rng = np.random.default_rng(seed)
    tiles, seeds = [], []
    for i in range(n_tiles):
        N = int(rng.choice([128, 256, 512, 1024, 2048]))
        th = rng.uniform(0, 2 * math.pi)
        tiles.append(og.Params(N=N, L=f32(rng.uniform(100, 4000)), amplitude=f32(rng.uniform(0.5, 8)),
                               wind_speed=f32(rng.uniform(5, 40)), wind_dir_x=f32(math.cos(th)),
                               wind_dir_y=f32(math.sin(th)), choppiness=f32(rng.uniform(0, 2)),
                               suppression=f32(0.1), gravity=f32(9.81)))
        seeds.append(1000 + i)
    times = rng.uniform(0, 600, size=n_tiles * samples).tolist()
    return tiles, seeds, times


def fit_params(A=3.0, V=22.0, theta_deg=50.0, lam=1.1) -> og.Params:
    a = math.radians(theta_deg)
    return og.Params(N=512, L=1500.0, amplitude=A, wind_speed=V, wind_dir_x=f32(math.cos(a)),
                     wind_dir_y=f32(math.sin(a)), choppiness=f32(lam), suppression=f32(0.1), gravity=f32(9.81))


ADJ_N, ADJ_T, ADJ_DT = 2048, 64, 0.05


def adjoint_sets(n_sets: int = 16):
    """[(params, noise seed)] of the full-spectrum adjoint sets."""
    rng = np.random.default_rng(10)
    out = []
    for s in range(n_sets):
        a = rng.uniform(0, 2 * math.pi)
        p = og.Params(N=ADJ_N, L=3000.0, amplitude=f32(rng.uniform(1, 6)), wind_speed=f32(rng.uniform(10, 35)),
                      wind_dir_x=f32(math.cos(a)), wind_dir_y=f32(math.sin(a)),
                      choppiness=f32(rng.uniform(0.5, 1.5)), suppression=f32(0.1), gravity=f32(9.81))
        out.append((p, 10 + s))
    return out


def perturb_seed(s: int) -> int:
    return 5000 + s
