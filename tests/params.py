"""Parameter sets of the benchmark configurations (seeded synthetic noise).

Every value is rounded to float32 first, because the library takes float32
parameters; the FP64 oracle is then fed exactly the same numbers.
"""
import math

import numpy as np


def f32(x):
    return float(np.float32(x))


def c1():
    """Plain single tile N=256: L=1000, A=4, V=40 along (1,1)/sqrt2, lambda=1,
    l = Lw/1000, seed 0, t = 1.0."""
    V = 40.0
    l = (V * V / 9.81) / 1000.0
    return dict(N=256, L=1000.0, amplitude=4.0, wind_speed=V, wind_x=f32(1 / math.sqrt(2)),
                wind_y=f32(1 / math.sqrt(2)), choppiness=1.0, suppression=f32(l), seed=0)


def c2(N):
    """Plain drop-in throughput tile: L=2000, A=2, V=30 at 30 deg, lambda=1.3,
    l=0.1, seed 1."""
    a = math.radians(30.0)
    return dict(N=N, L=2000.0, amplitude=2.0, wind_speed=30.0, wind_x=f32(math.cos(a)),
                wind_y=f32(math.sin(a)), choppiness=f32(1.3), suppression=f32(0.1), seed=1)


def reference_default(N=256):
    """The reference demo's own defaults (main.cpp:1631-1646)."""
    return dict(N=N, L=1000.0, amplitude=2.0, wind_speed=80.0, wind_x=1.0, wind_y=1.0,
                choppiness=f32(0.75), suppression=f32(0.1), seed=0)


def oracle_params(d, literal_conj=False):
    from oracle import oracle
    return oracle.Params(N=d["N"], L=d["L"], amplitude=d["amplitude"], wind_speed=d["wind_speed"],
                         wind_x=d["wind_x"], wind_y=d["wind_y"], choppiness=d["choppiness"],
                         suppression=d["suppression"], gravity=f32(9.81), literal_conj=literal_conj)


def lib_params(d, literal_conj=False):
    import ocean_gb300
    return ocean_gb300.Params(N=d["N"], L=d["L"], amplitude=d["amplitude"], wind_speed=d["wind_speed"],
                              wind_dir_x=d["wind_x"], wind_dir_y=d["wind_y"], choppiness=d["choppiness"],
                              suppression=d["suppression"], gravity=f32(9.81), literal_conj=literal_conj)


def oracle_from_lib(p):
    """oracle.Params carrying exactly an ocean_gb300.Params' values."""
    from oracle import oracle
    return oracle.Params(N=p.N, L=p.L, amplitude=p.amplitude, wind_speed=p.wind_speed, wind_x=p.wind_dir_x,
                         wind_y=p.wind_dir_y, choppiness=p.choppiness, suppression=p.suppression,
                         gravity=p.gravity, literal_conj=p.literal_conj)
