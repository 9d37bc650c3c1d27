"""Generate the golden fixtures from the reference's own shader code.

Runs the reference's hot-path compute shaders (compiled for the CPU by
oracle/build_ref.py from the reference sources, which must be present) in the
order src/main.cpp dispatches them, on seeded noise, and writes:

  ref_tables.npz        bit-reversed indices (main.cpp:29-64,733-744) for
                        N = 32..2048 and the twiddle texture
                        (twiddle_factors_cs.glsl) for N = 32, 64, 256
  ref_frame_N32.npz     h0k, h0minusk (tilde_h0_k_cs.glsl) and frames
  ref_frame_N64.npz     (tilde_h0_t_cs + butterfly_cs + inversion_cs +
                        normal_map_cs) at several times
  ref_sky.npz           sky environment cube maps (sky_envmap_fs.glsl with
                        atmosphere.glsl) on seeded synthetic tables
                        (sky_tables(seed): the reference's inscatter.raw is
                        missing), for two sun angles and camera heights

Each file records its parameters and the sha256 of the shader sources used.
The shaders' DC mode is NaN (normalize(0), tilde_h0_k_cs.glsl:44); as in the
library it is set to 0 before the per-frame shaders run, and the raw NaN is
kept in the stored h0 so tests can see it.

Usage: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, oracle, ref  # noqa: E402

CASES = [
    # the reference demo's defaults (main.cpp:1641-1646) on a 32 x 32 grid
    dict(name="ref_frame_N32", N=32, L=1000, A=2.0, V=80.0, wx=1.0, wy=1.0, l=0.1, seed=11,
         times=[0.0, 1.5, 40.25]),
    # the N=256 benchmark tile's spectrum (A=4, V=40, l=Lw/1000) on a 64 x 64 grid
    dict(name="ref_frame_N64", N=64, L=1000, A=4.0, V=40.0, wx=1.0, wy=1.0, l=(40.0 ** 2 / 9.81) / 1000.0,
         seed=0, times=[1.0, 7.75]),
]


SKY_CASES = [
    # sun 0.4 rad above the horizon, camera 10 m up (sun disk on the -Z face)
    dict(name="high_sun", camera=(0.0, 10.0, 0.0), angle=-0.4, S=32, seed=5),
    # sun at the horizon seen from 2 km: rays through the ground and the disk's edge
    dict(name="low_sun", camera=(30.0, 2000.0, -50.0), angle=-0.02, S=24, seed=6),
]


def sky_tables(seed):
    """Seeded stand-ins for the sky tables: transmittance U(0,1), inscatter
    U(0.001, 0.051), float32 (numpy PCG64)."""
    rng = np.random.default_rng(seed)
    tr = rng.random((64, 256, 4), dtype=np.float32)
    ins = (rng.random((32, 128, 256, 4), dtype=np.float32) * np.float32(0.05) + np.float32(1e-3)).astype(np.float32)
    return tr, ins


def sky_prm(c):
    d = oracle.sky_sun_direction(c["angle"])
    s = oracle.SKY_DEFAULTS
    return np.array([*c["camera"], *d, *s["earth_pos"], *s["beta_r"], s["mie_g"], s["sun_intensity"]], np.float32)


def shader_hashes():
    out = {}
    for s in build_ref.SHADERS:
        with open(os.path.join(build_ref.REF, "src", "shader", s), "rb") as fh:
            out[s] = hashlib.sha256(fh.read()).hexdigest()
    with open(os.path.join(build_ref.REF, "src", "main.cpp"), "rb") as fh:
        out["main.cpp"] = hashlib.sha256(fh.read()).hexdigest()
    return out


def main():
    build_ref.build()
    hashes = shader_hashes()
    tables = {}
    for N in (32, 64, 128, 256, 512, 1024, 2048):
        tables[f"bitrev_{N}"] = ref.bit_reversed(N)
    for N in (32, 64, 256):
        tables[f"twiddle_{N}"] = ref.twiddle_image(N)
    np.savez_compressed(os.path.join(HERE, "ref_tables.npz"), meta=json.dumps({"sha256": hashes}), **tables)

    for c in CASES:
        N = c["N"]
        f32 = lambda v: float(np.float32(v))
        nz = oracle.noise(c["seed"], N)
        h0k, h0mk = ref.h0(N, c["L"], c["A"], c["V"], c["wx"], c["wy"], f32(c["l"]), nz)
        raw_k, raw_mk = h0k.copy(), h0mk.copy()
        h0k[N // 2, N // 2] = 0.0
        h0mk[N // 2, N // 2] = 0.0
        arrs = {"h0k": raw_k, "h0minusk": raw_mk, "times": np.array(c["times"], np.float32)}
        for i, t in enumerate(c["times"]):
            fr = ref.frame(N, c["L"], t, h0k, h0mk)
            for k in ("dx", "dy", "dz", "normal"):
                arrs[f"{k}_{i}"] = fr[k]
        meta = {k: v for k, v in c.items() if k != "name"}
        meta["l"] = f32(c["l"])
        meta["noise"] = "oracle.noise(seed, N): splitmix64 24-bit uniforms, planes [4][N][N]"
        meta["sha256"] = hashes
        np.savez_compressed(os.path.join(HERE, c["name"] + ".npz"), meta=json.dumps(meta), **arrs)
        print("wrote", c["name"])

    sky = {}
    for c in SKY_CASES:
        tr, ins = sky_tables(c["seed"])
        sky[c["name"] + "_prm"] = sky_prm(c)
        sky[c["name"]] = ref.sky_envmap(sky[c["name"] + "_prm"], c["S"], tr, ins)
    np.savez_compressed(os.path.join(HERE, "ref_sky.npz"), meta=json.dumps({"cases": SKY_CASES, "sha256": hashes}),
                        **sky)
    print("wrote ref_sky")


if __name__ == "__main__":
    main()
