"""The sky environment cube map's oracle (orc_sky_envmap: FP32 in the
shader's operation order) against the reference's own sky_envmap_fs.glsl +
atmosphere.glsl run on the CPU: the committed golden maps (seeded synthetic
tables, since the reference's inscatter.raw is missing) and, where the
reference sources are present, the live harness on its real transmittance
table.  Plus analytic cases and the .raw table loader."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402  (sky_tables, sky_prm, SKY_CASES)


def _oracle_map(oracle_mod, prm, S, tr, ins):
    return oracle_mod.sky_envmap(prm[0:3], prm[3:6], tr, ins, S, earth_pos=prm[6:9], beta_r=prm[9:12],
                                 mie_g=float(prm[12]), sun_intensity=float(prm[13]))


def _assert_close(got, want, max_flips=2):
    """Equal up to libm ulps (atanf, powf, tanf may differ between C
    libraries); a texel on the sun disk's rim may flip."""
    err = np.abs(got.astype(np.float64) - want.astype(np.float64))
    bad = err > 1e-5 * (1.0 + np.abs(want))
    assert bad.sum() <= 4 * max_flips, (bad.sum(), err.max())
    ok = ~bad.any(axis=-1)
    d = got[ok].astype(np.float64) - want[ok]
    assert np.sqrt((d * d).sum() / max((want[ok].astype(np.float64) ** 2).sum(), 1e-30)) < 1e-6


@pytest.mark.parametrize("case", [c["name"] for c in make_golden.SKY_CASES])
def test_oracle_matches_reference_sky_golden(oracle_mod, case):
    g = np.load(os.path.join(HERE, "golden", "ref_sky.npz"))
    meta = json.loads(str(g["meta"]))
    c = next(x for x in meta["cases"] if x["name"] == case)
    tr, ins = make_golden.sky_tables(c["seed"])
    prm = g[case + "_prm"]
    want = g[case]
    assert want.shape == (6, c["S"], c["S"], 4) and np.isfinite(want).all()
    _assert_close(_oracle_map(oracle_mod, prm, c["S"], tr, ins), want)


def test_oracle_bit_exact_with_reference_shader_on_real_transmittance(oracle_mod):
    from oracle import build_ref, ref
    if not build_ref.available():
        pytest.skip("reference sources not present")
    import ocean_gb300 as og
    tabs = og.load_sky_tables(os.path.join(build_ref.REF, "data", "texture"))
    _, ins = make_golden.sky_tables(9)
    for angle, cam, S in ((-0.3, (0.0, 5.0, 0.0), 48), (-0.05, (100.0, 3000.0, 20.0), 40)):
        prm = make_golden.sky_prm(dict(camera=cam, angle=angle))
        got = _oracle_map(oracle_mod, prm, S, tabs["transmittance"], ins)
        want = ref.sky_envmap(prm, S, tabs["transmittance"], ins)
        assert np.array_equal(got, want)


def test_sky_table_loader():
    from oracle import build_ref
    d = os.path.join(build_ref.REF, "data", "texture")
    if not os.path.isdir(d):
        pytest.skip("reference data not present")
    import ocean_gb300 as og
    t = og.load_sky_tables(d)
    assert t["transmittance"].shape == (64, 256, 4) and t["irradiance"].shape == (16, 64, 4)
    assert t["inscatter"] is None                     # missing from the reference
    assert np.isfinite(t["transmittance"]).all() and t["transmittance"].min() >= 0.0
    assert t["transmittance"][..., :3].max() <= 1.0 + 1e-6


def test_sun_disk_only(oracle_mod):
    """Transmittance 1, no inscatter: exactly the texels within half a degree
    of the sun (sky_envmap_fs.glsl:29) carry the sun intensity."""
    S = 256
    tr = np.ones((64, 256, 4), np.float32)
    ins = np.zeros((32, 128, 256, 4), np.float32)
    sun = np.array(oracle_mod.sky_sun_direction(-0.4), np.float32)
    m = oracle_mod.sky_envmap((0.0, 10.0, 0.0), sun, tr, ins, S)
    lit = m[..., 0] > 0
    assert set(np.unique(m[..., :3])) <= {0.0, 100.0} and np.all(m[..., 3] == 1.0)
    # the texel directions, for an independent count
    i = (np.arange(S) + 0.5) / S * 2 - 1
    sc, tc = np.meshgrid(i, i)
    one = np.ones_like(sc)
    faces = [(one, -tc, -sc), (-one, -tc, sc), (sc, one, tc), (sc, -one, -tc), (sc, -tc, one), (-sc, -tc, -one)]
    d = np.stack([np.stack(f, -1) for f in faces])
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    expect = d @ sun.astype(np.float64) >= np.cos(np.float32(3.141592) / 360.0)
    assert abs(int(lit.sum()) - int(expect.sum())) <= 2 and lit.sum() > 0


def test_constant_inscatter_is_phase_functions(oracle_mod):
    """Constant inscatter c and transmittance T: away from the sun every texel
    is I * (c * phaseR(nu) + c * (betaR.r / betaR) * phaseM(nu))."""
    S, c, I = 32, 0.02, 100.0
    tr = np.full((64, 256, 4), 0.5, np.float32)
    ins = np.full((32, 128, 256, 4), c, np.float32)
    sun = np.array(oracle_mod.sky_sun_direction(-0.6), np.float64)
    m = oracle_mod.sky_envmap((0.0, 10.0, 0.0), sun, tr, ins, S).astype(np.float64)
    i = (np.arange(S) + 0.5) / S * 2 - 1
    sc, tc = np.meshgrid(i, i)
    one = np.ones_like(sc)
    d = np.stack([np.stack(f, -1) for f in [(one, -tc, -sc), (-one, -tc, sc), (sc, one, tc), (sc, -one, -tc),
                                            (sc, -tc, one), (-sc, -tc, -one)]])
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    nu = d @ sun
    g = 0.75
    pr = 3.0 / (16.0 * 3.141592) * (1 + nu * nu)
    pm = 1.5 / (4 * 3.141592) * (1 - g * g) * (1 + g * g - 2 * g * nu) ** -1.5 * (1 + nu * nu) / (2 + g * g)
    br = np.array([0.0058, 0.0135, 0.0331])
    want = I * (c * pr[..., None] + c * (br[0] / br)[None, None, None, :] * pm[..., None])
    away = nu < 0.99
    assert np.allclose(m[..., :3][away], want[away], rtol=2e-5, atol=0)
