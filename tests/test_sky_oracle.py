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


def look_at(eye, center, up):
    """glm::lookAt (right-handed) as a (4, 4) array indexed [column][row]."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    M = np.eye(4)
    M[0, 0], M[1, 0], M[2, 0] = s
    M[0, 1], M[1, 1], M[2, 1] = u
    M[0, 2], M[1, 2], M[2, 2] = -f
    M[3, 0], M[3, 1], M[3, 2] = -s @ eye, -u @ eye, f @ eye
    return M


def perspective(fovy, aspect, near, far):
    """glm::perspective (right-handed, depth -1..1), [column][row]."""
    t = np.tan(fovy / 2)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = 1 / (aspect * t), 1 / t
    P[2, 2], P[2, 3], P[3, 2] = -(far + near) / (far - near), -1.0, -2 * far * near / (far - near)
    return P


def np_cube_sample(sky, d):
    """Independent cube-map lookup (OpenGL face selection and orientation,
    bilinear within the face, edges clamped) for directions d (..., 3)."""
    S = sky.shape[1]
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    ax, ay, az = np.abs(x), np.abs(y), np.abs(z)
    xm = (ax >= ay) & (ax >= az)
    ym = ~xm & (ay >= az)
    face = np.where(xm, np.where(x >= 0, 0, 1), np.where(ym, np.where(y >= 0, 2, 3), np.where(z >= 0, 4, 5)))
    ma = np.where(xm, ax, np.where(ym, ay, az))
    sc = np.select([face == 0, face == 1, face == 2, face == 3, face == 4], [-z, z, x, x, x], -x)
    tc = np.select([face == 0, face == 1, face == 2, face == 3, face == 4], [-y, -y, z, -z, -y], -y)
    s = 0.5 * (sc / ma + 1) * S - 0.5
    t = 0.5 * (tc / ma + 1) * S - 0.5
    s0, t0 = np.floor(s), np.floor(t)
    ws, wt = (s - s0)[..., None], (t - t0)[..., None]
    cl = lambda v: np.clip(v, 0, S - 1).astype(int)
    a, b = cl(s0), cl(s0 + 1)
    c, e = cl(t0), cl(t0 + 1)
    top = sky[face, c, a, :3] * (1 - ws) + sky[face, c, b, :3] * ws
    bot = sky[face, e, a, :3] * (1 - ws) + sky[face, e, b, :3] * ws
    return top * (1 - wt) + bot * wt


def np_skybox(sky, eye, center, up, fovy, W, H):
    """Per pixel: the view-space ray (x t a, y t, -1) rotated to world by the
    transpose of the view's rotation (no matrix inverse), the cube map, tone."""
    t = np.tan(fovy / 2)
    xs = (2 * (np.arange(W) + 0.5) / W - 1) * t * (W / H)
    ys = (2 * (np.arange(H) + 0.5) / H - 1) * t
    X, Y = np.meshgrid(xs, ys)
    v = np.stack([X, Y, -np.ones_like(X)], -1)
    Rm = look_at(eye, center, up).T[:3, :3]          # [row][column]
    w = v @ Rm                                       # = (Rm^T v) per pixel
    c = np_cube_sample(sky, w)
    out = np.ones((H, W, 4))
    out[..., :3] = (c / (c + 1)) ** (1 / 2.2)
    return out


SKYBOX_CAMERAS = [((0.0, 10.0, 0.0), (1.0, 9.5, -2.0), (0.0, 1.0, 0.0), 1.0),
                  ((5.0, 2.0, 3.0), (-3.0, 8.0, 1.0), (0.0, 1.0, 0.0), 0.6)]


@pytest.mark.parametrize("cam", range(len(SKYBOX_CAMERAS)))
def test_skybox_oracle_vs_numpy(oracle_mod, cam):
    eye, center, up, fovy = SKYBOX_CAMERAS[cam]
    W, H = 48, 32
    rng = np.random.default_rng(cam)
    sky = rng.random((6, 24, 24, 4)) * 5.0
    V, P = look_at(eye, center, up), perspective(fovy, W / H, 0.1, 1000.0)
    got = oracle_mod.skybox(sky, V, P, W, H)
    assert np.allclose(got, np_skybox(sky, eye, center, up, fovy, W, H), rtol=1e-9, atol=1e-12)
