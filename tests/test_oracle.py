"""CPU tests of the oracle itself: the FP64 restatement against independent
mathematics (naive DFT, single-mode known answers, Parseval, periodicity) and
the FP32 port of the reference algorithm against the FP64 oracle."""
import math

import numpy as np
import pytest

from conftest import rel_l2
import params as P


def _naive_idft2_real(spec):
    """O(N^4) evaluation of d(x,y) = (-1)^(x+y) Re sum X[y'][x'] e^{+2 pi i (x'x + y'y)/N} / N^2."""
    N = spec.shape[0]
    n = np.arange(N)
    out = np.zeros((N, N))
    for y in range(N):
        for x in range(N):
            ph = np.exp(2j * np.pi * (n[:, None] * y + n[None, :] * x) / N)  # [y'][x']
            out[y, x] = ((-1) ** (x + y)) * np.real(np.sum(spec * ph)) / N ** 2
    return out


@pytest.mark.parametrize("N", [8, 16])
def test_ifft2_matches_naive_dft(oracle_mod, N):
    rng = np.random.default_rng(N)
    spec = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    d = oracle_mod.ifft2_real(spec)
    assert rel_l2(d, _naive_idft2_real(spec)) < 1e-13


@pytest.mark.parametrize("N", [8, 32, 128])
def test_ifft2_matches_numpy(oracle_mod, N):
    rng = np.random.default_rng(100 + N)
    spec = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    n = np.arange(N)
    sgn = (-1.0) ** (n[None, :] + n[:, None])
    ref = sgn * np.real(np.fft.ifft2(spec))
    assert rel_l2(oracle_mod.ifft2_real(spec), ref) < 1e-13


def test_single_mode_known_answer(oracle_mod):
    """One mode at centred index (ix, iz) with value a gives
    d(x,y) = Re(a e^{2 pi i (ix x + iz y)/N}) / N^2: the (-1)^(x+y) of
    inversion_cs.glsl turns the stored index x' = ix + N/2 into the centred one."""
    N, ix, iz = 16, 3, -5
    a = 0.7 - 0.2j
    spec = np.zeros((N, N), complex)
    spec[iz + N // 2, ix + N // 2] = a
    d = oracle_mod.ifft2_real(spec)
    y, x = np.mgrid[0:N, 0:N]
    ref = np.real(a * np.exp(2j * np.pi * (ix * x + iz * y) / N)) / N ** 2
    assert np.abs(d - ref).max() < 1e-15


def test_parseval(oracle_mod):
    """For a Hermitian spectrum the output is the full inverse transform and
    sum d^2 = sum |X|^2 / N^2 (unnormalised inverse with 1/N^2)."""
    N = 32
    rng = np.random.default_rng(7)
    X = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    Xh = 0.5 * (X + np.conj(np.roll(np.flip(X, (0, 1)), 1, (0, 1))))
    d = oracle_mod.ifft2_real(Xh)
    assert abs(np.sum(d ** 2) - np.sum(np.abs(Xh) ** 2) / N ** 2) < 1e-12 * np.sum(d ** 2)


def test_h0_statistics_and_dc(oracle_mod):
    d = P.c1()
    p = P.oracle_params(d)
    h = oracle_mod.h0(p, oracle_mod.noise(d["seed"], d["N"]))
    N = d["N"]
    assert np.isfinite(h).all()
    assert np.all(h[N // 2, N // 2] == 0.0)               # DC pinned (Q3)
    # h0k and h0minusk share the amplitude a(k) (tilde_h0_k_cs.glsl:87-88)
    a1 = np.hypot(h[..., 0], h[..., 1])
    a2 = np.hypot(h[..., 2], h[..., 3])
    assert np.corrcoef(a1.ravel(), a2.ravel())[0, 1] > 0.5


def test_clamp_counts(oracle_mod):
    """The +-4000 amplitude clamp is active (16 modes at the N=256 config,
    20 at the N=512 / N=1024 configs)."""
    assert oracle_mod.count_clamped(P.oracle_params(P.c1())) == 16
    assert oracle_mod.count_clamped(P.oracle_params(P.c2(512))) == 20
    assert oracle_mod.count_clamped(P.oracle_params(P.c2(1024))) == 20


def test_noise_generator(oracle_mod):
    n = oracle_mod.noise(0, 64)
    assert n.dtype == np.float32 and n.shape == (4, 64, 64)
    assert n.min() > 0.0 and n.max() <= 1.0
    assert abs(float(n.mean()) - 0.5) < 0.01
    # 24-bit grid
    assert np.all(np.round(n.astype(np.float64) * 2 ** 24) == n.astype(np.float64) * 2 ** 24)


def test_spectrum_time_periodicity(oracle_mod):
    """A single-|k| spectrum repeats with period 2 pi / w."""
    d = P.c2(32)
    p = P.oracle_params(d)
    N = 32
    h = np.zeros((N, N, 4))
    ix, iz = 3, 4                                        # |k| = 5 * 2 pi / L
    h[iz + N // 2, ix + N // 2] = [0.3, -0.1, 0.2, 0.05]
    w = math.sqrt(p.gravity * 5 * 2 * math.pi / p.L)
    s0 = oracle_mod.spectrum(p, h, 0.37)
    s1 = oracle_mod.spectrum(p, h, 0.37 + 2 * math.pi / w)
    assert np.abs(s0 - s1).max() < 1e-12


def test_hermitian_h0_gives_real_transform(oracle_mod):
    """With textbook h0(-k) (h0minusk(k) = h0k(-k)) and conj(), h(k,t) is
    Hermitian and the discarded imaginary part of the IFFT is ~0."""
    N = 32
    d = P.c2(N)
    p = P.oracle_params(d)
    h = oracle_mod.h0(p, oracle_mod.noise(5, N))
    hk = h[..., 0] + 1j * h[..., 1]
    neg = np.roll(np.flip(hk, (0, 1)), 1, (0, 1))        # hk at -k (periodic)
    h2 = h.copy()
    h2[..., 2] = neg.real
    h2[..., 3] = neg.imag
    spec = oracle_mod.spectrum(p, h2, 2.5)[1]
    full = np.fft.ifft2(spec)
    assert np.abs(full.imag).max() < 1e-12 * np.abs(full.real).max()


@pytest.mark.parametrize("literal", [False, True])
def test_translation_and_superposition(oracle_mod, literal):
    """A phase ramp on h0 shifts every output map by whole texels. With
    phi = 2 pi (ix sx + iz sz) / N, h0k takes e^{-i phi}. h0minusk takes e^{+i phi},
    because it enters conjugated; with the literal conjugate it takes e^{-i phi}.
    dx, dy, dz are also linear in h0.  The GPU tests check both properties at
    full size."""
    N, sx, sz, t = 32, 5, -3, 7.25
    p = P.oracle_params(P.c2(N), literal_conj=literal)
    h = oracle_mod.h0(p, oracle_mod.noise(1, N))
    ix = np.arange(N) - N // 2
    w = np.exp(1j * 2 * np.pi * (ix[None, :] * sx + ix[:, None] * sz) / N)
    hk = (h[..., 0] + 1j * h[..., 1]) * np.conj(w)
    hm = (h[..., 2] + 1j * h[..., 3]) * (np.conj(w) if literal else w)
    hs = np.stack([hk.real, hk.imag, hm.real, hm.imag], -1)
    a, b = oracle_mod.update(p, h, t), oracle_mod.update(p, hs, t)
    for k in ("dx", "dy", "dz", "nj"):
        assert rel_l2(b[k], np.roll(a[k], (sz, sx), axis=(0, 1))) < 1e-13
    c = oracle_mod.update(p, h + hs, t)
    for k in ("dx", "dy", "dz"):
        assert rel_l2(c[k], a[k] + b[k]) < 1e-13


def test_outputs_stencils(oracle_mod):
    """finish(): lambda scaling, Sobel normal and Jacobian against direct numpy."""
    N = 16
    p = P.oracle_params(P.c2(N))
    rng = np.random.default_rng(3)
    raw = rng.standard_normal((3, N, N))
    o = oracle_mod.finish(p, raw)
    lam = p.choppiness
    dy = raw[1]
    sh = lambda a, dx, dy_: np.roll(np.roll(a, -dy_, 0), -dx, 1)   # a[y+dy_][x+dx]
    z = {(-1, -1): 0, (0, -1): 1, (1, -1): 2, (-1, 0): 3, (1, 0): 4, (-1, 1): 5, (0, 1): 6, (1, 1): 7}
    zz = {v: sh(dy, k[0], k[1]) for k, v in z.items()}
    nz = zz[0] + 2 * zz[1] + zz[2] - zz[5] - 2 * zz[6] - zz[7]
    nx = zz[0] + 2 * zz[3] + zz[5] - zz[2] - 2 * zz[4] - zz[7]
    n = np.stack([nx, np.ones_like(nx), nz], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    assert np.abs(o["nj"][..., :3] - n).max() < 1e-14
    Dx, Dz = lam * raw[0], lam * raw[2]
    h = 2 * p.L / N
    dxx = (sh(Dx, 1, 0) - sh(Dx, -1, 0)) / h
    dxz = (sh(Dx, 0, 1) - sh(Dx, 0, -1)) / h
    dzx = (sh(Dz, 1, 0) - sh(Dz, -1, 0)) / h
    dzz = (sh(Dz, 0, 1) - sh(Dz, 0, -1)) / h
    J = (1 - dxx) * (1 - dzz) - dxz * dzx
    assert np.abs(o["nj"][..., 3] - J).max() < 1e-13
    assert np.abs(o["dx"] - Dx).max() == 0 and np.abs(o["dy"] - dy).max() == 0


@pytest.mark.parametrize("literal", [False, True])
def test_port_matches_oracle_c1(oracle_mod, literal):
    """The FP32 port of the reference's table-driven radix-2 algorithm agrees
    with the FP64 oracle on the N=256 configuration at t = 1 s."""
    d = P.c1()
    p = P.oracle_params(d, literal_conj=literal)
    nz = oracle_mod.noise(d["seed"], d["N"])
    h = oracle_mod.h0(p, nz)
    ref = oracle_mod.update(p, h, 1.0)
    port = oracle_mod.Port(p, nz)
    assert rel_l2(port.h0(), h) < 1e-6
    o = port.frame(1.0)
    for k in ("dx", "dy", "dz"):
        assert rel_l2(o[k], ref[k]) < 1e-5, k
    assert rel_l2(o["nj"][..., :3], ref["nj"][..., :3]) < 1e-5
    assert rel_l2(o["nj"][..., 3], ref["nj"][..., 3]) < 1e-5
    port.close()


def test_fp32_phase_fails_at_large_t(oracle_mod):
    """The reference's FP32 w*t (main.cpp:599, tilde_h0_t_cs.glsl:96-97) drifts
    at t = 1e5 s: the FP32 port is far from the FP64 oracle there, which is why
    the library reduces the phase in double-float."""
    d = P.c2(256)
    p = P.oracle_params(d)
    nz = oracle_mod.noise(d["seed"], 256)
    h = oracle_mod.h0(p, nz)
    ref = oracle_mod.update(p, h, 1e5)
    port = oracle_mod.Port(p, nz)
    assert rel_l2(port.frame(1e5)["dy"], ref["dy"]) > 1e-3
    port.close()


def test_literal_conj_differs(oracle_mod):
    d = P.c1()
    nz = oracle_mod.noise(0, 256)
    pa, pb = P.oracle_params(d), P.oracle_params(d, literal_conj=True)
    h = oracle_mod.h0(pa, nz)
    a = oracle_mod.update(pa, h, 1.0)["dy"]
    b = oracle_mod.update(pb, h, 1.0)["dy"]
    assert rel_l2(a, b) > 0.1


def test_tables(oracle_mod):
    """Bit reversal and the butterfly table (twiddle_factors_cs.glsl:34-69):
    driving the table with the reference's radix-2 ping-pong is an
    unnormalised inverse DFT."""
    for N in (8, 64, 256):
        br = oracle_mod.bit_reversed(N)
        lg = N.bit_length() - 1
        assert all(int(format(i, f"0{lg}b")[::-1], 2) == br[i] for i in range(N))
    N = 32
    T = oracle_mod.twiddle_table(N)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    a = x.copy()
    for s in range(N.bit_length() - 1):
        b = np.empty_like(a)
        for i in range(N):
            w = T[s, i, 0] + 1j * T[s, i, 1]
            b[i] = a[int(T[s, i, 2])] + w * a[int(T[s, i, 3])]
        a = b
    assert np.abs(a - np.fft.ifft(x) * N).max() < 1e-12


@pytest.mark.parametrize("literal", [False, True])
def test_oracle_adjoint_matches_finite_differences(oracle_mod, literal):
    """FP64 adjoint (orc_backward) against central finite differences of the
    FP64 forward, for L = sum_t sum_f <g_f(t), D_f(t)> with fixed random g."""
    N = 16
    base = dict(N=N, L=800.0, amplitude=3.0, wind_speed=22.0, wind_x=math.cos(0.9), wind_y=math.sin(0.9),
                choppiness=1.1, suppression=0.1, literal_conj=literal)
    nz = oracle_mod.noise(3, N)
    times = [0.3, 1.7, 4.0]
    rng = np.random.default_rng(0)
    g = [rng.standard_normal((3, N, N)) for _ in range(3)]

    def loss(prm, h=None):
        p = oracle_mod.Params(**prm)
        hh = oracle_mod.h0(p, nz) if h is None else h
        s = 0.0
        for j, t in enumerate(times):
            o = oracle_mod.update(p, hh, t)
            s += np.sum(g[0][j] * o["dx"]) + np.sum(g[1][j] * o["dy"]) + np.sum(g[2][j] * o["dz"])
        return s

    p = oracle_mod.Params(**base)
    h = oracle_mod.h0(p, nz)
    dh0, gr = oracle_mod.backward(p, h, times, *g)
    for name, key in (("dA", "amplitude"), ("dV", "wind_speed"), ("dlambda", "choppiness")):
        e = 1e-5 * base[key]
        a, b = dict(base), dict(base)
        a[key] += e
        b[key] -= e
        fd = (loss(a) - loss(b)) / (2 * e)
        assert abs(fd - gr[name]) <= 1e-6 * abs(fd), (name, fd, gr[name])
    e = 1e-6
    a, b = dict(base), dict(base)
    a["wind_x"], a["wind_y"] = math.cos(0.9 + e), math.sin(0.9 + e)
    b["wind_x"], b["wind_y"] = math.cos(0.9 - e), math.sin(0.9 - e)
    fd = (loss(a) - loss(b)) / (2 * e)
    assert abs(fd - gr["dtheta"]) <= 1e-6 * abs(fd)
    for (yy, xx, c) in [(5, 7, 0), (12, 3, 1), (1, 14, 2), (8, 8, 3), (0, 0, 2)]:
        e = 1e-4
        ha, hb = h.copy(), h.copy()
        ha[yy, xx, c] += e
        hb[yy, xx, c] -= e
        fd = (loss(base, ha) - loss(base, hb)) / (2 * e)
        assert abs(fd - dh0[yy, xx, c]) <= 1e-6 * max(1.0, abs(fd)), (yy, xx, c, fd, dh0[yy, xx, c])
