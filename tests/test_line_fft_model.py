"""The line FFT of csrc/fft_line.cuh restated in numpy, index for index, and
checked against numpy's FFT for every decomposition the kernels instantiate.

Covered here:
  - the R1-point in-register first pass on x[t + r*G];
  - each Stockham exchange: the writes to buf[pad(idxD + r*NSP)] and the reads
    of buf[pad(j + r*N/RN)];
  - the twiddle plan as k_twiddles builds it (plan_entry in
    csrc/ocean_kernels.cu);
  - the output positions of LineOut::pos.

The GPU parity tests check whole frames. This test pins the line transform on
its own, for both signs.
"""
import numpy as np
import pytest

# LineFor (rows, adjoint) and ColLineFor (k_col_fft): (N, R1, R2, R3)
DECOMPS = sorted({(32, 8, 4, 1), (64, 8, 8, 1), (128, 16, 8, 1), (256, 16, 16, 1), (512, 16, 16, 2),
                  (1024, 16, 16, 4), (2048, 16, 16, 8), (1024, 32, 32, 1), (2048, 32, 8, 8)})


def plan(N, R1, R2, R3):
    """k_twiddles' plan: entry i < P2 is W_N^((i%R1)*(i/R1)*N/(R1*R2)); entry
    P2 + i is W_N^((i%P2)*(i/P2)), W_N = exp(+2 pi i/N)."""
    P2 = R1 * R2
    P3 = R1 * R2 * R3 if R3 > 1 else 0
    i = np.arange(P2 + P3)
    e = np.where(i < P2, (i % R1) * (i // R1) * (N // (R1 * R2)), ((i - P2) % P2) * ((i - P2) // P2))
    return np.exp(2j * np.pi * (e % N) / N)


def dft(v, sign):
    """In-register R-point DFT along axis 1, natural order in and out."""
    R = v.shape[1]
    n = np.arange(R)
    return v @ np.exp(sign * 2j * np.pi * np.outer(n, n) / R)


def stockham_pass(v, N, R1, G, RP, NSP, RN, T, sign):
    """T: this pass's twiddle plan, entry r*NSN + k (NSN = NSP*RP)."""
    pad = lambda i: i + i // R1
    buf = np.full(N + N // R1, np.nan + 0j)
    t = np.arange(G)
    for b in range(R1 // RP):
        j = t + b * G
        idxD = (j // NSP) * NSP * RP + (j % NSP)
        for r in range(RP):
            buf[pad(idxD + r * NSP)] = v[:, b * RP + r]
    out = np.empty_like(v)
    NSN = NSP * RP
    for b in range(R1 // RN):
        j = t + b * G
        k = j % NSN
        blk = np.stack([buf[pad(j + r * (N // RN))] for r in range(RN)], axis=1)
        for r in range(1, RN):
            w = T[r * NSN + k]
            blk[:, r] *= w if sign > 0 else np.conj(w)
        out[:, b * RN:(b + 1) * RN] = dft(blk, sign)
    assert not np.isnan(out).any()
    return out


def line_fft(x, N, R1, R2, R3, sign):
    G = N // R1
    tw = plan(N, R1, R2, R3)
    t = np.arange(G)[:, None]
    v = x[t + np.arange(R1)[None, :] * G]                         # v[r] = x[t + r*G]
    v = dft(v, sign)
    v = stockham_pass(v, N, R1, G, R1, 1, R2, tw, sign)
    if R3 > 1:
        v = stockham_pass(v, N, R1, G, R2, R1, R3, tw[R1 * R2:], sign)
    RL = R3 if R3 > 1 else R2
    e = np.arange(R1)[None, :]
    pos = (t + (e // RL) * G) + (e % RL) * (N // RL)            # LineOut::pos(t, e)
    X = np.empty(N, complex)
    X[pos.ravel()] = v.ravel()
    assert np.array_equal(np.sort(pos.ravel()), np.arange(N))     # every output once
    return X


@pytest.mark.parametrize("N,R1,R2,R3", DECOMPS)
@pytest.mark.parametrize("sign", [+1, -1])
def test_line_fft_matches_numpy(N, R1, R2, R3, sign):
    rng = np.random.default_rng(N + R1)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    got = line_fft(x, N, R1, R2, R3, sign)
    ref = np.fft.ifft(x) * N if sign > 0 else np.fft.fft(x)
    assert np.abs(got - ref).max() < 1e-9 * np.abs(ref).max()


def test_decompositions_are_valid():
    """The static_asserts of LineCfg: radices multiply to N, each <= 32 and
    dividing R1."""
    for N, R1, R2, R3 in DECOMPS:
        assert R1 * R2 * R3 == N
        assert R1 <= 32 and R2 <= R1 and R3 <= R1 and R1 % R2 == 0 and R1 % R3 == 0
