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

# LineFor (rows, adjoint), ColLineFor (k_col_fft) and the 8-point-first row
# lines (RowLine<N, 2>): (N, R1, R2, R3, R4)
DECOMPS = sorted({(32, 8, 4, 1, 1), (64, 8, 8, 1, 1), (128, 16, 8, 1, 1), (256, 16, 16, 1, 1),
                  (512, 16, 16, 2, 1), (1024, 16, 16, 4, 1), (2048, 16, 16, 8, 1), (1024, 32, 32, 1, 1),
                  (2048, 32, 8, 8, 1), (512, 8, 8, 8, 1), (1024, 8, 8, 4, 4), (2048, 8, 8, 8, 4)})


def plan(N, R1, R2, R3, R4=1):
    """k_twiddles' plan (plan_entry): segment p (pass 2, 3, 4) with butterfly
    stride NS and radix R holds W_N^(k*r*N/(NS*R)) at r*NS + k, W_N =
    exp(+2 pi i/N)."""
    segs = [(R1, R2)] + ([(R1 * R2, R3)] if R3 > 1 else []) + ([(R1 * R2 * R3, R4)] if R4 > 1 else [])
    out = []
    for ns, r in segs:
        i = np.arange(ns * r)
        e = (i % ns) * (i // ns) * (N // (ns * r))
        out.append(np.exp(2j * np.pi * (e % N) / N))
    return np.concatenate(out)


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


def line_fft(x, N, R1, R2, R3, sign, R4=1):
    G = N // R1
    tw = plan(N, R1, R2, R3, R4)
    t = np.arange(G)[:, None]
    v = x[t + np.arange(R1)[None, :] * G]                         # v[r] = x[t + r*G]
    v = dft(v, sign)
    v = stockham_pass(v, N, R1, G, R1, 1, R2, tw, sign)
    if R3 > 1:
        v = stockham_pass(v, N, R1, G, R2, R1, R3, tw[R1 * R2:], sign)
    if R4 > 1:
        v = stockham_pass(v, N, R1, G, R3, R1 * R2, R4, tw[R1 * R2 + R1 * R2 * R3:], sign)
    RL = R4 if R4 > 1 else (R3 if R3 > 1 else R2)
    e = np.arange(R1)[None, :]
    pos = (t + (e // RL) * G) + (e % RL) * (N // RL)            # LineOut::pos(t, e)
    X = np.empty(N, complex)
    X[pos.ravel()] = v.ravel()
    assert np.array_equal(np.sort(pos.ravel()), np.arange(N))     # every output once
    return X


@pytest.mark.parametrize("N,R1,R2,R3,R4", DECOMPS)
@pytest.mark.parametrize("sign", [+1, -1])
def test_line_fft_matches_numpy(N, R1, R2, R3, R4, sign):
    rng = np.random.default_rng(N + R1)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    got = line_fft(x, N, R1, R2, R3, sign, R4)
    ref = np.fft.ifft(x) * N if sign > 0 else np.fft.fft(x)
    assert np.abs(got - ref).max() < 1e-9 * np.abs(ref).max()


def test_decompositions_are_valid():
    """The static_asserts of LineCfg: radices multiply to N, each <= 32 and
    dividing R1."""
    for N, R1, R2, R3, R4 in DECOMPS:
        assert R1 * R2 * R3 * R4 == N
        assert R1 <= 32 and max(R2, R3, R4) <= R1 and R1 % R2 == 0 and R1 % R3 == 0 and R1 % R4 == 0
        assert R4 == 1 or R3 > 1
