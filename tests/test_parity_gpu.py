"""GPU parity: the CUDA path through the C ABI against the FP64 oracle on the
same seeded noise.  Tolerance: relative L2 <= 1e-5 per output field (Dx, Dy,
Dz, normal xyz, Jacobian) and <= 1e-6 for h0."""
import math

import numpy as np
import pytest

from conftest import rel_l2
import params as P

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _run(torch, ocean_lib, d, times, literal=False):
    """Create the tile through the C ABI, run frames, return host copies."""
    N = d["N"]
    lp = P.lib_params(d, literal_conj=literal)
    dev = torch.device("cuda")
    outs = []
    with ocean_lib.Ocean(lp, seed=d["seed"]) as oc:
        h0 = torch.empty((N, N, 4), dtype=torch.float32, device=dev)
        oc.get_h0(h0)
        dx, dy, dz = (torch.empty((N, N), dtype=torch.float32, device=dev) for _ in range(3))
        nj = torch.empty((N, N, 4), dtype=torch.float32, device=dev)
        for t in times:
            oc.update(t, dx, dy, dz, nj)
            torch.cuda.synchronize()
            outs.append({"dx": dx.cpu().numpy().copy(), "dy": dy.cpu().numpy().copy(),
                         "dz": dz.cpu().numpy().copy(), "nj": nj.cpu().numpy().copy()})
        h0h = h0.cpu().numpy()
    return h0h, outs


def _check(o, ref, tol=TOL):
    errs = {k: rel_l2(o[k], ref[k]) for k in ("dx", "dy", "dz")}
    errs["normal"] = rel_l2(o["nj"][..., :3], ref["nj"][..., :3])
    errs["J"] = rel_l2(o["nj"][..., 3], ref["nj"][..., 3])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, errs
    # J is O(1): bound its absolute error by a few FP32 ulps of its magnitude too
    jref = ref["nj"][..., 3]
    dj = np.abs(o["nj"][..., 3].astype(np.float64) - jref).max()
    assert dj < 5e-7 * max(1.0, float(np.abs(jref).max())), dj
    return errs


@pytest.mark.parametrize("N", [32, 64, 128, 256, 512, 1024, 2048])
def test_parity_sizes(torch_cuda, ocean_lib, oracle_mod, N):
    d = P.c2(N)
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], N))
    times = [0.0, 1.0 / 60.0, 7.25]
    h0g, outs = _run(torch_cuda, ocean_lib, d, times)
    assert rel_l2(h0g, h0ref) < 1e-6
    for t, o in zip(times, outs):
        _check(o, oracle_mod.update(p, h0ref, t))


def test_parity_c1(torch_cuda, ocean_lib, oracle_mod):
    """The N=256 configuration at t = 1 s."""
    d = P.c1()
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], d["N"]))
    h0g, outs = _run(torch_cuda, ocean_lib, d, [1.0])
    assert rel_l2(h0g, h0ref) < 1e-6
    _check(outs[0], oracle_mod.update(p, h0ref, 1.0))


def test_parity_literal_conj(torch_cuda, ocean_lib, oracle_mod):
    """OCEAN_FLAG_LITERAL_CONJ reproduces the shader's no-op conjugate()."""
    d = P.c1()
    p = P.oracle_params(d, literal_conj=True)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], d["N"]))
    _, outs = _run(torch_cuda, ocean_lib, d, [1.0, 33.3], literal=True)
    _check(outs[0], oracle_mod.update(p, h0ref, 1.0))
    _check(outs[1], oracle_mod.update(p, h0ref, 33.3))


@pytest.mark.parametrize("N", [512, 1024])
def test_phase_precision_large_t(torch_cuda, ocean_lib, oracle_mod, N):
    """t = 1e5 s: FP32 w*t would be off by ~0.03 rad; the double-float phase
    keeps the FP64-oracle tolerance."""
    d = P.c2(N)
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], N))
    _, outs = _run(torch_cuda, ocean_lib, d, [1e5, 1e5 + 1.0 / 60.0])
    _check(outs[0], oracle_mod.update(p, h0ref, 1e5))
    _check(outs[1], oracle_mod.update(p, h0ref, 1e5 + 1.0 / 60.0))


def test_reference_defaults(torch_cuda, ocean_lib, oracle_mod):
    """The reference demo's own parameters (V=80, A=2, L=1000, N=256)."""
    d = P.reference_default(256)
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], 256))
    _, outs = _run(torch_cuda, ocean_lib, d, [12.5])
    _check(outs[0], oracle_mod.update(p, h0ref, 12.5))


@pytest.mark.parametrize("name", ["ref_frame_N32", "ref_frame_N64"])
def test_matches_reference_shader_golden(torch_cuda, ocean_lib, name):
    """The CUDA path in literal-conjugate mode with lambda = 1 against frames the
    reference's own compute shaders produced (tests/golden/make_golden.py)."""
    import json
    import os
    from conftest import ROOT
    z = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    meta = json.loads(str(z["meta"]))
    d = dict(N=meta["N"], L=float(meta["L"]), amplitude=meta["A"], wind_speed=meta["V"], wind_x=meta["wx"],
             wind_y=meta["wy"], choppiness=1.0, suppression=meta["l"], seed=meta["seed"])
    h0g, outs = _run(torch_cuda, ocean_lib, d, [float(t) for t in z["times"]], literal=True)
    N = d["N"]
    g = np.concatenate([z["h0k"], z["h0minusk"]], -1).astype(np.float64)
    g[N // 2, N // 2] = 0.0
    assert rel_l2(h0g, g) < 2e-6
    for i, o in enumerate(outs):
        for k in ("dx", "dy", "dz"):
            assert rel_l2(o[k], z[f"{k}_{i}"]) < 1e-5, k
        assert rel_l2(o["nj"][..., :3], z[f"normal_{i}"][..., :3]) < 1e-5


@pytest.mark.parametrize("N", [512, 1024])
def test_repeated_row_pass_is_stream_ordered(torch_cuda, ocean_lib, N):
    """Two row passes on one handle with no column stage between them (the
    second would overwrite the intermediate while the first still writes it
    if it overlapped): the column stage then sees the second time's frame, bit
    for bit, also right after a back-to-back frame."""
    torch = torch_cuda
    d = P.c2(N)
    dev = torch.device("cuda")
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        outs = lambda: [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
        ref = outs()
        oc.update(9.25, *ref)
        torch.cuda.synchronize()
        got = outs()
        scratch = outs()
        oc.update(0.5, *scratch)                 # a frame in flight before the two row passes
        oc.update_rows(3.0)
        oc.update_rows(9.25)
        oc.update_columns_outputs(*got)
        torch.cuda.synchronize()
        oc.device_status()
        for a, b in zip(got, ref):
            assert torch.equal(a, b)


@pytest.mark.parametrize("N", [64, 512, 1024, 2048])
def test_back_to_back_frames_bitwise(torch_cuda, ocean_lib, N):
    """Frames launched back to back with no host synchronisation (the stages
    of a frame are chained by programmatic dependent launch, the next frame
    overwrites the same scratch) give bit-identical outputs to frames run one
    at a time: alternating times, every frame into its own output set, some
    frames through the staged entry points."""
    torch = torch_cuda
    d = P.c2(N)
    dev = torch.device("cuda")
    times = (0.25, 7.5)
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        # one at a time, through ocean_update and through the staged entry
        # points (those run the column side as two kernels; ocean_update may
        # fuse them, whose normal map rounds differently at the CTA edges)
        ref, ref_staged = [], []
        for t in times:
            o = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
            oc.update(t, *o)
            torch.cuda.synchronize()
            ref.append(o)
            o = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
            oc.update_rows(t)
            oc.update_columns()
            oc.update_outputs(*o)
            torch.cuda.synchronize()
            ref_staged.append(o)
        F = 12
        sets = [[torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
                for _ in range(F)]
        for k in range(F):
            if k % 3 == 2:                       # the staged API, also back to back
                oc.update_rows(times[k % 2])
                oc.update_columns()
                oc.update_outputs(*sets[k])
            else:
                oc.update(times[k % 2], *sets[k])
        torch.cuda.synchronize()
        oc.device_status()
        for k in range(F):
            for a, b in zip(sets[k], (ref_staged if k % 3 == 2 else ref)[k % 2]):
                assert torch.equal(a, b), (N, k)


@pytest.mark.parametrize("N", [64, 1024])
def test_calm_sea_is_exact(torch_cuda, ocean_lib, N):
    """Amplitude 0: h0 = 0, so every displacement is exactly 0, every normal
    exactly (0, 1, 0) and the Jacobian exactly 1, at any time."""
    d = dict(P.c2(N), amplitude=0.0)
    _, outs = _run(torch_cuda, ocean_lib, d, [0.0, 123.456])
    for o in outs:
        for k in ("dx", "dy", "dz"):
            assert not np.any(o[k]), k
        nj = o["nj"]
        assert np.all(nj[..., 0] == 0.0) and np.all(nj[..., 1] == 1.0) and np.all(nj[..., 2] == 0.0)
        assert np.all(nj[..., 3] == 1.0)


@pytest.mark.parametrize("N", [64, 1024])
def test_no_choppiness(torch_cuda, ocean_lib, oracle_mod, N):
    """lambda = 0: the horizontal displacements are exactly 0 and the Jacobian
    exactly 1; the height field still matches the oracle."""
    d = dict(P.c2(N), choppiness=0.0)
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], N))
    _, outs = _run(torch_cuda, ocean_lib, d, [2.5])
    o = outs[0]
    assert not np.any(o["dx"]) and not np.any(o["dz"])
    assert np.all(o["nj"][..., 3] == 1.0)
    ref = oracle_mod.update(p, h0ref, 2.5)
    assert rel_l2(o["dy"], ref["dy"]) <= TOL
    assert rel_l2(o["nj"][..., :3], ref["nj"][..., :3]) <= TOL


@pytest.mark.parametrize("N", [32, 1024])
def test_negative_time(torch_cuda, ocean_lib, oracle_mod, N):
    """Negative t runs the spectrum backwards, as the formula does."""
    d = P.c2(N)
    p = P.oracle_params(d)
    h0ref = oracle_mod.h0(p, oracle_mod.noise(d["seed"], N))
    _, outs = _run(torch_cuda, ocean_lib, d, [-3.75])
    _check(outs[0], oracle_mod.update(p, h0ref, -3.75))


def test_update_argument_errors(torch_cuda, ocean_lib):
    """Non-finite times and misaligned output pointers are refused before any
    launch; the handle keeps working afterwards."""
    torch = torch_cuda
    N = 64
    d = P.c2(N)
    dev = torch.device("cuda")
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        dx, dy, dz = (torch.zeros((N, N), device=dev) for _ in range(3))
        nj = torch.zeros((N, N, 4), device=dev)
        for t in (float("nan"), float("inf"), -float("inf")):
            with pytest.raises(ocean_lib.OceanError):
                oc.update(t, dx, dy, dz, nj)
        flat = torch.zeros(N * N + 1, device=dev)
        with pytest.raises(ocean_lib.OceanError):
            oc.update(1.0, flat[1:].view(N, N), dy, dz, nj)      # 4-byte offset: not 16-byte aligned
        torch.cuda.synchronize()
        assert not torch.any(dx) and not torch.any(nj)
        oc.update(1.0, dx, dy, dz, nj)
        torch.cuda.synchronize()
        oc.device_status()
        assert torch.any(dy)


def test_outputs_in_pinned_host_memory(torch_cuda, ocean_lib):
    """Output pointers may be pinned host memory (unified addressing): the
    output kernel then writes across the host link, with the same values as
    into device buffers."""
    torch = torch_cuda
    N = 256
    d = P.c2(N)
    dev = torch.device("cuda")
    with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
        dv = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
        hv = [torch.empty((N, N), pin_memory=True) for _ in range(3)] + [torch.empty((N, N, 4), pin_memory=True)]
        oc.update(3.5, *dv)
        oc.update(3.5, *hv)
        torch.cuda.synchronize()
        oc.device_status()
        for a, b in zip(dv, hv):
            assert torch.equal(a.cpu(), b)


@pytest.mark.parametrize("N", [1024, 2048])
def test_amplitude_scaling_is_exact(torch_cuda, ocean_lib, N):
    """Size-independent property at full size.  h0 is proportional to
    sqrt(A). Away from the +-4000 clamp, 4A therefore doubles h0 exactly, and
    every later step is linear with scalings by 2 that commute with FP32
    rounding, so dx, dy and dz double bit for bit."""
    torch = torch_cuda
    dev = torch.device("cuda")
    outs = []
    for A in (0.02, 0.08):
        d = dict(P.c2(N), amplitude=A)
        with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
            o = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
            oc.update(123.25, *o)
            torch.cuda.synchronize()
            oc.device_status()
            outs.append(o)
    for a, b in zip(outs[0][:3], outs[1][:3]):
        assert torch.any(a != 0)
        assert torch.equal(2.0 * a, b)


def _frame(torch, oc, N, t):
    dev = torch.device("cuda")
    o = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
    oc.update(t, *o)
    torch.cuda.synchronize()
    oc.device_status()
    return o


def _rel(torch, a, b):
    a, b = a.double(), b.double()
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def _maps(o):
    """dx, dy, dz, the normal (xyz) and the Jacobian of one frame."""
    return [o[0], o[1], o[2], o[3][..., :3], o[3][..., 3]]


@pytest.mark.parametrize("N,literal", [(2048, False), (1024, True)])
def test_translation_full_size(torch_cuda, ocean_lib, N, literal):
    """Size-independent property at full size.  With phi = 2 pi (ix sx + iz sz) / N,
    multiply h0k by e^{-i phi} and h0minusk by e^{+i phi}; with the literal conjugate,
    h0minusk also takes e^{-i phi}, because it enters unconjugated.  This shifts every
    output map by (sx, sz) texels: dx, dy, dz, the Sobel normal and the Jacobian."""
    torch = torch_cuda
    d = P.c2(N)
    sx, sz, t = 5, -3, 77.5
    with ocean_lib.Ocean(P.lib_params(d, literal_conj=literal), seed=d["seed"]) as oc:
        h0 = torch.empty((N, N, 4), device="cuda")
        oc.get_h0(h0)
        a = _frame(torch, oc, N, t)
        ix = torch.arange(N, dtype=torch.float64, device="cuda") - N // 2
        phi = 2.0 * math.pi * (ix[None, :] * sx + ix[:, None] * sz) / N
        w = torch.polar(torch.ones_like(phi), phi)
        hk = torch.complex(h0[..., 0].double(), h0[..., 1].double()) * w.conj()
        hm = torch.complex(h0[..., 2].double(), h0[..., 3].double()) * (w.conj() if literal else w)
        oc.set_h0(torch.stack([hk.real, hk.imag, hm.real, hm.imag], -1).float().contiguous())
        b = _frame(torch, oc, N, t)
    for x, y in zip(_maps(a), _maps(b)):
        assert _rel(torch, y, torch.roll(x, (sz, sx), dims=(0, 1))) < 2 * TOL


def test_superposition_full_size(torch_cuda, ocean_lib):
    """Size-independent property at full size: dx, dy, dz are linear in h0, so
    the frame of h0a + h0b is the sum of the frames of h0a and h0b."""
    torch = torch_cuda
    N, t = 2048, 31.0
    frames, h0s = [], []
    for seed in (1, 2):
        d = dict(P.c2(N), seed=seed)
        with ocean_lib.Ocean(P.lib_params(d), seed=seed) as oc:
            h0 = torch.empty((N, N, 4), device="cuda")
            oc.get_h0(h0)
            h0s.append(h0)
            frames.append(_frame(torch, oc, N, t))
    with ocean_lib.Ocean(P.lib_params(P.c2(N)), seed=1) as oc:
        oc.set_h0((h0s[0] + h0s[1]).contiguous())
        s = _frame(torch, oc, N, t)
    for k in range(3):
        assert _rel(torch, s[k], frames[0][k] + frames[1][k]) < 2 * TOL


@pytest.mark.parametrize("N", [512, 1024])
def test_fused_column_kernel_matches_two_kernels(torch_cuda, ocean_lib, N):
    """The fused column kernel (the tuning's col_fused: 2 or 4 column pairs
    per CTA) against the column FFT + output kernels on the same frames,
    launched back to back on one handle: dx, dy, dz bit for bit (same
    arithmetic), normal_j within 1e-6 relative L2 (its halo columns come from
    a differently paired transform, which rounds differently)."""
    torch = torch_cuda
    d = P.c2(N)
    dev = torch.device("cuda")
    times = [0.5 + 3.25 * k for k in range(6)]
    outs = {}
    saved = ocean_lib.get_tuning(N)
    try:
        for fused in (0, 2, 4):
            ocean_lib.set_tuning(N, col_fused=fused)
            assert ocean_lib.get_tuning(N)["col_fused"] == fused
            with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
                sets = [[torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
                        for _ in times]
                for t, o in zip(times, sets):
                    oc.update(t, *o)
                torch.cuda.synchronize()
                oc.device_status()
                outs[fused] = [[x.cpu().numpy() for x in o] for o in sets]
    finally:
        ocean_lib.set_tuning(N, **saved)
    for fused in (2, 4):
        for a, b in zip(outs[0], outs[fused]):
            for k in range(3):
                assert np.array_equal(a[k], b[k]), fused
            assert rel_l2(b[3], a[3]) < 1e-6, fused


@pytest.mark.parametrize("N", [512, 1024, 2048])
def test_row_pass_variants_agree(torch_cuda, ocean_lib, oracle_mod, N):
    """The row-pass kernels the tuning chooses between at N >= 512 (the
    warp-specialised k_row_ws with 16- or 8-point-first lines or, at N = 1024,
    32 x 32 lines, and k_row_pass with every warp on the prepass and then its
    line, with the default or 32 x 32 lines) give the same frames, back to back
    on one handle, and match the FP64 oracle."""
    torch = torch_cuda
    d = P.c2(N)
    dev = torch.device("cuda")
    times = [0.25, 9.5, 1.0e5]
    outs = {}
    variants = (0, 1, 2, 3, 4, 5) if N == 1024 else (0, 1, 2)
    saved = ocean_lib.get_tuning(N)
    try:
        for variant in variants:
            ocean_lib.set_tuning(N, row_variant=variant)
            assert ocean_lib.get_tuning(N)["row_variant"] == variant
            with ocean_lib.Ocean(P.lib_params(d), seed=d["seed"]) as oc:
                sets = [[torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
                        for _ in times]
                for t, o in zip(times, sets):
                    oc.update(t, *o)
                torch.cuda.synchronize()
                oc.device_status()
                outs[variant] = [[x.cpu().numpy() for x in o] for o in sets]
    finally:
        ocean_lib.set_tuning(N, **saved)
    for variant in variants[1:]:
        for a, b in zip(outs[0], outs[variant]):
            for k in range(4):
                assert rel_l2(b[k], a[k]) < 1e-6, (variant, k)
    op = P.oracle_params(d)
    ref = oracle_mod.update(op, oracle_mod.h0(op, oracle_mod.noise(d["seed"], N)), times[1])
    for variant in variants[1:]:
        _check({"dx": outs[variant][1][0], "dy": outs[variant][1][1], "dz": outs[variant][1][2],
                "nj": outs[variant][1][3]}, ref)
