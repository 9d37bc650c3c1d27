"""ocean_update_noalloc: the frame update for callers that cannot allocate
device memory (plug-in hosts that own the context, code running under a locked
or exhausted allocator, fixed load-time memory budgets).  Its scratch is a
static device array, so it takes the spectrum from the caller; its output must
match ocean_update's on the same spectrum and time, call after call.

This file is collected last so that, if it fails, a run stopping at the first
failure has already run every other test."""
import numpy as np
import pytest

from conftest import rel_l2
import params as P

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the per-field tolerance of the parity tests


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _bufs(torch, N):
    dev = torch.device("cuda")
    return [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]


@pytest.mark.parametrize("N,literal", [(1024, False), (256, True), (32, False)])
def test_noalloc_matches_ocean_update(torch_cuda, ocean_lib, N, literal):
    torch = torch_cuda
    d = P.c2(N)
    lp = P.lib_params(d, literal_conj=literal)
    with ocean_lib.Ocean(lp, seed=d["seed"]) as oc:
        h0 = torch.empty((N, N, 4), device=torch.device("cuda"))
        oc.get_h0(h0)
        for t in (0.75, 12345.6):                         # two calls in a row
            want = _bufs(torch, N)
            got = _bufs(torch, N)
            oc.update(t, *want)
            ocean_lib.update_noalloc(lp, h0, t, *got)
            torch.cuda.synchronize()
            for g, w in zip(got, want):
                assert rel_l2(g.cpu().numpy(), w.cpu().numpy()) < TOL


def test_noalloc_rejects_large_n(torch_cuda, ocean_lib):
    torch = torch_cuda
    N = 2048
    lp = P.lib_params(P.c2(N))
    h0 = torch.zeros((N, N, 4), device=torch.device("cuda"))
    with pytest.raises(ocean_lib.OceanError) as e:
        ocean_lib.update_noalloc(lp, h0, 1.0, *_bufs(torch, N))
    assert e.value.code == ocean_lib.OCEAN_ERR_INVALID and "N <= 1024" in str(e.value)


def test_noalloc_device_status_after_frames(torch_cuda, ocean_lib):
    """ocean_noalloc_device_status reads (and clears) the status word of the
    static path: OK after ordinary frames, and again on a second read."""
    torch = torch_cuda
    N = 256
    d = P.c2(N)
    lp = P.lib_params(d)
    with ocean_lib.Ocean(lp, seed=d["seed"]) as oc:
        h0 = torch.empty((N, N, 4), device=torch.device("cuda"))
        oc.get_h0(h0)
        for t in (0.5, 1.5):
            ocean_lib.update_noalloc(lp, h0, t, *_bufs(torch, N))
        ocean_lib.noalloc_device_status()
        ocean_lib.noalloc_device_status()


def test_noalloc_refuses_table_rebuild_inside_a_capture(torch_cuda, ocean_lib):
    """The first call after a change of N rebuilds the static twiddle table;
    inside a stream capture that would run only at graph launch, so the call
    is refused (nothing is enqueued) and the same call outside the capture
    then succeeds and matches ocean_update."""
    torch = torch_cuda
    dev = torch.device("cuda")
    small, other = P.c2(32), P.c2(64)
    lp32, lp64 = P.lib_params(small), P.lib_params(other)
    h32 = torch.empty((32, 32, 4), device=dev)
    h64 = torch.empty((64, 64, 4), device=dev)
    with ocean_lib.Ocean(lp32, seed=1) as a, ocean_lib.Ocean(lp64, seed=1) as b:
        a.get_h0(h32)
        b.get_h0(h64)
        ocean_lib.update_noalloc(lp32, h32, 1.0, *_bufs(torch, 32))   # the table now holds N = 32
        torch.cuda.synchronize()
        got, want = _bufs(torch, 64), _bufs(torch, 64)
        s = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        x = torch.zeros(1, device=dev)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
                x.add_(1.0)
                with pytest.raises(ocean_lib.OceanError) as e:
                    ocean_lib.update_noalloc(lp64, h64, 2.0, *got, stream=s)
        assert e.value.code == ocean_lib.OCEAN_ERR_INVALID and "capture" in str(e.value)
        ocean_lib.update_noalloc(lp64, h64, 2.0, *got)
        b.update(2.0, *want)
        torch.cuda.synchronize()
        ocean_lib.noalloc_device_status()
        for gg, w in zip(got, want):
            assert rel_l2(gg.cpu().numpy(), w.cpu().numpy()) < TOL
