"""Failure paths without a GPU fault: every device allocation of ocean_create
and ocean_batch_create is made to fail in turn (ocean_debug_fail_allocations);
each call must report OCEAN_ERR_NOMEM, release what it had allocated, and
leave the library usable."""
import pytest

import params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _free(torch):
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_create_fails_cleanly_at_every_allocation(torch_cuda, ocean_lib):
    torch = torch_cuda
    d = P.c2(512)
    lp = P.lib_params(d)
    with ocean_lib.Ocean(lp, seed=1):
        pass                                           # warm-up: the context and kernels are loaded
    base = _free(torch)
    failures = 0
    try:
        for k in range(12):
            ocean_lib.debug_fail_allocations(k)
            try:
                with ocean_lib.Ocean(lp, seed=1):
                    pass
                break                                  # k >= the number of allocations: it succeeded
            except ocean_lib.OceanError as e:
                failures += 1
                assert "alloc" in str(e)
    finally:
        ocean_lib.debug_fail_allocations(-1)
    assert failures >= 7                               # h0, spectrum, intermediate, maps, status, noise, twiddles
    assert abs(_free(torch) - base) <= 64 << 20       # nothing of the failed creates is left allocated
    with ocean_lib.Ocean(lp, seed=1) as oc:           # and the library still works
        oc.update(1.0)
        oc.device_status()


def test_batch_create_fails_cleanly_at_every_allocation(torch_cuda, ocean_lib):
    torch = torch_cuda
    tiles = [P.lib_params(P.c2(n)) for n in (64, 128, 64)]
    ocean_lib.OceanBatch(tiles, seeds=[1, 2, 3], samples=2).close()   # warm-up
    base = _free(torch)
    failures = 0
    try:
        for k in range(20):
            ocean_lib.debug_fail_allocations(k)
            try:
                b = ocean_lib.OceanBatch(tiles, seeds=[1, 2, 3], samples=2)
                b.close()
                break
            except ocean_lib.OceanError:
                failures += 1
    finally:
        ocean_lib.debug_fail_allocations(-1)
    assert failures >= 8
    assert abs(_free(torch) - base) <= 64 << 20
