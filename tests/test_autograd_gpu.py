"""torch.autograd wrappers over the C ABI (fft-ocean-waves_gb300/ocean_autograd.py):
wiring checks and the parameter-fit workload (N=512, T=32 frames at dt=0.1 s,
hidden A=3, V=22 m/s at 50 deg, lambda=1.1, L=1500 m, noise seed 3, target
noise sigma=0.02 m, MSE, 200 Adam steps from A=1, V=10, 0 deg, lambda=0.5)."""
import math

import numpy as np
import pytest

from conftest import rel_l2
import params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _base(N):
    return P.lib_params(dict(N=N, L=1500.0, amplitude=3.0, wind_speed=22.0, wind_x=P.f32(math.cos(math.radians(50))),
                             wind_y=P.f32(math.sin(math.radians(50))), choppiness=P.f32(1.1),
                             suppression=P.f32(0.1), seed=3))


def test_param_frames_gradient_wiring(torch_cuda, ocean_lib):
    import ocean_autograd as oa
    torch = torch_cuda
    N, times = 64, [0.0, 0.1, 0.2]
    oc = ocean_lib.Ocean(_base(N), seed=3)
    theta = torch.tensor([3.0, 22.0, math.radians(50), 1.1], dtype=torch.float64, requires_grad=True)
    D = oa.OceanParamFrames.apply(theta, oc, times)
    w = torch.randn_like(D)
    (D * w).sum().backward()
    r = oc.backward(times, w[:, 0].contiguous(), w[:, 1].contiguous(), w[:, 2].contiguous())
    g = theta.grad.numpy()
    assert np.allclose(g, [r["dA"], r["dV"], r["dtheta"], r["dlambda"]], rtol=1e-6)
    oc.close()


def test_h0_loss_gradient_matches_oracle(torch_cuda, ocean_lib, oracle_mod):
    """dMSE/dh0 with frames recomputed in the backward, against the FP64
    adjoint applied to FP64 residuals."""
    import ocean_autograd as oa
    torch = torch_cuda
    N, times = 128, [0.0, 0.05, 0.1, 0.15]
    lp = _base(N)
    oc = ocean_lib.Ocean(lp, seed=10)
    tgt = ocean_lib.Ocean(lp, seed=10)
    dev = torch.device("cuda")
    h0 = torch.empty((N, N, 4), dtype=torch.float32, device=dev)
    oc.get_h0(h0)
    gen = torch.Generator(device="cpu").manual_seed(0)
    h0t = h0 * (1 + 0.05 * torch.randn(h0.shape, generator=gen).to(dev))
    tgt.set_h0(h0t)
    h0 = h0.clone().requires_grad_(True)
    loss = oa.OceanH0Loss.apply(h0, oc, tgt, times)
    loss.backward()
    # FP64 reference
    op = oracle_mod.Params(N=N, L=lp.L, amplitude=lp.amplitude, wind_speed=lp.wind_speed, wind_x=lp.wind_dir_x,
                           wind_y=lp.wind_dir_y, choppiness=lp.choppiness, suppression=lp.suppression,
                           gravity=lp.gravity)
    ha = h0.detach().cpu().numpy().astype(np.float64)
    hb = h0t.cpu().numpy().astype(np.float64)
    n = len(times) * 3 * N * N
    res = {k: [] for k in ("dx", "dy", "dz")}
    L64 = 0.0
    for t in times:
        a, b = oracle_mod.update(op, ha, t), oracle_mod.update(op, hb, t)
        for k in res:
            res[k].append(2.0 / n * (a[k] - b[k]))
            L64 += np.sum((a[k] - b[k]) ** 2) / n
    dh0_ref, _ = oracle_mod.backward(op, ha, times, np.array(res["dx"]), np.array(res["dy"]), np.array(res["dz"]))
    assert abs(float(loss.detach()) - L64) < 1e-4 * L64
    assert rel_l2(h0.grad.cpu().numpy(), dh0_ref) < 1e-4
    oc.close()
    tgt.close()


def test_parameter_fit_converges(torch_cuda, ocean_lib):
    """200 Adam steps of the N=512 fit reach the noise floor of the target
    (MSE = sigma^2 = 4e-4) from an initial MSE about 18x higher."""
    import ocean_autograd as oa
    torch = torch_cuda
    N, T = 512, 32
    times = [0.1 * j for j in range(T)]
    lp = _base(N)
    hidden = ocean_lib.Ocean(lp, seed=3)
    target = oa._frames(hidden, times).clone()
    gen = torch.Generator(device="cpu").manual_seed(123)
    target += 0.02 * torch.randn(target.shape, generator=gen).to(target.device)
    hidden.close()
    model = ocean_lib.Ocean(oa.params_with(lp, 1.0, 10.0, 0.0, 0.5), seed=3)
    # optimise in scaled coordinates: (log A, V/10, theta, lambda)
    z = torch.tensor([0.0, 1.0, 0.0, 0.5], dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([z], lr=0.05)
    losses = []
    for it in range(200):
        opt.zero_grad()
        th = torch.stack([z[0].exp(), 10.0 * z[1], z[2], z[3]])
        D = oa.OceanParamFrames.apply(th, model, times)
        loss = ((D - target) ** 2).mean()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    model.close()
    sigma2 = 0.02 ** 2
    assert losses[0] > 10 * sigma2
    assert losses[-1] < 1.05 * sigma2, (losses[0], losses[-1])
