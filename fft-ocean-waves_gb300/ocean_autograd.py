"""torch.autograd wrappers over the C ABI (ocean_update / ocean_backward).

``OceanParamFrames``  D(t_j) for T frames as a function of the spectrum
                      parameters (A, V, theta, lambda); backward calls
                      ocean_backward for dL/d(A, V, theta, lambda).
``OceanH0Loss``       an MSE between this tile's frames and a target tile's
                      frames as a function of the per-mode spectrum h0
                      (N, N, 4); neither forward nor backward keeps frames:
                      the forward accumulates the loss frame by frame and the
                      backward recomputes each frame's residual from h0 (the
                      only saved tensor) and feeds it to ocean_backward.

Both take an ``ocean_gb300.Ocean`` handle whose state they set (parameters or
h0) before running.  Device work goes to torch's current stream.
"""
from __future__ import annotations

import math

import torch

import ocean_gb300 as og


def _frames(oc: og.Ocean, times, out=None):
    N = oc.params.N
    dev = torch.device("cuda", torch.cuda.current_device())
    T = len(times)
    D = out if out is not None else torch.empty((T, 3, N, N), dtype=torch.float32, device=dev)
    nj = torch.empty((N, N, 4), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream()
    for j, t in enumerate(times):
        oc.update(t, D[j, 0], D[j, 1], D[j, 2], nj, stream=st)
    return D


def params_with(base: og.Params, A, V, theta, lam) -> og.Params:
    return og.Params(N=base.N, L=base.L, amplitude=float(A), wind_speed=float(V),
                     wind_dir_x=math.cos(float(theta)), wind_dir_y=math.sin(float(theta)),
                     choppiness=float(lam), suppression=base.suppression, gravity=base.gravity,
                     literal_conj=base.literal_conj)


class OceanParamFrames(torch.autograd.Function):
    """theta4 = (A, V, theta, lambda) (CPU float64 tensor) -> frames (T, 3, N, N)
    holding (Dx, Dy, Dz) per frame."""

    @staticmethod
    def forward(ctx, theta4, oc: og.Ocean, times):
        A, V, th, lam = (float(x) for x in theta4.detach().cpu())
        oc.set_params(params_with(oc.params, A, V, th, lam))
        ctx.oc, ctx.times = oc, list(times)
        return _frames(oc, times)

    @staticmethod
    def backward(ctx, gD):
        # ocean_backward takes each field's gradients frame-major and contiguous
        g = [gD[:, f].contiguous() for f in range(3)]
        r = ctx.oc.backward(ctx.times, g[0], g[1], g[2], stream=torch.cuda.current_stream())
        g = torch.tensor([r["dA"], r["dV"], r["dtheta"], r["dlambda"]], dtype=torch.float64)
        return g, None, None


class OceanH0Loss(torch.autograd.Function):
    """h0 (N, N, 4) device tensor -> sum over frames of mean squared error
    between this tile's (Dx, Dy, Dz) and the target tile's, normalised by the
    number of values (T * 3 * N * N)."""

    @staticmethod
    def forward(ctx, h0, oc: og.Ocean, target: og.Ocean, times):
        oc.set_h0(h0, stream=torch.cuda.current_stream())
        N = oc.params.N
        n = len(times) * 3 * N * N
        D = torch.empty((1, 3, N, N), dtype=torch.float32, device=h0.device)
        Dt = torch.empty_like(D)
        loss = torch.zeros((), dtype=torch.float64, device=h0.device)
        for t in times:
            _frames(oc, [t], D)
            _frames(target, [t], Dt)
            loss += ((D - Dt).double() ** 2).sum()
        ctx.save_for_backward(h0)
        ctx.oc, ctx.target, ctx.times, ctx.n = oc, target, list(times), n
        return loss / n

    @staticmethod
    def backward(ctx, gl):
        (h0,) = ctx.saved_tensors
        oc, target = ctx.oc, ctx.target
        oc.set_h0(h0, stream=torch.cuda.current_stream())
        N = oc.params.N
        D = torch.empty((1, 3, N, N), dtype=torch.float32, device=h0.device)
        Dt = torch.empty_like(D)
        dh0 = torch.zeros_like(h0)
        scale = (2.0 / ctx.n) * float(gl)
        for j, t in enumerate(ctx.times):
            _frames(oc, [t], D)                        # recomputed from h0
            _frames(target, [t], Dt)
            G = (D - Dt) * scale                       # one frame: each field slice is contiguous
            oc.backward([t], G[0, 0], G[0, 1], G[0, 2], dh0=dh0, accumulate=j > 0,
                        stream=torch.cuda.current_stream())
        return dh0, None, None, None
