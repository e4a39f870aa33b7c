"""Adjoint (Hellmann-Feynman) gradients through torch.autograd, checked against
central finite differences of the CUDA solver (the Morse+bump adjoint
workload at reduced size: loss = sum_v w_v (E_v - T_v)^2, T_v the levels with
every bump amplitude scaled by 1.1)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from epseon_backend_gb300 import autograd as AG
from epseon_backend_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _setup(method, B=3, N=6144, n_trial=2048):
    b = synth.bump_adjoint(B=B, N=N, n_trial=n_trial)
    t = synth.bump_adjoint(B=B, N=N, n_trial=n_trial, amp_scale=1.1)
    g = AG.Grids(b.N.copy(), b.r_min.copy(), b.r_max.copy(), b.mu.copy(), b.e_cap.copy(), n_trial, 256, method)
    P = torch.from_numpy(capi.batch_params(b)).cuda()
    Pt = torch.from_numpy(capi.batch_params(t)).cuda()
    return b, g, P, Pt


def _loss(P, Pt, kind, g, solver, w):
    V = AG.tabulate(P, kind, g, solver=solver)
    E, mask = AG.levels(V, g, solver)
    with torch.no_grad():
        Et, mt = AG.levels(AG.tabulate(Pt, kind, g, solver=solver), g, solver)
    m = mask & mt
    return torch.sum(torch.where(m, w * (E - Et) ** 2, torch.zeros_like(E))), V


@pytest.mark.parametrize("method", [capi.METHOD_FAST_FP32C, capi.METHOD_PLAIN_FP64])
def test_parameter_gradients_match_fd(method):
    b, g, P, Pt = _setup(method)
    solver = AG.Solver()
    w = torch.from_numpy(synth.loss_weights(len(b) * 256).reshape(len(b), 256)).cuda()
    Pr = P.clone().requires_grad_(True)
    L, _ = _loss(Pr, Pt, b.kind, g, solver, w)
    L.backward()
    grad = Pr.grad.cpu().numpy()
    h = 1e-6
    checked = 0
    # 1e-6 relative to the potential's gradient scale: a component that nearly
    # cancels across levels sits below the finite-difference noise floor
    # (energy error ~1e-14 against a difference of ~1e-9)
    for p in range(len(b)):
        for j in [0, 1, 2, 3, 4, 5]:
            if j >= 3 and P[p, j].item() == 0.0:
                continue
            # central differences with h = 1e-6 (absolute, FP64)
            Pp, Pm = P.clone(), P.clone()
            Pp[p, j] += h
            Pm[p, j] -= h
            with torch.no_grad():
                Lp, _ = _loss(Pp, Pt, b.kind, g, solver, w)
                Lm, _ = _loss(Pm, Pt, b.kind, g, solver, w)
            fd = (Lp.item() - Lm.item()) / (2 * h)
            an = grad[p, j]
            gscale = np.max(np.abs(grad[p, :6]))
            assert abs(an - fd) <= 1e-6 * max(abs(fd), gscale), (p, j, an, fd, gscale)
            checked += 1
    assert checked >= 10


def test_potential_gradient_matches_fd():
    b, g, P, Pt = _setup(capi.METHOD_FAST_FP32C, B=2, N=4096, n_trial=1024)
    solver = AG.Solver()
    with torch.no_grad():
        V0 = AG.tabulate(P, b.kind, g, solver=solver)
    V = V0.clone().requires_grad_(True)
    E, mask = AG.levels(V, g, solver)
    w = torch.rand_like(E)
    L = torch.sum(torch.where(mask, w * E, torch.zeros_like(E)))
    L.backward()
    gV = V.grad.cpu().numpy()
    N0 = int(g.N[0])
    Vnp = V0.cpu().numpy()
    for i in np.argsort(-np.abs(gV[:N0]))[:6]:
        d = 1e-6
        Vp, Vm = Vnp.copy(), Vnp.copy()
        Vp[i] += d
        Vm[i] -= d
        with torch.no_grad():
            Ep, mp = AG.levels(torch.from_numpy(Vp).cuda(), g, solver)
            Em, mm = AG.levels(torch.from_numpy(Vm).cuda(), g, solver)
        fd = torch.sum(torch.where(mask, w * (Ep - Em), torch.zeros_like(Ep))).item() / (2 * d)
        assert abs(gV[i] - fd) <= 1e-6 * abs(fd) + 1e-10, (i, gV[i], fd)
