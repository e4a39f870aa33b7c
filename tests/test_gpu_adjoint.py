"""Adjoint (Hellmann-Feynman) gradients of the CUDA solver, through the C ABI
and torch.autograd, against central finite differences of the FP64 oracle
re-solved on perturbed potentials (the reference solver's role: the
reference has no numerics of its own, its algorithm slot is
VibwaAlgorithm<FP>::run, cpp/gpu/include/epseon/gpu/algorithms/vibwa.hpp:605-637).

* dL/dV_i for both methods on Morse+bump grids (N = 4096);
* dL/dtheta through the parameter chain for every kind: Morse (De, a, re),
  shifted Lennard-Jones (eps, sigma) and Morse + Gaussian bumps through the
  natural cubic spline (S^T, then the knot-level derivatives), with the
  adjoint workload's loss sum_v w_v (E_v - T_v)^2;
* the long grid (one heavy Morse, N = 2^20): gradients of the top 50 levels.

Bar: 1e-6 relative.  The finite-difference noise floor, measured with the
oracle alone (its Hellmann-Feynman gradient from its own wavefunctions
against its own central differences): a single V_i on a 4096-point grid with
h = 1e-6, 3e-9 relative; parameters with h = 1e-6 (absolute, FP64), below
1e-8; on the 2^20-point grid a single point is too noisy for the bar (2.6e-5
at h = 1e-6, 1.4e-6 at h = 1e-5: the level shift is ~1e-11 against a
polished-energy noise of ~1e-14), so there the derivative is taken along a
direction supported on 2000 sampled points in the well, h = 1e-5, noise
2e-9 relative.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from epseon_backend_gb300 import autograd as AG
from epseon_backend_gb300 import capi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-6


def _oracle_E(V, b, i, n_trial, **kw):
    return O.solve_batch([V], b.r_min[i], b.r_max[i], b.mu[i], b.e_cap[i], n_trial, **kw)[0].energy_polished


def _well_points(gV, k_min, rng, count):
    well = np.where(gV > 1e-3 * gV.max())[0]
    well = well[np.abs(well - k_min) > 8]  # the minimum sets the cut-offs: leave it alone
    return np.sort(rng.choice(well, count, replace=False))


@pytest.mark.parametrize("method", [capi.METHOD_FAST_FP32C, capi.METHOD_PLAIN_FP64])
def test_potential_gradient_matches_oracle_fd(method):
    b = synth.bump_adjoint(B=2, N=4096, n_trial=1024)
    g = AG.Grids(b.N.copy(), b.r_min.copy(), b.r_max.copy(), b.mu.copy(), b.e_cap.copy(), b.n_trial, 128, method)
    solver = AG.Solver()
    P = torch.from_numpy(capi.batch_params(b)).cuda()
    with torch.no_grad():
        V0 = AG.tabulate(P, b.kind, g, solver=solver)
    V = V0.clone().requires_grad_(True)
    E, mask = AG.levels(V, g, solver)
    rng = np.random.default_rng(3)
    w = torch.from_numpy(rng.uniform(0.5, 1.0, tuple(E.shape))).cuda()
    L = torch.sum(torch.where(mask, w * E, torch.zeros_like(E)))
    L.backward()
    gV = V.grad.cpu().numpy()
    Vh = V0.cpu().numpy()  # the device-tabulated potentials, re-solved by the oracle
    off = g.offsets
    wn = w.cpu().numpy()
    checked = 0
    for i in range(len(b)):
        N = int(b.N[i])
        Vi = Vh[off[i]: off[i] + N]
        gi = gV[off[i]: off[i] + N]
        n = int(mask[i].sum())
        k_min = int(np.argmin(Vi))
        top = np.argsort(-np.abs(gi))[:3]
        pts = np.unique(np.concatenate([top, _well_points(np.abs(gi), k_min, rng, 4)]))
        for j in pts:
            if abs(j - k_min) <= 8:
                continue
            hfd = 1e-6
            Vp, Vm = Vi.copy(), Vi.copy()
            Vp[j] += hfd
            Vm[j] -= hfd
            Ep, Em = _oracle_E(Vp, b, i, b.n_trial), _oracle_E(Vm, b, i, b.n_trial)
            assert Ep.size == Em.size == n
            fd = float(np.sum(wn[i, :n] * (Ep - Em)) / (2 * hfd))
            assert abs(gi[j] - fd) <= REL * abs(fd), (i, int(j), gi[j], fd)
            checked += 1
    assert checked >= 10


def _kind_batch():
    """Two potentials of each kind (Morse, shifted LJ, Morse + bumps via the
    spline) from the mixed-batch generator, grids of 3000 - 6000 points."""
    b = synth.mixed_batch(B=60, n_min=3000, n_max=6000, seed=9)
    idx = []
    for kind in (synth.KIND_MORSE, synth.KIND_LJ, synth.KIND_SPLINE):
        idx += list(np.where(b.kind == kind)[0][:2])
    bb = b.subset(idx)
    bb.n_trial = 2048
    return bb


def _targets(kind, P):
    """Target parameters: bump amplitudes x 1.1 (the adjoint workload's
    targets); Morse and LJ well depths x 1.01."""
    T = P.copy()
    for i in range(T.shape[0]):
        if int(kind[i]) == synth.KIND_SPLINE:
            T[i, 3::3] *= 1.1
        else:
            T[i, 0] *= 1.01
    return T


@pytest.mark.parametrize("method", [capi.METHOD_FAST_FP32C, capi.METHOD_PLAIN_FP64])
def test_parameter_gradients_match_oracle_fd(method):
    b = _kind_batch()
    cap = 256
    g = AG.Grids(b.N.copy(), b.r_min.copy(), b.r_max.copy(), b.mu.copy(), b.e_cap.copy(), b.n_trial, cap, method)
    P = capi.batch_params(b)
    T = _targets(b.kind, P)
    n = len(b)
    nt = b.n_trial

    def oracle_levels(i, row):
        V = synth.tabulate_params(b.kind[i], row, b.N[i], b.r_min[i], b.r_max[i])
        return _oracle_E(V, b, i, nt)

    # targets: the oracle's levels of the target parameters (constants)
    Et = [oracle_levels(i, T[i]) for i in range(n)]
    w = synth.loss_weights(n * cap).reshape(n, cap)
    Tt = np.zeros((n, cap))
    Tm = np.zeros((n, cap), bool)
    for i in range(n):
        Tt[i, : Et[i].size] = Et[i]
        Tm[i, : Et[i].size] = True
    Tt_d, Tm_d, w_d = (torch.from_numpy(x).cuda() for x in (Tt, Tm, w))

    solver = AG.Solver()
    Pr = torch.from_numpy(P).cuda().requires_grad_(True)
    E, mask = AG.levels(AG.tabulate(Pr, b.kind, g, solver=solver), g, solver)
    m = mask & Tm_d
    L = torch.sum(torch.where(m, w_d * (E - Tt_d) ** 2, torch.zeros_like(E)))
    L.backward()
    grad = Pr.grad.cpu().numpy()
    mn = m.cpu().numpy()

    def loss_i(i, row):
        Ei = oracle_levels(i, row)
        k = int(mn[i].sum())
        assert Ei.size >= k
        return float(np.sum(w[i, :k] * (Ei[:k] - Tt[i, :k]) ** 2))

    h = 1e-6
    checked = {synth.KIND_MORSE: 0, synth.KIND_LJ: 0, synth.KIND_SPLINE: 0}
    for i in range(n):
        kind = int(b.kind[i])
        active = [0, 1] if kind == synth.KIND_LJ else [0, 1, 2]
        if kind == synth.KIND_SPLINE:
            active += [3 + c for c in range(9) if P[i, 3 + 3 * (c // 3)] != 0.0]
        # 1e-6 of the potential's gradient scale: a component that nearly
        # cancels across levels sits below the finite-difference noise floor
        gscale = np.max(np.abs(grad[i, active]))
        for j in active:
            Pp, Pm = P[i].copy(), P[i].copy()
            Pp[j] += h
            Pm[j] -= h
            fd = (loss_i(i, Pp) - loss_i(i, Pm)) / (2 * h)
            assert abs(grad[i, j] - fd) <= REL * max(abs(fd), gscale), (i, kind, j, grad[i, j], fd, gscale)
            checked[kind] += 1
    assert all(c >= 4 for c in checked.values()), checked


def test_long_grid_top50_gradient(ctx):
    """The long grid (one heavy Morse, N = 2^20, 280 bound levels): the
    fast method's levels 230..279 with their wavefunctions, and the adjoint
    of L = sum_v w_v E_v to every V(r_i): pointwise against the oracle's
    Hellmann-Feynman gradient, and along a direction on 2000 sampled well
    points against the oracle's central difference."""
    b = synth.morse_long(n_trial=2048)
    V = b.V(0)
    lo, hi = 230, 279
    sol = ctx.solve([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_FAST_FP32C, min_level=lo,
                    max_level=hi, level_capacity=hi - lo + 1, want_psi=True)
    assert sol.n_total[0] == 280 and sol.n_out[0] == 50
    rng = np.random.default_rng(11)
    w = rng.uniform(0.5, 1.0, 50)
    gV = ctx.adjoint(w[None, :], V.size)
    ref = O.solve_batch([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, min_level=lo, max_level=hi,
                        want_psi=True)[0]
    assert ref.energy.size == 50
    g_ref = (w[:, None] * ref.psi ** 2).sum(0) * ref.grid.h
    assert np.max(np.abs(gV - g_ref)) <= REL * np.max(np.abs(g_ref))
    idx = _well_points(g_ref, int(ref.grid.k_scan), rng, 2000)
    d = np.zeros_like(V)
    d[idx] = rng.uniform(0.5, 1.5, idx.size)
    an = float(gV @ d)
    hfd = 1e-5
    kw = dict(min_level=lo, max_level=hi)
    Ep = O.solve_batch([V + hfd * d], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, **kw)[0].energy_polished
    Em = O.solve_batch([V - hfd * d], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, **kw)[0].energy_polished
    fd = float(np.sum(w * (Ep - Em)) / (2 * hfd))
    assert abs(an - fd) <= REL * abs(fd), (an, fd)


def test_autograd_psi_exact_size_and_recompute():
    """The autograd solve keeps its wavefunctions in a buffer of exactly the
    size the levels need (sum over potentials of levels x grid points, read
    back by the library after its level set-up), not capacity x points.  With
    a memory budget below that size the forward keeps none and the backward
    recomputes them in chunks of potentials that fit; the parameter gradients
    agree with the stored-psi ones far below the finite-difference bar (the
    chunks are re-solved as smaller batches, which may take a level through
    the other pass of the same method: ~1e-12 relative)."""
    b = synth.bump_adjoint(B=6, N=4096, n_trial=1024)
    g = AG.Grids(b.N.copy(), b.r_min.copy(), b.r_max.copy(), b.mu.copy(), b.e_cap.copy(), b.n_trial, 128,
                 capi.METHOD_FAST_FP32C)
    P = torch.from_numpy(capi.batch_params(b)).cuda()
    w = torch.from_numpy(synth.loss_weights(len(b) * 128).reshape(len(b), 128)).cuda()

    def grads(solver):
        Pr = P.clone().requires_grad_(True)
        E, mask = AG.levels(AG.tabulate(Pr, b.kind, g, solver=solver), g, solver)
        L = torch.sum(torch.where(mask, w * E, torch.zeros_like(E)))
        rec = solver.last
        L.backward()
        return Pr.grad.cpu().numpy(), rec

    stored, rec = grads(AG.Solver())
    need = int(np.sum(rec.n_out.astype(np.int64) * b.N.astype(np.int64)))
    assert rec.psi is not None and rec.psi.numel() == need == rec.psi_required
    assert need < g.total * g.capacity // 2
    recomputed, rec2 = grads(AG.Solver(psi_budget_bytes=need * 8 // 3))
    assert rec2.psi is None and rec2.V is not None
    assert np.max(np.abs(recomputed - stored)) <= 1e-10 * np.max(np.abs(stored))
