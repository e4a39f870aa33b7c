"""Pins the FP64 oracle (test infrastructure) against independent truths.

The reference (epseon_backend) has no solver and no golden data, so parity
with it is unpinned; the oracle is pinned here against
  * the dense symmetric eigen-decomposition of the same discretisation,
  * the analytic Morse spectrum (O(h^4) discretisation error),
  * node count == level index,
  * Hellmann-Feynman derivatives vs central finite differences,
  * the frozen golden vectors in tests/golden (regression).
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from epseon_backend_gb300 import synth
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def dense_levels(V, g, mu, n):
    i0, i1, h = g.i0, g.i1, g.h
    m = i1 - i0 + 1
    D2 = np.diag(-2.0 * np.ones(m)) + np.diag(np.ones(m - 1), 1) + np.diag(np.ones(m - 1), -1)
    B = np.eye(m) + D2 / 12.0
    H = np.diag(V[i0 : i1 + 1]) - np.linalg.solve(B, D2) / (2.0 * mu * h * h)
    H = 0.5 * (H + H.T)
    w, U = np.linalg.eigh(H)
    return w[:n], U[:, :n] / np.sqrt(h)


def test_morse_single_against_dense_and_analytic():
    b = synth.morse_single()
    V = b.V(0)
    s = O.solve_batch([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, want_psi=True)[0]
    assert s.n_total == 14 and s.status == 0
    an = synth.analytic_morse_levels(0.1, 1.0, 1000.0, b.e_cap[0])
    assert an.size == 14
    # O(h^4) discretisation error of Numerov on this grid
    assert np.max(np.abs(s.energy_polished - an)) < 5e-9
    # dense eigen-decomposition of the same discretisation on a coarser grid
    b = synth.morse_single(N=1400)
    V = b.V(0)
    s = O.solve_batch([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, want_psi=True)[0]
    assert s.n_total == 14
    w, U = dense_levels(V, s.grid, b.mu[0], 14)
    assert np.max(np.abs(s.energy_polished - w)) < 1e-12
    assert np.max(np.abs(s.energy - w)) < 1e-12  # bisection to 1e-12
    assert np.array_equal(s.nodes, np.arange(14))
    h = s.grid.h
    for v in range(14):
        u = U[:, v].copy()
        if u[0] < 0:
            u = -u
        psi = s.psi[v, s.grid.i0 : s.grid.i1 + 1]
        assert np.sqrt(np.sum((u - psi) ** 2) * h) < 1e-8
        assert abs(np.sum(s.psi[v] ** 2) * h - 1.0) < 1e-12


@pytest.mark.parametrize("seed", [11, 14, 18])
def test_mixed_kinds_against_dense(seed):
    b = synth.mixed_batch(B=16, n_min=500, n_max=1100, seed=seed)
    for i in range(len(b)):
        V = b.V(i)
        s = O.solve_batch([V], b.r_min[i], b.r_max[i], b.mu[i], b.e_cap[i], 512)[0]
        if s.n_total == 0:
            continue
        w, _ = dense_levels(V, s.grid, b.mu[i], s.n_total + 1)
        # level counts and energies are exact (Sturm counts) even on grids too
        # coarse for the wavelength (status UNDER_RESOLVED)
        assert np.sum(w < b.e_cap[i]) == s.n_total
        assert np.max(np.abs(s.energy_polished - w[: s.n_total])) < 1e-13
        assert np.max(np.abs(s.energy - w[: s.n_total])) < 1e-12
        if not (s.status & O.UNDER_RESOLVED):
            assert np.array_equal(s.nodes, np.arange(s.n_total))


def test_count_is_monotone_and_exact():
    b = synth.morse_single(N=1024, n_trial=256)
    V = b.V(0)
    g = O.grid(V, b.r_min[0], b.r_max[0], b.mu[0], b.e_cap[0], 256)
    w, _ = dense_levels(V, g, b.mu[0], 14)
    Es = np.linspace(g.e_lo + 1e-6, b.e_cap[0], 300)
    for k in (g.k_scan, g.i0, g.i1, (g.i0 + g.i1) // 2):
        c = [O.count(V, g, E, k) for E in Es]
        assert np.all(np.diff(c) >= 0)
        assert c == [int(np.sum(w < E)) for E in Es]


def test_hellmann_feynman_matches_fd():
    b = synth.morse_single(N=1500, n_trial=256)
    V = b.V(0).copy()
    s = O.solve_batch([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, want_psi=True)[0]
    h = s.grid.h
    for v in (0, 5, 11):
        for i in (300, 420, 600):
            d = 1e-5
            Vp, Vm = V.copy(), V.copy()
            Vp[i] += d
            Vm[i] -= d
            ep = O.solve_batch([Vp], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)[0].energy_polished[v]
            em = O.solve_batch([Vm], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)[0].energy_polished[v]
            fd = (ep - em) / (2 * d)
            hf = s.psi[v, i] ** 2 * h
            assert abs(fd - hf) <= 1e-6 * max(abs(hf), 1e-4)


def test_double_well_inner_level_wavefunction():
    # Morse with a tall Gaussian barrier: a double well whose inner levels are
    # invisible at the outer turning point; the match point must move.
    r = np.linspace(0.5, 12.0, 1500)
    V = synth.morse(r, 0.1, 1.0, 2.0) + synth.bumps_at(r, [(0.08, 0.25, 2.6)])
    s = O.solve_batch([V], 0.5, 12.0, 2000.0, 0.0999, 512, want_psi=True)[0]
    g = s.grid
    w, U = dense_levels(V, g, 2000.0, s.n_total)
    assert np.max(np.abs(s.energy_polished - w)) < 1e-11
    assert np.array_equal(s.nodes, np.arange(s.n_total))
    for v in range(s.n_total):
        u = U[:, v].copy()
        if u[0] < 0:
            u = -u
        assert np.sqrt(np.sum((u - s.psi[v, g.i0 : g.i1 + 1]) ** 2) * g.h) < 1e-7


def test_golden_vectors():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        gold = json.load(f)
    for case in gold["cases"]:
        b = getattr(synth, case["workload"])(**case.get("kwargs", {}))
        idx = case["indices"]
        sel = np.array(idx)
        sols = O.solve_batch([b.V(i) for i in idx], b.r_min[sel], b.r_max[sel], b.mu[sel], b.e_cap[sel], case["n_trial"])
        for s, ref in zip(sols, case["results"]):
            assert s.n_total == ref["n_total"]
            # the plain method's bits are platform independent (explicit fma, no contraction)
            assert np.max(np.abs(s.energy - np.array(ref["energy"]))) <= 2e-13
            assert np.array_equal(s.counts[:: case["count_stride"]], np.array(ref["counts_strided"]))
