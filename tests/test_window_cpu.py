"""Decay windows of the fast method (CPU check of the rule, no GPU).

The fast method's scan and per-level passes run on a window [j0, j1] of the
grid instead of the oracle's [i0, i1]: beyond the classical turning points of
an energy E_up the discrete solution decays at least by acosh(1 + 6 t_i) per
step (t_i = a (V_i - E_up)), and the window ends where that exponent, summed
from the turning point, reaches 36.  This file restates the kernels' rule in
numpy (in FP64; the kernels sum it in FP32 with block minima rounded down) and
checks on dense eigen-decompositions of the discrete problem that the cut
leaves every eigenvalue below E_up unchanged to FP64 rounding and the
eigenvectors unchanged far below the 1e-8 L2 tolerance, while the window is
much shorter than the grid for most energies.
"""
from __future__ import annotations

import numpy as np
import pytest

from epseon_backend_gb300 import synth
from oracle import oracle as O

DECAY = 36.0


def decay_window(V, g, mu, Eu, decay=DECAY):
    """[j0, j1] of the kernels' decay window at energy Eu (within [i0, i1]).

    The kernels sum the decay over whole 32-point blocks beyond the block of
    each turning point, a block of n points counting n acosh(1 + 6 t) with t
    from the block's minimum of a V: a lower bound of the point-wise sum."""
    i0, i1, h = g.i0, g.i1, g.h
    a = mu * h * h / 6.0
    allowed = np.nonzero(V[i0 : i1 + 1] <= Eu)[0]
    t_in, t_out = i0 + allowed[0], i0 + allowed[-1]

    def block_decay(B):
        lo, hi = max(32 * B, i0), min(32 * B + 31, i1)
        t = a * V[lo : hi + 1].min() - a * Eu
        return (hi - lo + 1) * np.arccosh(1.0 + 6.0 * max(t, 0.0))

    j1, X = i1, 0.0
    for B in range(t_out // 32 + 1, i1 // 32 + 1):
        X += block_decay(B)
        if X >= decay:
            j1 = min(32 * B + 31, i1)
            break
    j0, X = i0, 0.0
    for B in range(t_in // 32 - 1, i0 // 32 - 1, -1):
        X += block_decay(B)
        if X >= decay:
            j0 = max(32 * B, i0)
            break
    if j1 - j0 < 4:
        return i0, i1
    return int(j0), int(j1)


def dense(V, lo, hi, h, mu):
    m = hi - lo + 1
    D2 = np.diag(-2.0 * np.ones(m)) + np.diag(np.ones(m - 1), 1) + np.diag(np.ones(m - 1), -1)
    B = np.eye(m) + D2 / 12.0
    H = np.diag(V[lo : hi + 1]) - np.linalg.solve(B, D2) / (2.0 * mu * h * h)
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    return w, U / np.sqrt(h)


@pytest.mark.parametrize("seed", [5, 9])
def test_window_leaves_levels_unchanged(seed):
    b = synth.mixed_batch(B=12, n_min=600, n_max=1200, seed=seed)
    cut_any = False
    for i in range(len(b)):
        V = b.V(i)
        g = O.grid(V, b.r_min[i], b.r_max[i], b.mu[i], b.e_cap[i], 512)
        mu = b.mu[i]
        w_full, U_full = dense(V, g.i0, g.i1, g.h, mu)
        n_bound = int(np.sum(w_full < b.e_cap[i]))
        if n_bound < 2:
            continue
        for frac in (0.3, 1.0):
            v_top = max(0, int(frac * n_bound) - 1)
            Eu = 0.5 * (w_full[v_top] + (w_full[v_top + 1] if v_top + 1 < w_full.size else b.e_cap[i]))
            j0, j1 = decay_window(V, g, mu, Eu)
            assert g.i0 <= j0 < j1 <= g.i1
            if j1 - j0 < 0.8 * (g.i1 - g.i0):
                cut_any = True
            w_win, U_win = dense(V, j0, j1, g.h, mu)
            n = v_top + 1
            # eigenvalues below E_up: unchanged to rounding
            assert np.max(np.abs(w_win[:n] - w_full[:n])) < 1e-12, (i, frac, j0, j1)
            # eigenvectors: zero outside the window, unchanged inside
            for v in range(n):
                full = U_full[:, v]
                win = np.zeros_like(full)
                win[j0 - g.i0 : j1 - g.i0 + 1] = U_win[:, v]
                if np.dot(full, win) < 0:
                    win = -win
                assert np.sqrt(np.sum((full - win) ** 2) * g.h) < 1e-10, (i, frac, v)
    assert cut_any


def test_window_is_monotone_in_energy():
    """Windows grow with the energy, so the window of a block's highest trial
    energy contains the windows of every energy of the block."""
    b = synth.morse_batch(B=3, N=4096, n_trial=256, seed=7)
    for i in range(len(b)):
        V = b.V(i)
        g = O.grid(V, b.r_min[i], b.r_max[i], b.mu[i], b.e_cap[i], 256)
        prev = None
        for E in np.linspace(V.min() + 1e-4, b.e_cap[i], 24):
            j0, j1 = decay_window(V, g, b.mu[i], E)
            if prev is not None:
                assert j0 <= prev[0] and j1 >= prev[1]
            prev = (j0, j1)
