"""Edge cases of the CUDA solver through the C ABI, both methods, against the
FP64 oracle where a result exists: non-finite input, no bound level, a grid
too short for the cut-offs, level windows and capacities smaller than the
spectrum, a single trial energy (every level in one scan bracket), a psi
buffer too small, and a ragged batch mixing all of these with ordinary
potentials (one bad potential must not disturb the others).
"""
from __future__ import annotations

import numpy as np
import pytest

from epseon_backend_gb300 import capi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = {capi.METHOD_PLAIN_FP64: 1e-10, capi.METHOD_FAST_FP32C: 1e-10}
METHODS = [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C]


def _morse(N=3000, De=0.1, a=1.0, re=2.0, mu=1500.0):
    r0, r1 = 0.5, re + 30.0 / a
    r = np.linspace(r0, r1, N)
    return synth.morse(r, De, a, re), r0, r1, mu, 0.999 * De


@pytest.mark.parametrize("method", METHODS)
def test_ragged_batch_with_bad_potentials(ctx, method):
    good1 = _morse()
    good2 = _morse(N=5000, De=0.05, a=0.8, re=3.0, mu=20000.0)
    nan = list(_morse())
    nan[0] = nan[0].copy()
    nan[0][1234] = np.nan
    shallow = list(_morse())
    shallow[4] = -1.0  # cap below the minimum: no bound level
    short = (10.0 * np.array([1.0, 0.0, 1.0, 1.0, 1.0]), 0.5, 1.0, 1500.0, 0.1)  # one point survives the cut
    pots = [good1, nan, shallow, good2, short]
    Vs = [p[0] for p in pots]
    r0, r1, mu, cap = (np.array([p[k] for p in pots]) for k in (1, 2, 3, 4))
    sol = ctx.solve(Vs, r0, r1, mu, cap, 2048, method=method, level_capacity=256, want_psi=True)
    # the bad ones: nothing found, flagged
    for q in (1, 2, 4):
        assert sol.n_total[q] == 0 and sol.n_out[q] == 0
        assert sol.status[q, 0] & capi.LEVEL_BAD_INPUT
        assert sol.status[q, 0] & capi.LEVEL_NOT_FOUND
    assert sol.status[1, 0] & capi.LEVEL_NONFINITE
    # the good ones: as the oracle
    for q in (0, 3):
        V, a0, a1, m, c = pots[q]
        ref = O.solve_batch([V], a0, a1, m, c, 2048)[0]
        n = sol.n_out[q]
        assert n == ref.n_total and n > 0
        assert np.array_equal(sol.nodes[q, :n], np.arange(n))
        assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < E_TOL[method]


@pytest.mark.parametrize("method", METHODS)
def test_level_window_and_capacity(ctx, method):
    V, r0, r1, mu, cap = _morse(N=4000, mu=3000.0)
    ref = O.solve_batch([V], r0, r1, mu, cap, 2048)[0]
    nt = ref.n_total
    assert nt > 12
    # window [3, 7]
    sol = ctx.solve([V], r0, r1, mu, cap, 2048, method=method, min_level=3, max_level=7, level_capacity=5)
    assert sol.n_total[0] == nt and sol.n_out[0] == 5
    assert np.array_equal(sol.nodes[0, :5], np.arange(3, 8))
    assert np.max(np.abs(sol.energy[0, :5] - ref.energy_polished[3:8])) < E_TOL[method]
    # capacity below the spectrum: the lowest `cap` levels, the total still reported
    sol = ctx.solve([V], r0, r1, mu, cap, 2048, method=method, level_capacity=4)
    assert sol.n_total[0] == nt and sol.n_out[0] == 4
    assert np.max(np.abs(sol.energy[0, :4] - ref.energy_polished[:4])) < E_TOL[method]
    # window beyond the spectrum: nothing out, the total still reported
    sol = ctx.solve([V], r0, r1, mu, cap, 2048, method=method, min_level=nt + 3, max_level=nt + 5, level_capacity=3)
    assert sol.n_total[0] == nt and sol.n_out[0] == 0


@pytest.mark.parametrize("method", METHODS)
def test_single_trial_energy(ctx, method):
    """One trial energy (at the cap): every level starts in the same scan
    bracket; counts and the refinement still separate them."""
    V, r0, r1, mu, cap = _morse(N=2500, mu=1000.0)
    ref = O.solve_batch([V], r0, r1, mu, cap, 1024)[0]
    sol = ctx.solve([V], r0, r1, mu, cap, 1, method=method, level_capacity=64)
    n = sol.n_out[0]
    assert n == ref.n_total
    assert np.array_equal(sol.nodes[0, :n], np.arange(n))
    assert np.max(np.abs(sol.energy[0, :n] - ref.energy_polished)) < E_TOL[method]


@pytest.mark.parametrize("method", METHODS)
def test_psi_buffer_too_small(ctx, method):
    V, r0, r1, mu, cap = _morse(N=3000)
    with pytest.raises(RuntimeError, match="psi buffer too small|capacity"):
        ctx.solve([V], r0, r1, mu, cap, 1024, method=method, level_capacity=64, want_psi=True, psi_capacity=3000)
    # the context stays usable
    sol = ctx.solve([V], r0, r1, mu, cap, 1024, method=method, level_capacity=64)
    assert sol.n_out[0] > 0


def test_bisection_scan_batch(ctx):
    """A batch large enough for the bisection scan (counts only where they
    change: the coarse grid of every 16th trial energy, then a count round
    inside the cells whose end counts differ)
    gives every level of the plain FP64 solver (itself bit-exact with the
    oracle) within the fast method's tolerance, with its node count."""
    b = synth.mixed_batch(B=640, n_min=2048, n_max=6144, seed=11)
    b.n_trial = 2048
    Vs = b.potentials()
    ref = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_PLAIN_FP64, level_capacity=256)
    sol = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_FAST_FP32C, level_capacity=256)
    # a second solve gives the same bits (the count round's lists, and so the
    # refinement's first energies, do not depend on thread scheduling)
    again = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_FAST_FP32C, level_capacity=256)
    assert np.array_equal(again.energy, sol.energy, equal_nan=True)
    assert np.array_equal(sol.n_total, ref.n_total)
    assert np.array_equal(sol.n_out, ref.n_out)
    checked = 0
    for q in range(len(b)):
        n = sol.n_out[q]
        if n == 0:
            continue
        if not (ref.status[q, 0] & capi.LEVEL_UNDER_RESOLVED):
            assert np.array_equal(sol.nodes[q, :n], ref.nodes[q, :n])
        assert np.max(np.abs(sol.energy[q, :n] - ref.energy[q, :n])) < E_TOL[capi.METHOD_FAST_FP32C]
        checked += n
    assert checked > 10000
