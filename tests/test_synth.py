"""Seeded synthetic workloads: reproducible, in range, and the spline
tabulation interpolates its knots."""
from __future__ import annotations

import numpy as np

from epseon_backend_gb300 import synth


def test_seeded_and_reproducible():
    a = synth.mixed_batch(B=60)
    b = synth.mixed_batch(B=60)
    assert np.array_equal(a.N, b.N) and np.array_equal(a.mu, b.mu) and np.array_equal(a.kind, b.kind)
    c = synth.mixed_batch(B=60, seed=103)
    assert not np.array_equal(a.mu, c.mu)


def test_ranges():
    b = synth.mixed_batch()
    assert len(b) == 2048
    assert b.N.min() >= 2048 and b.N.max() <= 65536
    assert b.mu.min() >= 500 and b.mu.max() <= 1e5
    counts = np.bincount(b.kind, minlength=3)
    assert np.all(np.abs(counts - 2048 / 3) <= 1)
    mb = synth.morse_batch()
    assert np.all((mb.morse[:, 0] >= 0.02) & (mb.morse[:, 0] <= 0.2))
    assert np.allclose(mb.r_max, mb.morse[:, 2] + 30.0 / mb.morse[:, 1])


def test_spline_interpolates_knots_and_is_smooth():
    b = synth.mixed_batch(B=30, n_min=4097, n_max=4097)
    for i in np.where(b.kind == synth.KIND_SPLINE)[0][:3]:
        rk, yk = synth.knot_values(b, i)
        hk = rk[1] - rk[0]
        M = synth.natural_spline_second_derivs(yk, hk)
        y = synth.spline_eval(rk, rk[0], hk, yk, M)
        assert np.max(np.abs(y - yk)) < 1e-12 * max(1.0, np.abs(yk).max())
        assert M[0] == 0.0 and M[-1] == 0.0


def test_analytic_morse_levels():
    E = synth.analytic_morse_levels(0.1, 1.0, 1000.0, 0.0999)
    assert E.size == 14 and np.all(np.diff(E) > 0)
