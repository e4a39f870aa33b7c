"""Index arithmetic of the bisection scan (CPU restatement, no GPU).

The fast method's large-batch scan takes counts at every kBisectCoarse-th
trial energy (and the last), then, round by round, at the midpoints of the
cells of width W = kBisectCoarse, kBisectCoarse/2, ..., 2 whose end counts
differ (scan.cu: bisect_plan_kernel); the bracket kernel then descends the
same cells (prepare.cu: bracket_kernel).  This file restates both in Python
and checks, on monotone count sequences with clustered and degenerate levels
and on awkward trial counts, that the descent returns the bracket a binary
search over the full count array returns, reading only counts the rounds
took.
"""
from __future__ import annotations

import numpy as np
import pytest

COARSE = 8  # kBisectCoarse


def rounds(full: np.ndarray) -> np.ndarray:
    """Counts the bisection scan takes (-1 where it takes none)."""
    n_trial = full.size
    last = n_trial - 1
    c = -np.ones(n_trial, np.int64)
    K = (n_trial + COARSE - 1) // COARSE
    for k in range(1, K + 1):  # the strided scan32 launch
        j = min(k * COARSE - 1, last)
        c[j] = full[j]
    W = COARSE
    while W > 1:  # plan + count rounds
        mids = []
        for t in range((n_trial + W - 1) // W):
            a = t * W - 1
            ca = 0 if a < 0 else c[a]
            cb = c[min(a + W, last)]
            mid = a + W // 2
            if ca >= 0 and cb > ca and mid < last:
                mids.append(mid)
        for m in mids:
            c[m] = full[m]
        W //= 2
    return c


def descend(c: np.ndarray, v: int) -> int:
    """First trial index with a count above v (n_trial: none), reading c."""
    n_trial = c.size
    last = n_trial - 1
    ctop = c[last]
    assert ctop >= 0
    if v >= ctop:
        return n_trial
    K = (n_trial + COARSE - 1) // COARSE
    kl, kh = 1, K
    while kl < kh:
        km = (kl + kh) // 2
        x = c[min(km * COARSE - 1, last)]
        assert x >= 0
        if x > v:
            kh = km
        else:
            kl = km + 1
    a = (kl - 1) * COARSE - 1
    W = COARSE
    while W > 1:
        mid = a + W // 2
        x = ctop if mid >= last else c[mid]
        assert x >= 0, "the descent read a count the rounds did not take"
        if x <= v:
            a = mid
        W //= 2
    lo = min(a + 1, last)
    # the bracket's end counts are taken too
    assert c[lo] >= 0 and (lo == 0 or c[lo - 1] >= 0)
    return lo


def full_search(full: np.ndarray, v: int) -> int:
    return int(np.searchsorted(full, v, side="right"))


@pytest.mark.parametrize("n_trial", [1, 2, 7, 8, 9, 63, 64, 65, 1000, 1024, 8191, 8192])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_descent_matches_full_scan(n_trial, seed):
    rng = np.random.default_rng(seed + 31 * n_trial)
    n_levels = int(rng.integers(0, 3 * n_trial // 2 + 3))
    # level energies in trial units: uniform, plus a dense cluster and
    # degenerate pairs (several levels inside one trial spacing)
    x = rng.uniform(-0.5, n_trial + 0.5, n_levels)
    if n_levels > 4:
        x[: n_levels // 4] = rng.uniform(0.3 * n_trial, 0.3 * n_trial + 2, n_levels // 4)
        x[n_levels // 4 : n_levels // 4 + 2] = x[0]
    full = np.array([int(np.sum(x < j + 1)) for j in range(n_trial)], np.int64)  # count below E_j
    c = rounds(full)
    taken = int(np.sum(c >= 0))
    for v in range(int(full[-1]) + 2):
        assert descend(c, v) == full_search(full, v), (n_trial, v)
    if n_trial >= 1024 and full[-1] < n_trial // 16:
        assert taken < n_trial // 3  # far fewer counts than the full scan


def test_counts_taken_on_a_mixed_batch_spectrum():
    """~45 levels over 8192 trial energies: the rounds take ~1/6 of the counts."""
    n_trial = 8192
    E = np.cumsum(np.linspace(400, 60, 45))  # a Morse-like ladder in trial units
    full = np.array([int(np.sum(E < j + 1)) for j in range(n_trial)], np.int64)
    c = rounds(full)
    assert np.sum(c >= 0) < n_trial // 6
    for v in range(int(full[-1])):
        assert descend(c, v) == full_search(full, v)


def test_descent_on_oracle_counts():
    """The FP64 oracle's scan counts of real potentials (Morse, LJ, bumps):
    the bisection rounds and the descent give the full scan's bracket of
    every level."""
    from epseon_backend_gb300 import synth
    from oracle import oracle as O

    b = synth.mixed_batch(B=6, n_min=2048, n_max=4096, n_trial=1000, seed=13)
    Vs = [b.V(i) for i in range(len(b))]
    refs = O.solve_batch(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)
    for ref in refs:
        full = np.asarray(ref.counts, np.int64)
        assert full.size == b.n_trial and np.all(np.diff(full) >= 0)
        c = rounds(full)
        for v in range(int(full[-1])):
            assert descend(c, v) == full_search(full, v)
