"""Index arithmetic of the bisection scan (CPU restatement, no GPU).

The fast method's large-batch scan takes counts at every kBisectCoarse-th
trial energy (and the last), then in one round inside the coarse cells whose
end counts differ (scan.cu: bisect_plan_kernel): a cell with two or more
levels is cut into kBisectSplit parts (a count at every trial energy inside
it), a cell with exactly one level into kBisectSingle parts.  The bracket
kernel (prepare.cu: bracket_kernel) then descends the cell's halves while
their midpoints have a count; the level's bracket is the last cell it
reached.  This file restates both in Python and checks, on monotone count
sequences with clustered and degenerate levels and on awkward trial counts,
that the descent reads only counts the round took, that its bracket holds
the level alone when it is wider than one trial spacing, and that it is the
full scan's one-spacing bracket wherever a cell holds more than one level.
"""
from __future__ import annotations

import numpy as np
import pytest

COARSE = 16  # kBisectCoarse
SPLIT = 16  # kBisectSplit
SINGLE = 4  # kBisectSingle


def rounds(full: np.ndarray, single: int = SINGLE) -> np.ndarray:
    """Counts the bisection scan takes (-1 where it takes none)."""
    n_trial = full.size
    last = n_trial - 1
    c = -np.ones(n_trial, np.int64)
    K = (n_trial + COARSE - 1) // COARSE
    for k in range(1, K + 1):  # the strided scan32 launch
        j = min(k * COARSE - 1, last)
        c[j] = full[j]
    pts = []
    for t in range((n_trial + COARSE - 1) // COARSE):  # the plan of the round
        a = t * COARSE - 1
        ca = 0 if a < 0 else c[a]
        cb = c[min(a + COARSE, last)]
        parts = min(single, SPLIT) if cb - ca == 1 else SPLIT
        if ca >= 0 and cb > ca:
            for q in range(1, parts):
                pt = a + q * (COARSE // parts)
                if pt < last:
                    pts.append(pt)
    for p in pts:  # the count round
        c[p] = full[p]
    return c


def descend(c: np.ndarray, v: int) -> tuple[int, int]:
    """The level's bracket (lo, top) of trial indices: E_{lo-1} < E_v <= E_top
    (lo = n_trial: no level v), reading c as the bracket kernel does."""
    n_trial = c.size
    last = n_trial - 1
    ctop = c[last]
    assert ctop >= 0
    if v >= ctop:
        return n_trial, n_trial
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
        if x < 0:
            break  # no count taken there: the bracket is (a, a + W]
        if x <= v:
            a = mid
        W //= 2
    lo = min(a + 1, last)
    top = max(min(a + W, last), lo)
    # the bracket's end counts are taken
    assert c[top] >= 0 and (lo == 0 or c[lo - 1] >= 0)
    return lo, top


def full_search(full: np.ndarray, v: int) -> int:
    return int(np.searchsorted(full, v, side="right"))


def check_brackets(full: np.ndarray, c: np.ndarray, single: int = SINGLE) -> None:
    n_trial = full.size
    for v in range(int(full[-1]) + 2):
        j = full_search(full, v)
        lo, top = descend(c, v)
        if j >= n_trial:
            assert lo == n_trial
            continue
        assert lo <= j <= top, (n_trial, v, lo, j, top)
        assert top - lo + 1 <= max(1, COARSE // single)
        n_in = int(c[top] - (0 if lo == 0 else c[lo - 1]))
        if top > lo:
            assert n_in == 1  # a bracket wider than one spacing holds its level alone
        else:
            assert lo == j  # the full scan's bracket


@pytest.mark.parametrize("n_trial", [1, 2, 7, 8, 9, 63, 64, 65, 1000, 1024, 8191, 8192])
@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("single", [1, 2, 4, 8, 16])
def test_descent_brackets_every_level(n_trial, seed, single):
    rng = np.random.default_rng(seed + 31 * n_trial)
    n_levels = int(rng.integers(0, 3 * n_trial // 2 + 3))
    # level energies in trial units: uniform, plus a dense cluster and
    # degenerate pairs (several levels inside one trial spacing)
    x = rng.uniform(-0.5, n_trial + 0.5, n_levels)
    if n_levels > 4:
        x[: n_levels // 4] = rng.uniform(0.3 * n_trial, 0.3 * n_trial + 2, n_levels // 4)
        x[n_levels // 4 : n_levels // 4 + 2] = x[0]
    full = np.array([int(np.sum(x < j + 1)) for j in range(n_trial)], np.int64)  # count below E_j
    c = rounds(full, single)
    check_brackets(full, c, single)
    if single == SPLIT:  # every cell with a level cut to single spacings: the full scan's brackets
        for v in range(int(full[-1])):
            assert descend(c, v)[0] == full_search(full, v)
    taken = int(np.sum(c >= 0))
    if n_trial >= 1024 and full[-1] < n_trial // 16:
        assert taken < n_trial // 3  # far fewer counts than the full scan


def test_counts_taken_on_a_mixed_batch_spectrum():
    """A Morse-like ladder over 8192 trial energies (levels 60 or more trial
    spacings apart, each alone in its coarse cell): the round takes
    kBisectSingle - 1 counts per level instead of kBisectSplit - 1."""
    n_trial = 8192
    E = np.cumsum(np.linspace(400, 60, 45))  # a Morse-like ladder in trial units
    full = np.array([int(np.sum(E < j + 1)) for j in range(n_trial)], np.int64)
    n_lev = int(full[-1])
    coarse = (n_trial + COARSE - 1) // COARSE
    c = rounds(full)
    assert np.sum(c >= 0) == coarse + n_lev * (SINGLE - 1)
    check_brackets(full, c)
    assert np.sum(rounds(full, SPLIT) >= 0) == coarse + n_lev * (SPLIT - 1)


def test_descent_on_oracle_counts():
    """The FP64 oracle's scan counts of real potentials (Morse, LJ, bumps):
    every level's bracket holds it (alone, when wider than one spacing)."""
    from epseon_backend_gb300 import synth
    from oracle import oracle as O

    b = synth.mixed_batch(B=6, n_min=2048, n_max=4096, n_trial=1000, seed=13)
    Vs = [b.V(i) for i in range(len(b))]
    refs = O.solve_batch(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)
    for ref in refs:
        full = np.asarray(ref.counts, np.int64)
        assert full.size == b.n_trial and np.all(np.diff(full) >= 0)
        for single in (1, 2, 8):
            check_brackets(full, rounds(full, single), single)
