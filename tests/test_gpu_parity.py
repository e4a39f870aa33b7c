"""Parity of the CUDA solver (through the C ABI) with the FP64 oracle.

Tolerances (the reference CPU path's bars): node counts bit-exact; energies
within 1e-10 Hartree for both methods (the plain FP64 method is bit-exact
here, same arithmetic as the oracle; the FP32-compensated method measures
~6e-13 on the 2048-potential mixed batch); normalised wavefunctions within
1e-8 in L2 (sqrt(sum (psi - psi_ref)^2 h)).
"""
from __future__ import annotations

import numpy as np
import pytest

from epseon_backend_gb300 import capi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL_PLAIN = 1e-10
E_TOL_FAST = 1e-10
PSI_TOL = 1e-8


def _oracle(b, want_psi=False, idx=None):
    idx = range(len(b)) if idx is None else idx
    Vs = [b.V(i) for i in idx]
    sel = np.array(list(idx))
    return O.solve_batch(Vs, b.r_min[sel], b.r_max[sel], b.mu[sel], b.e_cap[sel], b.n_trial, want_psi=want_psi)


def _gpu(ctx, b, method, want_psi=False, idx=None, cap=512):
    idx = list(range(len(b))) if idx is None else list(idx)
    Vs = [b.V(i) for i in idx]
    sel = np.array(idx)
    return ctx.solve(Vs, b.r_min[sel], b.r_max[sel], b.mu[sel], b.e_cap[sel], b.n_trial, method=method,
                     want_psi=want_psi, level_capacity=cap)


def _psi_l2(a, b, h):
    return float(np.sqrt(np.sum((a - b) ** 2) * h))


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_morse_single(ctx, method):
    b = synth.morse_single()
    ref = _oracle(b, want_psi=True)[0]
    sol = _gpu(ctx, b, method, want_psi=True, cap=32)
    assert sol.n_total[0] == ref.n_total == 14
    n = sol.n_out[0]
    assert n == 14
    assert np.array_equal(sol.nodes[0, :n], np.arange(n))
    assert np.all(sol.status[0, :n] == 0)
    if method == capi.METHOD_PLAIN_FP64:
        # same arithmetic as the oracle: identical bits
        assert np.array_equal(sol.energy[0, :n], ref.energy)
    else:
        assert np.max(np.abs(sol.energy[0, :n] - ref.energy_polished)) < E_TOL_FAST
    h = ref.grid.h
    psi = sol.wavefunctions(0)
    for v in range(n):
        assert _psi_l2(psi[v], ref.psi[v], h) < PSI_TOL
        assert abs(np.sum(psi[v] ** 2) * h - 1.0) < 1e-12


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_morse_batch_subset(ctx, method):
    b = synth.morse_batch()
    idx = [0, 5, 17, 42]
    refs = _oracle(b, idx=idx)
    sol = _gpu(ctx, b, method, idx=idx)
    for q, ref in enumerate(refs):
        n = sol.n_out[q]
        assert sol.n_total[q] == ref.n_total
        assert n == ref.energy.size
        assert np.array_equal(sol.nodes[q, :n], np.arange(n))
        if method == capi.METHOD_PLAIN_FP64:
            assert np.array_equal(sol.energy[q, :n], ref.energy)
        else:
            assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < E_TOL_FAST


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_mixed_subset(ctx, method):
    b = synth.mixed_batch()
    # one of each kind, short grids so the oracle finishes in seconds
    idx = []
    for kind in (synth.KIND_MORSE, synth.KIND_LJ, synth.KIND_SPLINE):
        cand = np.where((b.kind == kind) & (b.N < 6000))[0]
        idx += list(cand[:2])
    bb = b.subset(idx)
    bb.n_trial = 2048
    refs = _oracle(bb)
    sol = _gpu(ctx, bb, method)
    for q, ref in enumerate(refs):
        n = sol.n_out[q]
        assert sol.n_total[q] == ref.n_total
        assert np.array_equal(sol.nodes[q, :n], np.arange(n))
        if method == capi.METHOD_PLAIN_FP64:
            assert np.array_equal(sol.energy[q, :n], ref.energy)
        else:
            assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < E_TOL_FAST


def test_tabulate_matches_host(ctx):
    b = synth.mixed_batch(B=12, n_min=2048, n_max=8192)
    Vd = ctx.tabulate(b.kind, capi.batch_params(b), b.N, b.r_min, b.r_max)
    for i in range(len(b)):
        Vh = b.V(i)
        scale = np.maximum(1.0, np.abs(Vh))
        assert np.max(np.abs(Vd[i] - Vh) / scale) < 1e-11


def test_adjoint_matches_finite_differences(ctx):
    b = synth.morse_single(N=2048, n_trial=512)
    V = b.V(0).copy()
    sol = ctx.solve([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_PLAIN_FP64,
                    want_psi=True, level_capacity=16)
    n = sol.n_out[0]
    rng = np.random.default_rng(0)
    w = rng.uniform(0.5, 1.0, n)
    gE = np.zeros((1, 16))
    gE[0, :n] = w
    gV = ctx.adjoint(gE, V.size)
    g = O.grid(V, b.r_min[0], b.r_max[0], b.mu[0], b.e_cap[0], b.n_trial)
    for i in [g.i0 + 200, 300, 500, 700]:
        hfd = 1e-6
        Vp, Vm = V.copy(), V.copy()
        Vp[i] += hfd
        Vm[i] -= hfd
        rp = O.solve_batch([Vp], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)[0]
        rm = O.solve_batch([Vm], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)[0]
        fd = np.sum(w * (rp.energy_polished - rm.energy_polished)) / (2 * hfd)
        assert abs(gV[i] - fd) <= 1e-6 * max(abs(fd), 1e-3)


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_adjoint_recompute_equals_stored(ctx, method):
    """The adjoint with psi recomputed (nothing stored by the solve) equals the
    adjoint on the stored wavefunctions, for both methods."""
    b = synth.mixed_batch(B=9, n_min=2048, n_max=6000)
    b.n_trial = 2048
    Vs = b.potentials()
    cap = 256
    s1 = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=method, want_psi=True, level_capacity=cap)
    rng = np.random.default_rng(5)
    gE = rng.uniform(0.5, 1.0, (len(b), cap)) * (np.arange(cap)[None, :] < s1.n_out[:, None])
    total = int(sum(v.size for v in Vs))
    g_stored = ctx.adjoint(gE, total)
    s2 = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=method, level_capacity=cap)
    g_recomp = ctx.adjoint(gE, total, recompute=True)
    g_again = ctx.adjoint(gE, total, recompute=True)
    assert np.array_equal(np.nan_to_num(s1.energy), np.nan_to_num(s2.energy))
    scale = np.abs(g_stored).max()
    assert np.max(np.abs(g_recomp - g_stored)) <= 1e-12 * scale
    assert np.array_equal(g_recomp, g_again)
    # psi kept in device memory by a host-buffer solve (EPSCU_KEEP_PSI): the
    # adjoint needs no recompute and equals the one on the returned psi
    s3 = ctx.solve(capi.Concatenated(*capi.concat(Vs)), b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=method,
                   level_capacity=cap, keep_psi=True)
    assert np.array_equal(np.nan_to_num(s1.energy), np.nan_to_num(s3.energy))
    g_kept = ctx.adjoint(gE, total, recompute=False)
    assert np.max(np.abs(g_kept - g_stored)) <= 1e-12 * scale


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_bump_wavefunctions_all_levels(ctx, method):
    """Every level of Morse+bump potentials (double wells, near-degenerate
    pairs): energies, node counts and psi against the oracle."""
    b = synth.bump_adjoint(B=3, N=6144, n_trial=2048)
    refs = _oracle(b, want_psi=True)
    sol = _gpu(ctx, b, method, want_psi=True, cap=256)
    for q, ref in enumerate(refs):
        n = sol.n_out[q]
        assert n == ref.n_total
        assert np.array_equal(sol.nodes[q, :n], np.arange(n))
        tol = E_TOL_PLAIN if method == capi.METHOD_PLAIN_FP64 else E_TOL_FAST
        assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < tol
        psi = sol.wavefunctions(q)
        errs = [_psi_l2(psi[v], ref.psi[v], ref.grid.h) for v in range(n)]
        worst = int(np.argmax(errs))
        assert errs[worst] < PSI_TOL, (q, worst, errs[worst])


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_long_grid_top_levels(ctx, method):
    """Long grid (one heavy Morse, N = 2^20, ~280 bound levels): the lowest three
    levels (windows of ~4e4 points: one lane per level), a middle band and the
    ten highest (windows of 9e4 - 6.5e5 points: the fast method's CTA-per-level
    passes) against the oracle, with a reduced number of trial energies so the
    oracle finishes in seconds."""
    b = synth.morse_long(n_trial=4096)
    V = b.V(0)
    for lo, hi in ((0, 2), (100, 104), (270, 279)):
        ref = O.solve_batch([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, min_level=lo, max_level=hi,
                            want_psi=True)[0]
        assert ref.n_total == 280
        sol = ctx.solve([V], b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=method, min_level=lo,
                        max_level=hi, want_psi=True)
        n = sol.n_out[0]
        assert sol.n_total[0] == 280 and n == hi - lo + 1
        assert np.array_equal(sol.nodes[0, :n], np.arange(lo, hi + 1))
        tol = E_TOL_PLAIN if method == capi.METHOD_PLAIN_FP64 else E_TOL_FAST
        assert np.max(np.abs(sol.energy[0, :n] - ref.energy_polished)) < tol
        psi = sol.wavefunctions(0)
        for s in range(n):
            assert _psi_l2(psi[s], ref.psi[s], ref.grid.h) < PSI_TOL


def test_mixed_batch_path_with_psi(ctx):
    """The path the 2048-potential mixed batch takes, at its sizes: the first
    512 potentials of that batch (enough for the bisection scan: every 16th
    trial energy, then a count round inside the cells where the count
    changes), 8192 trial energies, grids of 2048 to
    65,536 points, long level windows on one CTA per level.  A seeded sample
    of 24 potentials, 8 of each kind (for each kind its three longest grids,
    so LJ and N > 32k are in it, and five drawn at random), is compared with
    the oracle: every level's energy (1e-10 Hartree), node count and
    normalised wavefunction (1e-8 in L2)."""
    full = synth.mixed_batch()
    b = full.subset(np.arange(512))
    assert b.n_trial == 8192 and len(b) >= 512
    rng = np.random.Generator(np.random.PCG64(17))
    sample = []
    for kind in (synth.KIND_MORSE, synth.KIND_LJ, synth.KIND_SPLINE):
        cand = np.where(b.kind == kind)[0]
        longest = cand[np.argsort(-b.N[cand])[:3]]
        rest = np.setdiff1d(cand, longest)
        sample += list(longest) + list(rng.choice(rest, 5, replace=False))
    sample = np.array(sorted(sample))
    assert np.any((b.kind[sample] == synth.KIND_LJ) & (b.N[sample] > 32768))
    Vs = b.potentials()
    args = (Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)
    probe = ctx.solve(*args, method=capi.METHOD_FAST_FP32C, level_capacity=512)
    sol = ctx.solve(*args, method=capi.METHOD_FAST_FP32C, level_capacity=512, want_psi=True,
                    psi_capacity=probe.psi_required)
    assert np.array_equal(sol.energy, probe.energy, equal_nan=True)
    refs = _oracle(b, want_psi=True, idx=sample)
    long_levels = 0
    for q, ref in zip(sample, refs):
        n = int(sol.n_out[q])
        assert sol.n_total[q] == ref.n_total and n == ref.energy.size, q
        assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < E_TOL_FAST, q
        if sol.status[q, 0] & capi.LEVEL_UNDER_RESOLVED:
            continue  # counts and energies exact; the shooting psi is not asserted
        assert np.array_equal(sol.nodes[q, :n], np.arange(n)), q
        psi = sol.wavefunctions(q)
        errs = np.array([_psi_l2(psi[v], ref.psi[v], ref.grid.h) for v in range(n)])
        assert errs.max() < PSI_TOL, (q, int(errs.argmax()), errs.max())
        long_levels += int(np.sum(np.count_nonzero(psi, axis=1) > 8192))
    assert long_levels > 0  # windows long enough for the CTA-per-level passes


def test_tabulate_adjoint_is_the_transpose(ctx):
    """epscu_tabulate_adjoint is the exact transpose of epscu_tabulate: for a
    random dL/dV and a random parameter direction d, <dL/dparams, d> equals
    the central difference of <dL/dV, V(params + t d)> (host FP64 tabulation;
    V is smooth in the parameters, so the difference with t = 1e-5 is exact to
    ~1e-9 relative).  Two calls give identical bits."""
    import ctypes as C

    b = synth.mixed_batch(B=15, n_min=2048, n_max=9000, seed=13)
    P = capi.batch_params(b)
    n = len(b)
    N = b.N.astype(np.int32)
    off = np.zeros(n, np.int64)
    off[1:] = np.cumsum(N[:-1].astype(np.int64))
    rng = np.random.default_rng(2)
    gV = rng.standard_normal(int(N.sum()))
    kind = b.kind.astype(np.int32)
    r0, r1 = np.ascontiguousarray(b.r_min), np.ascontiguousarray(b.r_max)

    def adj():
        gP = np.zeros((n, 12))
        o = capi.Opts(0, 0, 0.0, None, 0, 0)
        capi._check(capi.load().epscu_tabulate_adjoint(ctx.handle, n, capi._i(kind), capi._d(P), capi._l(off),
                                                       capi._i(N), capi._d(r0), capi._d(r1), 1024, capi._d(gV),
                                                       capi._d(gP), C.byref(o)))
        return gP

    gP = adj()
    assert np.array_equal(gP, adj())
    for i in range(n):
        g = gV[off[i]: off[i] + N[i]]
        active = np.array([0, 1]) if b.kind[i] == synth.KIND_LJ else np.array([0, 1, 2])
        if b.kind[i] == synth.KIND_SPLINE:
            active = np.concatenate([active, [3 + c for c in range(9) if P[i, 3 + 3 * (c // 3)] != 0.0]])
        assert np.all(gP[i, np.setdiff1d(np.arange(12), active)] == 0.0)
        d = np.zeros(12)
        d[active] = rng.uniform(0.5, 1.5, active.size) * np.maximum(np.abs(P[i, active]), 1e-2)
        t = 1e-5

        def f(s):
            return float(g @ synth.tabulate_params(b.kind[i], P[i] + s * d, b.N[i], b.r_min[i], b.r_max[i]))

        fd = (f(t) - f(-t)) / (2 * t)
        an = float(gP[i] @ d)
        assert abs(an - fd) <= 1e-7 * max(abs(fd), np.abs(gP[i] * d).max()), (i, int(b.kind[i]), an, fd)
