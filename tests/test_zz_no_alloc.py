"""epscu_count_levels_static: level counting for callers that cannot allocate
device memory (plugins inside another framework's memory pool or allocation
budget).  It runs the same trial-energy scan as epscu_solve on scratch held in
a static __device__ array of the library; here its counts are checked, through
the C ABI, against the bound levels epscu_solve returns for the same
potentials, on two calls in a row (the shared scratch is reused), at the
largest grid it accepts, with the device's free memory unchanged across a
call, and with inputs that fail on the device (every count -1).

This file is named to be collected last: a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# trial energies this close to a level may be counted on either side by the
# FP32 scan (its counts are reliable to ~1e-9 Hartree)
NEAR = 1e-8


def _ptr(t, ty):
    return C.cast(C.c_void_p(t.data_ptr()), ty)


def _expected(ctx, V, r_min, r_max, mu, e_cap, n_trial):
    from epseon_backend_gb300 import capi

    sol = ctx.solve([V], r_min, r_max, mu, e_cap, n_trial, method=capi.METHOD_PLAIN_FP64, level_capacity=1024)
    n = int(sol.n_out[0])
    assert n == int(sol.n_total[0])
    E = sol.energy[0, :n]
    e_lo = V.min()
    Ej = e_lo + (np.arange(n_trial) + 1) * ((e_cap - e_lo) / n_trial)
    near = np.zeros(n_trial, bool)
    if n:
        near = np.min(np.abs(Ej[:, None] - E[None, :]), axis=1) < NEAR
    return np.searchsorted(E, Ej), near, n


def _call(L, Vd, N, r_min, r_max, mu, e_cap, n_trial, counts, stream=None):
    from epseon_backend_gb300 import capi

    return L.epscu_count_levels_static(_ptr(Vd, capi._dp), int(N), float(r_min), float(r_max), float(mu),
                                       float(e_cap), int(n_trial), _ptr(counts, capi._ip), stream)


def test_static_counts_match_solve_twice():
    import torch

    from epseon_backend_gb300 import capi, synth

    L = capi.load()
    ctx = capi.Context(0)
    b = synth.mixed_batch(B=6, n_min=2048, n_max=8192, seed=21)
    n_trial = 2048
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for i in range(len(b)):
        V = np.ascontiguousarray(b.V(i))
        sol = ctx.solve([V], b.r_min[i], b.r_max[i], b.mu[i], b.e_cap[i], n_trial, method=capi.METHOD_PLAIN_FP64,
                        level_capacity=512)
        n = int(sol.n_out[0])
        assert n == int(sol.n_total[0])
        E = sol.energy[0, :n]
        e_lo = V.min()
        Ej = e_lo + (np.arange(n_trial) + 1) * ((b.e_cap[i] - e_lo) / n_trial)
        expect = np.searchsorted(E, Ej)  # levels below each trial energy
        near = np.zeros(n_trial, bool)
        if n:
            near = np.min(np.abs(Ej[:, None] - E[None, :]), axis=1) < NEAR
        Vd = torch.from_numpy(V).cuda()
        counts = torch.empty(n_trial, dtype=torch.int32, device="cuda")
        for call in range(2):
            counts.fill_(-1)
            rc = L.epscu_count_levels_static(_ptr(Vd, capi._dp), V.size, float(b.r_min[i]), float(b.r_max[i]),
                                             float(b.mu[i]), float(b.e_cap[i]), n_trial, _ptr(counts, capi._ip),
                                             stream)
            assert rc == capi.EPSCU_OK, L.epscu_last_error()
            torch.cuda.synchronize()
            c = counts.cpu().numpy()
            assert np.all((c == expect) | near), (i, call, np.where((c != expect) & ~near)[0][:5])
            assert c[-1] == n


def test_static_rejects_oversized_grid():
    import torch

    from epseon_backend_gb300 import capi

    L = capi.load()
    V = torch.zeros(65537, dtype=torch.float64, device="cuda")
    counts = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = L.epscu_count_levels_static(_ptr(V, capi._dp), V.numel(), 0.5, 10.0, 1000.0, 0.1, 16,
                                     _ptr(counts, capi._ip), None)
    assert rc == capi.ERR_CAPACITY
    assert b"exceeds the static scratch" in L.epscu_last_error()


def test_static_largest_grid_and_no_allocation():
    """N = 65536, the largest grid the scratch holds (the last 2048-point TMA
    tile ends exactly at the end of the scratch), compared with epscu_solve;
    the device's free memory is the same before and after a call."""
    import torch

    from epseon_backend_gb300 import capi, synth

    L = capi.load()
    ctx = capi.Context(0)
    b = synth.morse_batch(B=2, N=65536, seed=7)
    n_trial = 4096
    V = np.ascontiguousarray(b.V(1))
    assert V.size == 65536
    expect, near, n = _expected(ctx, V, b.r_min[1], b.r_max[1], b.mu[1], b.e_cap[1], n_trial)
    Vd = torch.from_numpy(V).cuda()
    counts = torch.full((n_trial,), -7, dtype=torch.int32, device="cuda")
    assert _call(L, Vd, V.size, b.r_min[1], b.r_max[1], b.mu[1], b.e_cap[1], n_trial, counts) == capi.EPSCU_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    reserved0 = torch.cuda.memory_reserved()
    counts.fill_(-7)
    assert _call(L, Vd, V.size, b.r_min[1], b.r_max[1], b.mu[1], b.e_cap[1], n_trial, counts) == capi.EPSCU_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0
    c = counts.cpu().numpy()
    assert np.all((c == expect) | near), np.where((c != expect) & ~near)[0][:5]
    assert c[-1] == n
    ctx.close()


def test_static_device_failures_give_minus_one():
    """Failures the host cannot see before the call returns (a NaN in the
    potential, an energy cap below the potential's minimum) set every count
    to EPSCU_STATIC_FAILED (-1); the next call with a good potential on the
    same scratch is correct again."""
    import torch

    from epseon_backend_gb300 import capi, synth

    L = capi.load()
    ctx = capi.Context(0)
    b = synth.morse_batch(B=1, N=8192, seed=3)
    V = np.ascontiguousarray(b.V(0))
    n_trial = 1024
    counts = torch.zeros(n_trial, dtype=torch.int32, device="cuda")
    bad = V.copy()
    bad[4000] = np.nan
    cases = [(bad, b.e_cap[0]), (V, V.min() - 1e-3)]
    for Vx, e_cap in cases:
        Vd = torch.from_numpy(Vx).cuda()
        counts.fill_(5)
        assert _call(L, Vd, Vx.size, b.r_min[0], b.r_max[0], b.mu[0], e_cap, n_trial, counts) == capi.EPSCU_OK
        torch.cuda.synchronize()
        assert np.all(counts.cpu().numpy() == -1)
    expect, near, n = _expected(ctx, V, b.r_min[0], b.r_max[0], b.mu[0], b.e_cap[0], n_trial)
    Vd = torch.from_numpy(V).cuda()
    assert _call(L, Vd, V.size, b.r_min[0], b.r_max[0], b.mu[0], b.e_cap[0], n_trial, counts) == capi.EPSCU_OK
    torch.cuda.synchronize()
    c = counts.cpu().numpy()
    assert np.all((c == expect) | near) and c[-1] == n
    ctx.close()
