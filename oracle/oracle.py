"""ctypes front end of the FP64 CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` import this module, and only as the checker or the timed CPU
baseline.  The product path (``epseon_backend_gb300``) never does.

Parity with the reference is unpinned (the reference has no solver); the
oracle is pinned against the dense eigen-decomposition of the same
discretisation, analytic Morse levels, node counts and Hellmann-Feynman
derivatives (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

OK, MAXITER, NONFINITE, UNDER_RESOLVED, NOT_FOUND, BAD_INPUT = 0, 1, 2, 4, 16, 32


class Problem(C.Structure):
    _fields_ = [
        ("V", C.POINTER(C.c_double)),
        ("N", C.c_int32),
        ("r_min", C.c_double),
        ("r_max", C.c_double),
        ("mu", C.c_double),
        ("e_cap", C.c_double),
        ("n_trial", C.c_int32),
        ("min_level", C.c_int32),
        ("max_level", C.c_int32),
        ("tol", C.c_double),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("h", C.c_double),
        ("a", C.c_double),
        ("e_lo", C.c_double),
        ("delta", C.c_double),
        ("i0", C.c_int32),
        ("i1", C.c_int32),
        ("k_scan", C.c_int32),
        ("n_bisect", C.c_int32),
        ("N", C.c_int32),
    ]


class Result(C.Structure):
    _fields_ = [
        ("capacity", C.c_int32),
        ("n_total", C.c_int32),
        ("n_out", C.c_int32),
        ("status", C.c_int32),
        ("energy", C.POINTER(C.c_double)),
        ("energy_polished", C.POINTER(C.c_double)),
        ("nodes", C.POINTER(C.c_int32)),
        ("level_status", C.POINTER(C.c_int32)),
        ("psi", C.POINTER(C.c_double)),
        ("counts", C.POINTER(C.c_int32)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.eo_prepare.argtypes = [C.POINTER(Problem), C.POINTER(Grid)]
        L.eo_prepare.restype = C.c_int
        L.eo_count.argtypes = [C.POINTER(C.c_double), C.POINTER(Grid), C.c_double, C.c_int32]
        L.eo_count.restype = C.c_int32
        L.eo_match_index.argtypes = [C.POINTER(C.c_double), C.POINTER(Grid), C.c_double]
        L.eo_match_index.restype = C.c_int32
        L.eo_cooley_pass.argtypes = [
            C.POINTER(C.c_double),
            C.POINTER(Grid),
            C.c_double,
            C.POINTER(C.c_int32),
        ]
        L.eo_cooley_pass.restype = C.c_double
        L.eo_wavefunction.argtypes = [
            C.POINTER(C.c_double),
            C.POINTER(Grid),
            C.c_double,
            C.POINTER(C.c_double),
        ]
        L.eo_wavefunction.restype = None
        L.eo_scan.argtypes = [C.POINTER(C.c_double), C.POINTER(Grid), C.c_int32, C.POINTER(C.c_int32)]
        L.eo_scan.restype = None
        L.eo_solve_batch.argtypes = [C.POINTER(Problem), C.POINTER(Result), C.c_int32, C.c_int32]
        L.eo_solve_batch.restype = C.c_int
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@dataclass
class Solution:
    """Oracle results for one potential (levels min_level .. min_level+n_out-1)."""

    n_total: int
    status: int
    energy: np.ndarray  # bisection energies (the plain method)
    energy_polished: np.ndarray  # Cooley-polished FP64 energies
    nodes: np.ndarray
    level_status: np.ndarray
    psi: np.ndarray | None
    counts: np.ndarray
    grid: Grid


def make_problem(V: np.ndarray, r_min, r_max, mu, e_cap, n_trial, min_level=0, max_level=-1, tol=1e-12):
    V = np.ascontiguousarray(V, dtype=np.float64)
    p = Problem(_dptr(V), V.size, r_min, r_max, mu, e_cap, n_trial, min_level, max_level, tol)
    return p, V


def grid(V, r_min, r_max, mu, e_cap, n_trial=1024, tol=1e-12) -> Grid:
    p, _keep = make_problem(V, r_min, r_max, mu, e_cap, n_trial, tol=tol)
    g = Grid()
    st = lib().eo_prepare(C.byref(p), C.byref(g))
    if st:
        raise ValueError(f"eo_prepare failed with status {st}")
    return g


def count(V, g: Grid, E: float, k: int | None = None) -> int:
    V = np.ascontiguousarray(V, dtype=np.float64)
    return int(lib().eo_count(_dptr(V), C.byref(g), E, g.k_scan if k is None else k))


def cooley(V, g: Grid, E: float):
    V = np.ascontiguousarray(V, dtype=np.float64)
    n = C.c_int32()
    dE = lib().eo_cooley_pass(_dptr(V), C.byref(g), E, C.byref(n))
    return dE, n.value


def wavefunction(V, g: Grid, E: float) -> np.ndarray:
    V = np.ascontiguousarray(V, dtype=np.float64)
    out = np.zeros(V.size)
    lib().eo_wavefunction(_dptr(V), C.byref(g), E, _dptr(out))
    return out


def solve_batch(
    Vs,
    r_min,
    r_max,
    mu,
    e_cap,
    n_trial,
    min_level=0,
    max_level=-1,
    tol=1e-12,
    want_psi=False,
    capacity=None,
    n_threads=0,
):
    """Solve a batch of potentials; scalar parameters broadcast over the batch."""
    n = len(Vs)

    def arr(x, dt=np.float64):
        a = np.asarray(x, dtype=dt)
        return np.broadcast_to(a, (n,)).copy() if a.ndim == 0 else a.astype(dt)

    r_min, r_max, mu, e_cap = arr(r_min), arr(r_max), arr(mu), arr(e_cap)
    n_trial, min_level, max_level = arr(n_trial, np.int32), arr(min_level, np.int32), arr(max_level, np.int32)
    probs = (Problem * n)()
    res = (Result * n)()
    keep = []
    outs = []
    for i, V in enumerate(Vs):
        V = np.ascontiguousarray(V, dtype=np.float64)
        cap = int(capacity) if capacity is not None else max(1, int(n_trial[i]))
        if max_level[i] >= 0:
            cap = min(cap, int(max_level[i]) - int(min_level[i]) + 1)
        cap = max(cap, 1)
        e = np.full(cap, np.nan)
        ep = np.full(cap, np.nan)
        nd = np.full(cap, -1, np.int32)
        ls = np.zeros(cap, np.int32)
        cnt = np.zeros(int(n_trial[i]), np.int32)
        psi = np.zeros((cap, V.size)) if want_psi else None
        keep.append((V, e, ep, nd, ls, cnt, psi))
        probs[i] = Problem(
            _dptr(V), V.size, r_min[i], r_max[i], mu[i], e_cap[i], int(n_trial[i]), int(min_level[i]), int(max_level[i]), tol
        )
        res[i] = Result(
            cap, 0, 0, 0, _dptr(e), _dptr(ep), _iptr(nd), _iptr(ls), _dptr(psi) if psi is not None else None, _iptr(cnt)
        )
    lib().eo_solve_batch(probs, res, n, n_threads)
    for i in range(n):
        V, e, ep, nd, ls, cnt, psi = keep[i]
        m = res[i].n_out
        g = Grid()
        lib().eo_prepare(C.byref(probs[i]), C.byref(g))
        outs.append(
            Solution(
                res[i].n_total,
                res[i].status,
                e[:m].copy(),
                ep[:m].copy(),
                nd[:m].copy(),
                ls[:m].copy(),
                psi[:m].copy() if psi is not None else None,
                cnt,
                g,
            )
        )
    return outs


def n_threads_default() -> int:
    return os.cpu_count() or 1
