"""torch.autograd.Function wrappers over the CUDA solver and its adjoint.

This is the only place PyTorch touches the product path; the forward solve,
the backward (Hellmann-Feynman) pass and the parameter chain are
libepseon_cuda kernels, called through the C ABI on the tensors' device
memory and the current stream.

* ``LevelEnergies`` -- V (concatenated grids, float64, cuda) -> level
  energies [n_potentials, capacity]; backward: dL/dV_i = sum_v dL/dE_v
  psi_v(r_i)^2 h, exact for the discrete problem.  The wavefunctions are
  kept in a buffer of exactly the size the solve needs (the library reads the
  size back after its level set-up and asks for the buffer through
  epscu_opts.psi_alloc).  When that size is above the solver's memory budget
  the forward keeps no wavefunctions and the backward recomputes them: it
  re-solves the potentials in chunks whose wavefunctions fit the budget and
  applies the adjoint chunk by chunk (the adjoint of one potential needs only
  that potential's wavefunctions).
* ``tabulate`` -- parameters -> V on the device (epscu_tabulate); backward is
  epscu_tabulate_adjoint: the analytic derivatives of the Morse and
  Lennard-Jones forms and, for Morse+bump potentials, the transpose of the
  natural-cubic-spline map from knots to grid (S^T) followed by the
  knot-level derivatives, for the whole batch in one kernel.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import capi

KIND_MORSE, KIND_LJ, KIND_SPLINE = capi.KIND_MORSE, capi.KIND_LJ, capi.KIND_SPLINE


@dataclass
class Grids:
    """Host description of a ragged batch of uniform grids."""

    N: np.ndarray  # int32 [n]
    r_min: np.ndarray
    r_max: np.ndarray
    mu: np.ndarray
    e_cap: np.ndarray
    n_trial: int
    capacity: int = 512
    method: int = capi.METHOD_FAST_FP32C

    @property
    def offsets(self) -> np.ndarray:
        off = np.zeros(self.N.size, np.int64)
        off[1:] = np.cumsum(self.N[:-1].astype(np.int64))
        return off

    @property
    def total(self) -> int:
        return int(self.N.astype(np.int64).sum())

    def subset(self, idx: np.ndarray) -> "Grids":
        return Grids(self.N[idx].copy(), self.r_min[idx].copy(), self.r_max[idx].copy(), self.mu[idx].copy(),
                     self.e_cap[idx].copy(), self.n_trial, self.capacity, self.method)


def _ptr(t, ty):
    return C.cast(C.c_void_p(t.data_ptr()), ty)


class Solver:
    """Owns an epscu context and the wavefunction buffers of its solves.

    psi_budget_bytes: the most device memory one solve's wavefunctions may
    take (None: half of the device's free memory at the time of the solve).
    Above it the forward keeps none and the backward recomputes them in
    chunks that fit."""

    def __init__(self, device: int | None = None, psi_budget_bytes: int | None = None):
        dev = torch.cuda.current_device() if device is None else device
        self.ctx = capi.Context(dev)
        self.psi_budget_bytes = psi_budget_bytes

    def _budget(self, dev) -> int:
        if self.psi_budget_bytes is not None:
            return int(self.psi_budget_bytes)
        free, _ = torch.cuda.mem_get_info(dev)
        return int(free) // 2

    def _solve(self, V: torch.Tensor, g: Grids, budget: int):
        """One device solve; the wavefunctions in a tensor of exactly the
        size the solve needs, or None when that is above `budget` bytes."""
        n, cap = int(g.N.size), int(g.capacity)
        dev = V.device
        n_total = torch.zeros(n, dtype=torch.int32, device=dev)
        n_out = torch.zeros(n, dtype=torch.int32, device=dev)
        E = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        nodes = torch.zeros((n, cap), dtype=torch.int32, device=dev)
        status = torch.zeros((n, cap), dtype=torch.int32, device=dev)
        err = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        keep = [np.ascontiguousarray(x) for x in (g.offsets, g.N.astype(np.int32), g.r_min, g.r_max, g.mu, g.e_cap)]
        off, N, r0, r1, mu, ec = keep
        psi_off = np.zeros(n, np.int64)
        held = {}

        def alloc(nbytes, user):
            if nbytes > budget:
                return None  # too large: no wavefunctions kept
            try:
                t = torch.empty((int(nbytes) + 7) // 8, dtype=torch.float64, device=dev)
            except torch.OutOfMemoryError:
                return None
            held["psi"] = t
            return t.data_ptr()

        cb = capi.ALLOC_FN(alloc)
        b = capi.Batch(n, _ptr(V, capi._dp), capi._l(off), capi._i(N), capi._d(r0), capi._d(r1), capi._d(mu),
                       capi._d(ec), int(g.n_trial), 0, -1)
        r = capi.Result(cap, _ptr(n_total, capi._ip), _ptr(n_out, capi._ip), _ptr(E, capi._dp),
                        _ptr(nodes, capi._ip), _ptr(status, capi._ip), _ptr(err, capi._dp), None, 0,
                        capi._l(psi_off), 0)
        o = capi.Opts(int(g.method), capi.MEM_DEVICE | capi.WANT_PSI, 1e-12,
                      C.c_void_p(torch.cuda.current_stream(dev).cuda_stream), 0, 0, 0, 0, 0, cb, None)
        capi._check(self.ctx._lib.epscu_solve(self.ctx.handle, C.byref(b), C.byref(r), C.byref(o)))
        return E, nodes, status, n_out, held.get("psi"), psi_off, int(r.psi_required)

    def solve(self, V: torch.Tensor, g: Grids):
        assert V.is_cuda and V.dtype == torch.float64 and V.is_contiguous()
        cap = int(g.capacity)
        E, nodes, status, n_out, psi, psi_off, need = self._solve(V, g, self._budget(V.device))
        mask = torch.arange(cap, device=V.device)[None, :] < n_out[:, None].long()
        E = torch.where(mask, E, torch.zeros_like(E))
        # everything the adjoint of this solve needs, independent of later
        # solves: the wavefunctions, or the potentials to recompute them from
        self.last = SolveRecord(g, psi, psi_off.copy(), n_out.cpu().numpy().astype(np.int32),
                                V if psi is None else None, need)
        return E, nodes, status, mask

    def _adjoint_psi(self, g: Grids, n_out: np.ndarray, psi: torch.Tensor, psi_off: np.ndarray,
                     gE: torch.Tensor, gV: torch.Tensor):
        keep = [np.ascontiguousarray(x) for x in (g.offsets, g.N.astype(np.int32), g.r_min, g.r_max, n_out,
                                                   psi_off)]
        off, N, r0, r1, no, po = keep
        o = capi.Opts(0, capi.MEM_DEVICE, 0.0, C.c_void_p(torch.cuda.current_stream(gE.device).cuda_stream), 0, 0)
        capi._check(self.ctx._lib.epscu_adjoint_psi(
            self.ctx.handle, int(N.size), capi._l(off), capi._i(N), capi._d(r0), capi._d(r1), capi._i(no),
            int(g.capacity), _ptr(psi, capi._dp), capi._l(po), _ptr(gE, capi._dp), _ptr(gV, capi._dp),
            C.byref(o)))

    def adjoint(self, gE: torch.Tensor, rec: "SolveRecord | None" = None) -> torch.Tensor:
        """dL/dV of a recorded solve (default: this solver's last one)."""
        rec = rec or self.last
        g = rec.grids
        gE = gE.to(torch.float64).contiguous()
        gV = torch.zeros(g.total, dtype=torch.float64, device=gE.device)
        if rec.psi is not None:
            self._adjoint_psi(g, rec.n_out, rec.psi, rec.psi_offsets, gE, gV)
            return gV
        # recompute: potentials in chunks whose wavefunctions fit the budget
        budget = self._budget(gE.device)
        per = rec.n_out.astype(np.int64) * g.N.astype(np.int64) * 8
        off = g.offsets
        first = 0
        n = int(g.N.size)
        while first < n:
            last, used = first, 0
            while last < n and (last == first or used + per[last] <= budget):
                used += int(per[last])
                last += 1
            idx = np.arange(first, last)
            gc = g.subset(idx)
            a, z = int(off[first]), int(off[last - 1] + g.N[last - 1])
            Vc = rec.V[a:z]
            _, _, _, n_out_c, psi_c, psi_off_c, _ = self._solve(Vc, gc, max(budget, int(per[idx].sum())))
            n_out_c = n_out_c.cpu().numpy().astype(np.int32)
            if psi_c is None or not np.array_equal(n_out_c, rec.n_out[idx]):
                raise RuntimeError("wavefunction recompute failed for potentials %d..%d" % (first, last - 1))
            gVc = torch.zeros(z - a, dtype=torch.float64, device=gE.device)
            self._adjoint_psi(gc, n_out_c, psi_c, psi_off_c, gE[first:last].contiguous(), gVc)
            gV[a:z] = gVc
            del psi_c
            first = last
        return gV


@dataclass
class SolveRecord:
    """Wavefunctions and layout of one solve (kept by autograd for its
    backward), or the potentials to recompute them from."""

    grids: Grids
    psi: torch.Tensor | None
    psi_offsets: np.ndarray
    n_out: np.ndarray
    V: torch.Tensor | None = None
    psi_required: int = 0  # doubles the wavefunctions take


class LevelEnergies(torch.autograd.Function):
    """E = levels(V); dL/dV by the Hellmann-Feynman adjoint kernel."""

    @staticmethod
    def forward(ctx, V: torch.Tensor, grids: Grids, solver: Solver):
        E, nodes, status, mask = solver.solve(V.detach().contiguous(), grids)
        ctx.solver = solver
        ctx.record = solver.last
        ctx.mark_non_differentiable(mask)
        return E, mask

    @staticmethod
    def backward(ctx, gE, gmask):
        return ctx.solver.adjoint(gE, ctx.record), None, None


def levels(V: torch.Tensor, grids: Grids, solver: Solver | None = None):
    """Differentiable level energies [n, capacity] and the mask of valid slots."""
    return LevelEnergies.apply(V, grids, solver or Solver(V.device.index))


# ------------------------------------------------------------- tabulation


def _tab_args(kind: np.ndarray, grids: Grids):
    return [np.ascontiguousarray(x) for x in (kind.astype(np.int32), grids.offsets, grids.N.astype(np.int32),
                                               grids.r_min, grids.r_max)]


class Tabulate(torch.autograd.Function):
    """V = tabulate(params) on the device; backward by epscu_tabulate_adjoint."""

    @staticmethod
    def forward(ctx, params: torch.Tensor, kind: np.ndarray, grids: Grids, n_knots: int, solver: Solver):
        P = params.detach().to(torch.float64).contiguous()
        n = int(grids.N.size)
        V = torch.zeros(grids.total, dtype=torch.float64, device=P.device)
        k, off, N, r0, r1 = _tab_args(kind, grids)
        o = capi.Opts(0, capi.MEM_DEVICE, 0.0, C.c_void_p(torch.cuda.current_stream(P.device).cuda_stream), 0, 0)
        capi._check(solver.ctx._lib.epscu_tabulate(
            solver.ctx.handle, n, capi._i(k), _ptr(P, capi._dp), capi._l(off), capi._i(N), capi._d(r0),
            capi._d(r1), int(n_knots), _ptr(V, capi._dp), C.byref(o)))
        ctx.save_for_backward(P)
        ctx.kind, ctx.grids, ctx.n_knots, ctx.solver = kind, grids, n_knots, solver
        return V

    @staticmethod
    def backward(ctx, gV):
        (P,) = ctx.saved_tensors
        grids = ctx.grids
        n = int(grids.N.size)
        gV = gV.to(torch.float64).contiguous()
        gP = torch.zeros_like(P)
        k, off, N, r0, r1 = _tab_args(ctx.kind, grids)
        o = capi.Opts(0, capi.MEM_DEVICE, 0.0, C.c_void_p(torch.cuda.current_stream(P.device).cuda_stream), 0, 0)
        capi._check(ctx.solver.ctx._lib.epscu_tabulate_adjoint(
            ctx.solver.ctx.handle, n, capi._i(k), _ptr(P, capi._dp), capi._l(off), capi._i(N), capi._d(r0),
            capi._d(r1), int(ctx.n_knots), _ptr(gV, capi._dp), _ptr(gP, capi._dp), C.byref(o)))
        return gP, None, None, None, None


def tabulate(params: torch.Tensor, kind: np.ndarray, grids: Grids, n_knots: int = 1024,
             solver: Solver | None = None) -> torch.Tensor:
    """Differentiable device tabulation of [n, 12] parameter rows (see epscu_tabulate)."""
    return Tabulate.apply(params, kind, grids, n_knots, solver or Solver(params.device.index))
