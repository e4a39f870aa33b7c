"""torch.autograd.Function wrappers over the CUDA solver and its adjoint.

This is the only place PyTorch touches the product path; the forward solve
and the backward (Hellmann-Feynman) pass are the libepseon_cuda kernels,
called through the C ABI on the tensors' device memory and the current
stream.

* ``LevelEnergies`` -- V (concatenated grids, float64, cuda) -> level
  energies [n_potentials, capacity]; backward: dL/dV_i = sum_v dL/dE_v
  psi_v(r_i)^2 h, exact for the discrete problem.
* ``tabulate`` -- parameters -> V on the device (epscu_tabulate); backward is
  the analytic derivative of the Morse / Lennard-Jones forms and, for
  Morse+bump potentials, the transpose of the natural-cubic-spline map from
  knots to grid (S^T) followed by the knot-level derivatives.
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


class Solver:
    """Owns an epscu context and the device outputs of the last solve."""

    def __init__(self, device: int | None = None):
        dev = torch.cuda.current_device() if device is None else device
        self.ctx = capi.Context(dev)

    def solve(self, V: torch.Tensor, g: Grids):
        assert V.is_cuda and V.dtype == torch.float64 and V.is_contiguous()
        n, cap = int(g.N.size), int(g.capacity)
        dev = V.device
        self.n_total = torch.zeros(n, dtype=torch.int32, device=dev)
        self.n_out = torch.zeros(n, dtype=torch.int32, device=dev)
        E = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        nodes = torch.zeros((n, cap), dtype=torch.int32, device=dev)
        status = torch.zeros((n, cap), dtype=torch.int32, device=dev)
        err = torch.zeros((n, cap), dtype=torch.float64, device=dev)
        psi = torch.empty(g.total * cap, dtype=torch.float64, device=dev)
        keep = [np.ascontiguousarray(x) for x in (g.offsets, g.N.astype(np.int32), g.r_min, g.r_max, g.mu, g.e_cap)]
        off, N, r0, r1, mu, ec = keep
        psi_off = np.zeros(n, np.int64)

        def p(t, ty):
            return C.cast(C.c_void_p(t.data_ptr()), ty)

        b = capi.Batch(n, p(V, capi._dp), capi._l(off), capi._i(N), capi._d(r0), capi._d(r1), capi._d(mu),
                       capi._d(ec), int(g.n_trial), 0, -1)
        r = capi.Result(cap, p(self.n_total, capi._ip), p(self.n_out, capi._ip), p(E, capi._dp),
                        p(nodes, capi._ip), p(status, capi._ip), p(err, capi._dp), p(psi, capi._dp),
                        int(psi.numel()), capi._l(psi_off), 0)
        o = capi.Opts(int(g.method), capi.MEM_DEVICE | capi.WANT_PSI, 1e-12,
                      C.c_void_p(torch.cuda.current_stream(dev).cuda_stream), 0, 0)
        capi._check(self.ctx._lib.epscu_solve(self.ctx.handle, C.byref(b), C.byref(r), C.byref(o)))
        mask = torch.arange(cap, device=dev)[None, :] < self.n_out[:, None].long()
        E = torch.where(mask, E, torch.zeros_like(E))
        # everything the adjoint of this solve needs, independent of later solves
        self.last = SolveRecord(g, psi, psi_off.copy(), self.n_out.cpu().numpy().astype(np.int32))
        return E, nodes, status, mask

    def adjoint(self, gE: torch.Tensor, rec: "SolveRecord | None" = None) -> torch.Tensor:
        """dL/dV of a recorded solve (default: this solver's last one)."""
        rec = rec or self.last
        g = rec.grids
        gE = gE.to(torch.float64).contiguous()
        gV = torch.zeros(g.total, dtype=torch.float64, device=gE.device)
        keep = [np.ascontiguousarray(x) for x in (g.offsets, g.N.astype(np.int32), g.r_min, g.r_max, rec.n_out,
                                                   rec.psi_offsets)]
        off, N, r0, r1, no, po = keep
        o = capi.Opts(0, capi.MEM_DEVICE, 0.0, C.c_void_p(torch.cuda.current_stream(gE.device).cuda_stream), 0, 0)
        capi._check(self.ctx._lib.epscu_adjoint_psi(
            self.ctx.handle, int(N.size), capi._l(off), capi._i(N), capi._d(r0), capi._d(r1), capi._i(no),
            int(g.capacity), C.cast(C.c_void_p(rec.psi.data_ptr()), capi._dp), capi._l(po),
            C.cast(C.c_void_p(gE.data_ptr()), capi._dp), C.cast(C.c_void_p(gV.data_ptr()), capi._dp), C.byref(o)))
        return gV


@dataclass
class SolveRecord:
    """Wavefunctions and layout of one solve (kept by autograd for its backward)."""

    grids: Grids
    psi: torch.Tensor
    psi_offsets: np.ndarray
    n_out: np.ndarray


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


def _spline_transpose_factory(n_knots: int, device):
    """Dense inverse of the natural-spline system tridiag(1, 4, 1) (K-2)^2."""
    m = n_knots - 2
    A = torch.diag(torch.full((m,), 4.0, dtype=torch.float64))
    A += torch.diag(torch.ones(m - 1, dtype=torch.float64), 1) + torch.diag(torch.ones(m - 1, dtype=torch.float64), -1)
    return torch.linalg.inv(A).to(device)


class Tabulate(torch.autograd.Function):
    """V = tabulate(params) on the device; analytic backward."""

    @staticmethod
    def forward(ctx, params: torch.Tensor, kind: np.ndarray, grids: Grids, n_knots: int, solver: Solver):
        P = params.detach().to(torch.float64).contiguous()
        n = int(grids.N.size)
        V = torch.zeros(grids.total, dtype=torch.float64, device=P.device)
        keep = [np.ascontiguousarray(x) for x in (kind.astype(np.int32), grids.offsets, grids.N.astype(np.int32),
                                                   grids.r_min, grids.r_max)]
        k, off, N, r0, r1 = keep
        o = capi.Opts(0, capi.MEM_DEVICE, 0.0, C.c_void_p(torch.cuda.current_stream(P.device).cuda_stream), 0, 0)
        capi._check(solver.ctx._lib.epscu_tabulate(
            solver.ctx.handle, n, capi._i(k), C.cast(C.c_void_p(P.data_ptr()), capi._dp), capi._l(off),
            capi._i(N), capi._d(r0), capi._d(r1), int(n_knots), C.cast(C.c_void_p(V.data_ptr()), capi._dp),
            C.byref(o)))
        ctx.save_for_backward(P)
        ctx.kind, ctx.grids, ctx.n_knots = kind, grids, n_knots
        return V

    @staticmethod
    def backward(ctx, gV):
        (P,) = ctx.saved_tensors
        grids, kind, K = ctx.grids, ctx.kind, ctx.n_knots
        dev = P.device
        gP = torch.zeros_like(P)
        off = grids.offsets
        Ainv = None
        for p in range(int(grids.N.size)):
            Np = int(grids.N[p])
            g = gV[int(off[p]): int(off[p]) + Np]
            r = grids.r_min[p] + torch.arange(Np, dtype=torch.float64, device=dev) * (
                (grids.r_max[p] - grids.r_min[p]) / (Np - 1))
            if int(kind[p]) == KIND_LJ:
                eps, sig = P[p, 0], P[p, 1]
                s6 = (sig / r) ** 6
                gP[p, 0] = torch.sum(g * (4.0 * (s6 * s6 - s6) + 1.0))
                gP[p, 1] = torch.sum(g * 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6) / sig)
                continue
            if int(kind[p]) == KIND_MORSE:
                gy, rk = g, r
            else:
                # g at the knots: S^T g for the natural cubic spline on K uniform knots
                if Ainv is None:
                    Ainv = _spline_transpose_factory(K, dev)
                hk = (grids.r_max[p] - grids.r_min[p]) / (K - 1)
                t = (r - grids.r_min[p]) / hk
                j = torch.clamp(torch.floor(t).long(), 0, K - 2)
                u = t - j
                w = 1.0 - u
                gy = torch.zeros(K, dtype=torch.float64, device=dev)
                gy.index_add_(0, j, g * w)
                gy.index_add_(0, j + 1, g * u)
                gM = torch.zeros(K, dtype=torch.float64, device=dev)
                h2 = hk * hk / 6.0
                gM.index_add_(0, j, g * h2 * (w ** 3 - w))
                gM.index_add_(0, j + 1, g * h2 * (u ** 3 - u))
                # M_int = Ainv @ (6/hk^2) D2 y  ->  gy += D2^T (6/hk^2) Ainv^T gM_int
                z = Ainv.T @ gM[1:-1] * (6.0 / (hk * hk))
                gy[:-2] += z
                gy[1:-1] -= 2.0 * z
                gy[2:] += z
                rk = grids.r_min[p] + torch.arange(K, dtype=torch.float64, device=dev) * hk
            De, a, re = P[p, 0], P[p, 1], P[p, 2]
            ex = torch.exp(-a * (rk - re))
            x = 1.0 - ex
            gP[p, 0] = torch.sum(gy * x * x)
            gP[p, 1] = torch.sum(gy * 2.0 * De * x * ex * (rk - re))
            gP[p, 2] = torch.sum(gy * -2.0 * De * x * ex * a)
            if int(kind[p]) == KIND_SPLINE:
                for q in range(3):
                    amp, wd, c = P[p, 3 + 3 * q], P[p, 4 + 3 * q], P[p, 5 + 3 * q]
                    gauss = torch.exp(-((rk - c) ** 2) / (2.0 * wd * wd))
                    gP[p, 3 + 3 * q] = torch.sum(gy * gauss)
                    gP[p, 4 + 3 * q] = torch.sum(gy * amp * gauss * (rk - c) ** 2 / wd ** 3)
                    gP[p, 5 + 3 * q] = torch.sum(gy * amp * gauss * (rk - c) / (wd * wd))
        return gP, None, None, None, None


def tabulate(params: torch.Tensor, kind: np.ndarray, grids: Grids, n_knots: int = 1024,
             solver: Solver | None = None) -> torch.Tensor:
    """Differentiable device tabulation of [n, 12] parameter rows (see epscu_tabulate)."""
    return Tabulate.apply(params, kind, grids, n_knots, solver or Solver(params.device.index))
