"""ctypes binding of the libepseon_cuda C ABI (``include/epscu.h``).

This is the thin Python view of the same entry points a cgo/JNI/ctypes user
would bind; the parity tests call the solver through it.  There is no CPU
fallback: if the CUDA library is missing or no device is present, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _build

EPSCU_OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_CANCELLED, ERR_CAPACITY, ERR_TIMEOUT = 1, 2, 3, 4, 5, 6
LEVEL_OK, LEVEL_MAXITER, LEVEL_NONFINITE, LEVEL_UNDER_RESOLVED = 0, 1, 2, 4
LEVEL_CANCELLED, LEVEL_NOT_FOUND, LEVEL_BAD_INPUT = 8, 16, 32
METHOD_PLAIN_FP64, METHOD_FAST_FP32C = 0, 1
KIND_MORSE, KIND_LJ, KIND_SPLINE = 0, 1, 2
MEM_DEVICE, WANT_PSI, STAGE_TIMING, KEEP_PSI = 1, 2, 4, 8

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class Batch(C.Structure):
    _fields_ = [
        ("n_potentials", C.c_int32),
        ("V", _dp),
        ("offsets", _lp),
        ("N", _ip),
        ("r_min", _dp),
        ("r_max", _dp),
        ("mu", _dp),
        ("e_cap", _dp),
        ("n_trial", C.c_int32),
        ("min_level", C.c_int32),
        ("max_level", C.c_int32),
    ]


ALLOC_FN = C.CFUNCTYPE(C.c_void_p, C.c_int64, C.c_void_p)


class Opts(C.Structure):
    _fields_ = [
        ("method", C.c_int32),
        ("flags", C.c_int32),
        ("tol", C.c_double),
        ("stream", C.c_void_p),
        ("tune", C.c_int32),
        ("long_window", C.c_int32),
        ("wait_polls", C.c_int32),
        ("max_iter", C.c_int32),
        ("mid_window", C.c_int32),
        ("psi_alloc", ALLOC_FN),
        ("psi_alloc_user", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("level_capacity", C.c_int32),
        ("n_total", _ip),
        ("n_out", _ip),
        ("energy", _dp),
        ("nodes", _ip),
        ("status", _ip),
        ("err_est", _dp),
        ("psi", _dp),
        ("psi_capacity", C.c_int64),
        ("psi_offsets", _lp),
        ("psi_required", C.c_int64),
    ]


class DeviceInfo(C.Structure):
    _fields_ = [
        ("name", C.c_char * 256),
        ("ordinal", C.c_int32),
        ("pci_device_id", C.c_int32),
        ("pci_bus_id", C.c_int32),
        ("cc_major", C.c_int32),
        ("cc_minor", C.c_int32),
        ("sm_count", C.c_int32),
        ("total_global_mem", C.c_int64),
        ("shared_mem_per_block_optin", C.c_int32),
        ("max_threads_per_block", C.c_int32),
        ("max_grid_dim", C.c_int32 * 3),
        ("max_block_dim", C.c_int32 * 3),
        ("l2_cache_size", C.c_int32),
        ("driver_version", C.c_int32),
        ("runtime_version", C.c_int32),
        ("uuid", C.c_uint8 * 16),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("ms_prepare", C.c_float),
        ("ms_scan", C.c_float),
        ("ms_refine32", C.c_float),
        ("ms_polish64", C.c_float),
        ("ms_write", C.c_float),
        ("ms_total", C.c_float),
        ("scan_point_updates", C.c_int64),
        ("refine_point_updates", C.c_int64),
        ("fp64_point_updates", C.c_int64),
        ("psi_bytes", C.c_int64),
        ("n_levels", C.c_int64),
        ("kernel_launches", C.c_int32),
        ("fallbacks", C.c_int32),
        ("twist_searches", C.c_int32),
        ("norm_redos", C.c_int32),
        ("refine_max_level_updates", C.c_int64),
        ("df_max_level_updates", C.c_int64),
        ("refine_max_iters", C.c_int32),
        ("reserved", C.c_int32),
        ("ms_refine_long", C.c_float),
        ("reserved2", C.c_int32),
        ("long_fp32_point_updates", C.c_int64),
        ("long_df_point_updates", C.c_int64),
        ("ms_zero_psi", C.c_float),
        ("reserved3", C.c_int32),
        ("psi_zero_points", C.c_int64),
        ("psi_window_points", C.c_int64),
    ]


# every symbol the header declares (checked by the CPU test suite)
EXPORTED = [
    "epscu_abi_version",
    "epscu_device_count",
    "epscu_get_device_info",
    "epscu_last_error",
    "epscu_create",
    "epscu_destroy",
    "epscu_set_arena_block",
    "epscu_solve",
    "epscu_adjoint",
    "epscu_adjoint_psi",
    "epscu_tabulate",
    "epscu_tabulate_adjoint",
    "epscu_cancel",
    "epscu_cancel_clear",
    "epscu_last_stats",
    "epscu_measure_fma_peaks",
    "epscu_count_levels_static",
]

_lib = None


class EpscuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"epscu error {code}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libepseon_cuda.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError(f"{_build.LIB} is not built")
        _build.build_cuda()
    L = C.CDLL(_build.LIB)
    L.epscu_abi_version.restype = C.c_int32
    L.epscu_last_error.restype = C.c_char_p
    L.epscu_device_count.argtypes = [_ip]
    L.epscu_get_device_info.argtypes = [C.c_int32, C.POINTER(DeviceInfo)]
    L.epscu_create.argtypes = [C.c_int32, C.POINTER(C.c_void_p)]
    L.epscu_destroy.argtypes = [C.c_void_p]
    L.epscu_set_arena_block.argtypes = [C.c_void_p, C.c_int64]
    L.epscu_solve.argtypes = [C.c_void_p, C.POINTER(Batch), C.POINTER(Result), C.POINTER(Opts)]
    L.epscu_adjoint.argtypes = [C.c_void_p, _dp, _dp, C.c_int32, C.POINTER(Opts)]
    L.epscu_adjoint_psi.argtypes = [C.c_void_p, C.c_int32, _lp, _ip, _dp, _dp, _ip, C.c_int32, _dp, _lp, _dp, _dp,
                                    C.POINTER(Opts)]
    L.epscu_tabulate.argtypes = [C.c_void_p, C.c_int32, _ip, _dp, _lp, _ip, _dp, _dp, C.c_int32, _dp, C.POINTER(Opts)]
    L.epscu_tabulate_adjoint.argtypes = [C.c_void_p, C.c_int32, _ip, _dp, _lp, _ip, _dp, _dp, C.c_int32, _dp, _dp,
                                         C.POINTER(Opts)]
    L.epscu_cancel.argtypes = [C.c_void_p]
    L.epscu_cancel_clear.argtypes = [C.c_void_p]
    L.epscu_last_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.epscu_measure_fma_peaks.argtypes = [C.c_void_p, _dp, _dp]
    L.epscu_count_levels_static.argtypes = [_dp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_int32, _ip, C.c_void_p]
    for name in EXPORTED:
        if name not in ("epscu_abi_version", "epscu_last_error"):
            getattr(L, name).restype = C.c_int32
    _lib = L
    return L


def _check(code: int):
    if code != EPSCU_OK:
        raise EpscuError(code, load().epscu_last_error().decode(errors="replace"))


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _l(a):
    return a.ctypes.data_as(_lp)


def device_count() -> int:
    c = C.c_int32()
    rc = load().epscu_device_count(C.byref(c))
    return c.value if rc == EPSCU_OK else 0


def device_info(ordinal: int) -> DeviceInfo:
    info = DeviceInfo()
    _check(load().epscu_get_device_info(ordinal, C.byref(info)))
    return info


@dataclass
class Solution:
    """Levels of a batch in [potential x capacity] layout (slot s = level min_level + s)."""

    n_total: np.ndarray
    n_out: np.ndarray
    energy: np.ndarray
    nodes: np.ndarray
    status: np.ndarray
    err_est: np.ndarray
    psi: np.ndarray | None
    psi_offsets: np.ndarray
    N: np.ndarray
    rc: int = 0  # status code of the solve (epscu_solve's return value)
    psi_required: int = 0  # doubles the wavefunctions of this solve need

    def levels(self, p: int) -> np.ndarray:
        return self.energy[p, : self.n_out[p]]

    def wavefunctions(self, p: int) -> np.ndarray:
        o = int(self.psi_offsets[p])
        n, N = int(self.n_out[p]), int(self.N[p])
        return self.psi[o : o + n * N].reshape(n, N)


class Concatenated(tuple):
    """(V, offsets, N) of a batch already laid out contiguously (e.g. in pinned
    memory): passed to Context.solve as is, without a host-side copy."""

    def __new__(cls, V, offsets, N):
        return super().__new__(cls, (np.ascontiguousarray(V, np.float64), np.asarray(offsets, np.int64),
                                     np.asarray(N, np.int32)))


def concat(Vs):
    if isinstance(Vs, Concatenated):
        return Vs
    N = np.array([v.size for v in Vs], np.int32)
    offsets = np.zeros(len(Vs), np.int64)
    offsets[1:] = np.cumsum(N[:-1].astype(np.int64))
    return np.ascontiguousarray(np.concatenate([np.asarray(v, np.float64) for v in Vs])), offsets, N


class Context:
    """One epscu context on one device."""

    def __init__(self, device: int = 0):
        self._lib = load()
        self._h = C.c_void_p()
        _check(self._lib.epscu_create(int(device), C.byref(self._h)))
        self.device = device

    def close(self):
        if self._h:
            self._lib.epscu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_arena_block(self, nbytes: int):
        _check(self._lib.epscu_set_arena_block(self._h, int(nbytes)))

    def cancel(self):
        _check(self._lib.epscu_cancel(self._h))

    def cancel_clear(self):
        _check(self._lib.epscu_cancel_clear(self._h))

    def stats(self) -> Stats:
        s = Stats()
        _check(self._lib.epscu_last_stats(self._h, C.byref(s)))
        return s

    def measure_fma_peaks(self):
        a, b = C.c_double(), C.c_double()
        _check(self._lib.epscu_measure_fma_peaks(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def solve(
        self,
        Vs,
        r_min,
        r_max,
        mu,
        e_cap,
        n_trial: int,
        method: int = METHOD_FAST_FP32C,
        min_level: int = 0,
        max_level: int = -1,
        level_capacity: int | None = None,
        want_psi: bool = False,
        psi_capacity: int | None = None,
        tol: float = 1e-12,
        tune: bool = False,
        long_window: int = 0,
        keep_psi: bool = False,
        out: Solution | None = None,
        wait_polls: int = 0,
        max_iter: int = 0,
        check: bool = True,
        mid_window: int = 0,
    ) -> Solution:
        """Solve a batch of host potentials (host buffers through the C ABI).

        out: a Solution of this batch's shape whose result arrays are written
        in place (for instance page-locked buffers reused across solves, so
        the device-to-host copies run at full speed); its psi is not used.
        wait_polls / max_iter: epscu_opts bounds (0: the defaults); mid_window:
        the warp-per-level tier's threshold (> 0; 0 or < 0: off, the default).
        check=False returns the Solution with the status code in .rc instead
        of raising on a non-zero code."""
        V, offsets, N = concat(Vs)
        n = int(N.size)

        def arr(x):
            a = np.asarray(x, np.float64)
            return np.ascontiguousarray(np.broadcast_to(a, (n,)) if a.ndim == 0 else a)

        r_min, r_max, mu, e_cap = arr(r_min), arr(r_max), arr(mu), arr(e_cap)
        if level_capacity is None:
            level_capacity = (max_level - min_level + 1) if max_level >= 0 else 512
        cap = int(level_capacity)
        if out is not None:
            def own(a, shape, dtype):
                if a.shape != shape or a.dtype != dtype or not a.flags.c_contiguous:
                    raise ValueError(f"out array of shape {a.shape} {a.dtype}, expected {shape} {np.dtype(dtype)}")
                return a
            n_total = own(out.n_total, (n,), np.int32)
            n_out = own(out.n_out, (n,), np.int32)
            energy = own(out.energy, (n, cap), np.float64)
            nodes = own(out.nodes, (n, cap), np.int32)
            status = own(out.status, (n, cap), np.int32)
            err = own(out.err_est, (n, cap), np.float64)
            psi_off = own(out.psi_offsets, (n,), np.int64)
        else:
            n_total = np.zeros(n, np.int32)
            n_out = np.zeros(n, np.int32)
            energy = np.zeros((n, cap))
            nodes = np.zeros((n, cap), np.int32)
            status = np.zeros((n, cap), np.int32)
            err = np.zeros((n, cap))
            psi_off = np.zeros(n, np.int64)
        psi = None
        if want_psi:
            if psi_capacity is None:
                psi_capacity = int(N.astype(np.int64).sum()) * cap
            psi = np.zeros(int(psi_capacity))
        b = Batch(n, _d(V), _l(offsets), _i(N), _d(r_min), _d(r_max), _d(mu), _d(e_cap), int(n_trial), int(min_level), int(max_level))
        r = Result(
            cap,
            _i(n_total),
            _i(n_out),
            _d(energy),
            _i(nodes),
            _i(status),
            _d(err),
            _d(psi) if psi is not None else None,
            int(psi.size) if psi is not None else 0,
            _l(psi_off),
            0,
        )
        flags = (WANT_PSI if want_psi else 0) | (KEEP_PSI if keep_psi and not want_psi else 0)
        o = Opts(int(method), flags, float(tol), None, 1 if tune else 0, int(long_window), int(wait_polls),
                 int(max_iter), int(mid_window))
        rc = self._lib.epscu_solve(self._h, C.byref(b), C.byref(r), C.byref(o))
        if check:
            _check(rc)
        sol = Solution(n_total, n_out, energy, nodes, status, err, psi, psi_off, N)
        sol.rc = int(rc)
        sol.psi_required = int(r.psi_required)
        return sol

    def adjoint(self, dL_dE: np.ndarray, total_points: int, recompute: bool = False,
                out: np.ndarray | None = None) -> np.ndarray:
        g = np.ascontiguousarray(dL_dE, np.float64)
        if out is None:
            out = np.zeros(int(total_points))
        o = Opts(0, 0, 0.0, None, 0, 0)
        _check(self._lib.epscu_adjoint(self._h, _d(g), _d(out), 1 if recompute else 0, C.byref(o)))
        return out

    def tabulate_adjoint(self, kind, params, N, r_min, r_max, dL_dV, n_knots: int = 1024,
                         out: np.ndarray | None = None) -> np.ndarray:
        """dL/dparams [n, 12] from dL/dV (host arrays; epscu_tabulate_adjoint)."""
        kind = np.ascontiguousarray(kind, np.int32)
        params = np.ascontiguousarray(params, np.float64).reshape(-1, 12)
        N = np.ascontiguousarray(N, np.int32)
        offsets = np.zeros(N.size, np.int64)
        offsets[1:] = np.cumsum(N[:-1].astype(np.int64))
        r_min = np.ascontiguousarray(r_min, np.float64)
        r_max = np.ascontiguousarray(r_max, np.float64)
        g = np.ascontiguousarray(dL_dV, np.float64)
        if out is None:
            out = np.zeros((N.size, 12))
        o = Opts(0, 0, 0.0, None, 0, 0)
        _check(self._lib.epscu_tabulate_adjoint(self._h, int(N.size), _i(kind), _d(params), _l(offsets), _i(N),
                                                _d(r_min), _d(r_max), int(n_knots), _d(g), _d(out), C.byref(o)))
        return out

    def tabulate(self, kind, params, N, r_min, r_max, n_knots: int = 1024) -> list:
        kind = np.ascontiguousarray(kind, np.int32)
        params = np.ascontiguousarray(params, np.float64).reshape(-1, 12)
        N = np.ascontiguousarray(N, np.int32)
        offsets = np.zeros(N.size, np.int64)
        offsets[1:] = np.cumsum(N[:-1].astype(np.int64))
        r_min = np.ascontiguousarray(r_min, np.float64)
        r_max = np.ascontiguousarray(r_max, np.float64)
        V = np.zeros(int(N.astype(np.int64).sum()))
        o = Opts(0, 0, 0.0, None, 0, 0)
        _check(
            self._lib.epscu_tabulate(
                self._h, int(N.size), _i(kind), _d(params), _l(offsets), _i(N), _d(r_min), _d(r_max), int(n_knots), _d(V), C.byref(o)
            )
        )
        return [V[offsets[i] : offsets[i] + N[i]] for i in range(N.size)]


def batch_params(b) -> np.ndarray:
    """[n, 12] parameter rows of a synth.PotentialBatch for epscu_tabulate."""
    n = len(b)
    P = np.zeros((n, 12))
    for i in range(n):
        if int(b.kind[i]) == KIND_LJ:
            P[i, 0:2] = b.lj[i]
        else:
            P[i, 0:3] = b.morse[i]
            P[i, 3:12] = b.bumps[i].reshape(-1)
    return P


class DeviceBatch:
    """A batch resident in device memory (torch tensors) with persistent output
    buffers, solved through the C ABI with EPSCU_MEM_DEVICE; repeated solves of
    the same DeviceBatch replay the context's captured CUDA graph."""

    def __init__(self, ctx: Context, Vs, r_min, r_max, mu, e_cap, n_trial: int, level_capacity: int,
                 min_level: int = 0, max_level: int = -1, want_psi: bool = True, psi_capacity: int | None = None,
                 device: str = "cuda"):
        import torch

        self.ctx = ctx
        V, offsets, N = concat(Vs)
        n = int(N.size)

        def arr(x):
            a = np.asarray(x, np.float64)
            return np.ascontiguousarray(np.broadcast_to(a, (n,)) if a.ndim == 0 else a)

        self.n = n
        self.N = N
        self.offsets = offsets
        self.r_min, self.r_max, self.mu, self.e_cap = arr(r_min), arr(r_max), arr(mu), arr(e_cap)
        self.n_trial = int(n_trial)
        self.cap = int(level_capacity)
        self.min_level, self.max_level = int(min_level), int(max_level)
        self.total_points = int(V.size)
        self.V = torch.from_numpy(V).to(device)
        self.n_total = torch.zeros(n, dtype=torch.int32, device=device)
        self.n_out = torch.zeros(n, dtype=torch.int32, device=device)
        self.energy = torch.zeros((n, self.cap), dtype=torch.float64, device=device)
        self.nodes = torch.zeros((n, self.cap), dtype=torch.int32, device=device)
        self.status = torch.zeros((n, self.cap), dtype=torch.int32, device=device)
        self.err = torch.zeros((n, self.cap), dtype=torch.float64, device=device)
        self.want_psi = want_psi
        if want_psi:
            if psi_capacity is None:
                psi_capacity = int(N.astype(np.int64).sum()) * self.cap
            self.psi = torch.zeros(int(psi_capacity), dtype=torch.float64, device=device)
        else:
            self.psi = None
        self.psi_offsets = np.zeros(n, np.int64)
        self.gV = torch.zeros(self.total_points, dtype=torch.float64, device=device)
        self.psi_required = 0

    def _ptr(self, t, ty):
        return C.cast(C.c_void_p(t.data_ptr()), ty) if t is not None else None

    def solve(self, method: int = METHOD_FAST_FP32C, tune: bool = False, stage_timing: bool = False, stream=None,
              long_window: int = 0, mid_window: int = 0):
        import torch

        b = Batch(self.n, self._ptr(self.V, _dp), _l(self.offsets), _i(self.N), _d(self.r_min), _d(self.r_max),
                  _d(self.mu), _d(self.e_cap), self.n_trial, self.min_level, self.max_level)
        r = Result(self.cap, self._ptr(self.n_total, _ip), self._ptr(self.n_out, _ip), self._ptr(self.energy, _dp),
                   self._ptr(self.nodes, _ip), self._ptr(self.status, _ip), self._ptr(self.err, _dp),
                   self._ptr(self.psi, _dp), int(self.psi.numel()) if self.psi is not None else 0,
                   _l(self.psi_offsets), 0)
        flags = MEM_DEVICE | (WANT_PSI if self.want_psi else 0) | (STAGE_TIMING if stage_timing else 0)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        o = Opts(int(method), flags, 1e-12, C.c_void_p(s), 1 if tune else 0, int(long_window), 0, 0, int(mid_window))
        _check(self.ctx._lib.epscu_solve(self.ctx.handle, C.byref(b), C.byref(r), C.byref(o)))
        self.psi_required = r.psi_required

    def param_adjoint(self, kind, params, gP=None, n_knots: int = 1024, stream=None):
        """dL/dparams [n, 12] (device) from self.gV through epscu_tabulate_adjoint;
        params: the [n, 12] float64 cuda tensor the potentials were tabulated from."""
        import torch

        kind = np.ascontiguousarray(kind, np.int32)
        if gP is None:
            gP = torch.zeros((self.n, 12), dtype=torch.float64, device=self.gV.device)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        o = Opts(0, MEM_DEVICE, 0.0, C.c_void_p(s), 0, 0)
        _check(self.ctx._lib.epscu_tabulate_adjoint(
            self.ctx.handle, self.n, _i(kind), self._ptr(params, _dp), _l(self.offsets), _i(self.N),
            _d(self.r_min), _d(self.r_max), int(n_knots), self._ptr(self.gV, _dp), self._ptr(gP, _dp), C.byref(o)))
        return gP

    def adjoint(self, gE, recompute: bool = False, stream=None):
        """dL/dV into self.gV (device) for dL/dE = gE ([n, cap] float64 cuda tensor)."""
        import torch

        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        o = Opts(0, MEM_DEVICE, 0.0, C.c_void_p(s), 0, 0)
        g = gE.contiguous()
        _check(self.ctx._lib.epscu_adjoint(self.ctx.handle, self._ptr(g, _dp), self._ptr(self.gV, _dp),
                                           1 if recompute else 0, C.byref(o)))
        return self.gV
