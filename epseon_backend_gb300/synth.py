"""Seeded synthetic potential batches (atomic units: Hartree, bohr, m_e).

The reference has no potential data of its own: MorsePotentialGenerator and
PotentialFileLoader both return ``{}`` (cpp/gpu/include/epseon/gpu/
task_configurator/potential_source.hpp:89-91, :223-225) and its tests carry
only un-asserted Morse parameters (python/test/test_device/test_gpu/
test_libepseon_gpu.py:183-208).  These generators produce the five workloads
the solver is measured on, from numpy's PCG64 with a fixed seed per workload:

* ``morse_single``: De=0.1, a=1, re=2, mu=1000, N=4096 on [0.5, re+25/a],
  1024 trial energies.
* ``morse_batch``: 64 Morse, De~U[0.02,0.2], a~U[0.5,1.5], re~U[1.5,4],
  mu~logU[500,1e5], N=16384 on [0.5, re+30/a], 8192 trial energies.
* ``mixed_batch``: 2048 potentials, a third each Morse (ranges above), shifted
  Lennard-Jones 12-6 (eps~U[0.01,0.1], sigma~U[2,5], grid [0.5, 12 sigma]) and
  Morse plus 1-3 Gaussian bumps (amplitude~U[-0.2,0.2] De, width~U[0.1,0.5],
  centre~U[re-0.5,re+3]) tabulated on 1024 uniform knots and natural-cubic-
  spline interpolated; N~logU[2048,65536]; 8192 trial energies.
* ``bump_adjoint``: 256 Morse+bump potentials on N=32768 with loss weights
  w_v~U[0.5,1]; targets from the same potentials with bump amplitudes x1.1.
* ``morse_long``: De=0.15, a=0.6, re=4, mu=1e5, N=2^20 on [0.5, 54],
  65536 trial energies.

Every potential has its minimum at 0 (Morse, shifted LJ) or near it (bumps)
and its asymptote at De (eps for LJ); the energy window is capped at
0.999 De.  A Gaussian bump is ``A exp(-(r-c)^2 / (2 w^2))``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

KIND_MORSE, KIND_LJ, KIND_SPLINE = 0, 1, 2
CAP_FRACTION = 0.999
N_KNOTS = 1024


@dataclass
class PotentialBatch:
    """Host description of a batch of potentials on uniform grids."""

    kind: np.ndarray  # int32 [B]
    N: np.ndarray  # int32 [B]
    r_min: np.ndarray  # float64 [B]
    r_max: np.ndarray  # float64 [B]
    mu: np.ndarray  # float64 [B]
    De: np.ndarray  # asymptote above the minimum [B]
    e_cap: np.ndarray  # top of the energy window [B]
    n_trial: int
    # parameters: Morse (De, a, re), LJ (eps, sigma), bumps (amp, width, centre) x3
    morse: np.ndarray = field(default=None)  # [B, 3]
    lj: np.ndarray = field(default=None)  # [B, 2]
    bumps: np.ndarray = field(default=None)  # [B, 3, 3] (amp, width, centre); amp 0 = unused
    name: str = ""
    _V: list | None = None

    def __len__(self) -> int:
        return int(self.kind.size)

    @property
    def total_points(self) -> int:
        return int(self.N.sum())

    def V(self, i: int) -> np.ndarray:
        """FP64 tabulation of potential i on its grid (host)."""
        if self._V is None:
            self._V = [None] * len(self)
        if self._V[i] is None:
            self._V[i] = tabulate(self, i)
        return self._V[i]

    def potentials(self) -> list:
        return [self.V(i) for i in range(len(self))]

    def subset(self, idx) -> "PotentialBatch":
        idx = np.asarray(idx)
        out = PotentialBatch(
            self.kind[idx].copy(),
            self.N[idx].copy(),
            self.r_min[idx].copy(),
            self.r_max[idx].copy(),
            self.mu[idx].copy(),
            self.De[idx].copy(),
            self.e_cap[idx].copy(),
            self.n_trial,
            None if self.morse is None else self.morse[idx].copy(),
            None if self.lj is None else self.lj[idx].copy(),
            None if self.bumps is None else self.bumps[idx].copy(),
            self.name + "[subset]",
        )
        if self._V is not None:
            out._V = [self._V[int(i)] for i in idx]
        return out


def morse(r, De, a, re):
    x = 1.0 - np.exp(-a * (r - re))
    return De * x * x


def lennard_jones_shifted(r, eps, sigma):
    s6 = (sigma / r) ** 6
    return 4.0 * eps * (s6 * s6 - s6) + eps


def bumps_at(r, bumps):
    out = np.zeros_like(r)
    for amp, width, centre in bumps:
        if amp != 0.0:
            out += amp * np.exp(-((r - centre) ** 2) / (2.0 * width * width))
    return out


def natural_spline_second_derivs(y: np.ndarray, hk: float) -> np.ndarray:
    """Second derivatives M of the natural cubic spline through uniform knots.

    Solves (M_{k-1} + 4 M_k + M_{k+1}) = 6 (y_{k+1} - 2 y_k + y_{k-1}) / hk^2,
    M_0 = M_{K-1} = 0, by the Thomas algorithm (same sweep as the device
    tabulation kernel).
    """
    K = y.size
    M = np.zeros(K)
    if K < 3:
        return M
    rhs = 6.0 * (y[2:] - 2.0 * y[1:-1] + y[:-2]) / (hk * hk)
    n = K - 2
    cp = np.zeros(n)
    dp = np.zeros(n)
    cp[0] = 1.0 / 4.0
    dp[0] = rhs[0] / 4.0
    for i in range(1, n):
        den = 4.0 - cp[i - 1]
        cp[i] = 1.0 / den
        dp[i] = (rhs[i] - dp[i - 1]) / den
    x = np.zeros(n)
    x[-1] = dp[-1]
    for i in range(n - 2, -1, -1):
        x[i] = dp[i] - cp[i] * x[i + 1]
    M[1:-1] = x
    return M


def spline_eval(r: np.ndarray, r0: float, hk: float, y: np.ndarray, M: np.ndarray) -> np.ndarray:
    K = y.size
    t = (r - r0) / hk
    k = np.clip(np.floor(t).astype(np.int64), 0, K - 2)
    u = t - k
    w = 1.0 - u
    h2 = hk * hk / 6.0
    return w * y[k] + u * y[k + 1] + h2 * ((w * w * w - w) * M[k] + (u * u * u - u) * M[k + 1])


def knot_values(b: PotentialBatch, i: int, n_knots: int = N_KNOTS):
    rk = np.linspace(b.r_min[i], b.r_max[i], n_knots)
    De, a, re = b.morse[i]
    return rk, morse(rk, De, a, re) + bumps_at(rk, b.bumps[i])


def grid(b: PotentialBatch, i: int) -> np.ndarray:
    N = int(b.N[i])
    return b.r_min[i] + np.arange(N) * ((b.r_max[i] - b.r_min[i]) / (N - 1))


def tabulate(b: PotentialBatch, i: int) -> np.ndarray:
    r = grid(b, i)
    k = int(b.kind[i])
    if k == KIND_MORSE:
        De, a, re = b.morse[i]
        return morse(r, De, a, re)
    if k == KIND_LJ:
        eps, sigma = b.lj[i]
        return lennard_jones_shifted(r, eps, sigma)
    rk, yk = knot_values(b, i)
    hk = (b.r_max[i] - b.r_min[i]) / (rk.size - 1)
    M = natural_spline_second_derivs(yk, hk)
    return spline_eval(r, b.r_min[i], hk, yk, M)


def tabulate_params(kind: int, P: np.ndarray, N: int, r_min: float, r_max: float,
                    n_knots: int = N_KNOTS) -> np.ndarray:
    """Host tabulation of one [12] parameter row in the layout epscu_tabulate
    takes: Morse (De, a, re) or LJ (eps, sigma) at P[0:3], bumps (amp, width,
    centre) x 3 at P[3:12] (Morse + bumps through the natural spline)."""
    P = np.asarray(P, np.float64)
    r = r_min + np.arange(int(N)) * ((r_max - r_min) / (int(N) - 1))
    if int(kind) == KIND_MORSE:
        return morse(r, P[0], P[1], P[2])
    if int(kind) == KIND_LJ:
        return lennard_jones_shifted(r, P[0], P[1])
    rk = np.linspace(r_min, r_max, n_knots)
    yk = morse(rk, P[0], P[1], P[2]) + bumps_at(rk, P[3:12].reshape(3, 3))
    hk = (r_max - r_min) / (n_knots - 1)
    return spline_eval(r, r_min, hk, yk, natural_spline_second_derivs(yk, hk))


def _loguniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def _empty(B, n_trial, name):
    return PotentialBatch(
        np.zeros(B, np.int32),
        np.zeros(B, np.int32),
        np.zeros(B),
        np.zeros(B),
        np.zeros(B),
        np.zeros(B),
        np.zeros(B),
        n_trial,
        np.zeros((B, 3)),
        np.zeros((B, 2)),
        np.zeros((B, 3, 3)),
        name,
    )


def _finish(b: PotentialBatch) -> PotentialBatch:
    b.e_cap = CAP_FRACTION * b.De
    return b


def morse_single(N: int = 4096, n_trial: int = 1024) -> PotentialBatch:
    b = _empty(1, n_trial, "morse_single")
    b.kind[0] = KIND_MORSE
    b.N[0] = N
    b.morse[0] = (0.1, 1.0, 2.0)
    b.r_min[0], b.r_max[0] = 0.5, 2.0 + 25.0
    b.mu[0] = 1000.0
    b.De[0] = 0.1
    return _finish(b)


def morse_batch(B: int = 64, N: int = 16384, n_trial: int = 8192, seed: int = 2) -> PotentialBatch:
    rng = np.random.Generator(np.random.PCG64(seed))
    b = _empty(B, n_trial, "morse_batch")
    De = rng.uniform(0.02, 0.2, B)
    a = rng.uniform(0.5, 1.5, B)
    re = rng.uniform(1.5, 4.0, B)
    mu = _loguniform(rng, 500.0, 1e5, B)
    b.kind[:] = KIND_MORSE
    b.N[:] = N
    b.morse[:] = np.stack([De, a, re], 1)
    b.r_min[:] = 0.5
    b.r_max[:] = re + 30.0 / a
    b.mu[:] = mu
    b.De[:] = De
    return _finish(b)


def mixed_batch(B: int = 2048, n_trial: int = 8192, seed: int = 3, n_min: int = 2048, n_max: int = 65536) -> PotentialBatch:
    rng = np.random.Generator(np.random.PCG64(seed))
    b = _empty(B, n_trial, "mixed_batch")
    kinds = np.arange(B) % 3
    rng.shuffle(kinds)
    b.kind[:] = kinds
    b.N[:] = np.rint(_loguniform(rng, n_min, n_max, B)).astype(np.int32)
    b.mu[:] = _loguniform(rng, 500.0, 1e5, B)
    De = rng.uniform(0.02, 0.2, B)
    a = rng.uniform(0.5, 1.5, B)
    re = rng.uniform(1.5, 4.0, B)
    eps = rng.uniform(0.01, 0.1, B)
    sigma = rng.uniform(2.0, 5.0, B)
    nb = rng.integers(1, 4, B)
    amp = rng.uniform(-0.2, 0.2, (B, 3))
    width = rng.uniform(0.1, 0.5, (B, 3))
    centre = rng.uniform(-0.5, 3.0, (B, 3))
    for i in range(B):
        if kinds[i] == KIND_LJ:
            b.lj[i] = (eps[i], sigma[i])
            b.r_min[i], b.r_max[i] = 0.5, 12.0 * sigma[i]
            b.De[i] = eps[i]
        else:
            b.morse[i] = (De[i], a[i], re[i])
            b.r_min[i], b.r_max[i] = 0.5, re[i] + 30.0 / a[i]
            b.De[i] = De[i]
            if kinds[i] == KIND_SPLINE:
                for j in range(nb[i]):
                    b.bumps[i, j] = (amp[i, j] * De[i], width[i, j], re[i] + centre[i, j])
    return _finish(b)


def bump_adjoint(B: int = 256, N: int = 32768, n_trial: int = 8192, seed: int = 4, amp_scale: float = 1.0):
    """Morse+bump batch; returns (batch, weights_rng_seeded) for the adjoint loss."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = _empty(B, n_trial, "bump_adjoint")
    b.kind[:] = KIND_SPLINE
    b.N[:] = N
    De = rng.uniform(0.02, 0.2, B)
    a = rng.uniform(0.5, 1.5, B)
    re = rng.uniform(1.5, 4.0, B)
    b.mu[:] = _loguniform(rng, 500.0, 1e5, B)
    nb = rng.integers(1, 4, B)
    amp = rng.uniform(-0.2, 0.2, (B, 3))
    width = rng.uniform(0.1, 0.5, (B, 3))
    centre = rng.uniform(-0.5, 3.0, (B, 3))
    for i in range(B):
        b.morse[i] = (De[i], a[i], re[i])
        b.r_min[i], b.r_max[i] = 0.5, re[i] + 30.0 / a[i]
        b.De[i] = De[i]
        for j in range(nb[i]):
            b.bumps[i, j] = (amp_scale * amp[i, j] * De[i], width[i, j], re[i] + centre[i, j])
    return _finish(b)


def loss_weights(n_levels: int, seed: int = 4) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    return rng.uniform(0.5, 1.0, n_levels)


def morse_long(N: int = 1 << 20, n_trial: int = 65536) -> PotentialBatch:
    b = _empty(1, n_trial, "morse_long")
    b.kind[0] = KIND_MORSE
    b.N[0] = N
    b.morse[0] = (0.15, 0.6, 4.0)
    b.r_min[0], b.r_max[0] = 0.5, 54.0
    b.mu[0] = 1e5
    b.De[0] = 0.15
    return _finish(b)


def analytic_morse_levels(De: float, a: float, mu: float, e_cap: float) -> np.ndarray:
    """E_v = w (v+1/2) - w^2 (v+1/2)^2 / (4 De), w = a sqrt(2 De / mu), below e_cap."""
    w = a * np.sqrt(2.0 * De / mu)
    out = []
    v = 0
    while True:
        x = v + 0.5
        if x > 2.0 * De / w:
            break
        E = w * x - w * w * x * x / (4.0 * De)
        if E >= e_cap:
            break
        out.append(E)
        v += 1
    return np.array(out)
