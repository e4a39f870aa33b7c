"""Integer forms of prepare_kernel's per-point work (CPU restatement of
prepare.cu dkey0 / split_double_rn and of its cut-off and argmin, no GPU).

The kernel replaces FP64 comparisons by comparisons of order-preserving
integer images of the doubles and the double-to-float-pair split by integer
rounding.  Both must give exactly what the FP64 forms (and the oracle's
eo_prepare loops) give: the minimum of V, the cut-offs a (V_i - V_min) <= 1/2
(found through a threshold image located once per potential by bisection on
the images), the first argmin on [i0, i1], and (__double2float_rn(w),
__double2float_rn(w - hi)).
"""
from __future__ import annotations

import numpy as np
import pytest

M64 = (1 << 64) - 1
KEY_MAX = M64


def dkey0(x: float) -> int:
    u = int(np.float64(x).view(np.uint64))
    if (u << 1) & M64 == 0:
        u = 0
    return (~u) & M64 if u >> 63 else u | (1 << 63)


def dkey_inv(k: int) -> float:
    u = (k & ((1 << 63) - 1)) if k >> 63 else (~k) & M64
    return float(np.uint64(u).view(np.float64))


def split_double_rn(w: float) -> tuple[np.float32, np.float32]:
    u = int(np.float64(w).view(np.uint64))
    e = ((u >> 52) & 0x7FF) - 1023
    if e < -60 or e > 100:
        hi = np.float32(w)
        return hi, np.float32(np.float64(w) - np.float64(hi))
    sgn = (u >> 32) & 0x80000000
    mant = u & ((1 << 52) - 1)
    r = mant & 0x1FFFFFFF
    hb = ((e + 127) << 23) | (mant >> 29)
    up = 1 if (r > 0x10000000 or (r == 0x10000000 and (hb & 1))) else 0
    hb += up
    rr = r - (0x20000000 if up else 0)
    lo = np.float32(0.0)
    if rr != 0:
        lo = np.float32(rr)  # one rounding to 24 bits, ties to even
        lo = np.float32(lo * np.float32(2.0 ** -52))
        lo = np.float32(lo * np.float32(2.0 ** e))
        if sgn:
            lo = -lo
    hi = np.uint32(sgn | hb).view(np.float32)
    return hi, lo


def _bits32(x) -> int:
    return int(np.float32(x).view(np.uint32))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_split_matches_the_conversions(seed):
    rng = np.random.default_rng(seed)
    # random doubles over the integer path's exponent range and beyond
    e = rng.integers(-70, 110, 3000)
    w = rng.uniform(1.0, 2.0, 3000) * 2.0 ** e.astype(np.float64)
    w *= rng.choice([-1.0, 1.0], 3000)
    # exact ties of the 29 dropped bits (even and odd kept significands), and
    # significands that carry into the exponent when rounded up
    base = rng.integers(0, 1 << 23, 200)
    ties = [(1 << 52 | (int(m) << 29) | (1 << 28)) for m in base]
    carry = [(1 << 52) | ((1 << 52) - 1), (1 << 52) | ((1 << 52) - 2)]
    extra = [float(np.uint64(((1023 + int(x)) << 52) | (m & ((1 << 52) - 1))).view(np.float64))
             for m in ties + carry for x in (-3, 0, 7)]
    for x in list(w) + extra + [-v for v in extra]:
        hi, lo = split_double_rn(float(x))
        rhi = np.float32(x)
        rlo = np.float32(np.float64(x) - np.float64(rhi))
        assert _bits32(hi) == _bits32(rhi), x
        assert _bits32(lo) == _bits32(rlo), x


def oracle_prepare(V: np.ndarray, a: float):
    """eo_prepare's loops (oracle/numerov_oracle.c)."""
    vmin = V[0]
    for v in V:
        if v < vmin:
            vmin = v
    first = last = -1
    for i, v in enumerate(V):
        if a * (v - vmin) <= 0.5:
            if first < 0:
                first = i
            last = i
    N = len(V)
    i0 = 1 if first < 1 else first
    i1 = N - 2 if last > N - 2 else last
    k = i0
    for i in range(i0, i1 + 1):
        if V[i] < V[k]:
            k = i
    return vmin, i0, i1, k


def keyed_prepare(V: np.ndarray, a: float):
    """prepare_kernel's integer forms."""
    keys = [dkey0(v) for v in V]
    kmin = min(keys)
    vmin = dkey_inv(kmin)
    lo, hi = kmin, KEY_MAX
    while hi - lo > 1:
        mid = lo + (hi - lo) // 2
        if np.float64(a) * (np.float64(dkey_inv(mid)) - np.float64(vmin)) <= 0.5:
            lo = mid
        else:
            hi = mid
    kt = lo
    inside = [i for i, k in enumerate(keys) if k <= kt]
    N = len(V)
    first = inside[0] if inside else N
    last = inside[-1] if inside else -1
    i0 = 1 if first < 1 else first
    i1 = N - 2 if last > N - 2 else last
    k_scan = N
    if i1 >= i0:
        seg = keys[i0:i1 + 1]
        m = min(seg)
        k_scan = i0 + seg.index(m)
    return vmin, i0, i1, k_scan


@pytest.mark.parametrize("seed", range(6))
def test_cutoffs_and_argmin_match_the_oracle_loops(seed):
    rng = np.random.default_rng(100 + seed)
    N = int(rng.integers(16, 400))
    r = np.linspace(0.5, 6.0, N)
    V = 0.05 * (1.0 - np.exp(-1.3 * (r - 2.0))) ** 2
    if seed % 2:
        V = np.round(V, 4)  # repeated values: ties at the minimum and at the cut-off
    if seed == 3:
        V[N // 3] = 0.0
        V[N // 2] = -0.0  # both zeros at the minimum
    a = float(rng.uniform(2.0, 200.0))
    if seed >= 4:
        # put grid values exactly at the cut-off threshold and one ulp either side
        vmin = V.min()
        t = vmin + 0.5 / a
        for j, d in zip(rng.choice(N, 3, replace=False), (0, 1, -1)):
            V[j] = np.nextafter(t, np.inf if d > 0 else -np.inf) if d else t
    ov, oi0, oi1, ok = oracle_prepare(V, a)
    kv, ki0, ki1, kk = keyed_prepare(V, a)
    assert ov == kv
    assert (oi0, oi1) == (ki0, ki1)
    if oi1 >= oi0:
        assert ok == kk
