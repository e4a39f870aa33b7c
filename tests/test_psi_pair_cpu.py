"""The tagged float pair that holds psi-hat between the norm pass and
scale_psi, and the integer assembly of a double from a double-float pair
(CPU restatement of dfpass.cuh psi_tag / store_psi_pair / load_psi_pair and
dfloat.cuh df_pair_to_double; no GPU).

psi-hat = (h + l) 2^X is stored as (h 2^x, l 2^x) in two floats with
X = 64 r + x, x in [-32, 31], and r in the five low bits of the second float.
The round trip must keep psi-hat to ~2^-43 relative for every X the passes
can reach, and the assembled double must be within one unit in its last
place of h + l.
"""
from __future__ import annotations

import numpy as np


def psi_tag(X: int):
    X = max(-1000, min(X, 990))
    r = (X + 32) >> 6  # floor division
    x = X - 64 * r
    assert -32 <= x <= 31 and -16 <= r <= 15
    return np.float32(2.0 ** x), r


def store(h: np.float32, l: np.float32, X: int):
    sc, r = psi_tag(X)
    hs = np.float32(h * sc)
    ls = np.float32(l * sc)
    lt = (int(ls.view(np.uint32)) & ~31 & 0xFFFFFFFF) | (r & 31)
    return hs, np.uint32(lt).view(np.float32)


def load(hs: np.float32, lt: np.float32):
    bits = int(np.float32(lt).view(np.uint32))
    r5 = bits & 31
    r = r5 - 32 if r5 >= 16 else r5
    l = np.uint32(bits & ~31 & 0xFFFFFFFF).view(np.float32)
    return hs, l, r


def pair_to_double(h: np.float32, l: np.float32) -> float:
    """Integer assembly: h's significand at the top of 53 bits, l's below."""
    uh, ul = int(np.float32(h).view(np.uint32)), int(np.float32(l).view(np.uint32))
    eh, el = (uh >> 23) & 0xFF, (ul >> 23) & 0xFF
    if eh in (0, 0xFF) or el == 0xFF:
        return float(h) + float(l)
    M = ((uh & 0x7FFFFF) | 0x800000) << 29
    if el != 0:
        d = eh - el
        if d < 24:
            return float(h) + float(l)
        ml = (ul & 0x7FFFFF) | 0x800000
        sh = 29 - d
        add = ml << sh if sh >= 0 else (ml >> -sh if -sh < 64 else 0)
        M = M - add if (uh ^ ul) >> 31 else M + add
    e = eh + 896
    if not (M >> 52):
        M <<= 1
        e -= 1
    bits = ((uh >> 31) << 63) | (e << 52) | (M & ((1 << 52) - 1))
    return float(np.uint64(bits).view(np.float64))


def df_split(x: float):
    h = np.float32(x)
    return h, np.float32(x - float(h))


def test_round_trip_over_the_exponent_range():
    rng = np.random.default_rng(0)
    for X in list(range(-1000, 991, 7)) + [-1000, -33, -32, -31, -1, 0, 1, 31, 32, 33, 990]:
        for _ in range(20):
            v = rng.uniform(0.25, 1.0) * rng.choice([-1.0, 1.0])
            h, l = df_split(v)
            hs, lt = store(h, l, X)
            h2, l2, r = load(hs, lt)
            got = (float(h2) + float(l2)) * 2.0 ** (64 * r)
            want = (float(h) + float(l)) * 2.0 ** max(-1000, min(X, 990))
            assert abs(got - want) <= 2.0 ** -42 * abs(want), (X, v)


def test_zero_and_tiny_values_decode_to_zero_or_near():
    for X in (-40, 0, 70, 500):
        hs, lt = store(np.float32(0.0), np.float32(0.0), X)
        h2, l2, r = load(hs, lt)
        assert float(h2) + float(l2) == 0.0
        assert r == psi_tag(X)[1]


def test_pair_to_double_within_one_ulp():
    rng = np.random.default_rng(1)
    for _ in range(20000):
        x = rng.uniform(-1.0, 1.0) * 2.0 ** int(rng.integers(-60, 60))
        h, l = df_split(x)
        got = pair_to_double(h, l)
        exact = float(h) + float(l)  # h + l rounded to nearest double
        assert abs(got - exact) <= np.spacing(abs(exact)), (x, got, exact)
    # a power of two minus a small low part: the one-bit renormalisation
    h, l = np.float32(1.0), np.float32(-2.0 ** -30)
    assert abs(pair_to_double(h, l) - (1.0 - 2.0 ** -30)) <= np.spacing(1.0)
