"""Generates tests/golden/golden.json from the FP64 oracle (run from the repo root).

The reference ships no numeric fixtures for this path (its tests only carry
un-asserted Morse parameters), so these vectors freeze the oracle's own
output on seeded workloads; tests/test_oracle.py checks the oracle against
dense eigen-decompositions and analytic levels before trusting them, and the
GPU parity tests compare against the same values.
"""
from __future__ import annotations

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from epseon_backend_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = [
    dict(workload="morse_single", kwargs={}, indices=[0], n_trial=1024, count_stride=16),
    dict(workload="morse_batch", kwargs={}, indices=[0, 9, 33], n_trial=8192, count_stride=128),
    dict(workload="mixed_batch", kwargs=dict(B=30, n_min=2048, n_max=4096), indices=list(range(0, 30, 5)), n_trial=2048,
         count_stride=64),
]


def main():
    out = {"generator": "tests/golden/make_golden.py", "oracle": "oracle/numerov_oracle.c", "cases": []}
    for case in CASES:
        b = getattr(synth, case["workload"])(**case["kwargs"])
        idx = case["indices"]
        sel = np.array(idx)
        sols = O.solve_batch([b.V(i) for i in idx], b.r_min[sel], b.r_max[sel], b.mu[sel], b.e_cap[sel], case["n_trial"])
        res = []
        for s in sols:
            res.append(
                dict(
                    n_total=int(s.n_total),
                    energy=[float(x) for x in s.energy],
                    energy_polished=[float(x) for x in s.energy_polished],
                    counts_strided=[int(x) for x in s.counts[:: case["count_stride"]]],
                )
            )
        c = dict(case)
        c["results"] = res
        out["cases"].append(c)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
