"""Failure detection in forms that leave the GPU usable, through the C ABI and
the task API:

* a bounded wait of the TMA scan made to run out (epscu_opts.wait_polls < 0:
  every scan item waits on a barrier that no copy completes, then gives up
  as on a lost copy, draining the copies in flight): the solve reports
  EPSCU_ERR_TIMEOUT and no levels, and the next solve on the same context is
  exact;
* cooperative cancellation (the reference's TaskHandle::cancel,
  cpp/gpu/include/epseon/gpu/task_handle.hpp:136-144): a request made before a
  solve stops that solve and is consumed by it, a withdrawn request stops
  nothing, a request made while a solve runs stops it, and a cancelled task
  leaves the device interface usable for the next task;
* the refinement's iteration cap (epscu_opts.max_iter): levels that reach it
  carry EPSCU_LEVEL_MAXITER, and the levels that do not are still exact.

No GPU fault, trap or unbounded wait is involved: every failure is a bound
that runs out or a flag set by the host.
"""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from epseon_backend_gb300 import capi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL_FAST = 1e-10


def _small():
    b = synth.morse_batch()
    return b.subset([0, 5, 17, 42])


def _solve(ctx, b, method=capi.METHOD_FAST_FP32C, **kw):
    return ctx.solve(b.potentials(), b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=method,
                     level_capacity=512, **kw)


def _assert_exact(sol, b):
    refs = O.solve_batch(b.potentials(), b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)
    for q, ref in enumerate(refs):
        n = int(sol.n_out[q])
        assert n == ref.n_total == ref.energy.size
        assert np.array_equal(sol.nodes[q, :n], np.arange(n))
        assert np.max(np.abs(sol.energy[q, :n] - ref.energy_polished)) < E_TOL_FAST


def test_scan_wait_timeout_reports_and_context_stays_usable(ctx):
    b = _small()
    sol = _solve(ctx, b, wait_polls=-64, check=False)
    assert sol.rc == capi.ERR_TIMEOUT
    assert b"bounded wait" in capi.load().epscu_last_error()
    assert np.all(sol.n_out == 0)  # incomplete counts give no levels
    # the same context, default bounds: every level exact
    good = _solve(ctx, b)
    assert good.rc == capi.EPSCU_OK
    _assert_exact(good, b)


@pytest.mark.parametrize("method", [capi.METHOD_PLAIN_FP64, capi.METHOD_FAST_FP32C])
def test_cancel_before_solve_is_consumed_by_it(ctx, method):
    b = _small()
    ctx.cancel()
    sol = _solve(ctx, b, method=method, check=False)
    assert sol.rc == capi.ERR_CANCELLED
    assert np.all(sol.n_out == 0)
    # the request was consumed: the next solve runs to the end
    again = _solve(ctx, b, method=method)
    assert again.rc == capi.EPSCU_OK
    _assert_exact(again, b)


def test_withdrawn_cancel_stops_nothing(ctx):
    b = _small()
    ctx.cancel()
    ctx.cancel_clear()
    sol = _solve(ctx, b, check=False)
    assert sol.rc == capi.EPSCU_OK
    _assert_exact(sol, b)


def test_cancel_during_solve(ctx):
    # the plain method on 256 grids of 16384 points takes about a second; the
    # request comes 0.1 s in, from another thread (ctypes releases the GIL)
    b = synth.morse_batch()
    Vs = b.potentials() * 4
    n = len(Vs)
    rep = lambda x: np.tile(x, 4)  # noqa: E731
    out = {}

    def run():
        t0 = time.perf_counter()
        out["sol"] = ctx.solve(Vs, rep(b.r_min), rep(b.r_max), rep(b.mu), rep(b.e_cap), b.n_trial,
                               method=capi.METHOD_PLAIN_FP64, level_capacity=512, check=False)
        out["s"] = time.perf_counter() - t0

    t = threading.Thread(target=run)
    t.start()
    time.sleep(0.1)
    ctx.cancel()
    t.join()
    sol = out["sol"]
    assert sol.rc == capi.ERR_CANCELLED, (sol.rc, out["s"])
    # a level the solve set up before the request is either finished or
    # marked cancelled; none is reported as a plain success with a wrong count
    for p in range(n):
        k = int(sol.n_out[p])
        st = sol.status[p, :k]
        ok = (st & capi.LEVEL_CANCELLED) == 0
        assert np.array_equal(sol.nodes[p, :k][ok], np.arange(k)[ok])
    # and the context is usable afterwards
    small = _small()
    _assert_exact(_solve(ctx, small), small)


def test_iteration_cap_reports_maxiter(ctx):
    b = _small()
    capped = _solve(ctx, b, max_iter=1)
    flagged = 0
    refs = O.solve_batch(b.potentials(), b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial)
    for q, ref in enumerate(refs):
        n = int(capped.n_out[q])
        assert n == ref.n_total
        st = capped.status[q, :n]
        cap_hit = (st & capi.LEVEL_MAXITER) != 0
        flagged += int(cap_hit.sum())
        clean = st == 0
        # a level without a flag is exact even under the cap
        if clean.any():
            assert np.max(np.abs(capped.energy[q, :n][clean] - ref.energy_polished[clean])) < E_TOL_FAST
    assert flagged > 0
    # the default caps on the same context: no flags, every level exact
    sol = _solve(ctx, b)
    assert not np.any(sol.status[:, :] & capi.LEVEL_MAXITER)
    _assert_exact(sol, b)


def test_task_cancel_then_next_task_runs():
    import epseon_backend_gb300.device.cuda as m

    iface = m.EpseonComputeContext.create().get_device_interface(0)

    def configure(cfg, count, max_level):
        pots = [m.MorsePotentialConfig(dissociation_energy=5500.0, equilibrium_bond_distance=0.6, well_width=10,
                                       min_r=0.0, max_r=10.0, point_count=16500)] * count
        return (cfg.set_hardware_config(potential_buffer_size=16500, group_size=16,
                                        allocation_block_size=1 << 24)
                .set_morse_potential(pots)
                .set_vibwa_algorithm(mass_atom_0=87.62, mass_atom_1=87.62, integration_step=0.1,
                                     min_distance_to_asymptote=0.1, min_level=0, max_level=max_level))

    # 256 plain-method potentials in groups of 16: several seconds of work
    big = iface.submit_task(configure(iface.get_task_configurator("float64"), 256, 60))
    time.sleep(0.05)
    assert big.cancel() is True
    big.wait()
    assert big.is_done()
    assert big.get_status_message() == "cancelled"
    # the next task on the same device interface is not stopped by that request
    small = iface.submit_task(configure(iface.get_task_configurator("float64"), 2, 5))
    small.wait()
    assert small.get_status_message().startswith("done")
    r = small.get_results()
    assert len(r["energies"]) == 2 and r["energies"][0].size == 6
