"""The ``cuda`` device's Python surface, mirroring the reference's binding
tests (python/test/test_device/test_gpu/test_libepseon_gpu.py:38-339) and
extending them with numerical checks of the task results."""
from __future__ import annotations

import gc
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COMPUTE_GROUP_AXES_COUNT = 3


def _m():
    import epseon_backend_gb300.device.cuda as m

    return m


def _configure(configurator, point_count=16500, min_level=0, max_level=0):
    m = _m()
    return (
        configurator.set_hardware_config(potential_buffer_size=16500, group_size=512,
                                         allocation_block_size=16 * 1024 * 1024)
        .set_morse_potential([
            m.MorsePotentialConfig(dissociation_energy=5500.0, equilibrium_bond_distance=0.6, well_width=10,
                                   min_r=0.0, max_r=10.0, point_count=point_count),
            m.MorsePotentialConfig(dissociation_energy=5500.0, equilibrium_bond_distance=0.6, well_width=10,
                                   min_r=0.0, max_r=10.0, point_count=point_count),
        ])
        .set_vibwa_algorithm(mass_atom_0=87.62, mass_atom_1=87.62, integration_step=0.1,
                             min_distance_to_asymptote=0.1, min_level=min_level, max_level=max_level)
    )


def test_create_context_and_version():
    ctx = _m().EpseonComputeContext.create()
    assert repr(ctx)
    assert re.match(r"\d+\.\d+\.\d+\.\d+", ctx.get_vulkan_version()) is not None


def test_physical_device_info():
    ctx = _m().EpseonComputeContext.create()
    devs = list(ctx.get_physical_device_info())
    assert len(devs) > 0
    for d in devs:
        p = d.device_properties
        assert isinstance(p.api_version, str) and isinstance(p.driver_version, str)
        assert isinstance(p.vendor_id, int) and isinstance(p.device_id, int)
        assert p.device_type in ("INTEGRATED_GPU", "DISCRETE_GPU", "VIRTUAL_GPU", "CPU", "OTHER")
        assert isinstance(p.device_name, str) and len(p.device_name) > 0
        assert isinstance(p.pipeline_cache_uuid, list)
        assert isinstance(p.limits.max_compute_shared_memory_size, int)
        assert isinstance(p.limits.max_compute_work_group_count, tuple)
        assert len(p.limits.max_compute_work_group_count) == COMPUTE_GROUP_AXES_COUNT
        assert isinstance(p.limits.max_compute_work_group_invocations, int)
        assert isinstance(p.limits.max_compute_work_group_size, int)
        assert hasattr(p, "sparse_properties")
        assert hasattr(d, "memory_properties")
        assert len(d.memory_properties.memory_heaps) >= 1
        assert d.memory_properties.memory_heaps[0].size > 0


def _interface():
    ctx = _m().EpseonComputeContext.create()
    info = next(iter(ctx.get_physical_device_info()))
    return ctx.get_device_interface(info.device_properties.device_id)


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_configurator_chaining_same_object(precision):
    iface = _interface()
    configurator = iface.get_task_configurator(precision)
    m = _m()
    a = configurator.set_hardware_config(potential_buffer_size=16500, group_size=4096,
                                         allocation_block_size=64 * 1024 * 1024)
    b = a.set_morse_potential([m.MorsePotentialConfig(5500.0, 0.6, 10, 0.0, 10.0, 16500)])
    c = b.set_vibwa_algorithm(87.62, 87.62, 0.1, 0.1, 0, 0)
    assert id(a) == id(b) == id(c) == id(configurator)
    assert c.is_configured()


def test_unknown_precision():
    with pytest.raises(ValueError, match='Invalid PrecisionType literal in string: "float80"'):
        _interface().get_task_configurator("float80")


def test_mixed_point_counts_rejected():
    m = _m()
    cfg = _interface().get_task_configurator("float32")
    with pytest.raises(RuntimeError):
        cfg.set_morse_potential([m.MorsePotentialConfig(5500.0, 0.6, 10, 0.0, 10.0, 100),
                                 m.MorsePotentialConfig(5500.0, 0.6, 10, 0.0, 10.0, 200)])


def test_submit_unconfigured_raises():
    iface = _interface()
    cfg = iface.get_task_configurator("float64")
    with pytest.raises(RuntimeError):
        iface.submit_task(cfg)


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_submit_task_with_ctx_going_out_of_scope(precision):
    ctx = _m().EpseonComputeContext.create()
    info = next(iter(ctx.get_physical_device_info()))
    iface = ctx.get_device_interface(info.device_properties.device_id)
    del ctx
    gc.collect()
    handle = iface.submit_task(_configure(iface.get_task_configurator(precision)))
    assert isinstance(handle.get_status_message(), str)
    handle.wait()
    assert handle.is_done()


def test_results_match_between_precisions_and_analytic():
    from epseon_backend_gb300 import synth

    iface = _interface()
    res = {}
    for precision in ("float32", "float64"):
        h = iface.submit_task(_configure(iface.get_task_configurator(precision), max_level=40))
        h.wait()
        assert h.is_done()
        assert h.get_status_message().startswith("done")
        res[precision] = h.get_results()
    e32, e64 = res["float32"]["energies"], res["float64"]["energies"]
    assert len(e32) == len(e64) == 2
    for a, b in zip(e32, e64):
        assert a.size == b.size > 5
        # 1e-9 Hartree in cm^-1
        assert np.max(np.abs(a - b)) < 1e-9 * 219474.6313632
    for nd in res["float64"]["nodes"]:
        assert np.array_equal(nd, np.arange(nd.size))
    # Sr2-like Morse in spectroscopic units: analytic levels to O(h^4)
    hartree, bohr, dalton = 219474.6313632, 0.529177210903, 1822.888486209
    mu = 87.62 / 2 * dalton
    an = synth.analytic_morse_levels(5500.0 / hartree, 10 * bohr, mu, (5500.0 - 0.1) / hartree) * hartree
    n = min(an.size, e64[0].size)
    assert np.max(np.abs(e64[0][:n] - an[:n])) < 0.05  # cm^-1


def test_cancel_and_wavefunctions():
    iface = _interface()
    cfg = _configure(iface.get_task_configurator("float32"), max_level=5)
    cfg.set_wavefunction_output(True)
    h = iface.submit_task(cfg)
    h.wait()
    r = h.get_results()
    psi = r["wavefunctions"][0]
    rgrid = r["r"][0]
    dr = rgrid[1] - rgrid[0]
    assert psi.shape == (6, rgrid.size)
    assert np.allclose(np.sum(psi ** 2, axis=1) * dr, 1.0, atol=1e-10)
    # cancelling a finished task is a no-op; cancelling a running one stops it
    assert h.cancel() is False
    big = _configure(iface.get_task_configurator("float64"), max_level=60)
    h2 = iface.submit_task(big)
    h2.cancel()
    h2.wait()
    assert h2.is_done()
    assert isinstance(h2.get_status_message(), str)


def test_tabulated_and_file_potentials(tmp_path):
    from epseon_backend_gb300 import synth

    iface = _interface()
    # Morse curve tabulated on the host in cm^-1 / angstrom
    r = np.linspace(0.05, 10.0, 6000)
    V = 5500.0 * (1 - np.exp(-10 * (r - 0.6))) ** 2
    f = tmp_path / "morse.dat"
    np.savetxt(f, np.stack([r, V], 1), header="r[A] V[cm-1]")
    outs = []
    for how in ("tab", "file"):
        cfg = iface.get_task_configurator("float64").set_hardware_config(
            potential_buffer_size=6000, group_size=8, allocation_block_size=1 << 24)
        if how == "tab":
            cfg.set_tabulated_potential([V], min_r=0.05, max_r=10.0, asymptote=5500.0)
        else:
            cfg.set_potential_files([str(f)])
        cfg.set_vibwa_algorithm(87.62, 87.62, 0.5, 0.1, 0, 4)
        h = iface.submit_task(cfg)
        h.wait()
        outs.append(h.get_results()["energies"][0])
    assert np.allclose(outs[0], outs[1], atol=1e-6)
    assert outs[0].size == 5


HARTREE_CM, BOHR_A, DALTON_ME = 219474.6313632, 0.529177210903, 1822.888486209


def test_nonuniform_file_matches_oracle(tmp_path):
    """A two-column (r [angstrom], V [cm^-1]) file on a non-uniform grid takes
    the loader's resampling branch: a natural cubic spline through the file's
    points, evaluated on as many uniform points over [r_first, r_last]
    (potential_source.hpp:44-100 is the reference's stub of this loader).
    Both precisions against the oracle on the same resampled curve (scipy's
    natural spline); energies within 1e-10 Hartree, nodes exact."""
    scipy_interp = pytest.importorskip("scipy.interpolate")
    from oracle import oracle as O

    t = np.linspace(0.0, 1.0, 4000)
    r = 2.0 + 10.0 * t ** 1.4  # denser near the inner wall
    De, a, re = 5000.0, 1.2, 3.0
    V = De * (1 - np.exp(-a * (r - re))) ** 2 + 0.15 * De * np.exp(-((r - 4.2) ** 2) / (2 * 0.3 ** 2))
    f = tmp_path / "nonuniform.dat"
    with open(f, "w") as fh:
        fh.write("# r[A]\tV[cm-1]\n")
        for x, y in zip(r, V):
            fh.write(f"{x:.17g}\t{y:.17g}\n")
    xs = r[0] + (r[-1] - r[0]) / (r.size - 1) * np.arange(r.size)
    xs[-1] = r[-1]
    Vu = scipy_interp.CubicSpline(r, V, bc_type="natural")(xs)
    dist = 0.1
    mu = 87.62 / 2 * DALTON_ME
    e_cap = (Vu[-1] - dist) / HARTREE_CM
    ref = O.solve_batch([Vu / HARTREE_CM], r[0] / BOHR_A, r[-1] / BOHR_A, mu, e_cap, 4096)[0]
    assert ref.n_total > 20
    iface = _interface()
    for precision in ("float64", "float32"):
        cfg = iface.get_task_configurator(precision).set_hardware_config(
            potential_buffer_size=4000, group_size=1, allocation_block_size=1 << 24)
        cfg.set_potential_files([str(f)])
        cfg.set_vibwa_algorithm(87.62, 87.62, 0.5, dist, 0, ref.n_total + 10)
        h = iface.submit_task(cfg)
        h.wait()
        res = h.get_results()
        E = res["energies"][0] / HARTREE_CM
        assert res["n_total"][0] == ref.n_total and E.size == ref.n_total
        assert np.array_equal(res["nodes"][0], np.arange(E.size))
        assert np.max(np.abs(E - ref.energy_polished)) < 1e-10, precision


def _six_morse(m, point_count=6000):
    rng = np.random.default_rng(4)
    return [m.MorsePotentialConfig(dissociation_energy=float(rng.uniform(3000, 6000)),
                                   equilibrium_bond_distance=float(rng.uniform(2.5, 4.0)),
                                   well_width=float(rng.uniform(0.8, 1.5)), min_r=1.0, max_r=20.0,
                                   point_count=point_count) for _ in range(6)]


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_group_size_splits_reproduce_unsplit_batch(precision):
    """HardwareConfig.group_size (hardware_config.hpp:16-18) is the number of
    potentials per device batch.  Splitting a batch into groups of 1 and 4
    reproduces the unsplit batch: bit for bit with the plain FP64 method (its
    arithmetic is per potential, and the trial grid follows the whole task),
    within 1e-10 Hartree with the fast method (the long-window threshold
    follows the batch's level count, so a split may route a level through the
    other pass of the same precision)."""
    m = _m()
    iface = _interface()
    out = {}
    for group in (6, 4, 1):
        cfg = iface.get_task_configurator(precision).set_hardware_config(
            potential_buffer_size=6000, group_size=group, allocation_block_size=1 << 24)
        cfg.set_morse_potential(_six_morse(m)).set_vibwa_algorithm(87.62, 87.62, 0.5, 0.1, 0, 80)
        h = iface.submit_task(cfg)
        h.wait()
        out[group] = h.get_results()
    base = out[6]
    for group in (4, 1):
        r = out[group]
        assert list(r["n_total"]) == list(base["n_total"])
        for a, b, na, nb in zip(r["energies"], base["energies"], r["nodes"], base["nodes"]):
            assert np.array_equal(na, nb)
            if precision == "float64":
                assert np.array_equal(a, b)
            else:
                assert np.max(np.abs(a - b)) < 1e-10 * HARTREE_CM


def test_potential_buffer_size_rejects_longer_grids():
    """HardwareConfig.potential_buffer_size is the longest grid a task
    accepts: a longer one fails the task with a clear message."""
    iface = _interface()
    cfg = _configure(iface.get_task_configurator("float64"))
    cfg.set_hardware_config(potential_buffer_size=1000, group_size=2, allocation_block_size=1 << 24)
    h = iface.submit_task(cfg)
    h.wait()
    assert h.get_status_message().startswith("failed")
    with pytest.raises(RuntimeError, match="exceeds potential_buffer_size"):
        h.get_results()
