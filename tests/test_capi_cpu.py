"""CPU-side checks of the drop-in boundary: the C-ABI library loads and exports
every entry point include/epscu.h declares (no compute calls without a GPU),
and the Python extension exposes the reference's class and method names."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from epseon_backend_gb300 import _build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "epscu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(epscu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    _build.build_cuda()
    return C.CDLL(_build.LIB)


def test_header_declarations_are_all_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(capi.EXPORTED) == names


def test_abi_version_and_errors_without_device(lib):
    L = capi.load()
    assert L.epscu_abi_version() == 2
    # invalid arguments are rejected before any CUDA call
    assert L.epscu_create(0, None) == capi.ERR_INVALID
    assert b"NULL" in L.epscu_last_error()
    assert L.epscu_solve(None, None, None, None) == capi.ERR_INVALID


def test_extension_mirrors_reference_names():
    _build.build_pymodule()
    import epseon_backend_gb300.device.cuda as m

    for cls in ("EpseonComputeContext", "ComputeDeviceInterface", "TaskConfiguratorFloat32",
                "TaskConfiguratorFloat64", "TaskHandleFloat32", "TaskHandleFloat64", "MorsePotentialConfig",
                "PhysicalDeviceInfo", "PhysicalDeviceProperties", "PhysicalDeviceSparseProperties", "MemoryHeap",
                "MemoryType"):
        assert hasattr(m, cls), cls
    for meth in ("create", "get_vulkan_version", "get_physical_device_info", "get_device_interface"):
        assert hasattr(m.EpseonComputeContext, meth)
    for meth in ("get_task_configurator", "submit_task"):
        assert hasattr(m.ComputeDeviceInterface, meth)
    for cfg in (m.TaskConfiguratorFloat32, m.TaskConfiguratorFloat64):
        for meth in ("set_hardware_config", "set_morse_potential", "set_vibwa_algorithm", "is_configured",
                     "set_lj_potential", "set_tabulated_potential", "set_potential_files"):
            assert hasattr(cfg, meth), meth
    for h in (m.TaskHandleFloat32, m.TaskHandleFloat64):
        for meth in ("get_status_message", "is_done", "wait", "cancel", "is_running", "get_results"):
            assert hasattr(h, meth)
    c = m.MorsePotentialConfig(dissociation_energy=5500.0, equilibrium_bond_distance=0.6, well_width=10,
                               min_r=0.0, max_r=10.0, point_count=16500)
    assert c.point_count == 16500


def test_context_without_device_raises():
    import epseon_backend_gb300.device.cuda as m

    if capi.device_count() > 0:
        pytest.skip("a device is present")
    with pytest.raises(RuntimeError):
        m.EpseonComputeContext.create()


def test_reference_import_path():
    """The reference's package path for devices (epseon_backend.device.<name>)
    reaches the GB300 device and its extension module unchanged."""
    _build.build_pymodule()
    import importlib

    m = importlib.import_module("epseon_backend.device.cuda")
    ext = importlib.import_module("epseon_backend.device.cuda._libepseon_cuda")
    import epseon_backend_gb300.device.cuda as own

    assert m.EpseonComputeContext is own.EpseonComputeContext
    assert ext.TaskConfiguratorFloat32 is own.TaskConfiguratorFloat32
    for name in own.__all__:
        assert getattr(m, name) is getattr(own, name)
