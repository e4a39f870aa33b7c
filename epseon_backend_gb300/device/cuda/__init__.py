"""The ``cuda`` device: a drop-in for ``epseon_backend.device.gpu``.

``_libepseon_cuda`` exposes the reference's object model
(EpseonComputeContext -> ComputeDeviceInterface -> TaskConfigurator{Float32,
Float64} -> TaskHandle{Float32,Float64}) on the GB300 solver.  "float32"
selects the FP32-compensated solver with FP64 polish, "float64" the plain FP64
solver.  Units: cm^-1, angstrom, unified atomic mass units.
"""
from __future__ import annotations

from ._libepseon_cuda import (  # noqa: F401
    ComputeDeviceInterface,
    EpseonComputeContext,
    LennardJonesPotentialConfig,
    MemoryHeap,
    MemoryType,
    MorsePotentialConfig,
    PhysicalDeviceInfo,
    PhysicalDeviceProperties,
    PhysicalDeviceSparseProperties,
    TaskConfiguratorFloat32,
    TaskConfiguratorFloat64,
    TaskHandleFloat32,
    TaskHandleFloat64,
)

__all__ = [
    "ComputeDeviceInterface",
    "EpseonComputeContext",
    "LennardJonesPotentialConfig",
    "MemoryHeap",
    "MemoryType",
    "MorsePotentialConfig",
    "PhysicalDeviceInfo",
    "PhysicalDeviceProperties",
    "PhysicalDeviceSparseProperties",
    "TaskConfiguratorFloat32",
    "TaskConfiguratorFloat64",
    "TaskHandleFloat32",
    "TaskHandleFloat64",
]
