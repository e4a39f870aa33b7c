"""The reference's import path for the ``cuda`` device.

User code written against epseon_backend imports devices as
``epseon_backend.device.<name>`` (python/epseon_backend/device/gpu/__init__.py
in the reference).  This package gives the GB300 device that path:
``epseon_backend.device.cuda`` and ``epseon_backend.device.cuda._libepseon_cuda``
resolve to ``epseon_backend_gb300.device.cuda``.  In an installation that
already has the reference's ``epseon_backend`` package, its
``device/cuda/__init__.py`` below is the one file to add to that package.
"""
from __future__ import annotations

__version__ = "0.1.0"
