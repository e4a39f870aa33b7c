"""Shared fixtures; registers the ``gpu`` marker (tests that need a GB300)."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a) and the built libepseon_cuda")


@pytest.fixture(scope="session")
def ctx():
    from epseon_backend_gb300 import capi

    if capi.device_count() < 1:
        pytest.fail("no CUDA device visible: the gpu tests must run on a GB300")
    c = capi.Context(0)
    yield c
    c.close()
