"""Interfaces of compute devices (the ``cuda`` device only in this tree)."""
from __future__ import annotations
