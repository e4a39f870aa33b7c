"""Compute devices of epseon_backend_gb300 (only ``cuda``)."""
