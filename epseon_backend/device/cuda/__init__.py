"""``epseon_backend.device.cuda``: the GB300 device under the reference's
package path (the sibling of ``epseon_backend.device.gpu``).  The extension
module is registered as ``epseon_backend.device.cuda._libepseon_cuda`` too, so
both ``import epseon_backend.device.cuda._libepseon_cuda`` and
``from epseon_backend.device.cuda import EpseonComputeContext`` work
unchanged."""
from __future__ import annotations

import sys

from epseon_backend_gb300.device.cuda import _libepseon_cuda
from epseon_backend_gb300.device.cuda import *  # noqa: F401,F403
from epseon_backend_gb300.device.cuda import __all__ as _names  # noqa: F401

sys.modules[__name__ + "._libepseon_cuda"] = _libepseon_cuda
__all__ = list(_names)
