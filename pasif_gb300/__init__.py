"""pasif_gb300: GB300-native (sm_103a) engine for PASIf's hot path.

Batched fixed-step RK4 integration of polynomial first-order systems driven
by sampled excitations (forward), the reference's __GpuDriver API as a
drop-in (PASIfgpu), an exact discrete adjoint behind torch.autograd
(pasif_gb300.autograd) and the reference's own _getGradient semantics.
"""
from __future__ import annotations

import sys

from .system import Pattern, reducers_c

__all__ = ["Pattern", "Plan", "Signals", "Batch", "forward", "install_dropin", "reducers_c"]


def __getattr__(name):
    """The batch interface (and with it libpasif_gb300.so) is loaded on first
    use: importing the package for its pattern or synthetic-workload helpers
    maps no native library."""
    if name in ("Batch", "Plan", "Signals", "forward"):
        from . import batch
        return getattr(batch, name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")


def install_dropin() -> None:
    """Make `from PASIfgpu import __GpuDriver` (PASIf.py:17) resolve to this
    package's drop-in class."""
    from . import PASIfgpu
    sys.modules["PASIfgpu"] = PASIfgpu
