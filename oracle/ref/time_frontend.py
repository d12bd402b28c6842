"""Time the front-end packing: the reference's PASIf.setSystems (pure-Python
block-diagonal unfolding and -M^-1 preprocessing, PASIf.py:202-402,
475-633) against pasif_gb300.frontend.PASIf.setSystems (vectorised), on the
same seeded 2-DOF coupled systems, with the driver calls replaced by no-ops
(only the packing is timed; tests/test_frontend_ref.py checks that both hand
the driver the same arrays bit for bit).

    python oracle/ref/time_frontend.py [systems ...]      (default 1024 4096 16384)

Reads the reference's PASIf.py from $PASIF_REF (default /root/reference);
without it, only ours is timed.  CPU only.
"""
from __future__ import annotations

import json
import os
import sys
import time
import types

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from pasif_gb300 import PASIfgpu, frontend  # noqa: E402
from tests import frontend_cases as FC  # noqa: E402

REF = os.environ.get("PASIF_REF", "/root/reference")


def silence_driver():
    cls = getattr(PASIfgpu, "__GpuDriver")
    cls.__init__ = lambda self, *a, **k: None
    cls.__del__ = lambda self: None
    for name in FC.DRIVER_METHODS:
        setattr(cls, name, lambda self, *a: 0)


def reference_module():
    if not os.path.exists(os.path.join(REF, "PASIf.py")):
        return None
    mpi = types.ModuleType("mpi4py")
    mpi.MPI = types.SimpleNamespace(COMM_WORLD=types.SimpleNamespace(Get_rank=lambda: 0))
    sys.modules["mpi4py"] = mpi
    sys.modules["PASIfgpu"] = PASIfgpu
    sys.path.insert(0, REF)
    import PASIf as ref
    return ref


def systems(ct, n_sys, seed=2):
    rng = np.random.default_rng(seed)
    sy = [FC._coupled_system(rng, ct) for _ in range(n_sys)]
    return [list(col) for col in zip(*sy)]


def time_set(cls, ct, n_sys):
    exc = FC.excitations(np.random.default_rng(1))
    p = cls(exc, 1000, 300)
    args = systems(ct, n_sys)
    t = time.perf_counter()
    p.setSystems(*args)
    return time.perf_counter() - t


def main(argv):
    sizes = [int(a) for a in argv] or [1024, 4096, 16384]
    silence_driver()
    ref = reference_module()
    for n in sizes:
        row = {"systems": n, "ours_s": round(time_set(frontend.PASIf, frontend.coo_tensor, n), 3)}
        if ref is not None:
            row["reference_s"] = round(time_set(ref.PASIf, ref.coo_tensor, n), 3)
            row["speedup"] = round(row["reference_s"] / row["ours_s"], 1)
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
