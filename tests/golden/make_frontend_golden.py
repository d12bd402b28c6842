"""Record what the REFERENCE's own front end hands its driver.

Run in a container that holds the PASIf sources (PASIF_REF, default
/root/reference), from the repository root:

    python tests/golden/make_frontend_golden.py

The reference's PASIf.py is imported unmodified: `mpi4py` is replaced by a
one-rank stand-in (PASIf.py:27-30) and the compiled module `PASIfgpu` by a
recording `__GpuDriver` (PASIf.py:17), so that setSystems / setJacobian /
setInterpolationMatrix (PASIf.py:202-402) run their block-diagonal
unfolding, -M^-1 preprocessing and CSR packing (PASIf.py:475-633) and call
the driver's setters.  Every call and its arguments are stored in
tests/golden/frontend_calls_<case>.npz; tests/test_frontend_ref.py checks that
pasif_gb300.frontend.PASIf makes the same calls with the same arrays, bit for
bit, and tests/test_gpu_dropin.py replays them on the drop-in driver.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from tests import frontend_cases as FC  # noqa: E402

REF = os.environ.get("PASIF_REF", "/root/reference")
OUT = os.path.join(ROOT, "tests", "golden")

CALLS: list = []


class _Rank0:
    def Get_rank(self):
        return 0


def _recording_driver():
    def make(name):
        def method(self, *args):
            CALLS.append((name, FC.as_arrays(args)))
            return 0
        return method

    def init(self, excitationSet, sampleRate, numsteps, dCompute=False, dSystem=False, dSolver=False, GPUId=0):
        CALLS.append(("__init__", FC.as_arrays([excitationSet, sampleRate, numsteps, dCompute, dSystem, dSolver,
                                                GPUId])))

    body = {name: make(name) for name in FC.DRIVER_METHODS}
    body["__init__"] = init
    return type("__GpuDriver", (), body)


def main():
    mpi = types.ModuleType("mpi4py")
    mpi.MPI = types.SimpleNamespace(COMM_WORLD=_Rank0())
    sys.modules["mpi4py"] = mpi
    drv = types.ModuleType("PASIfgpu")
    setattr(drv, "__GpuDriver", _recording_driver())
    sys.modules["PASIfgpu"] = drv
    sys.path.insert(0, REF)
    import PASIf as ref   # the reference's front end, unmodified

    for name in FC.CASES:
        CALLS.clear()
        FC.run_front_end(ref.PASIf, FC.make_case(name, ref.coo_tensor))
        arrays = {}
        for k, (meth, args) in enumerate(CALLS):
            arrays[f"c{k:02d}_{meth}_n"] = np.asarray(len(args))   # calls without arguments too
            for j, a in enumerate(args):
                arrays[f"c{k:02d}_{meth}_a{j}"] = np.asarray(a)
        path = os.path.join(OUT, f"frontend_calls_{name}.npz")
        np.savez_compressed(path, **arrays)
        print(path, len(CALLS), "calls")


if __name__ == "__main__":
    main()
