"""The front end against the REFERENCE's own front end (CPU).

tests/golden/frontend_calls_<case>.npz hold the driver calls that the
reference's unmodified PASIf.py makes for seeded inputs (recorded by
tests/golden/make_frontend_golden.py: block-diagonal unfolding, -M^-1
preprocessing, CSR packing, PASIf.py:202-402, 475-633).  Here
pasif_gb300.frontend.PASIf runs on the same inputs over a recording driver:
the same setters must be called in the same order with the same arrays, bit
for bit.  When the reference's sources are present, the reference's
PASIf.py is also run directly over our drop-in's recording driver."""
import os
import sys
import types

import numpy as np
import pytest

from pasif_gb300 import PASIfgpu, frontend
from tests import frontend_cases as FC

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_calls(case):
    z = np.load(os.path.join(GOLDEN, f"frontend_calls_{case}.npz"))
    calls = {}
    for key in z.files:
        k, rest = key[1:].split("_", 1)
        if rest.endswith("_n"):   # argument count (calls without arguments are recorded by it alone)
            calls.setdefault(int(k), (rest[:-2], {}))
            continue
        meth, arg = rest.rsplit("_a", 1)
        calls.setdefault(int(k), (meth, {}))[1][int(arg)] = z[key]
    return [(calls[k][0], [calls[k][1][j] for j in sorted(calls[k][1])]) for k in sorted(calls)]


@pytest.fixture
def recording_driver(monkeypatch):
    """Replaces the drop-in's driver methods by recorders (no device work)."""
    calls = []
    cls = getattr(PASIfgpu, "__GpuDriver")

    def init(self, excitationSet_, sampleRate_, numsteps_, dCompute_=False, dSystem_=False, dSolver_=False,
             GPUId_=0, precision="fp64"):
        calls.append(("__init__", FC.as_arrays([excitationSet_, sampleRate_, numsteps_, dCompute_, dSystem_,
                                                dSolver_, GPUId_])))

    def make(name):
        def method(self, *args):
            calls.append((name, FC.as_arrays(args)))
            return 0
        return method

    monkeypatch.setattr(cls, "__init__", init)
    monkeypatch.setattr(cls, "__del__", lambda self: None)
    for name in FC.DRIVER_METHODS:
        monkeypatch.setattr(cls, name, make(name))
    return calls


def assert_same_calls(got, ref):
    assert [m for m, _ in got] == [m for m, _ in ref]
    for (meth, ga), (_, ra) in zip(got, ref):
        assert len(ga) == len(ra), meth
        for j, (g, r) in enumerate(zip(ga, ra)):
            g, r = np.asarray(g), np.asarray(r)
            if g.dtype.kind in "iub" or r.dtype.kind in "iub":
                assert g.shape == r.shape and np.array_equal(g.astype(np.int64), r.astype(np.int64)), (meth, j)
            else:
                np.testing.assert_array_equal(g.astype(np.float64), r.astype(np.float64), err_msg=f"{meth} arg {j}")


@pytest.mark.parametrize("case", FC.CASES)
def test_front_end_hands_the_driver_what_the_reference_does(recording_driver, case):
    ref = load_calls(case)
    FC.run_front_end(frontend.PASIf, FC.make_case(case, frontend.coo_tensor))
    assert_same_calls(recording_driver, ref)


REF = os.environ.get("PASIF_REF", "/root/reference")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "PASIf.py")), reason="reference sources not present")
@pytest.mark.parametrize("case", FC.CASES)
def test_reference_front_end_runs_on_the_drop_in(recording_driver, monkeypatch, case):
    """The reference's PASIf.py, unmodified, imported with `PASIfgpu` resolved
    to this package's drop-in (mpi4py replaced by a one-rank stand-in): its
    calls equal the recorded ones (and therefore ours)."""
    mpi = types.ModuleType("mpi4py")
    mpi.MPI = types.SimpleNamespace(COMM_WORLD=types.SimpleNamespace(Get_rank=lambda: 0))
    monkeypatch.setitem(sys.modules, "mpi4py", mpi)
    monkeypatch.setitem(sys.modules, "PASIfgpu", PASIfgpu)
    monkeypatch.syspath_prepend(REF)
    monkeypatch.delitem(sys.modules, "PASIf", raising=False)
    import PASIf as ref
    FC.run_front_end(ref.PASIf, FC.make_case(case, ref.coo_tensor))
    assert_same_calls(recording_driver, load_calls(case))
