"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, validates arguments before touching CUDA, and NVRTC builds
the pattern-specialised kernels for sm_103a."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pasif_gb300 import _native as N
from pasif_gb300 import synth
from pasif_gb300.batch import Plan
from tests import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "pasif_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pasif_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    syms = header_symbols()
    assert len(syms) >= 40
    for s in syms:
        assert hasattr(N.lib, s), s
    assert set(syms) == set(N.EXPORTED)


def test_version_and_no_device_is_not_an_error():
    assert N.lib.pasif_version() == 100
    assert N.device_count() >= 0


def test_invalid_pattern_is_rejected_before_cuda():
    h = C.c_void_p()
    p = N.PatternC()
    p.n = 2
    kptr = np.array([0, 1, 2], np.int32)
    kcol = np.array([0, 5], np.int32)          # column 5 out of range
    p.k_nnz, p.k_ptr, p.k_col = 2, N.iptr(kptr), N.iptr(kcol)
    rc = N.lib.pasif_plan_create(C.byref(h), C.byref(p), 0, 0)
    assert rc == N.ERR_INVALID
    assert "column" in N.last_error()


def test_null_handles():
    assert N.lib.pasif_batch_forward(None, None, 1.0, 0, 1, None, None) == N.ERR_INVALID
    assert N.lib.pasif_driver_allocate_system(None) == N.ERR_INVALID
    assert N.lib.pasif_batch_reserve(None, 1, 1) == N.ERR_INVALID
    assert N.lib.pasif_batch_set_adjoint_storage(None, 0) == N.ERR_INVALID
    assert N.lib.pasif_batch_adjoint(None, None, 1.0, 1, None, None, None, None, None, 0, None) == N.ERR_INVALID
    rid, n = C.c_int(), C.c_int()
    assert N.lib.pasif_pool_admit(None, 1, None, None, None, None, 1, 1, 1, 0, 0, C.byref(rid)) == N.ERR_INVALID
    assert N.lib.pasif_pool_launch(None) == N.ERR_INVALID
    assert N.lib.pasif_pool_poll(None, None, 0, C.byref(n)) == N.ERR_INVALID
    assert N.lib.pasif_pool_harvest(None, 0, None, None, None) == N.ERR_INVALID
    assert "null" in N.last_error()


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32_kahan"])
def test_nvrtc_builds_specialised_kernel_config2(precision):
    """NVRTC compiles the generated sm_103a kernel (no device needed) and the
    bench kernel keeps every value in registers (no spills)."""
    w = synth.coupled2(n_sys=64, nsteps=10)
    rep = Plan(w.pattern, precision).jit_report(w.values)
    m = re.search(r"Used (\d+) registers", rep)
    assert m, rep
    assert re.search(r"\b0 bytes spill stores", rep), rep


@pytest.mark.parametrize("seed", range(3))
def test_nvrtc_builds_random_patterns(seed):
    rng = np.random.default_rng(seed)
    pat, v = cases.random_system(rng)
    vals, _ = cases.random_batch(rng, pat, v, 16)
    rep = Plan(pat, ["fp64", "fp32", "fp32_kahan"][seed]).jit_report(vals, max_mask=1, sq_mask=1)
    assert "registers" in rep


def test_plan_without_device_and_bad_precision():
    pat, v = cases.random_system(np.random.default_rng(1), 3)
    Plan(pat, "fp64")
    with pytest.raises(N.PasifError):
        Plan(pat, 7)


def test_sweep_chunk_rule():
    """Memory-bounded sweeps: all instances at once when they fit the budget,
    else as many per sequential batch as fit, none when one does not."""
    import ctypes as C
    from pasif_gb300 import _native as N
    out = C.c_longlong()

    def chunk(n, per, budget):
        N.check(N.lib.pasif_sweep_chunk(n, per, budget, C.byref(out)))
        return out.value

    assert chunk(1000, 100, 10 ** 6) == 1000
    assert chunk(1000, 100, 10_000) == 100
    assert chunk(1000, 100, 10_050) == 100
    assert chunk(1000, 100, 99) == 0
    assert chunk(0, 100, 10) == 0
    assert chunk(7, 0, 0) == 7
    assert N.lib.pasif_sweep_chunk(-1, 1, 1, C.byref(out)) == N.ERR_INVALID
