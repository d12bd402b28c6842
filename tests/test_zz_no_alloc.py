"""pasif_forward_noalloc: the forward solve for callers that cannot allocate
device memory (code running inside another framework's memory pool or under a
fixed memory budget, or code that must not trigger the device synchronisation
cudaMalloc/cudaFree can cause).  It works in a fixed array owned by the
library, so its results must equal the allocating entry point's, call after
call, although every call reuses (and leaves behind) the same work space.  It
queues its work without waiting for the device, so a bad excitation index is
found on the device: that system's row is NaN and the status getter counts it.

Named to be collected last: a failure here leaves every other test run."""
import ctypes as C

import numpy as np
import pytest

from pasif_gb300 import _native as N
from pasif_gb300 import synth
from pasif_gb300.batch import forward

pytestmark = pytest.mark.gpu


def noalloc(w, values, x0, torch, exc_index=None, window=None):
    dev = "cuda"
    window = w.window if window is None else window
    exc = w.exc_index if exc_index is None else exc_index
    tv = torch.tensor(values, dtype=torch.float64, device=dev).contiguous()
    tx = torch.tensor(x0, dtype=torch.float64, device=dev).contiguous()
    te = torch.tensor(exc, dtype=torch.int32, device=dev).contiguous()
    ts = torch.tensor(w.signals, dtype=torch.float64, device=dev).contiguous()
    ti = torch.tensor(np.asarray(w.im).reshape(-1), dtype=torch.float64, device=dev).contiguous()
    out = torch.empty((w.n_sys, w.pattern.n), dtype=torch.float64, device=dev)
    pc = w.pattern.to_c()
    stream = torch.cuda.current_stream()
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = N.lib.pasif_forward_noalloc(C.byref(pc), w.n_sys, p(tv), p(tx), p(te), p(ts), w.signals.shape[0],
                                     w.signals.shape[1], window, p(ti) if window else None, w.h, 0, w.nsteps, p(out),
                                     C.c_void_p(stream.cuda_stream))
    N.check(rc)
    bad, first = C.c_int(-1), C.c_int(-1)
    N.check(N.lib.pasif_forward_noalloc_status(C.byref(bad), C.byref(first), C.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    return out.cpu().numpy(), bad.value, first.value


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    w = synth.coupled2(n_sys=1000, nsteps=1500)
    rng = np.random.default_rng(77)
    runs = [(w.values, w.x0), (w.values * (1 + 0.01 * rng.standard_normal(w.values.shape)),
                                rng.normal(0, 0.1, w.x0.shape))]
    for values, x0 in runs:   # two calls in a row through the same static work space
        got, bad, first = noalloc(w, values, x0, torch)
        ref, _, _ = forward(w.pattern, values, x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im, "fp64")
        np.testing.assert_array_equal(got, ref)
        assert (bad, first) == (0, w.n_sys)


def test_noalloc_sample_and_hold(gpu):
    torch = pytest.importorskip("torch")
    w = synth.coupled2(n_sys=300, nsteps=900)
    for _ in range(2):
        got, bad, _ = noalloc(w, w.values, w.x0, torch, window=0)
        ref, _, _ = forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, 0, None, "fp64")
        np.testing.assert_array_equal(got, ref)
        assert bad == 0


def test_noalloc_out_of_range_index_found_on_device(gpu):
    torch = pytest.importorskip("torch")
    w = synth.coupled2(n_sys=200, nsteps=600)
    exc = w.exc_index.copy()
    exc[[17, 150]] = [w.signals.shape[0], -3]
    got, bad, first = noalloc(w, w.values, w.x0, torch, exc_index=exc)
    assert (bad, first) == (2, 17)
    assert np.isnan(got[[17, 150]]).all()
    keep = np.setdiff1d(np.arange(w.n_sys), [17, 150])
    ref, _, _ = forward(w.pattern, w.values[keep], w.x0[keep], exc[keep], w.signals, w.h, w.nsteps, w.window, w.im,
                        "fp64")
    np.testing.assert_array_equal(got[keep], ref)
    # the next call starts from a clear status
    got, bad, first = noalloc(w, w.values, w.x0, torch)
    assert (bad, first) == (0, w.n_sys) and np.isfinite(got).all()


def test_noalloc_rejects_oversized_batch(gpu):
    w = synth.coupled2(n_sys=8, nsteps=10)
    pc = w.pattern.to_c()
    rc = N.lib.pasif_forward_noalloc(C.byref(pc), 10 ** 7, None, None, None, C.c_void_p(1), 1, 10, 0, None, 1e-3, 0,
                                     1, None, None)
    assert rc == N.ERR_INVALID
    assert "exceeds" in N.last_error()
