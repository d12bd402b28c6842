"""Host logic of the serving loop, driven with fake pools and a fake adjoint
runner (no GPU): first-come-first-served admission by free slots and arena
space, refusal of requests that can never fit, the adjoint memory budget,
and latency bookkeeping."""
import threading
import time

import numpy as np
import pytest

from pasif_gb300 import _native as N
from pasif_gb300 import serving as S
from pasif_gb300.system import Pattern

PAT = Pattern.from_dense_lists(2, [0, 1], [1, 0], (), (), (), [1])[0]


class FakePool:
    """Slots and arena like pasif_pool: admit fails when either is short;
    launch advances every request by `chunk` steps."""

    def __init__(self, capacity, arena, chunk, log):
        self.capacity, self.arena, self.chunk = capacity, arena, chunk
        self.free, self.used_arena = capacity, 0
        self.reqs, self.next, self.log = {}, 1, log

    def admit(self, values, x0, exc_index, signals, nsteps, max_start=0, sq_start=0):
        m, t = len(values), np.asarray(signals).size
        if nsteps < 0:   # as pasif_pool_admit: invalid input is an error, not a wait
            raise N.PasifError(N.ERR_INVALID, "negative step count")
        np.asarray(x0, dtype=float).reshape(m, 2)   # as Pool.admit's shape checks
        if m > self.free or t > self.arena - self.used_arena:
            return None
        rid, self.next = self.next, self.next + 1
        self.free -= m
        self.used_arena += t
        self.reqs[rid] = [nsteps, m, t, np.asarray(values)]
        self.log.append(("admit", rid, self.capacity - self.free))
        return rid

    def launch(self):
        for r in self.reqs.values():
            r[0] -= self.chunk

    def poll(self):
        return [rid for rid, r in self.reqs.items() if r[0] <= 0]

    def harvest(self, rid, n_sys):
        _, m, t, v = self.reqs.pop(rid)
        self.free += m
        self.used_arena -= t
        return v[:, :2] * 2.0, v[:, :1], v[:, 0]


def make_server(capacity=8, arena=1000, budget=100, workers=2, runner=None, log=None):
    log = [] if log is None else log
    spec = S.ClassSpec(PAT, 0.01, 0, None, (0,), chunk=10)
    return S.Server({"a": spec}, capacity=capacity, arena_samples=arena, adjoint_budget=budget,
                    adjoint_workers=workers, pool_factory=lambda sp: FakePool(capacity, arena, sp.chunk, log),
                    adjoint_runner=runner or (lambda sp, rq, st: (rq.values * 3.0, rq.x0)),
                    stream_factory=lambda prio: None), log


def req(rid, kind, n, nsteps=25, table=10):
    return S.Request(rid, kind, "a", np.full((n, PAT.P), float(rid)), np.zeros((n, 2)), np.zeros(n, np.int32),
                     np.zeros((1, table)), nsteps)


def test_forward_admission_and_results():
    srv, log = make_server()
    srv.start()
    for i, n in enumerate([6, 6, 3, 8, 9]):
        srv.submit(req(i, "forward", n))
    assert srv.wait(10.0)
    srv.stop()
    res = srv.results()
    assert res[4].error and "larger than a serving pool" in res[4].error
    for i, n in enumerate([6, 6, 3, 8]):
        assert res[i].error is None
        np.testing.assert_array_equal(res[i].state, np.full((n, 2), 2.0 * i))
        assert res[i].t_arrival <= res[i].t_admit <= res[i].t_done
    assert max(busy for _, _, busy in log) <= 8          # never more slots than the pool has
    order = [rid for ev, rid, _ in log if ev == "admit"]
    assert order == sorted(order)                       # first come, first served


def test_arena_limits_admission():
    srv, log = make_server(capacity=64, arena=25)
    srv.start()
    for i in range(4):
        srv.submit(req(i, "forward", 1, table=10))      # two tables fit at a time
    srv.submit(req(9, "forward", 1, table=26))           # never fits
    assert srv.wait(10.0)
    srv.stop()
    res = srv.results()
    assert res[9].error is not None
    assert all(res[i].error is None for i in range(4))



def test_invalid_forward_request_fails_alone():
    """A request the pool rejects as invalid gets an error result; the
    class's pool goes on serving the others."""
    srv, log = make_server()
    srv.start()
    srv.submit(req(0, "forward", 2))
    srv.submit(req(1, "forward", 2, nsteps=-5))
    srv.submit(req(2, "forward", 3))
    bad = req(3, "forward", 2)
    bad.x0 = np.zeros((3, 2))   # three initial states for two systems
    srv.submit(bad)
    with pytest.raises(AttributeError):   # not a request at all: raised to the caller, not registered
        srv.submit(S.Request(4, "forward", "a", "not an array", None, None, np.zeros((1, 4)), 10))
    assert srv.wait(10.0)
    srv.stop()
    res = srv.results()
    assert res[1].error and "forward refused" in res[1].error
    assert res[3].error and "forward refused" in res[3].error
    assert 4 not in res
    assert res[0].error is None and res[2].error is None
    np.testing.assert_array_equal(res[2].state, np.full((3, 2), 4.0))

def test_unknown_class_or_failing_pool_fails_the_request():
    """A request of a class the server does not serve, or whose pool cannot be
    made, gets an error result at once: wait() does not wait for it."""
    srv, _ = make_server()
    srv.start()
    for kind in ("forward", "adjoint"):
        r = req(0 if kind == "forward" else 1, kind, 2)
        r.cls = "no such class"
        srv.submit(r)
    srv.submit(req(2, "forward", 2))
    assert srv.wait(5.0)
    res = srv.results()
    assert "unknown request class" in res[0].error and "unknown request class" in res[1].error
    assert res[2].error is None
    srv.stop()

    def broken(spec):
        raise RuntimeError("kernel build failed")
    srv = S.Server({"a": S.ClassSpec(PAT, 0.01, 0, None, (0,), chunk=10)}, capacity=8, arena_samples=1000,
                   adjoint_budget=100, adjoint_workers=1, pool_factory=broken,
                   adjoint_runner=lambda sp, rq, st: (rq.values, rq.x0), stream_factory=lambda prio: None)
    srv.start()
    srv.submit(req(5, "forward", 2))
    assert srv.wait(5.0)
    assert "unavailable" in srv.results()[5].error
    srv.stop()


def test_adjoint_budget():
    lock, state = threading.Lock(), {"now": 0, "peak": 0}
    need = S.adjoint_bytes(PAT, 4, 25, 10, "fp32_kahan")

    def runner(spec, rq, stream):
        with lock:
            state["now"] += need
            state["peak"] = max(state["peak"], state["now"])
        threading.Event().wait(0.02)
        with lock:
            state["now"] -= need
        return rq.values * 3.0, rq.x0

    srv, _ = make_server(budget=need + need // 2, workers=3, runner=runner)   # one adjoint at a time
    srv.start()
    for i in range(4):
        srv.submit(req(i, "adjoint", 4))
    srv.submit(req(7, "adjoint", 400))                   # larger than the whole budget
    assert srv.wait(10.0)
    srv.stop()
    res = srv.results()
    assert res[7].error is not None and "budget" in res[7].error
    for i in range(4):
        assert res[i].error is None
        np.testing.assert_array_equal(res[i].d_values, np.full((4, PAT.P), 3.0 * i))
    assert state["peak"] == need


def test_adjoint_errors():
    """A request whose solve returns an error status gets an error result and
    the worker serves the next; any other exception stops the server and is
    raised by wait()."""
    from pasif_gb300 import _native as N

    def runner(spec, rq, stream):
        if rq.rid == 0:
            raise N.PasifError(N.ERR_INVALID, "bad request")
        if rq.rid == 2:
            raise RuntimeError("boom")
        return rq.values, rq.x0

    srv, _ = make_server(budget=1 << 30, workers=1, runner=runner)
    srv.start()
    srv.submit(req(0, "adjoint", 1))
    srv.submit(req(1, "adjoint", 1))
    assert srv.wait(10.0)
    res = srv.results()
    assert "bad request" in res[0].error and res[1].error is None
    srv.submit(req(2, "adjoint", 1))
    with pytest.raises(RuntimeError, match="boom"):
        srv.wait(10.0)
    srv.stop()


def test_adjoint_classes_do_not_block_each_other():
    """Each class has its own adjoint queue and workers: a cheap request is
    served while long requests of another class are still running."""
    spec = S.ClassSpec(PAT, 0.01, 0, None, (0,), chunk=10)
    release = threading.Event()

    def runner(sp, rq, stream):
        if rq.cls == "slow":
            release.wait(10.0)
        return rq.values, rq.x0

    srv = S.Server({"slow": spec, "fast": spec}, adjoint_budget=1 << 30, adjoint_workers=1,
                   pool_factory=lambda sp: FakePool(8, 1000, sp.chunk, []), adjoint_runner=runner,
                   stream_factory=lambda prio: None)
    srv.start()
    for i in range(3):
        rq = req(i, "adjoint", 1)
        rq.cls = "slow"
        srv.submit(rq)
    fast = req(9, "adjoint", 1)
    fast.cls = "fast"
    srv.submit(fast)
    deadline = time.time() + 10.0
    while np.isnan(srv.results()[9].t_done) and time.time() < deadline:
        time.sleep(0.01)
    assert not np.isnan(srv.results()[9].t_done)          # done while the slow class is still blocked
    assert all(np.isnan(srv.results()[i].t_done) for i in range(3))
    release.set()
    assert srv.wait(10.0)
    srv.stop()


def test_percentile():
    assert S.percentile([3.0, 1.0, 2.0], 50) == 2.0
    assert S.percentile([1.0, 2.0], 99) == pytest.approx(1.99)


def test_served_stream_shape():
    from pasif_gb300 import synth
    st = synth.served_stream(rate=200.0, duration=2.0, seed=1)
    assert 300 < len(st) < 500
    assert all(1 <= r.n_sys <= 4096 and 10_000 <= r.nsteps <= 200_000 for r in st)
    assert all(a.arrival < b.arrival for a, b in zip(st, st[1:]))
    frac = sum(r.kind == "adjoint" for r in st) / len(st)
    assert 0.2 < frac < 0.4
    assert {r.dof for r in st} == set(synth.SERVED_DOFS)


def test_adjoint_bytes_stored_or_checkpointed():
    """A request whose forward trajectory fits the per-worker storage books
    the trajectory instead of checkpoints and the recomputed chunk; FP64
    slots hold the stage inputs too."""
    n, N, B = PAT.n, 1000, 8
    ck = S.adjoint_bytes(PAT, B, N, 10, "fp32_kahan")
    full = B * (N + 1) * n * 4
    st = S.adjoint_bytes(PAT, B, N, 10, "fp32_kahan", storage=full)
    # ceil(sqrt(1000)) = 32 steps per chunk, 32 chunks: checkpoints, 33 chunk slots, the replay state
    assert st - ck == full - B * 4 * (2 * n * 32 + 33 * n + n)
    assert S.adjoint_bytes(PAT, B, N, 10, "fp32_kahan", storage=full - 1) == ck
    full64 = B * (4 * N + 1) * n * 8
    assert S.adjoint_bytes(PAT, B, N, 10, "fp64", storage=full64) > S.adjoint_bytes(PAT, B, N, 10, "fp64")
