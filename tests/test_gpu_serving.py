"""Serving pools and the continuous-batching server on the GPU.

A request in a pool, with others joining and leaving between its chunks,
gives the same bits as the request run alone (a one-request batch, and the
oracle); the server's forward and adjoint results in a mixed stream equal
the same requests served one at a time."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300 import serving as S
from pasif_gb300 import synth
from pasif_gb300.batch import Batch, Plan, Signals
from tests import cases

pytestmark = pytest.mark.gpu


def alone(pat, prec, vals, x0, exc, x, W, im, h, N, max_comp, ms, sq_comp, ss):
    plan = Plan(pat, prec)
    b = Batch(plan, vals, x0, exc)
    b.forward(Signals(x, W, im, prec), h, N, max_comp=max_comp, max_start=ms, sq_comp=sq_comp, sq_start=ss)
    return b.get()


@pytest.mark.parametrize("slicing", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("seed,W", [(0, 4), (1, 0), (2, 8)])
def test_pool_requests_equal_alone(gpu, prec, seed, W, slicing):
    rng = np.random.default_rng(1100 + seed)
    pat, v = cases.random_system(rng)
    if slicing and pat.n < 2:
        pytest.skip("one component: nothing to slice")
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    max_comp, sq_comp, h = (0,), sorted({0, pat.n - 1}), 0.05
    pool = S.Pool(pat, prec, W, im, h, max_comp, sq_comp, capacity=40, arena_samples=4000, chunk=23,
                  slicing=slicing)
    reqs, live, done = [], {}, {}
    for j in range(12):
        m = int(rng.integers(1, 12))
        vals, x0 = cases.random_batch(rng, pat, v, m)
        rows, L = int(rng.integers(1, 4)), int(rng.integers(20, 120))
        reqs.append(dict(vals=vals, x0=x0, x=cases.signals(rng, rows, L), exc=rng.integers(0, rows, m),
                         N=int(rng.integers(10, 150)), ms=int(rng.integers(0, 30)), ss=int(rng.integers(0, 30))))
    pending = list(range(len(reqs)))
    launches = 0
    while pending or live:
        while pending:      # admit while it fits, between chunks
            r = reqs[pending[0]]
            rid = pool.admit(r["vals"], r["x0"], r["exc"], r["x"], r["N"], r["ms"], r["ss"])
            if rid is None:
                break
            live[rid] = pending.pop(0)
        pool.launch()
        launches += 1
        for rid in pool.poll():
            j = live.pop(rid)
            done[j] = pool.harvest(rid, len(reqs[j]["vals"]))
        assert launches < 1000
    assert pool.info()["active"] == 0 and pool.info()["free_slots"] == 40
    for j, r in enumerate(reqs):
        st, mx, sq = done[j]
        a = alone(pat, prec, r["vals"], r["x0"], r["exc"], r["x"], W, im, h, r["N"], max_comp, r["ms"], sq_comp,
                  r["ss"])
        o = O.batch_forward(pat, r["vals"], r["x0"], r["exc"], r["x"], h, r["N"], W, im, prec, 0, max_comp, r["ms"],
                            sq_comp, r["ss"])
        for got, al, orc in zip((st, mx, sq), a, o):
            np.testing.assert_array_equal(got, al)
            np.testing.assert_array_equal(got, orc)


def test_pool_refuses_when_full(gpu):
    w = synth.duffing(n_sys=8, nsteps=100)
    pool = S.Pool(w.pattern, "fp32_kahan", 2, w.im, w.h, (0,), (), capacity=8, arena_samples=3 * 102, chunk=50)
    from pasif_gb300 import _native as N
    a = pool.admit(w.values, w.x0, np.zeros(8, np.int32), w.signals[:1], 100)
    assert a is not None
    assert pool.admit(w.values[:1], w.x0[:1], [0], w.signals[:1], 100) is None      # no free slot
    pool.launch()
    with pytest.raises(N.PasifError) as e:                                          # 50 of 100 steps done
        pool.harvest(a, 8)
    assert e.value.code == N.ERR_STATE
    pool.launch()
    assert pool.poll() == [a]
    pool.harvest(a, 8)
    b = pool.admit(w.values[:4], w.x0[:4], [0, 0, 0, 0], w.signals[:3], 100)
    assert b is not None
    assert pool.admit(w.values[:1], w.x0[:1], [0], w.signals[:1], 100) is None      # arena full
    with pytest.raises(N.PasifError) as e:                                          # can never fit
        pool.admit(np.tile(w.values, (2, 1)), np.tile(w.x0, (2, 1)), np.zeros(16, np.int32), w.signals[:1], 100)
    assert e.value.code == N.ERR_INVALID


def small_stream(seed, n_req=24):
    """Mixed forward/adjoint requests of several classes, small enough to
    check one by one."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_req):
        out.append(synth.ServedRequest(i, "adjoint" if rng.random() < 0.3 else "forward",
                                       int(rng.choice([1, 2, 4, 8])), 0.0, int(rng.integers(1, 300)),
                                       int(rng.integers(500, 4000)), int(rng.integers(1 << 30))))
    return out


def test_server_alone_equals_mix(gpu):
    specs = S.served_specs([1, 2, 4, 8])
    for s in specs.values():
        s.chunk = 256
    stream = small_stream(7)
    reqs = [S.make_request(r, specs[r.dof]) for r in stream]
    srv = S.Server(specs, capacity=2048, arena_samples=1 << 20, adjoint_budget=1 << 30)
    srv.warm()
    out = S.serve_stream(srv, [(0.0, r) for r in reqs], realtime=False, timeout=600)
    srv.stop()
    assert out["complete"] and out["refused"] == 0
    mix = out["results"]
    for r in reqs:
        one = S.Server(specs, capacity=2048, arena_samples=1 << 20, adjoint_budget=1 << 30, adjoint_workers=1)
        o = S.serve_stream(one, [(0.0, r)], realtime=False, timeout=600)["results"][r.rid]
        one.stop()
        m = mix[r.rid]
        assert m.error is None and o.error is None
        if r.kind == "forward":
            np.testing.assert_array_equal(m.state, o.state)
            np.testing.assert_array_equal(m.amplitude, o.amplitude)
        else:
            np.testing.assert_array_equal(m.d_values, o.d_values)
            np.testing.assert_array_equal(m.d_x0, o.d_x0)


def test_served_fp32_kahan_within_bound(gpu):
    """Served FP32-Kahan amplitudes against the same requests in FP64."""
    specs = S.served_specs([2, 8])
    stream = [synth.ServedRequest(0, "forward", 2, 0.0, 200, 20_000, 11),
              synth.ServedRequest(1, "forward", 8, 0.0, 100, 20_000, 12)]
    res = {}
    for prec in ("fp32_kahan", "fp64"):
        srv = S.Server(specs, precision=prec, capacity=1024, arena_samples=1 << 20, adjoint_workers=0)
        out = S.serve_stream(srv, [(0.0, S.make_request(r, specs[r.dof])) for r in stream], realtime=False,
                             timeout=600)
        srv.stop()
        res[prec] = out["results"]
    for r in stream:
        a, b = res["fp32_kahan"][r.rid].amplitude, res["fp64"][r.rid].amplitude
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3)) <= 1e-5
