"""Served mixed stream: Poisson arrivals of forward and adjoint sweep requests
through the continuous-batching server, latency p50/p99 and throughput.

    python -m pasif_gb300.serve --rate 200 --duration 1.5

Prints one JSON object.  Requests (values, excitations) are generated before
the stream starts; the clock of each request runs from its arrival time to
the moment its result is on the host.  After the stream a sample of requests
is served again one at a time (same precision: must be bit-identical to the
result in the mix) and in FP64 (relative error of the FP32-Kahan amplitudes
and gradients)."""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import serving as S
from . import synth


def adjoint_workers_for(n: int) -> int:
    """Adjoint workers of a served class with n states (see run)."""
    if n >= 60:
        return 6
    if n >= 16:
        return 4
    return 3 if n >= 8 else 2


def run(rate=200.0, duration=1.5, seed=5, precision="fp32_kahan", dofs=None, capacity=16384,
        arena_samples=1 << 25, adjoint_budget=96 << 30, adjoint_workers=None, adjoint_storage=3 << 30, check=6,
        log=None) -> dict:
    dofs = tuple(dofs or synth.SERVED_DOFS)
    specs = S.served_specs(dofs)
    stream = synth.served_stream(rate, duration, seed, dofs=dofs)
    t = time.perf_counter()
    reqs = [(sr.arrival, S.make_request(sr, specs[sr.dof])) for sr in stream]
    t_gen = time.perf_counter() - t
    if adjoint_workers is None:
        # More workers where one adjoint is long and holds few SMs (the 32- and
        # 64-DOF classes, one block per SM).  Measured on GB300, this stream,
        # p99 over runs: 2/2/3/4/4/10/6 workers (1..64 DOF) 2.3-2.8 s; these
        # counts (2/2/3/4/4/6/6) 2.22-2.25 s, forward p99 1.1 s; 6 for the
        # 8-DOF class or 8 for the 64-DOF class changed nothing beyond the
        # run-to-run spread (2.05-2.75 s).
        adjoint_workers = {d: adjoint_workers_for(s.pattern.n) for d, s in specs.items()}
    srv = S.Server(specs, precision, capacity, arena_samples, adjoint_budget, adjoint_workers,
                   reserve=(4096, 200_000, 4 * 200_003), adjoint_storage=adjoint_storage)
    t = time.perf_counter()
    srv.warm()
    t_warm = time.perf_counter() - t
    if log:
        log(f"{len(reqs)} requests generated in {t_gen:.1f}s, kernels ready in {t_warm:.1f}s")
    out = S.serve_stream(srv, reqs, realtime=True)
    chunks = dict(srv.chunks)
    srv.stop()
    res = out["results"]
    by_id = {r.rid: (sr, r) for sr, (_, r) in zip(stream, reqs)}
    ok = [x for x in res.values() if x.error is None]
    work = sum(by_id[x.rid][0].n_sys * by_id[x.rid][0].nsteps for x in ok)
    lat = lambda kind: [x.latency * 1e3 for x in ok if x.kind == kind]
    summary = {
        "rate_per_s": rate, "arrival_window_s": duration, "requests": len(reqs),
        "completed": len(ok), "refused_or_failed": len(res) - len(ok),
        "forward": len(lat("forward")), "adjoint": len(lat("adjoint")),
        "p50_ms": round(out["p50_ms"], 2), "p99_ms": round(out["p99_ms"], 2),
        "forward_p50_ms": round(S.percentile(lat("forward"), 50), 2),
        "forward_p99_ms": round(S.percentile(lat("forward"), 99), 2),
        "adjoint_p50_ms": round(S.percentile(lat("adjoint"), 50), 2),
        "adjoint_p99_ms": round(S.percentile(lat("adjoint"), 99), 2),
        "wall_s": round(out["wall_s"], 3),
        "system_steps_per_s": work / out["wall_s"],
        "requests_per_s": len(ok) / out["wall_s"],
        "precision": precision, "chunk_launches": {str(k): v for k, v in sorted(chunks.items())},
        "kernels_ready_s": round(t_warm, 1),
        "adjoint_memory": {"budget_bytes": int(adjoint_budget), "stored_trajectory_bytes_per_worker": int(adjoint_storage),
                           "workers": {str(k): v for k, v in sorted(adjoint_workers.items())}
                           if isinstance(adjoint_workers, dict) else adjoint_workers},
        "errors": sorted({x.error for x in res.values() if x.error})[:5],
        "by_dof": {str(d): {kind: {"n": len(v), "p50_ms": round(S.percentile(v, 50), 1),
                                   "p99_ms": round(S.percentile(v, 99), 1)}
                            for kind in ("forward", "adjoint")
                            for v in [[x.latency * 1e3 for x in ok if x.kind == kind and by_id[x.rid][0].dof == d]]}
                   for d in dofs},
    }
    if check:
        summary.update(_check(specs, reqs, res, precision, check, seed))
    return summary


def _check(specs, reqs, res, precision, k, seed) -> dict:
    """Serve k requests of the stream (the smallest of each kind) alone, in
    the same precision and in FP64."""
    ok = sorted((r for _, r in reqs if res[r.rid].error is None), key=lambda r: r.n_sys * r.nsteps)
    pick = [r for r in ok if r.kind == "forward"][:(k + 1) // 2] + [r for r in ok if r.kind == "adjoint"][:k // 2]
    same, err_amp, err_grad = True, 0.0, 0.0
    for prec in (precision, "fp64"):
        srv = S.Server(specs, prec, 4096, 1 << 23, 8 << 30, 1)
        alone = {}
        for r in pick:
            alone[r.rid] = S.serve_stream(srv, [(0.0, r)], realtime=False)["results"][r.rid]
        srv.stop()
        for r in pick:
            a, m = alone[r.rid], res[r.rid]
            if r.kind == "forward":
                if prec == precision:
                    same &= bool(np.array_equal(a.state, m.state) and np.array_equal(a.amplitude, m.amplitude))
                else:
                    err_amp = max(err_amp, _rel(m.amplitude, a.amplitude))
            else:
                if prec == precision:
                    same &= bool(np.array_equal(a.d_values, m.d_values) and np.array_equal(a.d_x0, m.d_x0))
                else:
                    err_grad = max(err_grad, _rel(m.d_values, a.d_values))
    return {"checked": len(pick), "alone_equals_mix": same, "amplitude_max_rel_err_vs_fp64": err_amp,
            "gradient_max_rel_err_vs_fp64": err_grad}


def _rel(a, b) -> float:
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def main():
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")   # pools and adjoint workers on their own queues
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--duration", type=float, default=1.5)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--precision", default="fp32_kahan")
    ap.add_argument("--dofs", type=str, default="")
    ap.add_argument("--check", type=int, default=6)
    ap.add_argument("--adjoint-storage", type=float, default=3.0,
                    help="GiB per adjoint worker for stored forward trajectories (0: always checkpointed)")
    a = ap.parse_args()
    dofs = tuple(int(x) for x in a.dofs.split(",")) if a.dofs else None
    print(json.dumps(run(a.rate, a.duration, a.seed, a.precision, dofs, check=a.check,
                         adjoint_storage=int(a.adjoint_storage * (1 << 30)), log=lambda m: print(m, flush=True))))


if __name__ == "__main__":
    main()
