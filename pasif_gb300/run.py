"""Run one synthetic configuration's forward solve from the command line.

    python -m pasif_gb300.run --config coupled2 --systems 16384 --nsteps 20000 \
        --precision fp32_kahan --repeat 3

Builds the seeded workload of pasif_gb300.synth, uploads it once, runs the
forward solve `repeat` times on the current GPU and prints the device time of
the last solve, the throughput and a checksum of the final states.  Used to
profile one kernel on a chosen size.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import synth
from .batch import Batch, Plan, Signals


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="coupled2", choices=sorted(synth.CONFIGS))
    ap.add_argument("--systems", type=int, default=None)
    ap.add_argument("--nsteps", type=int, default=None)
    ap.add_argument("--precision", default="fp32_kahan", choices=["fp64", "fp32", "fp32_kahan", "fp32_ext"])
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--generic", action="store_true", help="use the pattern-interpreting kernel")
    ap.add_argument("--adjoint", action="store_true", help="run the exact adjoint (gradients) instead")
    a = ap.parse_args(argv)
    kw = {}
    if a.systems:
        kw["n_sys"] = a.systems
    if a.nsteps:
        kw["nsteps"] = a.nsteps
    w = synth.CONFIGS[a.config](**kw)
    plan = Plan(w.pattern, a.precision, generic_only=a.generic)
    sig = Signals(w.signals, w.window, w.im, a.precision)
    b = Batch(plan, w.values, w.x0, w.exc_index)
    dt = 0.0
    if a.adjoint:
        g_sq = np.ones(w.n_sys)
        for _ in range(max(1, a.repeat)):
            t0 = time.perf_counter()
            dv, dx = b.adjoint(sig, w.h, w.nsteps, g_sq=g_sq, sq_comp=w.sq_comp or (0,), sq_start=w.sq_start)
            dt = time.perf_counter() - t0
        print(json.dumps({"config": a.config, "systems": w.n_sys, "nsteps": w.nsteps, "precision": a.precision,
                          "adjoint_seconds_last": dt, "gradients_per_s": w.n_sys / dt,
                          "adjoint_system_steps_per_s": w.n_sys * w.nsteps / dt,
                          "checksum": float(np.sum(np.abs(dv)))}))
        return
    for _ in range(max(1, a.repeat)):
        t0 = time.perf_counter()
        b.forward(sig, w.h, w.nsteps, **w.forward_kwargs())
        st, mx, sq = b.get()
        dt = time.perf_counter() - t0
    print(json.dumps({"config": a.config, "systems": w.n_sys, "nsteps": w.nsteps, "precision": a.precision,
                      "kernel": b.kernel_info(), "seconds_last": dt,
                      "system_steps_per_s": w.n_sys * w.nsteps / dt, "checksum": float(np.sum(np.abs(st)))}))


if __name__ == "__main__":
    main()
