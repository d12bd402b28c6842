"""Small, fixed kernel runs for profiling (the commands in profiles/*.md).

    python -m pasif_gb300.profile_cases fwd coupled2 [nsteps]
    python -m pasif_gb300.profile_cases fwd banded32
    python -m pasif_gb300.profile_cases adj chain8
    python -m pasif_gb300.profile_cases fwd coupled2 20000 fp32_ext    (precision, default fp32_kahan)

Each run compiles the kernel, makes one short warm-up launch, then one launch
of the case (so `ncu -k regex:pk_fwd -s 1 -c 1` captures the case), and prints
the kernel kind and the rate measured outside any profiler.
"""
from __future__ import annotations

import sys
import time

import numpy as np

from . import synth
from .batch import Batch, Plan, Signals

FWD = {
    "coupled2": lambda ns: (synth.coupled2(nsteps=ns), ns),                                   # 16384 x 5 states
    "banded32": lambda ns: (synth.banded32(n_sys=2048, nsteps=10, sig_len=1 << 14), ns),      # 2048 x 64
    "chain64": lambda ns: (synth.chain8(n_sys=4096, nsteps=ns + 2, nd=64), ns),               # 4096 x 128
    "chain16": lambda ns: (synth.chain8(n_sys=16384, nsteps=ns + 2, nd=16), ns),              # 16384 x 32
}
ADJ = {
    "chain8": lambda ns: (synth.chain8(n_sys=4096, nsteps=ns + 2, nd=8), ns),                 # 4096 x 16
    "banded32": lambda ns: (synth.banded32(n_sys=2048, nsteps=10, sig_len=1 << 12), ns),
    "chain64": lambda ns: (synth.chain8(n_sys=4096, nsteps=ns + 2, nd=64), ns),
}


def run(mode: str, case: str, nsteps: int | None = None, precision: str = "fp32_kahan") -> float:
    table = FWD if mode == "fwd" else ADJ
    w, ns = table[case](nsteps or (20000 if case == "coupled2" else 2000))
    plan = Plan(w.pattern, precision)
    sig = Signals(w.signals, w.window, w.im, precision)
    b = Batch(plan, w.values, w.x0, w.exc_index)
    if mode == "fwd":
        kw = dict(max_comp=(0,), max_start=ns // 2)
        b.forward(sig, w.h, 64, **kw)
        b.get()
        t = time.perf_counter()
        b.forward(sig, w.h, ns, **kw)
        b.get()
    else:
        comps = tuple(range(min(w.pattern.n // 2, 64)))
        g = np.ones(w.n_sys)
        b.adjoint(sig, w.h, 16, g_sq=g, sq_comp=comps, sq_start=8)
        t = time.perf_counter()
        b.adjoint(sig, w.h, ns, g_sq=g, sq_comp=comps, sq_start=ns // 2)
    rate = w.n_sys * ns / (time.perf_counter() - t)
    print(mode, case, b.kernel_info(), f"{rate:.3e} system-steps/s")
    return rate


if __name__ == "__main__":
    run(sys.argv[1], sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else None,
        sys.argv[4] if len(sys.argv) > 4 else "fp32_kahan")
