"""Times the REFERENCE's own CUDA driver against this engine's drop-in on the
same concatenated system (measurement infrastructure; run on a GPU machine).

    REF_SRC=<dir holding PASIf's src/> bash oracle/ref/build_ref.sh
    python oracle/ref/time_ref.py

Workload: config-1 shaped Duffing systems (synth.duffing values), 128 of
them concatenated -- 128 cubic entries, the most the reference's SpTdV
kernel computes correctly (src/kernels.cu:55-56) -- replicated by the
reference over 8 excitation signals (its "parallelism through excitations",
src/__GpuDriver.cu:896-938): 1024 system instances x 1e5 RK4 steps at
h = 1e-4 with window-2 linear interpolation, FP64 (reel = double).  Both
sides run _getAmplitudes through the __GpuDriver API; the reference through
oracle/ref/ref_driver (the reference's sources compiled unmodified), this
engine through pasif_gb300.PASIfgpu.__GpuDriver.  Prints one JSON line: both
wall times, system-steps/s, and the largest relative difference of the
final states.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from pasif_gb300 import synth  # noqa: E402
from tests.golden.make_ref_golden import concat, sys_block  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def main(n_blocks: int = 128, n_exc: int = 8, nsteps: int = 100_000):
    d = synth.duffing(n_sys=n_blocks, nsteps=nsteps)
    fp, fv = concat([(d.pattern, d.values[b]) for b in range(n_blocks)])
    assert len(fp.l_idx) + len(fp.g_idx) + len(fp.p_idx) <= 128
    x = np.asarray(d.signals[:n_exc, :nsteps + 2], float)
    sr, W, im = 10_000, 2, np.asarray(d.im, float)
    x0 = np.zeros(fp.n)
    # the reference's driver on the case file
    parts = [f"{x.shape[0]} {x.shape[1]}", " ".join(repr(float(v)) for v in x.reshape(-1)), f"{sr} {nsteps}",
             f"{W} {im.size} " + " ".join(repr(float(v)) for v in im.reshape(-1))]
    fb, _ = sys_block(fp, fv)
    parts += [fb, f"{fp.n} " + " ".join(repr(float(v)) for v in x0), "0", "0"]
    with tempfile.TemporaryDirectory() as tmp:
        cf, of, tf = (os.path.join(tmp, f) for f in ("case.txt", "out.txt", "t.txt"))
        open(cf, "w").write("\n".join(parts) + "\n")
        t0 = time.perf_counter()
        r = subprocess.run([DRIVER, cf, of, tf], capture_output=True, text=True, timeout=3600)
        proc_s = time.perf_counter() - t0
        if r.returncode != 0:
            raise SystemExit(f"reference driver failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
        lines = open(of).read().split()
        ref_err, count = int(lines[0]), int(lines[1])
        ref_out = np.array([float(v) for v in lines[2:2 + count]])
        ref_s = float(open(tf).read())
    # this engine's drop-in, same calls
    from pasif_gb300 import PASIfgpu
    drv = getattr(PASIfgpu, "__GpuDriver")(list(x), sr, nsteps)
    kv = fv[:fp.k_nnz]
    o = fp.offsets()
    drv._setFwdK([fp.n, fp.n], kv, fp.k_col, fp.k_ptr)
    drv._setFwdGamma([fp.n] * 3, fv[o["Gamma"]:o["Lambda"]], fp.g_idx.reshape(-1))
    drv._setFwdLambda([fp.n] * 4, fv[o["Lambda"]:o["Psi"]], fp.l_idx.reshape(-1))
    drv._setFwdPsi([1] * 5, [], [])
    F = np.zeros(fp.n)
    F[fp.f_idx] = fv[o["F"]:o["end"]]
    drv._setFwdForcePattern(F)
    drv._setFwdInitialConditions(x0)
    drv._allocateSystemOnDevice()
    drv._setInterpolationMatrix(im.reshape(-1), W)
    t0 = time.perf_counter()
    first = np.asarray(drv._getAmplitudes())
    first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ours = np.asarray(drv._getAmplitudes())
    ours_s = time.perf_counter() - t0
    assert np.array_equal(first, ours)
    inst = n_blocks * n_exc
    scale = np.maximum(np.abs(ref_out), 1e-12 * np.abs(ref_out).max())
    print(json.dumps({
        "workload": f"{n_blocks} concatenated Duffing systems x {n_exc} excitations = {inst} instances x "
                    f"{nsteps} RK4 steps, FP64, window-2 interpolation (config-1 shape, <= 128 cubic entries)",
        "reference_driver": {"seconds": ref_s, "system_steps_per_s": inst * nsteps / ref_s,
                             "process_seconds": proc_s, "cuda_error": ref_err},
        "pasif_gb300_dropin": {"seconds": ours_s, "system_steps_per_s": inst * nsteps / ours_s,
                               "first_call_seconds": first_s},
        "speedup": ref_s / ours_s,
        "max_rel_diff_final_state": float(np.max(np.abs(ours - ref_out) / scale)),
    }))


if __name__ == "__main__":
    main()
