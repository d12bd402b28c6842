"""CPU check of the code generator: the NVRTC source of the pattern-specialised
forward kernel is compiled for the host (tests/hostemu/emu_main.cpp replaces
the CUDA intrinsics by correctly rounded host arithmetic) and must equal the
oracle bit for bit.  Covers the interval loop (prologue, whole intervals,
epilogue), the literal folding and the canonical accumulation order without
a GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300 import synth
from pasif_gb300.batch import Plan
from tests import cases

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pasif_gb300", "csrc")


def run_emulated(tmp_path, pat, vals, x0, exc, x, W, im, h, step0, nsteps, prec):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    src = Plan(pat, prec).jit_report(vals, window=W, im=im).split("// ---- source ----\n", 1)[1]
    d = str(tmp_path)
    open(os.path.join(d, "gen.cu"), "w").write(src)
    exe = os.path.join(d, "emu")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", f"-DGEN_SOURCE=\"gen.cu\"", "-I", CSRC,
                        "-I", d, os.path.join(HERE, "hostemu", "emu_main.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    dt = np.float64 if prec == "fp64" else np.float32
    B = vals.shape[0]
    np.ascontiguousarray(vals.T.astype(dt)).tofile(os.path.join(d, "vals.bin"))
    np.ascontiguousarray(x0.T.astype(dt)).tofile(os.path.join(d, "x0.bin"))
    np.asarray(exc, np.int32).tofile(os.path.join(d, "exc.bin"))
    np.asarray(x, dt).tofile(os.path.join(d, "x.bin"))
    (np.asarray(im, dt).reshape(-1) if W else np.zeros(0, dt)).tofile(os.path.join(d, "im.bin"))
    xs = np.asarray(x)
    r = subprocess.run([exe, d, str(B), str(pat.n), str(pat.P), str(xs.shape[0]), str(xs.shape[1]), str(W),
                        str(step0), str(nsteps), repr(float(h)), "0"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(os.path.join(d, "out.bin"), dtype=dt).reshape(pat.n, B).T.astype(np.float64)


@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("seed,W,step0,nsteps", [(0, 8, 3, 61), (1, 0, 0, 40), (2, 4, 1, 30), (3, 2, 0, 25)])
def test_generated_kernel_matches_oracle(tmp_path, prec, seed, W, step0, nsteps):
    rng = np.random.default_rng(500 + seed)
    pat, v = cases.random_system(rng)
    B = 40
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 3, 28)   # shorter than the run: exercises the gating
    exc = rng.integers(0, 3, B)
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    got = run_emulated(tmp_path, pat, vals, x0, exc, x, W, im, 0.05, step0, nsteps, prec)
    ref, _, _ = O.batch_forward(pat, vals, x0, exc, x, 0.05, nsteps, W, im, prec, step0)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("seed", range(3))
def test_generated_adjoint_matches_oracle(tmp_path, seed):
    """FP64 specialised adjoint (registers + FP64 gradient totals) equals the
    oracle's exact discrete adjoint bit for bit."""
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    rng = np.random.default_rng(700 + seed)
    pat, v = cases.random_system(rng)
    B = 24
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 90)
    exc = rng.integers(0, 2, B)
    N = [37, 64, 101][seed]
    sq = (0,) if pat.n == 1 else (0, pat.n - 1)
    mask = sum(1 << c for c in sq)
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    src = Plan(pat, "fp64").jit_report_adjoint(vals, sq_mask=mask).split("// ---- source ----\n", 1)[1]
    d = str(tmp_path)
    open(os.path.join(d, "gen.cu"), "w").write(src)
    exe = os.path.join(d, "emu")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-DEMU_ADJ", f"-DGEN_SOURCE=\"gen.cu\"",
                        "-I", CSRC, "-I", d, os.path.join(HERE, "hostemu", "emu_main.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    np.ascontiguousarray(vals.T).tofile(os.path.join(d, "vals.bin"))
    np.ascontiguousarray(x0.T).tofile(os.path.join(d, "x0.bin"))
    np.asarray(exc, np.int32).tofile(os.path.join(d, "exc.bin"))
    np.asarray(x, np.float64).tofile(os.path.join(d, "x.bin"))
    np.zeros(2 * 2).tofile(os.path.join(d, "im.bin"))
    np.ascontiguousarray(gs).tofile(os.path.join(d, "gsq.bin"))
    np.ascontiguousarray(gf.T).tofile(os.path.join(d, "gfin.bin"))
    im = np.array([[0, .5], [1, .5]])
    im.tofile(os.path.join(d, "im.bin"))
    r = subprocess.run([exe, d, str(B), str(pat.n), str(pat.P), "2", "90", "2", "0", str(N), repr(0.03), "0",
                        str(N // 3)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pbar = np.fromfile(os.path.join(d, "pbar.bin")).reshape(pat.P, B).T
    dx0 = np.fromfile(os.path.join(d, "dx0.bin")).reshape(pat.n, B).T
    odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, im, gf, gs, sq, N // 3)
    np.testing.assert_array_equal(pbar, odv)
    np.testing.assert_array_equal(dx0, odx)


def test_generated_kernel_config2(tmp_path):
    w = synth.coupled2(n_sys=64, nsteps=300)
    got = run_emulated(tmp_path, w.pattern, w.values, w.x0, w.exc_index, w.signals, w.window, w.im, w.h, 0, w.nsteps,
                       "fp32_kahan")
    ref, _, _ = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                "fp32_kahan")
    np.testing.assert_array_equal(got, ref)


def _pool_jobs(rng, pat, v, C, W):
    """Jobs of a host-emulated serving pool: slot, admit chunk, steps and a
    signal table of their own; slots are reused and admissions staggered."""
    jobs, free_at = [], [0] * C
    for j in range(14):
        m = int(rng.integers(1, 4))
        slots = sorted(range(C), key=lambda s: (free_at[s], s))[:m]
        start = max(free_at[s] for s in slots) + int(rng.integers(0, 2))
        nsteps = int(rng.integers(5, 70))
        rows, length = int(rng.integers(1, 3)), int(rng.integers(8, 40))
        vals, x0 = cases.random_batch(rng, pat, v, m)
        jobs.append(dict(slots=slots, start=start, nsteps=nsteps, vals=vals, x0=x0,
                         x=cases.signals(rng, rows, length), exc=rng.integers(0, rows, m),
                         ms=int(rng.integers(0, 10)), ss=int(rng.integers(0, 10))))
        for s in slots:   # the emulator harvests a slot before the chunk after its last one
            free_at[s] = start + -(-nsteps // 16) + 1
    return jobs


@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("seed,W", [(0, 4), (1, 0), (2, 2)])
def test_generated_pool_matches_oracle(tmp_path, prec, seed, W):
    """Serving-pool chunk kernel: every system of every job, run in 16-step
    chunks beside other jobs that join and leave, equals the oracle run of
    that job alone, bit for bit (state, max and sum-of-squares reducers)."""
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    rng = np.random.default_rng(900 + seed)
    pat, v = cases.random_system(rng)
    C, chunk = 7, 16
    jobs = _pool_jobs(rng, pat, v, C, W)
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    max_comp = (0,)
    sq_comp = (0,) if pat.n == 1 else (0, pat.n - 1)
    src = Plan(pat, prec).jit_report_pool(W, im, max_comp, sq_comp).split("// ---- source ----\n", 1)[1]
    d = str(tmp_path)
    open(os.path.join(d, "gen.cu"), "w").write(src)
    exe = os.path.join(d, "emu")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-DEMU_POOL", f"-DGEN_SOURCE=\"gen.cu\"",
                        "-I", CSRC, "-I", d, os.path.join(HERE, "hostemu", "emu_main.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    dt = np.float64 if prec == "fp64" else np.float32
    rows, tab, vals, x0, arena, off = [], [], [], [], [], 0
    for jb in jobs:
        x = np.asarray(jb["x"], np.float64)
        L = x.shape[1]
        for i, s in enumerate(jb["slots"]):
            rows.append([s, jb["start"], jb["nsteps"], off + int(jb["exc"][i]) * L, off + x.size, L, jb["ms"],
                         jb["ss"]])
            vals.append(jb["vals"][i])
            x0.append(jb["x0"][i])
        arena.append(x.reshape(-1))
        off += x.size
    T = max(r_[1] for r_ in rows) + 70 // chunk + 3
    np.asarray(rows, np.int64).tofile(os.path.join(d, "jobs.bin"))
    np.asarray(vals, dt).tofile(os.path.join(d, "vals.bin"))
    np.asarray(x0, dt).tofile(os.path.join(d, "x0.bin"))
    np.concatenate(arena).astype(dt).tofile(os.path.join(d, "arena.bin"))
    (np.asarray(im, dt).reshape(-1) if W else np.zeros(0, dt)).tofile(os.path.join(d, "im.bin"))
    r = subprocess.run([exe, d, str(C), str(pat.n), str(pat.P), str(off), str(W), str(chunk), repr(0.05),
                        str(len(rows)), str(T)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    J = len(rows)
    st = np.fromfile(os.path.join(d, "state.bin"), dtype=dt).reshape(J, pat.n).astype(np.float64)
    mx = np.fromfile(os.path.join(d, "mx.bin"), dtype=dt).reshape(J, pat.n).astype(np.float64)
    sq = np.fromfile(os.path.join(d, "sq.bin"), dtype=dt).astype(np.float64) * 0.05
    k = 0
    for jb in jobs:
        m = len(jb["slots"])
        ost, omx, osq = O.batch_forward(pat, jb["vals"], jb["x0"], jb["exc"], jb["x"], 0.05, jb["nsteps"], W, im, prec,
                                        0, max_comp, jb["ms"], sq_comp, jb["ss"])
        np.testing.assert_array_equal(st[k:k + m], ost)
        np.testing.assert_array_equal(mx[k:k + m, list(max_comp)], omx)
        np.testing.assert_array_equal(sq[k:k + m], osq)
        k += m
