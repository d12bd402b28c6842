"""CPU check of the code generator: the NVRTC source of the pattern-specialised
forward kernel is compiled for the host (tests/hostemu/emu_main.cpp replaces
the CUDA intrinsics by correctly rounded host arithmetic) and must equal the
oracle bit for bit.  Covers the interval loop (prologue, whole intervals,
epilogue), the literal folding and the canonical accumulation order without
a GPU."""
import os
import re
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


def build_emulator(d, src, define=None):
    """Compile a generated kernel source with the host harness; returns the
    executable and the environment that selects its launch shape."""
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    open(os.path.join(d, "gen.cu"), "w").write(src)
    exe = os.path.join(d, "emu")
    cmd = ["g++", "-O1", "-std=c++20", "-pthread", "-ffp-contract=off", f"-DGEN_SOURCE=\"gen.cu\"", "-I", CSRC,
           "-I", d, os.path.join(HERE, "hostemu", "emu_main.cpp"), "-o", exe]
    if define:
        cmd.insert(1, f"-D{define}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ)
    m = re.search(r"// ws-launch (\d+) (\d+)", src)
    if m:
        env["EMU_WS_L"] = str(int(m.group(1)) // 32)
        env["EMU_WS_SMEM"] = m.group(2)
    return exe, env


def hi_lo(a):
    """[B][k] FP64 -> [B][2k] FP32: high parts, then the low parts (the
    extended-state mode's split of values and initial states)."""
    a = np.asarray(a, np.float64)
    hi = a.astype(np.float32)
    return np.concatenate([hi, (a - hi.astype(np.float64)).astype(np.float32)], axis=1)


def run_emulated(tmp_path, pat, vals, x0, exc, x, W, im, h, step0, nsteps, prec, slicing=None):
    src = Plan(pat, prec, slicing=slicing).jit_report(vals, window=W, im=im).split("// ---- source ----\n", 1)[1]
    default_sliced = pat.n >= 28 if prec != "fp64" else pat.n >= 8 or (pat.n >= 3 and len(vals) <= 8192)
    if prec == "fp32_ext":   # fewer components per warp: sliced from n >= 28 as well
        default_sliced = pat.n >= 28
    assert ("warp-sliced" in src) == (bool(slicing) or (slicing is None and default_sliced))
    d = str(tmp_path)
    exe, env = build_emulator(d, src)
    dt = np.float64 if prec == "fp64" else np.float32
    B = vals.shape[0]
    ext = prec == "fp32_ext"
    if ext:
        env["EMU_EXT"] = "1"
    np.ascontiguousarray((hi_lo(vals) if ext else vals).T.astype(dt)).tofile(os.path.join(d, "vals.bin"))
    np.ascontiguousarray((hi_lo(x0) if ext else x0).T.astype(dt)).tofile(os.path.join(d, "x0.bin"))
    np.asarray(exc, np.int32).tofile(os.path.join(d, "exc.bin"))
    np.asarray(x, dt).tofile(os.path.join(d, "x.bin"))
    (np.asarray(im, dt).reshape(-1) if W else np.zeros(0, dt)).tofile(os.path.join(d, "im.bin"))
    xs = np.asarray(x)
    r = subprocess.run([exe, d, str(B), str(pat.n), str(pat.P), str(xs.shape[0]), str(xs.shape[1]), str(W),
                        str(step0), str(nsteps), repr(float(h)), "0"], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(os.path.join(d, "out.bin"), dtype=dt).astype(np.float64)
    if ext:   # high + low parts
        out = out.reshape(2, pat.n, B)
        return (out[0] + out[1]).T
    return out.reshape(pat.n, B).T


@pytest.mark.parametrize("slicing", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan", "fp32_ext"])
@pytest.mark.parametrize("seed,W,step0,nsteps", [(0, 8, 3, 61), (1, 0, 0, 40), (2, 4, 1, 30), (3, 2, 0, 25)])
def test_generated_kernel_matches_oracle(tmp_path, prec, seed, W, step0, nsteps, slicing):
    rng = np.random.default_rng(500 + seed)
    pat, v = cases.random_system(rng)
    B = 40
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 3, 28)   # shorter than the run: exercises the gating
    exc = rng.integers(0, 3, B)
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    if slicing and pat.n < 2:
        pytest.skip("one component: nothing to slice")
    got = run_emulated(tmp_path, pat, vals, x0, exc, x, W, im, 0.05, step0, nsteps, prec, slicing)
    ref, _, _ = O.batch_forward(pat, vals, x0, exc, x, 0.05, nsteps, W, im, prec, step0)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("prec", ["fp32", "fp32_kahan", "fp32_ext"])
@pytest.mark.parametrize("seed", range(3))
def test_packed_fp32_kernel_matches_oracle(tmp_path, monkeypatch, mode, prec, seed):
    """Packed-FP32 (f32x2) forward, forced on random patterns (mode 1:
    packed stages and scalar compensated update, 2: packed update too; the
    extended-state update is always scalar), with K values of exactly 1 and
    -1 folded as literals: the oracle's bits."""
    monkeypatch.setenv("PASIF_FP32X2", str(mode))
    rng = np.random.default_rng(900 + seed)
    pat, v = cases.random_system(rng, n=[2, 5, 6][seed])
    vals, x0 = cases.random_batch(rng, pat, v, 40)
    vals[:, 0], vals[:, 1] = 1.0, -1.0
    x = cases.signals(rng, 3, 28)
    exc = rng.integers(0, 3, 40)
    W = 8
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W])
    src = Plan(pat, prec).jit_report(vals, window=W, im=im)
    assert "packed FP32" in src.split("// ---- source ----\n", 1)[1].splitlines()[0]
    got = run_emulated(tmp_path, pat, vals, x0, exc, x, W, im, 0.05, 3, 61, prec)
    ref, _, _ = O.batch_forward(pat, vals, x0, exc, x, 0.05, 61, W, im, prec, 3)
    np.testing.assert_array_equal(got, ref)


def run_emulated_adjoint(d, pat, prec, slicing, vals, x0, exc, x, im, gf, gs, N, sq, sq_start, h=0.03, split=0,
                         stored=False):
    """split > 0: run it as the split launches of Batch::adjoint with `split`
    checkpoint intervals per launch.  stored: backward sweep over a stored
    trajectory (no checkpoint pass, no chunk recompute)."""
    mask = sum(1 << c for c in sq)
    src = Plan(pat, prec, slicing=slicing).jit_report_adjoint(vals, sq_mask=mask)
    src = src.split("// ---- source ----\n", 1)[1]
    if slicing is not None:
        assert ("warp-sliced" in src) == bool(slicing)
    exe, env = build_emulator(d, src, "EMU_ADJ")
    if split:
        env["EMU_ADJ_SPLIT"] = str(split)
    if stored:
        env["EMU_ADJ_STORED"] = "1"
    dt = np.float64 if prec == "fp64" else np.float32
    B = len(vals)
    ext = prec == "fp32_ext"
    if ext:
        env["EMU_EXT"] = "1"
    np.ascontiguousarray((hi_lo(vals) if ext else vals).T, dt).tofile(os.path.join(d, "vals.bin"))
    np.ascontiguousarray((hi_lo(x0) if ext else x0).T, dt).tofile(os.path.join(d, "x0.bin"))
    np.asarray(exc, np.int32).tofile(os.path.join(d, "exc.bin"))
    np.asarray(x, dt).tofile(os.path.join(d, "x.bin"))
    np.ascontiguousarray(gs, dt).tofile(os.path.join(d, "gsq.bin"))
    np.ascontiguousarray(gf.T, dt).tofile(os.path.join(d, "gfin.bin"))
    np.asarray(im, dt).tofile(os.path.join(d, "im.bin"))
    r = subprocess.run([exe, d, str(B), str(pat.n), str(pat.P), str(x.shape[0]), str(x.shape[1]), str(im.shape[1]),
                        "0", str(N), repr(h), "1" if prec == "fp32_kahan" else "0", str(sq_start)],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    pbar = np.fromfile(os.path.join(d, "pbar.bin")).reshape(pat.P, B).T
    dx0 = np.fromfile(os.path.join(d, "dx0.bin"), dtype=dt).reshape(pat.n, B).T.astype(np.float64)
    if ext:   # high + low parts of the adjoint state
        dx0 = dx0 + np.fromfile(os.path.join(d, "lamc.bin"), dtype=dt).reshape(pat.n, B).T.astype(np.float64)
    return pbar, dx0


def _adjoint_case(seed):
    rng = np.random.default_rng(700 + seed)
    pat, v = cases.random_system(rng, n=[2, 5, 7][seed])
    B = 24
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 90)
    exc = rng.integers(0, 2, B)
    N = [37, 64, 101][seed]
    sq = (0,) if pat.n == 1 else (0, pat.n - 1)
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    im = np.array([[0, .5], [1, .5]])
    return pat, vals, x0, exc, x, im, gf, gs, N, sq


@pytest.mark.parametrize("slicing", [False, True])
@pytest.mark.parametrize("seed", range(3))
def test_generated_adjoint_matches_oracle(tmp_path, seed, slicing):
    """FP64 specialised adjoint (registers + FP64 gradient totals; thread per
    system or warp-sliced with the gather-form VJP) equals the oracle's exact
    discrete adjoint bit for bit."""
    pat, vals, x0, exc, x, im, gf, gs, N, sq = _adjoint_case(seed)
    if slicing and pat.n < 2:
        pytest.skip("one component: nothing to slice")
    pbar, dx0 = run_emulated_adjoint(str(tmp_path), pat, "fp64", slicing, vals, x0, exc, x, im, gf, gs, N, sq, N // 3)
    odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, im, gf, gs, sq, N // 3)
    np.testing.assert_array_equal(pbar, odv)
    np.testing.assert_array_equal(dx0, odx)


@pytest.mark.parametrize("prec", ["fp32_kahan", "fp32_ext"])
@pytest.mark.parametrize("seed", range(3))
def test_generated_adjoint_fp32_sliced_equals_thread(tmp_path, seed, prec):
    """FP32 adjoint (per-step FP32 gradient sums into FP64 totals): the warp-
    sliced kernel equals the thread-per-system kernel bit for bit."""
    pat, vals, x0, exc, x, im, gf, gs, N, sq = _adjoint_case(seed)
    if pat.n < 2:
        pytest.skip("one component: nothing to slice")
    out = []
    for slicing in (False, True):
        d = os.path.join(str(tmp_path), str(slicing))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, pat, prec, slicing, vals, x0, exc, x, im, gf, gs, N, sq, N // 3))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("split", [0, 2])
@pytest.mark.parametrize("prec,slicing", [("fp64", False), ("fp64", True), ("fp32_kahan", False),
                                          ("fp32_kahan", True), ("fp32_ext", False), ("fp32_ext", True)])
def test_generated_adjoint_stored_equals_checkpointed(tmp_path, prec, slicing, split):
    """The backward sweep over a stored trajectory (one forward pass) gives
    the bits of the checkpointed adjoint (forward pass, then per-chunk
    recompute), in one launch and as split backward launches."""
    pat, vals, x0, exc, x, im, gf, gs, N, sq = _adjoint_case(1)
    out = []
    for stored in (False, True):
        d = os.path.join(str(tmp_path), str(stored))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, pat, prec, slicing, vals, x0, exc, x, im, gf, gs, N, sq, N // 3,
                                        split=split, stored=stored))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


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


@pytest.mark.parametrize("slicing,packed", [(False, False), (True, False), (False, True)])
@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("seed,W", [(0, 4), (1, 0), (2, 2)])
def test_generated_pool_matches_oracle(tmp_path, monkeypatch, prec, seed, W, slicing, packed):
    """Serving-pool chunk kernel: every system of every job, run in 16-step
    chunks beside other jobs that join and leave, equals the oracle run of
    that job alone, bit for bit (state, max and sum-of-squares reducers);
    `packed`: the packed-FP32 form forced on."""
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    if packed:
        if prec == "fp64":
            pytest.skip("packed FP32 only")
        monkeypatch.setenv("PASIF_FP32X2", "2")
    rng = np.random.default_rng(900 + seed)
    pat, v = cases.random_system(rng)
    if slicing and pat.n < 2:
        pytest.skip("one component: nothing to slice")
    src = _check_pool(tmp_path, rng, pat, v, prec, W, slicing)
    if packed and pat.n >= 2:
        assert "packed FP32" in src.splitlines()[0]


def test_generated_pool_banded32_pair_cut(tmp_path):
    """Serving-pool chunk kernel of the 64-state banded system (the served
    32-DOF class), FP32-Kahan, default layout: warp-sliced, cut by
    displacement/velocity pairs into 8 warps with shared slice code; every
    job equals the oracle run of that job alone, bit for bit."""
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    rng = np.random.default_rng(950)
    w = synth.banded32(n_sys=1, nsteps=10, sig_len=64)
    src = _check_pool(tmp_path, rng, w.pattern, w.values[0], "fp32_kahan", 2, None)
    assert "slices=8 " in src.splitlines()[0]
    assert 2 * _distinct_structs(src) <= 8


def _check_pool(tmp_path, rng, pat, v, prec, W, slicing):
    """Run random jobs of pattern `pat` (values around v) through the host-
    emulated pool kernel and compare every job with the oracle; returns the
    kernel source."""
    C, chunk = 7, 16
    jobs = _pool_jobs(rng, pat, v, C, W)
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    max_comp = (0,)
    sq_comp = (0,) if pat.n == 1 else (0, pat.n - 1)
    src = Plan(pat, prec, slicing=slicing).jit_report_pool(W, im, max_comp, sq_comp)
    src = src.split("// ---- source ----\n", 1)[1]
    if slicing is not None:
        assert ("warp-sliced" in src) == slicing
    d = str(tmp_path)
    exe, env = build_emulator(d, src, "EMU_POOL")
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
                        str(len(rows)), str(T)], capture_output=True, text=True, env=env)
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
    return src


@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan", "fp32_ext"])
def test_generated_warp_sliced_banded32(tmp_path, prec):
    """64-state banded system: the default kernel is warp-sliced (components
    crossing warps through shared memory); FP32-Kahan cuts it by
    displacement/velocity pairs into 8 warps whose interior slices share one
    struct.  Equals the oracle."""
    w = synth.banded32(n_sys=6, nsteps=150, sig_len=256)
    if prec == "fp32_kahan":
        src = Plan(w.pattern, prec).jit_report(w.values, window=w.window, im=w.im)
        src = src.split("// ---- source ----\n", 1)[1]
        assert "slices=8 " in src.splitlines()[0]
        assert _distinct_structs(src) <= 4
    got = run_emulated(tmp_path, w.pattern, w.values, w.x0, w.exc_index, w.signals, w.window, w.im, w.h, 0,
                       w.nsteps, prec, slicing=None if prec != "fp64" else True)
    ref, _, _ = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                prec)
    np.testing.assert_array_equal(got, ref)



def test_generated_adjoint_banded32_default_slices(tmp_path):
    """64-state banded system, FP32-Kahan: the default warp-sliced adjoint
    (16 warps of 2 displacement/velocity pairs, at most 8 distinct slice
    structs) gives the bits of the thread-per-system adjoint."""
    w = synth.banded32(n_sys=5, nsteps=30, sig_len=64)
    rng = np.random.default_rng(31)
    gf = rng.normal(size=(w.n_sys, w.pattern.n))
    gs = rng.normal(size=w.n_sys)
    sq, N = (0, 5), 30
    rep = Plan(w.pattern, "fp32_kahan").jit_report_adjoint(w.values, sq_mask=(1 << 0) | (1 << 5))
    rep = rep.split("// ---- source ----\n", 1)[1]
    assert "slices=16 " in rep.splitlines()[0]
    assert 2 * _distinct_structs(rep) <= 16
    out = []
    for slicing in (None, False):
        d = os.path.join(str(tmp_path), str(slicing))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, w.pattern, "fp32_kahan", slicing, w.values, w.x0, w.exc_index, w.signals,
                                        np.asarray(w.im), gf, gs, N, sq, N // 3, h=w.h))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert np.abs(out[0][0]).max() > 0


def _distinct_structs(src):
    return len(re.findall(r"^struct SL\d+ \{", src, flags=re.M))


@pytest.mark.parametrize("prec", ["fp32_kahan", "fp64", "fp32_ext"])
def test_shared_slices_chain_forward(tmp_path, prec):
    """32-DOF spring chain (64 states), default warp-sliced kernels: the
    interior slices are translates of one another and share one struct
    (runtime bases, per-warp value table); FP32-Kahan cuts the chain into 8
    warps, FP64 and the extended-state mode into 16.  Equal to the oracle."""
    w = synth.chain8(n_sys=5, nsteps=120, nd=32)
    src = Plan(w.pattern, prec).jit_report(w.values, window=w.window, im=w.im)
    src = src.split("// ---- source ----\n", 1)[1]
    L = int(re.search(r"slices=(\d+)", src).group(1))
    assert L == (8 if prec == "fp32_kahan" else 16)
    assert 2 * _distinct_structs(src) <= L, (_distinct_structs(src), L)
    got = run_emulated(tmp_path, w.pattern, w.values, w.x0, w.exc_index, w.signals, w.window, w.im, w.h, 0,
                       w.nsteps, prec)
    ref, _, _ = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                prec)
    np.testing.assert_array_equal(got, ref)


def test_shared_slices_chain_adjoint(tmp_path):
    """16-DOF spring chain (32 states), FP32-Kahan: the default adjoint cuts
    it into 8 warps whose interior slices share one struct; it gives the bits
    of the thread-per-system adjoint.  FP64, forced 16-warp split (shared
    structs too): the oracle's exact adjoint bit for bit."""
    w = synth.chain8(n_sys=4, nsteps=40, nd=16)
    rng = np.random.default_rng(41)
    gf = rng.normal(size=(w.n_sys, w.pattern.n))
    gs = rng.normal(size=w.n_sys)
    sq, N = (0, 3), 40
    mask = (1 << 0) | (1 << 3)
    rep = Plan(w.pattern, "fp32_kahan").jit_report_adjoint(w.values, sq_mask=mask).split("// ---- source ----\n", 1)[1]
    assert "slices=8 " in rep.splitlines()[0]
    assert 2 * _distinct_structs(rep) <= 8
    out = []
    for slicing in (None, False):
        d = os.path.join(str(tmp_path), str(slicing))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, w.pattern, "fp32_kahan", slicing, w.values, w.x0, w.exc_index, w.signals,
                                        np.asarray(w.im), gf, gs, N, sq, N // 3, h=w.h))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    rep64 = Plan(w.pattern, "fp64", slicing=True).jit_report_adjoint(w.values, sq_mask=mask)
    assert 2 * _distinct_structs(rep64.split("// ---- source ----\n", 1)[1]) <= 16
    d = os.path.join(str(tmp_path), "fp64")
    os.makedirs(d)
    dv, dx = run_emulated_adjoint(d, w.pattern, "fp64", True, w.values, w.x0, w.exc_index, w.signals,
                                  np.asarray(w.im), gf, gs, N, sq, N // 3, h=w.h)
    odv, odx = O.batch_adjoint(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, N, w.window, w.im, gf, gs, sq,
                               N // 3)
    np.testing.assert_array_equal(dv, odv)
    np.testing.assert_array_equal(dx, odx)


def test_default_fp64_adjoint_chain8_shared(tmp_path):
    """8-DOF spring chain (16 states, the config-3 system), FP64: the default
    adjoint is cut into 8 warps of 2 states, some of them sharing code (the
    slices holding the summed components differ), and gives the oracle's
    exact adjoint bit for bit."""
    w = synth.chain8(n_sys=4, nsteps=40, nd=8)
    rng = np.random.default_rng(43)
    gf = rng.normal(size=(w.n_sys, w.pattern.n))
    gs = rng.normal(size=w.n_sys)
    sq, N = (0, 3), 40
    rep = Plan(w.pattern, "fp64").jit_report_adjoint(w.values, sq_mask=(1 << 0) | (1 << 3))
    rep = rep.split("// ---- source ----\n", 1)[1]
    assert "slices=8 " in rep.splitlines()[0]
    assert _distinct_structs(rep) < 8
    dv, dx = run_emulated_adjoint(str(tmp_path), w.pattern, "fp64", None, w.values, w.x0, w.exc_index, w.signals,
                                  np.asarray(w.im), gf, gs, N, sq, N // 3, h=w.h)
    odv, odx = O.batch_adjoint(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, N, w.window, w.im, gf, gs, sq,
                               N // 3)
    np.testing.assert_array_equal(dv, odv)
    np.testing.assert_array_equal(dx, odx)


@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan", "fp32_ext"])
@pytest.mark.parametrize("slicing", [False, True])
@pytest.mark.parametrize("split", [1, 2])
def test_generated_adjoint_split_launches(tmp_path, prec, slicing, split):
    """The adjoint split into short launches (forward segments carrying the
    state in the checkpoints, backward chunk groups carrying the adjoint state
    and its compensation) equals the single launch bit for bit."""
    pat, vals, x0, exc, x, im, gf, gs, N, sq = _adjoint_case(2)
    out = []
    for sp in (0, split):
        d = os.path.join(str(tmp_path), str(sp))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, pat, prec, slicing, vals, x0, exc, x, im, gf, gs, N, sq, N // 3, split=sp))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("prec", ["fp32_kahan", "fp32_ext"])
def test_generated_adjoint_chain16_sliced_equals_thread(tmp_path, prec):
    """A 32-state chain (87 values): the gradient totals of both layouts do not
    fit registers and go through the compensated FP32 totals in memory; the
    warp-sliced and thread-per-system adjoints still agree bit for bit."""
    w = synth.chain8(n_sys=5, nsteps=45, nd=16)
    rng = np.random.default_rng(37)
    gf = rng.normal(size=(w.n_sys, w.pattern.n))
    gs = rng.normal(size=w.n_sys)
    out = []
    for slicing in (False, True):
        d = os.path.join(str(tmp_path), str(slicing))
        os.makedirs(d)
        out.append(run_emulated_adjoint(d, w.pattern, prec, slicing, w.values, w.x0, w.exc_index, w.signals,
                                        np.asarray(w.im), gf, gs, w.nsteps, (0, 3), 20, h=w.h))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert np.abs(out[0][0]).max() > 0


def _scattered_velocity_form(seed, nd=32):
    """x_i' = v_i; v_i' = linear in x_i, v_i and two random x_j; one cubic
    term per DOF on random components: first-order mechanical form whose
    couplings follow no band."""
    from pasif_gb300.system import Pattern
    rng = np.random.default_rng(seed)
    n = 2 * nd
    rows, cols, vals = [], [], []
    for i in range(nd):
        rows.append(i); cols.append(nd + i); vals.append(1.0)
    for i in range(nd):
        for j, v in ((i, -2.0), (nd + i, -0.05)):
            rows.append(nd + i); cols.append(j); vals.append(v)
        for j in rng.choice(nd, size=2, replace=False):
            if j != i:
                rows.append(nd + i); cols.append(int(j)); vals.append(0.1)
    lam = [(nd + i, int(rng.integers(nd)), int(rng.integers(nd)), int(rng.integers(nd))) for i in range(nd)]
    pat, order = Pattern.from_dense_lists(n, rows, cols, [], lam, [], [nd])
    v = np.concatenate([np.asarray(vals)[order], rng.normal(0, 0.1, len(lam)), [1.0]])
    return pat, np.repeat(v[None, :], 2, axis=0)


def test_pair_cut_only_where_it_shares(monkeypatch):
    """Velocity-form patterns are cut by displacement/velocity pairs only when
    that gives shared slice code: the banded 32-DOF system takes it (8
    forward warps, at most 4 structs; in the default order its 8 slices all
    differ), a system with scattered couplings keeps the default cut (its
    source is the same with the pair cut switched off)."""
    w = synth.banded32(n_sys=4, nsteps=10, sig_len=256)
    src = Plan(w.pattern, "fp32_kahan").jit_report(w.values, window=w.window, im=w.im)
    src = src.split("// ---- source ----\n", 1)[1]
    assert "slices=8 " in src.splitlines()[0]
    assert _distinct_structs(src) <= 4
    monkeypatch.setenv("PASIF_WS_SLICES_FWD", "8")
    monkeypatch.setenv("PASIF_WS_RCM", "1")
    rcm = Plan(w.pattern, "fp32_kahan").jit_report(w.values, window=w.window, im=w.im)
    assert _distinct_structs(rcm.split("// ---- source ----\n", 1)[1]) == 8
    monkeypatch.delenv("PASIF_WS_SLICES_FWD")
    monkeypatch.delenv("PASIF_WS_RCM")
    pat, vals = _scattered_velocity_form(7)
    out = []
    for rcm_only in (False, True):
        if rcm_only:
            monkeypatch.setenv("PASIF_WS_RCM", "1")
        for prec in ("fp32_kahan", "fp64"):
            rep = Plan(pat, prec).jit_report(vals)
            out.append(rep.split("// ---- source ----\n", 1)[1])
            rep = Plan(pat, prec).jit_report_adjoint(vals, sq_mask=1)
            out.append(rep.split("// ---- source ----\n", 1)[1])
    assert out[:4] == out[4:]
