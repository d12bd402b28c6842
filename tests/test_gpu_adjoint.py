"""Exact discrete adjoint on the GPU vs the oracle's adjoint (bit for bit in
FP64) and vs central finite differences of the GPU forward."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300 import synth
from pasif_gb300.batch import Batch, Plan, Signals
from tests import cases

pytestmark = pytest.mark.gpu


def gpu_adjoint(pat, vals, x0, exc, x, h, N, W, im, prec, gf, gs, sq_comp, sq_start, generic=False):
    plan = Plan(pat, prec, generic_only=generic)
    b = Batch(plan, vals, x0, exc)
    out = b.adjoint(Signals(x, W, im, prec), h, N, g_final=gf, g_sq=gs, sq_comp=sq_comp, sq_start=sq_start)
    assert b.kernel_info()["adjoint"] == ("generic" if generic else "specialised")
    return out


@pytest.mark.parametrize("generic", [False, True])
@pytest.mark.parametrize("seed", range(3))
def test_adjoint_bit_exact_fp64(gpu, seed, generic):
    rng = np.random.default_rng(300 + seed)
    pat, v = cases.random_system(rng)
    B = 40
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 120)
    exc = rng.integers(0, 2, B)
    N = [50, 97, 144][seed]
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    sq = (0,)
    dv, dx = gpu_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, [[0, .5], [1, .5]], "fp64", gf, gs, sq, N // 3, generic)
    odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, [[0, .5], [1, .5]], gf, gs, sq, N // 3)
    np.testing.assert_array_equal(dv, odv)
    np.testing.assert_array_equal(dx, odx)


def test_adjoint_config3_fd_and_fp32(gpu):
    w = synth.chain8(n_sys=8, nsteps=3000)
    B = w.n_sys
    gs = np.ones(B)
    args = (w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im)
    dv, _ = gpu_adjoint(*args, "fp64", None, gs, w.sq_comp, w.sq_start)
    # central differences of the GPU forward on a few parameters of system 0
    plan = Plan(w.pattern, "fp64")
    sig = Signals(w.signals, w.window, w.im, "fp64")
    eps = 1e-6
    for q in (0, 9, 20, w.pattern.offsets()["Gamma"], w.pattern.offsets()["Lambda"] + 3):
        vp, vm = w.values.copy(), w.values.copy()
        vp[0, q] += eps
        vm[0, q] -= eps
        out = []
        for vv in (vp, vm):
            b = Batch(plan, vv, w.x0, w.exc_index)
            b.forward(sig, w.h, w.nsteps, sq_comp=w.sq_comp, sq_start=w.sq_start)
            out.append(b.get()[2][0])
        fd = (out[0] - out[1]) / (2 * eps)
        assert dv[0, q] == pytest.approx(fd, rel=1e-6, abs=1e-9)
    # FP32 modes against FP64, per value relative to the system's largest gradient: within 1e-5
    for prec in ("fp32_kahan", "fp32_ext"):
        dv32, _ = gpu_adjoint(*args, prec, None, gs, w.sq_comp, w.sq_start)
        rel = np.max(np.abs(dv32 - dv), axis=1) / np.max(np.abs(dv), axis=1)
        assert rel.max() <= 1e-5, (prec, rel.max())


@pytest.mark.parametrize("seed", range(3))
def test_adjoint_warp_sliced_fp64(gpu, seed):
    """Warp-sliced adjoint (gather-form VJP across warps) forced on small
    random patterns, batch not a multiple of 32: equal to the oracle bit for
    bit in FP64."""
    rng = np.random.default_rng(310 + seed)
    pat, v = cases.random_system(rng, n=[3, 5, 8][seed])
    B = 45
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 120)
    exc = rng.integers(0, 2, B)
    N = [50, 97, 144][seed]
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    sq = (0, pat.n - 1)
    plan = Plan(pat, "fp64", slicing=True)
    b = Batch(plan, vals, x0, exc)
    im = [[0, .5], [1, .5]]
    dv, dx = b.adjoint(Signals(x, 2, im, "fp64"), 0.03, N, g_final=gf, g_sq=gs, sq_comp=sq, sq_start=N // 3)
    assert b.kernel_info()["adjoint"] == "specialised"
    odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, im, gf, gs, sq, N // 3)
    np.testing.assert_array_equal(dv, odv)
    np.testing.assert_array_equal(dx, odx)


@pytest.mark.parametrize("nd", [4, 16, 32])
def test_adjoint_warp_sliced_fp32_equals_thread(gpu, nd):
    """FP32-Kahan adjoint of spring chains: warp-sliced and thread-per-system
    kernels give the same bits (same per-step FP32 sums, same FP64 totals)."""
    w = synth.chain8(n_sys=50, nsteps=300, nd=nd)
    out = []
    for slicing in (True, False):
        plan = Plan(w.pattern, "fp32_kahan", slicing=slicing)
        b = Batch(plan, w.values, w.x0, w.exc_index)
        out.append(b.adjoint(Signals(w.signals, w.window, w.im, "fp32_kahan"), w.h, w.nsteps,
                             g_sq=np.ones(w.n_sys), sq_comp=tuple(range(nd)), sq_start=w.nsteps // 2))
        assert b.kernel_info()["adjoint"] == "specialised"
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_adjoint_fp32_within_bound(gpu):
    """FP32 adjoints against the FP64 adjoint on 256 8-DOF chains x 20000
    steps, per system max|g32 - g64| / max|g64|.  FP32-Kahan (compensated
    state and adjoint-state updates, per-step FP32 gradient sums into
    compensated totals): median <= 1e-6, at most 2 % of the systems above
    1e-5 (the ones whose trajectories amplify the FP32 rounding of the values
    and of h/6).  The extended-state mode removes those two roundings: every
    system <= 1e-5.  verified_adjoint (cross-check, FP64 recompute of the
    flagged systems): every system <= 1e-5.  The generic kernel performs the
    same adjoint-state operations: its d x0 equals the specialised kernels'
    bit for bit."""
    from pasif_gb300.batch import verified_adjoint
    w = synth.chain8(n_sys=256, nsteps=20_000)
    out = {}
    for prec, generic in (("fp32_kahan", False), ("fp32_kahan", True), ("fp32_ext", False), ("fp64", False)):
        plan = Plan(w.pattern, prec, generic_only=generic)
        b = Batch(plan, w.values, w.x0, w.exc_index)
        out[(prec, generic)] = b.adjoint(Signals(w.signals, w.window, w.im, prec), w.h, w.nsteps,
                                         g_sq=np.ones(w.n_sys), sq_comp=w.sq_comp, sq_start=w.sq_start)
    g64 = out[("fp64", False)][0]

    def err(g):
        return np.max(np.abs(g - g64), axis=1) / np.max(np.abs(g64), axis=1)

    e32 = err(out[("fp32_kahan", False)][0])
    assert np.median(e32) <= 1e-6, np.median(e32)
    assert (e32 > 1e-5).sum() <= 0.02 * w.n_sys, (e32 > 1e-5).sum()
    eext = err(out[("fp32_ext", False)][0])
    assert eext.max() <= 1e-5, eext.max()
    gv, _, _ = verified_adjoint(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                g_sq=np.ones(w.n_sys), sq_comp=w.sq_comp, sq_start=w.sq_start)
    assert err(gv).max() <= 1e-5, err(gv).max()
    np.testing.assert_array_equal(out[("fp32_kahan", False)][1], out[("fp32_kahan", True)][1])


@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("config,n_sys,nsteps,slicing", [
    ("chain8", 40, 300, None),       # warp-sliced, one launch
    ("chain8", 1024, 20_000, None),  # warp-sliced, split backward launches
    ("duffing", 4096, 5_000, None),   # thread per system, split backward launches
    ("chain8", 200, 997, False),     # thread per system, ragged last chunk
])
def test_adjoint_stored_equals_checkpointed(gpu, prec, config, n_sys, nsteps, slicing):
    """The adjoint over a stored trajectory (the forward kernel writes every
    state once) gives the bits of the checkpointed adjoint (checkpoint pass,
    per-chunk recompute)."""
    w = synth.CONFIGS[config](n_sys=n_sys, nsteps=nsteps)
    rng = np.random.default_rng(77)
    gf = rng.normal(size=(n_sys, w.pattern.n))
    out = []
    for storage in (0, 1 << 34):
        b = Batch(Plan(w.pattern, prec, slicing=slicing), w.values, w.x0, w.exc_index)
        b.adjoint_storage(storage)
        out.append(b.adjoint(Signals(w.signals, w.window, w.im, prec), w.h, w.nsteps, g_final=gf,
                             g_sq=np.ones(n_sys), sq_comp=(0,), sq_start=nsteps // 2))
        assert b.kernel_info()["adjoint"] == "specialised"
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_adjoint_storage_limit_validated(gpu):
    w = synth.chain8(n_sys=4, nsteps=10)
    b = Batch(Plan(w.pattern, "fp32_kahan"), w.values, w.x0, w.exc_index)
    from pasif_gb300 import _native as N
    with pytest.raises(N.PasifError) as e:
        b.adjoint_storage(-1)
    assert e.value.code == N.ERR_INVALID
    b.adjoint_storage(0)


@pytest.mark.parametrize("B", [70, 4200])
@pytest.mark.parametrize("prec", ["fp64", "fp32_kahan"])
@pytest.mark.parametrize("seed,W,N", [(0, 2, 97), (1, 0, 144), (2, 4, 230)])
def test_adjoint_replayed_matches(gpu, prec, seed, W, N, B):
    """Checkpointed adjoint replayed by the forward kernel (checkpoint pass,
    then per chunk its slots from the checkpoint with the Kahan compensation):
    FP64 equals the oracle bit for bit; both precisions equal the stored
    trajectory's gradients.  Signals shorter than the run, horizons not a
    multiple of the chunk.  4200 systems: 32 blocks or more in either layout;
    70 systems: a small grid, whose checkpoints run inside the adjoint kernel."""
    rng = np.random.default_rng(320 + seed)
    pat, v = cases.random_system(rng)
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 60)
    exc = rng.integers(0, 2, B)
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    out = []
    for storage in (0, 1 << 30):
        b = Batch(Plan(pat, prec), vals, x0, exc)
        b.adjoint_storage(storage)
        out.append(b.adjoint(Signals(x, W, im, prec), 0.03, N, g_final=gf, g_sq=gs, sq_comp=(0,), sq_start=N // 3))
        assert b.kernel_info()["adjoint"] == "specialised"
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    if prec == "fp64":
        odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, W, im, gf, gs, (0,), N // 3)
        np.testing.assert_array_equal(out[0][0], odv)
        np.testing.assert_array_equal(out[0][1], odx)


@pytest.mark.parametrize("storage", [0, 1 << 30])
@pytest.mark.parametrize("N,B", [(0, 5), (1, 5), (2, 1), (3, 33)])
def test_adjoint_short_horizons(gpu, N, B, storage):
    """Edge horizons: no step (d x0 = g_final, no value gradient), one step,
    a single system; FP64 equals the oracle bit for bit in every trajectory
    mode."""
    rng = np.random.default_rng(340 + N)
    pat, v = cases.random_system(rng, n=3)
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 20)
    exc = rng.integers(0, 2, B)
    gf = rng.normal(size=(B, pat.n))
    gs = rng.normal(size=B)
    im = [[0, .5], [1, .5]]
    b = Batch(Plan(pat, "fp64"), vals, x0, exc)
    b.adjoint_storage(storage)
    dv, dx = b.adjoint(Signals(x, 2, im, "fp64"), 0.03, N, g_final=gf, g_sq=gs, sq_comp=(0,), sq_start=0)
    odv, odx = O.batch_adjoint(pat, vals, x0, exc, x, 0.03, N, 2, im, gf, gs, (0,), 0)
    np.testing.assert_array_equal(dv, odv)
    np.testing.assert_array_equal(dx, odx)
    if N == 0:
        np.testing.assert_array_equal(dx, gf)
        assert not dv.any()


@pytest.mark.parametrize("storage", [0, 1 << 30])
def test_adjoint_banded32_default_slices(gpu, storage):
    """64-state banded system (the 32-DOF serving class), FP32-Kahan: the
    default warp-sliced adjoint (8 warps) and a 16-warp split give the same
    bits, replayed from checkpoints (2112 systems: 66 blocks) and stored; the
    gradients are finite and nonzero."""
    w = synth.banded32(n_sys=2112, nsteps=210, sig_len=256)
    rng = np.random.default_rng(41)
    gf = rng.normal(size=(w.n_sys, w.pattern.n))
    gs = rng.normal(size=w.n_sys)
    out = []
    for slicing in (None, True):
        b = Batch(Plan(w.pattern, "fp32_kahan", slicing=slicing), w.values, w.x0, w.exc_index)
        b.adjoint_storage(storage)
        out.append(b.adjoint(Signals(w.signals, w.window, w.im, "fp32_kahan"), w.h, 200, g_final=gf, g_sq=gs,
                             sq_comp=(0, 5), sq_start=60))
        assert b.kernel_info()["adjoint"] == "specialised"
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert np.isfinite(out[0][0]).all() and np.abs(out[0][0]).max() > 0


@pytest.mark.parametrize("nd,n_sys", [(32, 300), (64, 100)])
def test_shared_slice_code_same_bits(gpu, monkeypatch, nd, n_sys):
    """Spring chains of 32 and 64 DOF (64, 128 states): the default kernels,
    whose interior warp slices share one struct (finer cut: 8 / 16 warps),
    give the bits of kernels with one struct per warp, forward (states and
    running max) and FP32-Kahan adjoint (stored trajectory and checkpoints)."""
    w = synth.chain8(n_sys=n_sys, nsteps=602, nd=nd)
    comps = tuple(range(nd))
    out = {}
    for share in ("1", "0"):
        monkeypatch.setenv("PASIF_WS_SHARE", share)
        plan = Plan(w.pattern, "fp32_kahan")
        sig = Signals(w.signals, w.window, w.im, "fp32_kahan")
        b = Batch(plan, w.values, w.x0, w.exc_index)
        b.forward(sig, w.h, 600, max_comp=comps[:8], max_start=300)
        res = list(b.get())
        for storage in (0, 1 << 30):
            b.adjoint_storage(storage)
            res += list(b.adjoint(sig, w.h, 600, g_sq=np.ones(n_sys), sq_comp=comps, sq_start=300))
        assert b.kernel_info()["adjoint"] == "specialised"
        out[share] = res
    for a, c in zip(out["1"], out["0"]):
        np.testing.assert_array_equal(a, c)


@pytest.mark.parametrize("prec", ["fp32_kahan", "fp64"])
def test_replayed_chunks_ahead_of_the_sweep(gpu, prec):
    """Checkpointed adjoints of 4200 systems (replayed by the forward kernel,
    the replays of up to four chunks running ahead of the backward sweep on
    their own streams): horizons of 2, 3 and 30 chunks and a batch reused
    across them give the bits of the stored-trajectory adjoint."""
    rng = np.random.default_rng(808)
    pat, v = cases.random_system(rng, n=4)
    B = 4200
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, 2, 200)
    exc = rng.integers(0, 2, B)
    gs = rng.normal(size=B)
    reused = Batch(Plan(pat, prec), vals, x0, exc)
    reused.adjoint_storage(0)
    for N in (4, 9, 870):
        out = []
        for storage in (0, 1 << 30):
            b = Batch(Plan(pat, prec), vals, x0, exc)
            b.adjoint_storage(storage)
            out.append(b.adjoint(Signals(x, 2, [[0, .5], [1, .5]], prec), 0.02, N, g_sq=gs, sq_comp=(0,),
                                 sq_start=N // 2))
        again = reused.adjoint(Signals(x, 2, [[0, .5], [1, .5]], prec), 0.02, N, g_sq=gs, sq_comp=(0,),
                               sq_start=N // 2)
        for a, c, d in zip(out[0], out[1], again):
            np.testing.assert_array_equal(a, c)
            np.testing.assert_array_equal(a, d)
