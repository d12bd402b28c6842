"""GPU forward kernels vs the CPU oracle.

Both follow one canonical operation order with correctly rounded operations,
so the comparison is bit for bit, in every precision, for the pattern-
specialised (NVRTC) kernel and for the generic kernel."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300 import synth
from pasif_gb300.batch import Batch, Plan, Signals, forward
from pasif_gb300.system import Pattern
from tests import cases

pytestmark = pytest.mark.gpu

PRECS = ["fp64", "fp32", "fp32_kahan"]


def run_gpu(pat, vals, x0, exc, x, h, N, W, im, prec, generic=False, step0=0, **red):
    plan = Plan(pat, prec, generic_only=generic)
    sig = Signals(x, W, im, prec)
    b = Batch(plan, vals, x0, exc)
    b.forward(sig, h, N, step0=step0, **red)
    st, mx, sq = b.get()
    return st, mx, sq, b.kernel_info()


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("generic", [False, True])
@pytest.mark.parametrize("seed", range(4))
def test_forward_bit_exact_random_patterns(gpu, prec, generic, seed):
    rng = np.random.default_rng(100 + seed)
    pat, v = cases.random_system(rng)
    B, E, L = 96, 3, 90
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, E, L)
    exc = rng.integers(0, E, B)
    W = [0, 2, 8, 4][seed]
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    red = dict(max_comp=[0], max_start=40, sq_comp=sorted({0, pat.n - 1}), sq_start=10)
    step0 = [0, 3, 0, 17][seed]
    N = 120  # runs past the end of the signals
    st, mx, sq, info = run_gpu(pat, vals, x0, exc, x, 0.05, N, W, im, prec, generic, step0, **red)
    assert info["kind"] == ("generic" if generic else "specialised")
    ost, omx, osq = O.batch_forward(pat, vals, x0, exc, x, 0.05, N, W, im, prec, step0, **red)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(mx, omx)
    np.testing.assert_array_equal(sq, osq)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("prec", ["fp32", "fp32_kahan", "fp32_ext"])
@pytest.mark.parametrize("seed", range(4))
def test_packed_fp32_forward_bit_exact(gpu, monkeypatch, mode, prec, seed):
    """Packed-FP32 (f32x2) forward kernels forced on random patterns (mode 1:
    packed stages, scalar compensated update; 2: packed update too; the
    extended-state update is always scalar), K values
    of exactly 1 and -1 folded as literals, reducers on: equal to the oracle
    bit for bit (ptxas must not contract a packed product into an add)."""
    monkeypatch.setenv("PASIF_FP32X2", str(mode))
    rng = np.random.default_rng(700 + seed)
    pat, v = cases.random_system(rng, n=[2, 3, 5, 6][seed])
    B, E, L = 96, 3, 90
    vals, x0 = cases.random_batch(rng, pat, v, B)
    vals[:, 0], vals[:, 1] = 1.0, -1.0
    x = cases.signals(rng, E, L)
    exc = rng.integers(0, E, B)
    W = [0, 2, 8, 4][seed]
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    src = Plan(pat, prec).jit_report(vals, window=W, im=im)
    assert "packed FP32" in src.split("// ---- source ----\n", 1)[1].splitlines()[0]
    red = dict(max_comp=[0], max_start=40, sq_comp=sorted({0, pat.n - 1}), sq_start=10)
    st, mx, sq, info = run_gpu(pat, vals, x0, exc, x, 0.05, 120, W, im, prec, False, 5, **red)
    assert info["kind"] == "specialised"
    ost, omx, osq = O.batch_forward(pat, vals, x0, exc, x, 0.05, 120, W, im, prec, 5, **red)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(mx, omx)
    np.testing.assert_array_equal(sq, osq)


def test_packed_fp32_config2_default(gpu):
    """Config 2 in FP32 with compensated update compiles to the packed kernel
    by default, and its states equal the oracle's bit for bit over 20000
    steps (every forcing interval, the L2-resident table)."""
    w = synth.coupled2(n_sys=512, nsteps=20_000)
    src = Plan(w.pattern, "fp32_kahan").jit_report(w.values, window=w.window, im=w.im)
    assert "packed FP32" in src.split("// ---- source ----\n", 1)[1].splitlines()[0]
    st, mx, sq, info = run_gpu(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                               "fp32_kahan", **w.forward_kwargs())
    ost, omx, osq = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                    "fp32_kahan", 0, **w.forward_kwargs())
    np.testing.assert_array_equal(st, ost)


@pytest.mark.parametrize("name", ["duffing", "coupled2", "chain8", "banded32"])
def test_configs_small_bit_exact(gpu, name):
    kw = {"duffing": dict(n_sys=200, nsteps=3000), "coupled2": dict(n_sys=256, nsteps=4000),
          "chain8": dict(n_sys=64, nsteps=2000), "banded32": dict(n_sys=32, nsteps=1500, sig_len=4096)}[name]
    w = synth.CONFIGS[name](**kw)
    for prec in ("fp64", "fp32_kahan"):
        st, mx, sq, info = run_gpu(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                   prec, **w.forward_kwargs())
        assert info["kind"] == "specialised"
        ost, omx, osq = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window,
                                        w.im, prec, **w.forward_kwargs())
        np.testing.assert_array_equal(st, ost)
        np.testing.assert_array_equal(mx, omx)
        np.testing.assert_array_equal(sq, osq)


def test_one_shot_api_matches_batch(gpu):
    w = synth.coupled2(n_sys=130, nsteps=500)
    st, _, _ = forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                       "fp32_kahan")
    ost, _, _ = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                "fp32_kahan")
    np.testing.assert_array_equal(st, ost)


def test_edge_cases(gpu):
    rng = np.random.default_rng(9)
    # a single state with no dynamics but forcing, one sample, sample and hold
    pat, _ = Pattern.from_dense_lists(1, [], [], f=[0])
    st, _, _, _ = run_gpu(pat, [[2.0]], [[0.5]], [0], np.ones((1, 1)), 0.1, 10, 0, None, "fp64")
    assert st[0, 0] == 0.5          # sample 0 is never applied
    # empty batch
    pat2, v2 = cases.random_system(rng, 3)
    plan = Plan(pat2, "fp64")
    b = Batch(plan, np.zeros((0, pat2.P)), np.zeros((0, 3)), np.zeros(0, np.int32))
    b.forward(Signals(np.ones((1, 5))), 0.1, 10)
    st, _, _ = b.get()
    assert st.shape == (0, 3)
    # zero steps returns the initial state
    st, _, _, _ = run_gpu(pat2, v2[None], [[1.0, 2.0, 3.0]], [0], np.ones((1, 5)), 0.1, 0, 0, None, "fp64")
    np.testing.assert_array_equal(st, [[1.0, 2.0, 3.0]])
    # instance count not a multiple of the block size
    vals, x0 = cases.random_batch(rng, pat2, v2, 1000)
    x = cases.signals(rng, 2, 50)
    exc = rng.integers(0, 2, 1000)
    st, _, _, _ = run_gpu(pat2, vals, x0, exc, x, 0.05, 60, 2, [[0, .5], [1, .5]], "fp32")
    ost, _, _ = O.batch_forward(pat2, vals, x0, exc, x, 0.05, 60, 2, [[0, .5], [1, .5]], "fp32")
    np.testing.assert_array_equal(st, ost)


def test_bad_inputs_raise(gpu):
    rng = np.random.default_rng(2)
    pat, v = cases.random_system(rng, 3)
    plan = Plan(pat, "fp64")
    b = Batch(plan, v[None], np.zeros((1, 3)), [5])
    with pytest.raises(RuntimeError, match="excitation index"):
        b.forward(Signals(np.ones((2, 5))), 0.1, 3)
    with pytest.raises(RuntimeError, match="power of two"):
        Signals(np.ones((1, 8)), 3, np.ones((2, 3)))
    b2 = Batch(plan, v[None], np.zeros((1, 3)), [0])
    with pytest.raises(RuntimeError, match="components"):
        b2.forward(Signals(np.ones((1, 5))), 0.1, 3, max_comp=[7])


def test_config2_full_horizon_fp32_kahan_within_1e5(gpu):
    """Config 2 at full horizon on a slice of systems: the FP32-Kahan RMS
    amplitude is within 1e-5 relative of the FP64 path (itself bit-exact to
    the oracle on the small cases above)."""
    w = synth.coupled2(n_sys=2048)
    T = w.nsteps * w.h
    res = {}
    for prec in ("fp64", "fp32_kahan", "fp32"):
        st, _, _, _ = run_gpu(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                              prec)
        res[prec] = np.sqrt(st[:, 4] / T)
    rel_k = np.abs(res["fp32_kahan"] - res["fp64"]) / np.abs(res["fp64"])
    rel_p = np.abs(res["fp32"] - res["fp64"]) / np.abs(res["fp64"])
    assert rel_k.max() <= 1e-5, rel_k.max()
    assert rel_p.max() > rel_k.max()   # the compensation is what buys the bound


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("seed", range(4))
def test_forward_warp_sliced_bit_exact(gpu, prec, seed):
    """Warp-sliced kernel (several warps per 32 systems, components crossing
    warps through shared memory) forced on small random patterns, with a
    batch that is not a multiple of 32: equal to the oracle bit for bit."""
    rng = np.random.default_rng(300 + seed)
    pat, v = cases.random_system(rng)
    if pat.n < 2:
        pytest.skip("one component: nothing to slice")
    B, E, L = 83, 3, 90
    vals, x0 = cases.random_batch(rng, pat, v, B)
    x = cases.signals(rng, E, L)
    exc = rng.integers(0, E, B)
    W = [0, 2, 8, 4][seed]
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W]) if W else None
    red = dict(max_comp=[0], max_start=40, sq_comp=sorted({0, pat.n - 1}), sq_start=10)
    step0 = [0, 3, 0, 17][seed]
    N = 120
    plan = Plan(pat, prec, slicing=True)
    b = Batch(plan, vals, x0, exc)
    b.forward(Signals(x, W, im, prec), 0.05, N, step0=step0, **red)
    st, mx, sq = b.get()
    assert b.kernel_info()["kind"] == "specialised"
    ost, omx, osq = O.batch_forward(pat, vals, x0, exc, x, 0.05, N, W, im, prec, step0, **red)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(mx, omx)
    np.testing.assert_array_equal(sq, osq)


@pytest.mark.parametrize("nd", [14, 32, 64])
def test_forward_warp_sliced_chain(gpu, nd):
    """Spring chains of 28, 64 and 128 states (warp-sliced by default) with
    trajectory output: equal to the thread-per-system kernel and the oracle."""
    w = synth.chain8(n_sys=70, nsteps=400, nd=nd)
    red = dict(max_comp=list(range(min(nd, 8))), max_start=100, sq_comp=list(range(min(nd, 64))), sq_start=200)
    out = {}
    for slicing in (None, False):
        plan = Plan(w.pattern, "fp32_kahan", slicing=slicing)
        b = Batch(plan, w.values, w.x0, w.exc_index)
        b.forward(Signals(w.signals, w.window, w.im, "fp32_kahan"), w.h, w.nsteps, **red)
        out[slicing] = b.get()
    ost, omx, osq = O.batch_forward(w.pattern, w.values, w.x0, w.exc_index, w.signals, w.h, w.nsteps, w.window, w.im,
                                    "fp32_kahan", 0, **red)
    for got in out.values():
        np.testing.assert_array_equal(got[0], ost)
        np.testing.assert_array_equal(got[1], omx)
        np.testing.assert_array_equal(got[2], osq)


def test_reserve_requires_inputs_again(gpu):
    """Reserving grows the device buffers without keeping their contents: a
    solve before the inputs are set again is refused (PASIF_ERR_STATE), and
    after set a reused, resized batch equals a fresh one."""
    from pasif_gb300 import _native as N
    w = synth.chain8(n_sys=40, nsteps=302)
    sig = Signals(w.signals, w.window, w.im, "fp32_kahan")
    plan = Plan(w.pattern, "fp32_kahan", literals=False)
    b = Batch(plan, w.values[:7], w.x0[:7], w.exc_index[:7])
    b.reserve(4096, 200_000)
    with pytest.raises(N.PasifError) as e:
        b.forward(sig, w.h, 300)
    assert e.value.code == N.ERR_STATE
    with pytest.raises(N.PasifError):
        b.adjoint(sig, w.h, 300, g_sq=np.ones(7), sq_comp=(0,))
    b.set(w.values, w.x0, w.exc_index)               # resized to 40
    b.forward(sig, w.h, 300, max_comp=(0,))
    fresh = Batch(plan, w.values, w.x0, w.exc_index)
    fresh.forward(sig, w.h, 300, max_comp=(0,))
    for x, y in zip(b.get(), fresh.get()):
        np.testing.assert_array_equal(x, y)


def test_one_shot_forward_reuses_its_buffers(gpu):
    """pasif_forward keeps its device buffers for the next call with the same
    pattern, precision and forcing: a sequence of calls that changes the
    values, the number of systems, the signals, then the pattern, the
    precision and the window, and comes back, gives the oracle's bits each
    time."""
    rng = np.random.default_rng(321)
    pats = [cases.random_system(rng, n=3), cases.random_system(rng, n=5)]
    seq = [(0, "fp32_kahan", 2, 70), (0, "fp32_kahan", 2, 70), (0, "fp32_kahan", 2, 130), (1, "fp32_kahan", 2, 50),
           (1, "fp64", 2, 50), (1, "fp64", 4, 50), (0, "fp32_kahan", 2, 40)]
    for k, (pi, prec, W, B) in enumerate(seq):
        pat, v = pats[pi]
        vals, x0 = cases.random_batch(rng, pat, v, B)
        x = cases.signals(rng, 3, 60 + 10 * k)
        exc = rng.integers(0, 3, B)
        im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W])
        red = dict(max_comp=[0], max_start=20, sq_comp=[0], sq_start=10)
        st, mx, sq = forward(pat, vals, x0, exc, x, 0.04, 90, W, im, prec, 0, **red)
        ost, omx, osq = O.batch_forward(pat, vals, x0, exc, x, 0.04, 90, W, im, prec, 0, **red)
        np.testing.assert_array_equal(st, ost, err_msg=str(k))
        np.testing.assert_array_equal(mx, omx, err_msg=str(k))
        np.testing.assert_array_equal(sq, osq, err_msg=str(k))
