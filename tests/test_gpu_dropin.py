"""The __GpuDriver drop-in (and the PASIf front end above it) on the GPU vs the
oracle's restatement of _getAmplitudes / _getTrajectory / _getGradient on the
same concatenated system."""
import numpy as np
import pytest
from scipy.sparse import coo_matrix, dia_matrix

from oracle import pyoracle as O
from pasif_gb300.frontend import PASIf, coo_tensor
from pasif_gb300.system import Pattern
from tests import cases

pytestmark = pytest.mark.gpu


def oracle_system(K_csr, gam, lam, force, psi=None, n_sp=None):
    """Pattern + values of a concatenated system as the driver receives it."""
    n = K_csr.shape[0]
    fi = [i for i, v in enumerate(force) if abs(v) > np.finfo(float).eps]
    g = np.asarray(gam.indices, np.int32).reshape(-1, 3)
    l = np.asarray(lam.indices, np.int32).reshape(-1, 4)
    p = np.asarray(psi.indices, np.int32).reshape(-1, 5) if psi is not None else np.zeros((0, 5), np.int32)
    pat = Pattern(n=n, k_ptr=K_csr.indptr, k_col=K_csr.indices, g_idx=g, l_idx=l, p_idx=p, f_idx=fi, n_sp=n_sp or n)
    vals = np.concatenate([K_csr.data, np.asarray(gam.val, float), np.asarray(lam.val, float),
                           np.asarray(psi.val, float) if psi is not None else [], np.asarray(force)[fi]])
    return pat, vals


def probe_system():
    c = cases.one_dof_probe()
    M = dia_matrix(([1., 1., 1., 1.], [0]), shape=(4, 4))
    B = coo_matrix(([-1., -1.], ([0, 1], [2, 3])), shape=(4, 4))
    K = coo_matrix(([1.0, 1.0], ([2, 2], [0, 2])), shape=(4, 4))
    G = coo_tensor([4, 4, 4]); G.val = [-1.]; G.indices = [3, 0, 0]
    L = coo_tensor([4, 4, 4, 4]); L.val = [0]; L.indices = [0, 0, 0, 0]
    return M, B, K, G, L, np.array([0., 0., 1., 0.]), np.zeros(4)


def random_user_system(rng, n):
    M = dia_matrix((rng.uniform(0.5, 2.0, n), [0]), shape=(n, n))
    pat, v = cases.random_system(rng, n, with_psi=False)
    rows = np.repeat(np.arange(n), np.diff(pat.k_ptr))
    kv = v[:pat.k_nnz]
    Bm = coo_matrix((kv[::2], (rows[::2], pat.k_col[::2])), shape=(n, n))
    Km = coo_matrix((kv[1::2], (rows[1::2], pat.k_col[1::2])), shape=(n, n))
    o = pat.offsets()
    G = coo_tensor([n, n, n]); G.val = list(v[o["Gamma"]:o["Lambda"]]); G.indices = pat.g_idx.reshape(-1).tolist()
    L = coo_tensor([n, n, n, n]); L.val = list(v[o["Lambda"]:o["Psi"]]); L.indices = pat.l_idx.reshape(-1).tolist()
    F = np.zeros(n); F[pat.f_idx] = v[o["F"]:o["end"]]
    return M, Bm, Km, G, L, F, rng.normal(0, 0.2, n)


def build(rng, E=3, L=120, numsteps=150, interp=None, precision="fp64"):
    exc = [np.sin(0.05 * (e + 1) * np.arange(L)) + 0.1 * rng.standard_normal(L) for e in range(E)]
    p = PASIf(exc, 64, numsteps, precision=precision)
    systems = [probe_system(), random_user_system(rng, 3), probe_system(), random_user_system(rng, 2)]
    p.setSystems(*[list(z) for z in zip(*systems)])
    if interp is not None:
        p.setInterpolationMatrix(interp)
    return p, np.asarray(exc)


def test_amplitudes_bit_exact(gpu):
    rng = np.random.default_rng(21)
    p, exc = build(rng)
    got = np.asarray(p.getAmplitudes())
    K, Gam, Lam, F, IC = p.getMatrices()
    csr = K.tocsr(); csr.sort_indices()
    pat, vals = oracle_system(csr, Gam, Lam, F)
    ref = O.get_amplitudes(pat, vals, IC, exc, 1 / 64, 150)
    assert got.shape == ref.shape == (3 * pat.n,)
    np.testing.assert_array_equal(got, ref)
    assert p._lastKernel() == "specialised"
    # a second call starts from the initial conditions again (resetStatesVectors)
    np.testing.assert_array_equal(np.asarray(p.getAmplitudes()), ref)


def test_amplitudes_large_block_warp_sliced(gpu):
    """A 30-state user system next to a small one: the driver's split gives it
    its own block, solved by the warp-sliced kernel (from 28 states in FP32,
    24 in FP64), and the amplitudes equal the oracle's on the concatenated
    system (bit for bit in FP64, within 1e-5 in FP32-Kahan)."""
    rng = np.random.default_rng(25)
    E, L = 2, 120
    exc = [np.sin(0.05 * (e + 1) * np.arange(L)) + 0.1 * rng.standard_normal(L) for e in range(E)]
    for precision in ("fp64", "fp32_kahan"):
        p = PASIf(exc, 64, 150, precision=precision)
        systems = [random_user_system(np.random.default_rng(26), 30), probe_system()]
        p.setSystems(*[list(z) for z in zip(*systems)])
        got = np.asarray(p.getAmplitudes())
        K, Gam, Lam, F, IC = p.getMatrices()
        csr = K.tocsr(); csr.sort_indices()
        pat, vals = oracle_system(csr, Gam, Lam, F)
        if precision == "fp64":
            ref = O.get_amplitudes(pat, vals, IC, np.asarray(exc), 1 / 64, 150)
            np.testing.assert_array_equal(got, ref)
        else:
            ref64 = ref
            np.testing.assert_allclose(got, ref64, rtol=1e-5, atol=1e-7)


def test_amplitudes_with_interpolation_matrix(gpu):
    rng = np.random.default_rng(22)
    W = 8
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W])
    p, exc = build(rng, L=40, numsteps=200, interp=im)   # 200 steps > 40 samples * 4: gated tail
    got = np.asarray(p.getAmplitudes())
    K, Gam, Lam, F, IC = p.getMatrices()
    csr = K.tocsr(); csr.sort_indices()
    pat, vals = oracle_system(csr, Gam, Lam, F)
    ref = O.get_amplitudes(pat, vals, IC, exc, 1 / 64, 200, W, im)
    np.testing.assert_array_equal(got, ref)


def test_trajectory(gpu):
    rng = np.random.default_rng(23)
    p, exc = build(rng, numsteps=90)
    K, Gam, Lam, F, IC = p.getMatrices()
    csr = K.tocsr(); csr.sort_indices()
    pat, vals = oracle_system(csr, Gam, Lam, F)
    for save in (1, 4, 7):
        got = np.asarray(p._getTrajectory(save))
        ref = O.get_trajectory(pat, vals, IC, exc, 1 / 64, 90, save)
        np.testing.assert_array_equal(got, ref)
    tr = p.getTrajectory(3)
    assert tr.shape == (pat.n * 3 + 1, 30)


def adjoint_inputs():
    c = cases.one_dof_probe()
    n = 6
    M = dia_matrix((np.ones(n), [0]), shape=(n, n))
    B = coo_matrix(([-1, -1], ([1, 2], [4, 5])), shape=(n, n))
    K = coo_matrix(([], ([], [])), shape=(n, n))
    G = coo_tensor([n, n, 4]); G.val = []; G.indices = []
    L = coo_tensor([n, n, 4, 4]); L.val = [-1, -1]; L.indices = [4, 0, 0, 0, 5, 0, 1, 1]
    Psi = coo_tensor([n, n, 4, 4, 4]); Psi.val = [0]; Psi.indices = [1, 1, 1, 1, 1]
    return M, B, K, G, L, np.zeros(n), c["a0"].copy(), Psi


def test_gradient_reference_semantics(gpu):
    rng = np.random.default_rng(24)
    E, L = 2, 140
    exc = [1.0 + 0.2 * rng.standard_normal(L) for _ in range(E)]
    N = 117
    p = PASIf(exc, 16, N)
    sysl = [probe_system(), probe_system()]
    p.setSystems(*[list(z) for z in zip(*sysl)])
    adj = [adjoint_inputs(), adjoint_inputs()]
    p.setJacobian(*[list(z) for z in zip(*adj)])
    got = np.asarray(p.getGradient())
    K, Gam, Lam, F, IC = p.getMatrices()
    csr = K.tocsr(); csr.sort_indices()
    fpat, fvals = oracle_system(csr, Gam, Lam, F)
    bcsr = (p.jacobian_B + p.jacobian_K).tocsr(); bcsr.sort_indices()
    bpat, bvals = oracle_system(bcsr, p.jacobian_Gamma, p.jacobian_Lambda, p.jacobian_forcePattern, p.jacobian_Psi,
                                n_sp=fpat.n)
    a0 = np.asarray(p.jacobian_initialConditions, float)
    ref = O.get_gradient(fpat, fvals, IC, bpat, bvals, a0, np.asarray(exc), 1 / 16, N)
    np.testing.assert_array_equal(got, ref)
    # the terminal condition is chained into the next call (src/__GpuDriver.cu:743)
    got2 = np.asarray(p.getGradient())
    ref2 = np.concatenate([O.get_gradient(fpat, fvals, IC, bpat, bvals, ref[e * 12:(e + 1) * 12],
                                          np.asarray(exc)[e:e + 1], 1 / 16, N) for e in range(E)])
    np.testing.assert_array_equal(got2, ref2)


def test_gradient_with_generated_jacobian(gpu):
    """getGradient with backward systems generated from the forward systems
    (setGeneratedJacobian) equals the oracle's _getGradient on the same
    preprocessed backward system, bit for bit; the accumulators list the
    parameters of -M^-1 (B + K), Gamma, Lambda."""
    rng = np.random.default_rng(27)
    E, L = 2, 160
    exc = [np.sin(0.07 * (e + 1) * np.arange(L)) + 0.1 * rng.standard_normal(L) for e in range(E)]
    N = 140
    p = PASIf(exc, 32, N)
    sysl = [random_user_system(np.random.default_rng(28), 3), random_user_system(np.random.default_rng(29), 2)]
    p.setSystems(*[list(z) for z in zip(*sysl)])
    terminals = [rng.normal(size=3), rng.normal(size=2)]
    params = p.setGeneratedJacobian(terminals)
    assert [len(x) for x in params] == [p.jacobian_initialConditions.size - 5 - len(params[1]), len(params[1])]
    got = np.asarray(p.getGradient())
    K, Gam, Lam, F, IC = p.getMatrices()
    csr = K.tocsr(); csr.sort_indices()
    fpat, fvals = oracle_system(csr, Gam, Lam, F)
    bcsr = (p.jacobian_B + p.jacobian_K).tocsr(); bcsr.sort_indices()
    bpat, bvals = oracle_system(bcsr, p.jacobian_Gamma, p.jacobian_Lambda, p.jacobian_forcePattern, p.jacobian_Psi,
                                n_sp=fpat.n)
    a0 = np.asarray(p.jacobian_initialConditions, float)
    ref = O.get_gradient(fpat, fvals, IC, bpat, bvals, a0, np.asarray(exc), 1 / 32, N)
    np.testing.assert_array_equal(got, ref)


def test_error_behaviour(gpu):
    p = PASIf([np.ones(10), np.ones(10)], 16, 5)
    with pytest.raises(ValueError):
        p.getAmplitudes()
    assert p._loadExcitationsSet([np.ones(10), np.ones(9)], 16) == 1
    with pytest.raises(RuntimeError):
        p._getAmplitudes()
    with pytest.raises(ValueError):
        p._setInterpolationMatrix(np.ones(12), 6)


class _Rec:
    """A concatenated system as recorded from the setter arguments."""

    def __init__(self, calls, fwd=True):
        tag = "Fwd" if fwd else "Bwd"
        d = {m: a for m, a in calls}
        shape, data, ind, ptr = d[f"_set{tag}K"]
        self.K = csr_like(data, ind, ptr, shape)
        self.gam = tens(*d[f"_set{tag}Gamma"])
        self.lam = tens(*d[f"_set{tag}Lambda"])
        self.psi = tens(*d[f"_set{tag}Psi"])
        self.force = np.asarray(d[f"_set{tag}ForcePattern"][0], float)
        self.ic = np.asarray(d[f"_set{tag}InitialConditions"][0], float)


def csr_like(data, ind, ptr, shape):
    from scipy.sparse import csr_matrix
    return csr_matrix((np.asarray(data, float), np.asarray(ind), np.asarray(ptr)), shape=tuple(int(s) for s in shape))


def tens(dims, val, idx):
    t = coo_tensor([int(x) for x in dims])
    t.val = [float(x) for x in np.asarray(val).reshape(-1)]
    t.indices = [int(x) for x in np.asarray(idx).reshape(-1)]
    return t


@pytest.mark.parametrize("case", ["coupled2x6", "probe1", "jacobian2", "interp"])
def test_reference_front_end_calls_replayed_on_the_drop_in(gpu, case):
    """The driver calls the reference's own PASIf.py makes (recorded in
    tests/golden/frontend_calls_<case>.npz) replayed on the drop-in __GpuDriver:
    _getAmplitudes (and _getGradient with a jacobian) equal the oracle's
    restatement on the recorded concatenated system, bit for bit."""
    from pasif_gb300 import PASIfgpu
    from tests.test_frontend_ref import load_calls
    calls = load_calls(case)
    init = calls[0][1]
    exc = np.asarray(init[0], float)
    sr, N = int(init[1]), int(init[2])
    drv = getattr(PASIfgpu, "__GpuDriver")(list(exc), sr, N, bool(init[3]), bool(init[4]), bool(init[5]), int(init[6]))
    window, im = 0, None
    for meth, args in calls[1:]:
        if meth == "_setInterpolationMatrix":
            window, im = int(args[1]), np.asarray(args[0], float)
        getattr(drv, meth)(*args)
    f = _Rec(calls)
    fpat, fvals = oracle_system(f.K, f.gam, f.lam, f.force)
    imr = im[:2 * window].reshape(2, window) if window else None
    got = np.asarray(drv._getAmplitudes())
    ref = O.get_amplitudes(fpat, fvals, f.ic, exc, 1 / sr, N, window, imr)
    np.testing.assert_array_equal(got, ref)
    if any(m == "_setBwdK" for m, _ in calls):
        b = _Rec(calls, fwd=False)
        bpat, bvals = oracle_system(b.K, b.gam, b.lam, b.force, b.psi, n_sp=fpat.n)
        got = np.asarray(drv._getGradient(0))
        ref = O.get_gradient(fpat, fvals, f.ic, bpat, bvals, b.ic, exc, 1 / sr, N)
        np.testing.assert_array_equal(got, ref)


def test_memory_bounded_sweep_equals_one_batch(gpu):
    """A sweep run as sequential batches (small device-memory budget) equals
    the one-batch solve bit for bit: amplitudes, trajectory and gradient, every
    instance on its own signal (the reference's chunks read the wrong
    excitation offset, src/__GpuDriver.cu:912-924).  A budget below one
    instance is refused with a memory error."""
    rng = np.random.default_rng(41)
    E, L, N = 7, 160, 120
    exc = [np.sin(0.03 * (e + 1) * np.arange(L)) + 0.1 * rng.standard_normal(L) for e in range(E)]

    def make(budget, grad=False):
        p = PASIf(exc, 32, N)
        if grad:
            p.setSystems(*[list(z) for z in zip(*[probe_system(), probe_system(), probe_system()])])
            p.setJacobian(*[list(z) for z in zip(*[adjoint_inputs(), adjoint_inputs(), adjoint_inputs()])])
        else:
            p.setSystems(*[list(z) for z in zip(*[probe_system(), random_user_system(np.random.default_rng(42), 3),
                                                  probe_system()])])
        if budget:
            p._setMemoryBudget(budget)
        return p

    whole, split = make(0), make(2000)
    a0, a1 = np.asarray(whole.getAmplitudes()), np.asarray(split.getAmplitudes())
    assert split._lastChunks() > whole._lastChunks() >= 1
    np.testing.assert_array_equal(a0, a1)
    np.testing.assert_array_equal(np.asarray(whole._getTrajectory(7)), np.asarray(split._getTrajectory(7)))
    assert split._lastChunks() > whole._lastChunks()
    whole, split = make(0, True), make(3000, True)
    np.testing.assert_array_equal(np.asarray(whole.getGradient()), np.asarray(split.getGradient()))
    assert split._lastChunks() > whole._lastChunks()
    tiny = make(1)
    with pytest.raises(RuntimeError, match="memory"):
        tiny.getAmplitudes()
