"""Seeded front-end inputs in the reference's input format (PASIf.setSystems /
setJacobian / setInterpolationMatrix, PASIf.py:202-402): first-order systems
as (dia_matrix M, coo_matrix B, coo_matrix K, 3-D and 4-D COO tensors, force
pattern, initial conditions), built with a given coo_tensor class so that the
same inputs reach the reference's PASIf (when its source is at hand) and
pasif_gb300.frontend.PASIf.  Shared by tests/golden/make_frontend_golden.py,
which records what the reference's front end hands its driver, and by
tests/test_frontend_ref.py, which checks that ours hands the same."""
from __future__ import annotations

import numpy as np
from scipy.sparse import coo_matrix, dia_matrix

CASES = ("coupled2x6", "probe1", "jacobian2", "interp")


def _tensor(ct, dims, entries, vals):
    t = ct(list(dims))
    t.val = [float(v) for v in vals]
    t.indices = [int(i) for e in entries for i in e]
    return t


def _coupled_system(rng, ct):
    """Two coupled oscillators with an RMS probe, first-order state
    (x1, x2, v1, v2, p): M = diag(1, 1, m1, m2, 1), B the damping rows, K the
    x' = v identity (with the sign -M^-1 turns positive) and the stiffness rows,
    a duplicate entry in K (coo duplicates are summed by tocsr), quadratic
    (Gamma, with the probe term p' = x2^2) and cubic (Lambda) couplings."""
    n = 5
    m = rng.uniform(0.5, 2.0, 2)
    M = dia_matrix((np.array([1.0, 1.0, m[0], m[1], 1.0]), [0]), shape=(n, n))
    k = rng.uniform(0.5, 2.0, 3)
    c = rng.uniform(0.01, 0.1, 3)
    Brow, Bcol, Bval = [2, 2, 3, 3], [2, 3, 2, 3], [c[0] + c[2], -c[2], -c[2], c[1] + c[2]]
    B = coo_matrix((Bval, (Brow, Bcol)), shape=(n, n))
    Krow = [0, 1, 2, 2, 3, 3, 3]
    Kcol = [2, 3, 0, 1, 0, 1, 1]
    kd = rng.uniform(0.0, 0.1)
    Kval = [-1.0, -1.0, k[0] + k[2], -k[2], -k[2], k[1] + k[2] - kd, kd]
    K = coo_matrix((Kval, (Krow, Kcol)), shape=(n, n))
    G = _tensor(ct, (n, n, n), [(2, 0, 1), (3, 0, 0), (3, 1, 1), (4, 1, 1)],
                list(rng.normal(0.0, 0.2, 3)) + [-1.0])
    L = _tensor(ct, (n, n, n, n), [(2, 0, 0, 0), (3, 1, 1, 1), (2, 0, 1, 1), (3, 0, 0, 1)], rng.normal(0.0, 0.5, 4))
    F = np.array([0.0, 0.0, 0.05, 0.0, 0.0])
    IC = np.array([rng.normal(0.0, 0.1), 0.0, 0.0, rng.normal(0.0, 0.1), 0.0])
    return M, B, K, G, L, F, IC


def _probe_system(ct):
    """The 1-DOF probe system of the reference's examples: x'' + c x' + k x +
    g x^3 = u with a probe p' = x^2, state (x, v, p)."""
    n = 3
    M = dia_matrix((np.array([1.0, 1.3, 1.0]), [0]), shape=(n, n))
    B = coo_matrix(([0.07], ([1], [1])), shape=(n, n))
    K = coo_matrix(([-1.0, 1.7], ([0, 1], [1, 0])), shape=(n, n))
    G = _tensor(ct, (n, n, n), [(2, 0, 0)], [-1.0])
    L = _tensor(ct, (n, n, n, n), [(1, 0, 0, 0)], [0.4])
    return M, B, K, G, L, np.array([0.0, 1.0, 0.0]), np.array([0.2, 0.0, 0.0])


def _jacobian_system(rng, ct, nf):
    """An adjoint system of 2 nf components for a forward system of nf: the
    setpoint dimensions of Gamma, Lambda and Psi are the forward size."""
    na = 2 * nf
    M = dia_matrix((rng.uniform(0.5, 2.0, na), [0]), shape=(na, na))
    rows = rng.integers(0, na, 6)
    cols = rng.integers(0, na, 6)
    B = coo_matrix((rng.normal(size=6), (rows, cols)), shape=(na, na))
    K = coo_matrix((rng.normal(size=5), (rng.integers(0, na, 5), rng.integers(0, na, 5))), shape=(na, na))
    G = _tensor(ct, (na, na, nf), [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf)))
                                   for _ in range(3)], rng.normal(size=3))
    L = _tensor(ct, (na, na, nf, nf), [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf)),
                                        int(rng.integers(nf))) for _ in range(2)], rng.normal(size=2))
    P = _tensor(ct, (na, na, nf, nf, nf), [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf)),
                                            int(rng.integers(nf)), int(rng.integers(nf))) for _ in range(2)],
                rng.normal(size=2))
    F = np.zeros(na)
    IC = rng.normal(size=na)
    return M, B, K, G, L, F, IC, P


def excitations(rng, n_exc=3, length=400):
    return [np.sin(0.05 * (i + 1) * np.arange(length)) + 0.1 * rng.normal(size=length) for i in range(n_exc)]


def make_case(name: str, ct):
    """Inputs of one case: dict with the constructor arguments (excitations,
    sample rate, steps), `systems` (the seven setSystems lists), optionally
    `jacobian` (the eight setJacobian lists) and `interp` (the rows given to
    setInterpolationMatrix)."""
    rng = np.random.default_rng({"coupled2x6": 11, "probe1": 12, "jacobian2": 13, "interp": 14}[name])
    out = {"excitations": excitations(rng), "sample_rate": 1000, "numsteps": 300}
    if name == "probe1":
        sy = [_probe_system(ct)]
    else:
        sy = [_coupled_system(rng, ct) for _ in range({"coupled2x6": 6, "jacobian2": 2}.get(name, 4))]
    out["systems"] = [list(col) for col in zip(*sy)]
    if name == "jacobian2":
        # two systems: the reference's setJacobian concatenates the diagonal of
        # M with np.concatenate(...).flatten() and fails from a third system on
        # (PASIf.py:574: a 1-D and a 2-D array)
        jac = [_jacobian_system(rng, ct, 5) for _ in range(2)]
        out["jacobian"] = [list(col) for col in zip(*jac)]
    if name == "interp":
        W = 4
        k = np.arange(W) / W
        out["interp"] = [k, 1.0 - k, 0.5 * k, 0.25 * (1.0 - k)]
    return out


def run_front_end(pasif_cls, case: dict):
    """Drive a PASIf class (the reference's or ours) through the case."""
    p = pasif_cls(case["excitations"], case["sample_rate"], case["numsteps"])
    p.setSystems(*case["systems"])
    if "jacobian" in case:
        p.setJacobian(*case["jacobian"])
    if "interp" in case:
        p.setInterpolationMatrix(case["interp"])
    return p


# the driver methods a front end calls, in the reference binding's order
# (src/PASIfgpu.cpp:22-105)
DRIVER_METHODS = ("_setFwdK", "_setFwdGamma", "_setFwdLambda", "_setFwdPsi", "_setFwdForcePattern",
                  "_setFwdInitialConditions", "_allocateSystemOnDevice", "_setBwdK", "_setBwdGamma",
                  "_setBwdLambda", "_setBwdPsi", "_setBwdForcePattern", "_setBwdInitialConditions",
                  "_allocateAdjointOnDevice", "_loadExcitationsSet", "_setInterpolationMatrix",
                  "_setModulationBuffer")


def as_arrays(args):
    """Recorded arguments as numpy arrays (lists, tuples, arrays) or scalars."""
    out = []
    for a in args:
        if isinstance(a, (list, tuple, np.ndarray)):
            arr = np.asarray(a)
            out.append(arr.astype(np.float64) if arr.dtype.kind in "fc" or arr.dtype == object else arr)
        else:
            out.append(a)
    return out
