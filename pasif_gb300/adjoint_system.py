"""Adjoint-system generator: the backward system of PASIf's `getGradient`
built from a forward system.

The reference's gradient (`_getGradient`, src/__GpuDriver.cu:502-587) integrates
a user-supplied backward system A = [lambda; g] in reversed time with the same
RK4 (src/__GpuDriver.cu:715-783):

    A' = K_b A + Gamma_b:(A, q) + Lambda_b:(A, q, q) + Psi_b:(A, q, q, q)

with q the forward state (index roles dest, A-index, q-indices,
src/kernels.cu:163-196).  The operators come from an external modelling tool
(absent); this module derives them from the forward system itself.  For the
forward system as the driver sees it (after PASIf.py:607-618:
f(q) = K_e q + Gamma_e:(q, q) + Lambda_e:(q, q, q) + F_e u, with
K_e = -M^-1 (B + K), Gamma_e / Lambda_e rows scaled by -M^-1):

* lambda' = J(q)^T lambda (the reversed-time adjoint):
  K_b[j, i] = K_e[i, j]; each Gamma_e entry (i, a, b) gives
  Gamma_b[a, i, b] and Gamma_b[b, i, a]; each Lambda_e entry (i, a, b, c)
  gives Lambda_b[a, i, b, c], [b, i, a, c] and [c, i, a, b];
* one accumulator g_p per parameter, g_p' = lambda_i * d f_i / d p:
  K_e entry (i, j) -> Gamma_b[n + p, i, j] = 1; Gamma_e entry (i, a, b) ->
  Lambda_b[n + p, i, a, b] = 1; Lambda_e entry (i, a, b, c) ->
  Psi_b[n + p, i, a, b, c] = 1.

Parameters are numbered like the driver's values of the system: the entries
of K_e in CSR order, then Gamma_e, then Lambda_e in their COO order (the
forcing pattern has no accumulator: the backward system has no excitation).
The terminal condition is A(T) = [dL/dq(T); 0].  `jacobian_inputs` returns
the arrays `PASIf.setJacobian` takes for one system: PASIf.py:620-633 scales
them by -M_j^-1, so M_j = I and the operators are given negated.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.sparse import coo_matrix, csr_matrix, dia_matrix

from .frontend import coo_tensor


@dataclass
class BackwardOperators:
    """Driver-level backward system of one forward system."""
    n: int                  # forward state size
    n_par: int              # parameter accumulators
    K: csr_matrix           # [n + n_par, n + n_par]
    gamma: np.ndarray       # [e, 3] (dest, A-index, q)
    gamma_val: np.ndarray
    lam: np.ndarray         # [e, 4]
    lam_val: np.ndarray
    psi: np.ndarray         # [e, 5]
    psi_val: np.ndarray
    params: list            # per accumulator: ("K", i, j) / ("Gamma", i, a, b) / ("Lambda", i, a, b, c)

    @property
    def n_adj(self) -> int:
        return self.n + self.n_par


def effective_forward(M, B, K, Gamma, Lambda):
    """K_e (CSR, sorted), Gamma_e / Lambda_e (indices, values) as
    PASIf.__systemPreprocessing and the driver hand them to the kernels."""
    s = -1.0 / np.asarray(M.diagonal(), dtype=np.float64)
    S = dia_matrix((s, [0]), shape=M.shape)
    Ke = (coo_matrix(S.dot(B)) + coo_matrix(S.dot(K))).tocsr()
    Ke.sort_indices()
    g = np.asarray(Gamma.indices, dtype=np.int64).reshape(-1, 3)
    gv = np.asarray(Gamma.val, dtype=np.float64) * (s[g[:, 0]] if len(g) else 1.0)
    l4 = np.asarray(Lambda.indices, dtype=np.int64).reshape(-1, 4)
    lv = np.asarray(Lambda.val, dtype=np.float64) * (s[l4[:, 0]] if len(l4) else 1.0)
    return Ke, g, gv, l4, lv


def backward_operators(M, B, K, Gamma, Lambda) -> BackwardOperators:
    """Backward operators (driver level) of one forward system given as
    PASIf.setSystems takes it (M diagonal, B, K sparse, Gamma, Lambda
    coo_tensor)."""
    Ke, g, gv, l4, lv = effective_forward(M, B, K, Gamma, Lambda)
    n = Ke.shape[0]
    rows = np.repeat(np.arange(n), np.diff(Ke.indptr))
    cols = Ke.indices
    params = [("K", int(i), int(j)) for i, j in zip(rows, cols)]
    params += [("Gamma",) + tuple(int(x) for x in e) for e in g]
    params += [("Lambda",) + tuple(int(x) for x in e) for e in l4]
    n_par = len(params)
    na = n + n_par
    # lambda' = K_e^T lambda
    Kb = coo_matrix((Ke.data, (cols, rows)), shape=(na, na)).tocsr()
    Kb.sort_indices()
    gb, gbv, lb, lbv, pb, pbv = [], [], [], [], [], []
    for (i, a, b), v in zip(g, gv):
        gb += [(a, i, b), (b, i, a)]
        gbv += [v, v]
    for (i, a, b, c), v in zip(l4, lv):
        lb += [(a, i, b, c), (b, i, a, c), (c, i, a, b)]
        lbv += [v, v, v]
    # parameter accumulators
    for p, prm in enumerate(params):
        if prm[0] == "K":
            gb.append((n + p, prm[1], prm[2]))
            gbv.append(1.0)
        elif prm[0] == "Gamma":
            lb.append((n + p, prm[1], prm[2], prm[3]))
            lbv.append(1.0)
        else:
            pb.append((n + p, prm[1], prm[2], prm[3], prm[4]))
            pbv.append(1.0)
    arr = lambda x, k: np.asarray(x, dtype=np.int64).reshape(-1, k)
    return BackwardOperators(n, n_par, Kb, arr(gb, 3), np.asarray(gbv, float), arr(lb, 4), np.asarray(lbv, float),
                             arr(pb, 5), np.asarray(pbv, float), params)


def apply_backward(ops: BackwardOperators, A: np.ndarray, q: np.ndarray) -> np.ndarray:
    """A' of the backward system (the contraction roles of
    src/kernels.cu:163-196): for checking the generated operators."""
    out = ops.K @ A
    for (d, s, k), v in zip(ops.gamma, ops.gamma_val):
        out[d] += v * A[s] * q[k]
    for (d, s, k, l), v in zip(ops.lam, ops.lam_val):
        out[d] += v * A[s] * q[k] * q[l]
    for (d, s, k, l, m), v in zip(ops.psi, ops.psi_val):
        out[d] += v * A[s] * q[k] * q[l] * q[m]
    return out


def jacobian_inputs(M, B, K, Gamma, Lambda, terminal=None):
    """Arguments of PASIf.setJacobian for one system:
    (M_j, B_j, K_j, Gamma_j, Lambda_j, forcePattern_j, initialConditions_j,
    Psi_j), and the parameter list of the accumulators.  terminal: dL/dq(T)
    (length n), the lambda part of the initial condition."""
    ops = backward_operators(M, B, K, Gamma, Lambda)
    n, na = ops.n, ops.n_adj
    Mj = dia_matrix((np.ones(na), [0]), shape=(na, na))
    Kc = ops.K.tocoo()
    Bj = coo_matrix(([], ([], [])), shape=(na, na))
    Kj = coo_matrix((-Kc.data, (Kc.row, Kc.col)), shape=(na, na))

    def tensor(dims, idx, val):
        t = coo_tensor(dims)
        t.val = (-np.asarray(val, dtype=np.float64)).tolist()
        t.indices = np.asarray(idx, dtype=np.int64).reshape(-1).tolist()
        return t

    Gj = tensor([na, na, n], ops.gamma, ops.gamma_val)
    Lj = tensor([na, na, n, n], ops.lam, ops.lam_val)
    Pj = tensor([na, na, n, n, n], ops.psi, ops.psi_val)
    a0 = np.zeros(na)
    if terminal is not None:
        a0[:n] = np.asarray(terminal, dtype=np.float64)
    return (Mj, Bj, Kj, Gj, Lj, np.zeros(na), a0, Pj), ops.params
