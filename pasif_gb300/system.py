"""Host-side description of polynomial first-order systems.

A system is  dQ/dt = K.Q + Gamma:(Q,Qp) + Lambda:(Q,Qp,Qp) + Psi:(Q,Qp,Qp,Qp) + F u(t)
with the index roles of the reference's SpTdV kernel (src/kernels.cu:52,56,61):
Gamma[i, j, k] adds v * Q[j] * Qp[k] to dQ[i]; Lambda[i, j, k, l] adds
v * Q[j] * Qp[k] * Qp[l]; Psi adds v * Q[j] * Qp[k] * Qp[l] * Qp[m].  For a
forward system Qp is Q itself; for an adjoint system Qp is the forward state.

A Pattern is the sparsity structure; the values of one instance are a vector
of length P ordered [K in CSR order | Gamma | Lambda | Psi | F].
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np


def _i32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    if shape is not None:
        a = a.reshape(shape)
    return a


@dataclass
class Pattern:
    n: int
    k_ptr: np.ndarray
    k_col: np.ndarray
    g_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    l_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    p_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.int32))
    f_idx: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))
    n_sp: int = 0

    def __post_init__(self):
        self.n = int(self.n)
        self.n_sp = int(self.n_sp) if self.n_sp else self.n
        self.k_ptr = _i32(self.k_ptr)
        self.k_col = _i32(self.k_col)
        self.g_idx = _i32(self.g_idx, (-1, 3))
        self.l_idx = _i32(self.l_idx, (-1, 4))
        self.p_idx = _i32(self.p_idx, (-1, 5))
        self.f_idx = _i32(self.f_idx, (-1,))
        self._keep = None

    @property
    def k_nnz(self) -> int:
        return int(self.k_col.size)

    @property
    def P(self) -> int:
        return self.k_nnz + len(self.g_idx) + len(self.l_idx) + len(self.p_idx) + len(self.f_idx)

    def offsets(self) -> dict:
        """Start of each parameter group inside an instance's value vector."""
        k = self.k_nnz
        g = k + len(self.g_idx)
        l = g + len(self.l_idx)
        p = l + len(self.p_idx)
        return {"K": 0, "Gamma": k, "Lambda": g, "Psi": l, "F": p, "end": p + len(self.f_idx)}

    def to_c(self):
        from . import _native as N
        c = N.PatternC()
        c.n, c.n_sp = self.n, self.n_sp
        c.k_nnz, c.k_ptr, c.k_col = self.k_nnz, N.iptr(self.k_ptr), N.iptr(self.k_col)
        c.g_nnz, c.g_idx = len(self.g_idx), N.iptr(self.g_idx)
        c.l_nnz, c.l_idx = len(self.l_idx), N.iptr(self.l_idx)
        c.p_nnz, c.p_idx = len(self.p_idx), N.iptr(self.p_idx)
        c.f_nnz, c.f_idx = len(self.f_idx), N.iptr(self.f_idx)
        return c

    def flops_per_step(self, reduced: int = 0) -> int:
        """Algorithmic FLOPs of one RK4 step of one instance (FMA = 2):
        4 * (2 nnz_K + 3 nnz_Gamma + 4 nnz_Lambda + 5 nnz_Psi + 2 nnz_F + 3) + 13 n
        (+2 per reduced component)."""
        rhs = 2 * self.k_nnz + 3 * len(self.g_idx) + 4 * len(self.l_idx) + 5 * len(self.p_idx) + 2 * len(self.f_idx) + 3
        return 4 * rhs + 13 * self.n + 2 * reduced

    def adjoint_flops_per_step(self, reduced: int = 0) -> int:
        """Algorithmic FLOPs of one step of the exact discrete adjoint with
        sqrt(N) checkpoints (FMA = 2): two forward steps (the checkpoint pass
        and the chunk replay), the three stage inputs recomputed from the
        step's state (3 right-hand sides + 2n each), and four vector-Jacobian
        products, each with the parameter-gradient terms: per K entry 4
        (one fma into the adjoint, one into the gradient), per Gamma entry 9,
        Lambda 15, Psi 22, forcing 2; plus 10 n for the stage weights and the
        adjoint update (+2 per component of a sum-of-squares loss)."""
        rhs = 2 * self.k_nnz + 3 * len(self.g_idx) + 4 * len(self.l_idx) + 5 * len(self.p_idx) + 2 * len(self.f_idx) + 3
        vjp = 4 * self.k_nnz + 9 * len(self.g_idx) + 15 * len(self.l_idx) + 22 * len(self.p_idx) + 2 * len(self.f_idx)
        return 2 * self.flops_per_step() + 3 * (rhs + 2 * self.n) + 4 * vjp + 10 * self.n + 2 * reduced

    @staticmethod
    def from_dense_lists(n, k_rows, k_cols, g=(), l=(), p=(), f=(), n_sp=0):
        """Pattern from COO K entries (sorted into CSR order, stable) and tensor index lists.
        Returns (pattern, k_perm): k_perm maps CSR position -> input K entry."""
        k_rows = np.asarray(k_rows, dtype=np.int64)
        k_cols = np.asarray(k_cols, dtype=np.int64)
        order = np.lexsort((k_cols, k_rows))
        ptr = np.zeros(n + 1, dtype=np.int32)
        np.add.at(ptr, k_rows + 1, 1)
        ptr = np.cumsum(ptr).astype(np.int32)
        pat = Pattern(n=n, k_ptr=ptr, k_col=k_cols[order], g_idx=np.asarray(g, np.int32).reshape(-1, 3),
                      l_idx=np.asarray(l, np.int32).reshape(-1, 4), p_idx=np.asarray(p, np.int32).reshape(-1, 5),
                      f_idx=np.asarray(f, np.int32).reshape(-1), n_sp=n_sp)
        return pat, order


def reducers_c(max_comp=(), max_start=0, sq_comp=(), sq_start=0):
    """Build a ReducersC (component lists sorted ascending, unique)."""
    from . import _native as N
    mc = np.ascontiguousarray(np.unique(np.asarray(max_comp, dtype=np.int32)))
    sc = np.ascontiguousarray(np.unique(np.asarray(sq_comp, dtype=np.int32)))
    r = N.ReducersC()
    r.n_max, r.max_comp, r.max_start = int(mc.size), N.iptr(mc), int(max_start)
    r.n_sq, r.sq_comp, r.sq_start = int(sc.size), N.iptr(sc), int(sq_start)
    r._keep = (mc, sc)
    return r
