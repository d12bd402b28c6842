"""Python front end with the reference's `PASIf` interface (PASIf.py:148-434).

`PASIf` subclasses the drop-in `__GpuDriver` and builds the concatenated
system exactly as the reference's front end does -- block-diagonal
unfolding (PASIf.py:475-605), -M^-1 preprocessing (PASIf.py:607-633), CSR
packing (PASIf.py:250-255) -- with the per-index Python loops of
`coo_tensor.concatenateTensor` / `multiplyByDiagMatrix` replaced by numpy
array operations that produce the same arrays in the same order.  The scipy
calls that fix the floating-point results (inv, dot, + and tocsr) are the
reference's own.

Differences, on purpose: no mpi4py (the GPU index is an argument, default
0: the reference maps MPI rank -> GPU and exchanges no message,
PASIf.py:27-30,167), and the caller's lists are not mutated (the reference
writes the concatenated force pattern back into vecForcePattern[0]).
"""
from __future__ import annotations

import copy as cp
from dataclasses import dataclass

import numpy as np
from scipy.sparse import coo_matrix, csc_matrix, dia_matrix
from scipy.sparse.linalg import inv

from .PASIfgpu import __GpuDriver as _GpuDriver


@dataclass
class coo_tensor:
    """Sparse tensor in COO format, highest dimension first (PASIf.py:32-146):
    `indices` holds len(dimensions) integers per value."""

    def __init__(self, dimensions_: list = None):
        self.dimensions = list(dimensions_) if dimensions_ is not None else [2, 2]
        self.val = []
        self.indices = []

    dimensions: list
    val: list
    indices: list

    def concatenateTensor(self, tensor_: "coo_tensor"):
        if len(self.dimensions) != len(tensor_.dimensions):
            raise Exception("The number of dimensions of the two tensors are not the same")
        nd = len(self.dimensions)
        idx = np.asarray(tensor_.indices, dtype=np.int64).reshape(-1, nd) + np.asarray(self.dimensions)
        self.val = list(self.val) + list(tensor_.val)
        self.indices = list(self.indices) + idx.reshape(-1).tolist()
        self.dimensions = [a + b for a, b in zip(self.dimensions, tensor_.dimensions)]

    def multiplyByDiagMatrix(self, diagMatrix_):
        nd = len(self.dimensions)
        if len(self.val) == 0:
            return
        d = np.asarray(diagMatrix_).reshape(-1)
        dest = np.asarray(self.indices, dtype=np.int64).reshape(-1, nd)[:, 0]
        self.val = (np.asarray(self.val, dtype=np.float64) * d[dest]).tolist()

    def getIndicesDim(self, dim_: int):
        return np.asarray(self.indices).reshape(-1, len(self.dimensions))[:, dim_].tolist()

    def isSquare(self) -> bool:
        return all(d == self.dimensions[0] for d in self.dimensions)

    def extendDimmensions(self, extension_: int):
        self.dimensions = [d + extension_ for d in self.dimensions]

    def offsetDimmension(self, targetDim_: int, offset_: int):
        a = np.asarray(self.indices, dtype=np.int64).reshape(-1, len(self.dimensions))
        a[:, targetDim_] += offset_
        self.indices = a.reshape(-1).tolist()


def _concat_tensors(ts):
    """Block-diagonal concatenation of coo_tensors (PASIf.py:86-100 applied
    system after system), vectorised."""
    nd = len(ts[0].dimensions)
    dims = np.asarray([t.dimensions for t in ts], dtype=np.int64)
    offs = np.cumsum(dims, axis=0) - dims
    out = coo_tensor(dims.sum(axis=0).tolist())
    vals = [v for t in ts for v in t.val]
    idx = [np.asarray(t.indices, dtype=np.int64).reshape(-1, nd) + offs[s] for s, t in enumerate(ts)]
    out.val = vals
    out.indices = np.concatenate(idx).reshape(-1).tolist() if idx else []
    return out


def _neg_inverse(M):
    """-M^-1 as PASIf.py:609 and :625 compute it (-1 * scipy's sparse inv).
    A diagonal M -- the case the reference's later use of M.data (one value
    per row) presumes -- is inverted entry by entry: the same values as the
    sparse LU solve (one correctly rounded division per entry), without its
    G column solves, which dominate setup for thousands of systems."""
    c = csc_matrix(M)
    G = c.shape[0]
    if (c.shape == (G, G) and c.nnz == G and np.array_equal(c.indptr, np.arange(G + 1))
            and np.array_equal(c.indices, np.arange(G)) and np.all(c.data != 0)):
        return -1. * csc_matrix((1.0 / c.data, c.indices.copy(), c.indptr.copy()), shape=(G, G))
    return -1. * inv(M)


def _concat_coo(mats, sizes):
    offs = np.cumsum(sizes) - sizes
    data = np.concatenate([m.data for m in mats])
    row = np.concatenate([m.row + o for m, o in zip(mats, offs)])
    col = np.concatenate([m.col + o for m, o in zip(mats, offs)])
    return data, row, col


class PASIf(_GpuDriver):
    def __init__(self, excitationSet, sampleRate, numsteps_=0, dCompute_=False, dSystem_=False, dSolver_=False,
                 GPUId=0, precision="fp64"):
        self.numsteps = len(excitationSet[0]) if numsteps_ == 0 else numsteps_
        super().__init__(excitationSet, sampleRate, self.numsteps, dCompute_, dSystem_, dSolver_, GPUId,
                         precision=precision)
        self.sampleRate = sampleRate
        self.globalSystemSize = 0
        self.globalAdjointSize = 0
        self.interpolSize = 0
        self.saveSteps = 1
        self.n_excitations = len(excitationSet)
        self.systemSet = False
        self.numberOfSystems = 0
        self.jacobianSet = False

    def setExcitations(self, excitationSet, sampleRate):
        self.sampleRate = sampleRate
        self._loadExcitationsSet(excitationSet, self.sampleRate)

    # ---- checks (PASIf.py:439-473) ----
    def _check(self, vecM, vecB, vecK, vecGamma, vecLambda, vecF, vecIC, vecPsi=None):
        for i in range(len(vecM)):
            nd = vecM[i].shape[0]
            assert vecM[i].shape[0] == vecM[i].shape[1], "The matrix M must be squared."
            assert vecB[i].shape[0] == vecB[i].shape[1], "The matrix B must be squared."
            assert vecK[i].shape[0] == vecK[i].shape[1], "The matrix K must be squared."
            if vecPsi is None:
                assert len(set(vecGamma[i].dimensions)) == 1, "The System Gamma tensor must be squared."
                assert len(set(vecLambda[i].dimensions)) == 1, "The System Lambda tensor must be squared."
            assert vecB[i].shape[0] == nd, "The matrix B must have the same size as the matrix M."
            assert vecK[i].shape[0] == nd, "The matrix K must have the same size as the matrix M."
            assert vecGamma[i].dimensions[0] == nd, "The Gamma tensor must have the same size as the matrix M."
            assert vecLambda[i].dimensions[0] == nd, "The Lambda tensor must have the same size as the matrix M."
            assert vecF[i].shape[0] == nd, "The force pattern vector must have the same size as the matrix M."
            assert vecIC[i].shape[0] == nd, "The initial conditions vector must have the same size as the matrix M."
            if vecPsi is not None:
                assert vecPsi[i].dimensions[0] == nd, "The Psi tensor must have the same size as the matrix M."
                assert vecPsi[i].dimensions[0] == vecPsi[i].dimensions[1]
                assert vecPsi[i].dimensions[2] == vecPsi[i].dimensions[3] == vecPsi[i].dimensions[4]

    # ---- unfolding (PASIf.py:475-605) ----
    def _unfold(self, vecM, vecB, vecK, tensors, vecF, vecIC):
        sizes = np.asarray([m.shape[0] for m in vecM], dtype=np.int64)
        G = int(sizes.sum())
        if len(vecM) > 1:
            diagM = np.concatenate([np.asarray(m.data).reshape(-1) for m in vecM]).reshape(G)
            M = dia_matrix((diagM, [0]), shape=(G, G))
            d, r, c = _concat_coo([coo_matrix(b) for b in vecB], sizes)
            Bm = coo_matrix((d, (r, c)), shape=(G, G))
            d, r, c = _concat_coo([coo_matrix(k) for k in vecK], sizes)
            Km = coo_matrix((d, (r, c)), shape=(G, G))
            ts = [_concat_tensors(t) for t in tensors]
        else:
            M, Bm, Km = cp.deepcopy(vecM[0]), cp.deepcopy(vecB[0]), cp.deepcopy(vecK[0])
            ts = [cp.deepcopy(t[0]) for t in tensors]
        F = np.concatenate([np.asarray(f) for f in vecF], axis=0)
        IC = np.concatenate([np.asarray(x) for x in vecIC], axis=0)
        return G, M, Bm, Km, ts, F, IC

    def setSystems(self, vecM, vecB, vecK, vecGamma, vecLambda, vecForcePattern, vecInitialConditions):
        self.systemSet = False
        assert len(vecM) > 0
        assert len(vecM) == len(vecB) == len(vecK) == len(vecGamma) == len(vecLambda) == len(vecForcePattern) == len(
            vecInitialConditions), "The number of Systems in the input vectors must be the same."
        self._check(vecM, vecB, vecK, vecGamma, vecLambda, vecForcePattern, vecInitialConditions)
        self.numberOfSystems = len(vecM)
        self._user_systems = (list(vecM), list(vecB), list(vecK), list(vecGamma), list(vecLambda))
        G, M, Bm, Km, (Gam, Lam), F, IC = self._unfold(vecM, vecB, vecK, [vecGamma, vecLambda], vecForcePattern,
                                                       vecInitialConditions)
        self.globalSystemSize = G
        # PASIf.py:607-618
        M = _neg_inverse(M)
        Bm = coo_matrix(M.dot(Bm))
        Km = coo_matrix(M.dot(Km))
        Gam.multiplyByDiagMatrix(M.data)
        Lam.multiplyByDiagMatrix(M.data)
        F = F * (-1. * M.data)
        self.system_M, self.system_B, self.system_K = M, Bm, Km
        self.system_Gamma, self.system_Lambda = Gam, Lam
        self.system_forcePattern, self.system_initialConditions = F, IC
        csr = (Bm + Km).tocsr()
        csr.sort_indices()
        self._setFwdK(Km.shape, csr.data, csr.indices, csr.indptr)
        self._setFwdGamma(Gam.dimensions, Gam.val, Gam.indices)
        self._setFwdLambda(Lam.dimensions, Lam.val, Lam.indices)
        self._setFwdPsi([1] * 5, [], [])
        self._setFwdForcePattern(F)
        self._setFwdInitialConditions(IC)
        self.systemSet = True
        self._allocateSystemOnDevice()

    def setGeneratedJacobian(self, terminals=None):
        """setJacobian with backward systems generated from the systems given
        to setSystems (pasif_gb300.adjoint_system; the role of the external
        modelling tool).  terminals[i]: dL/dq(T) of system i (default 0).
        Returns, per system, the parameter of each gradient accumulator (the
        entries of -M^-1 (B + K) in CSR order, then Gamma, then Lambda)."""
        from .adjoint_system import jacobian_inputs
        if not self.systemSet:
            raise ValueError("The system must be set before the jacobian")
        ins, params = [], []
        for i, (M, B, K, G, L) in enumerate(zip(*self._user_systems)):
            t = None if terminals is None else terminals[i]
            j, p = jacobian_inputs(M, B, K, G, L, terminal=t)
            ins.append(j)
            params.append(p)
        self.setJacobian(*[list(z) for z in zip(*ins)])
        return params

    def setJacobian(self, vecM, vecB, vecK, vecGamma, vecLambda, vecForcePattern, vecInitialConditions, vecPsi):
        self.jacobianSet = False
        if not self.systemSet:
            raise ValueError("The system must be set before the jacobian")
        assert len(vecM) > 0
        assert len(vecM) == self.numberOfSystems, "The number of jacobian must be the same as the number of systems."
        self._check(vecM, vecB, vecK, vecGamma, vecLambda, vecForcePattern, vecInitialConditions, vecPsi)
        G, M, Bm, Km, (Gam, Lam, Psi), F, IC = self._unfold(vecM, vecB, vecK, [vecGamma, vecLambda, vecPsi],
                                                            vecForcePattern, vecInitialConditions)
        self.globalAdjointSize = G
        # PASIf.py:620-633 (the force pattern is not scaled)
        M = _neg_inverse(M)
        Bm = coo_matrix(M.dot(Bm))
        Km = coo_matrix(M.dot(Km))
        Gam.multiplyByDiagMatrix(M.data)
        Lam.multiplyByDiagMatrix(M.data)
        Psi.multiplyByDiagMatrix(M.data)
        self.jacobian_M, self.jacobian_B, self.jacobian_K = M, Bm, Km
        self.jacobian_Gamma, self.jacobian_Lambda, self.jacobian_Psi = Gam, Lam, Psi
        self.jacobian_forcePattern, self.jacobian_initialConditions = F, IC
        csr = (Bm + Km).tocsr()
        csr.sort_indices()
        self._setBwdK(Km.shape, csr.data, csr.indices, csr.indptr)
        self._setBwdGamma(Gam.dimensions, Gam.val, Gam.indices)
        self._setBwdLambda(Lam.dimensions, Lam.val, Lam.indices)
        self._setBwdForcePattern(F)
        self._setBwdInitialConditions(IC)
        self._setBwdPsi(Psi.dimensions, Psi.val, Psi.indices)
        self.jacobianSet = True
        self._allocateAdjointOnDevice()

    def setInterpolationMatrix(self, interpolationMatrix_):
        for row in interpolationMatrix_:
            if len(row) % 2 != 0:
                raise ValueError("The windows size must be even.")
            elif len(row) != len(interpolationMatrix_[0]):
                raise ValueError("The windows size must be the same for all the rows.")
        self.interpolSize = len(interpolationMatrix_)
        self.interpolationMatrix = np.array(interpolationMatrix_).flatten()
        self._setInterpolationMatrix(self.interpolationMatrix, len(interpolationMatrix_[0]))

    def setModulationBuffer(self, modulationBuffer_):
        if len(modulationBuffer_) == 0:
            raise ValueError("The modulation buffer must be non-empty.")
        elif len(modulationBuffer_) > 32000:
            raise ValueError("The modulation buffer don't fit in the GPU cst memory.")
        self.modulationBuffer = modulationBuffer_
        self._setModulationBuffer(self.modulationBuffer)

    def getAmplitudes(self):
        if not self.systemSet:
            raise ValueError("The system must be set before computing the amplitudes.")
        return self._getAmplitudes()

    def getTrajectory(self, saveSteps: int = 1):
        if not self.systemSet:
            raise ValueError("The system must be set before computing the trajectory.")
        self.saveSteps = saveSteps
        traj = np.asarray(self._getTrajectory(saveSteps))
        nsaved = int(self.numsteps / self.saveSteps)
        rows = self.globalSystemSize * self.n_excitations
        out = np.zeros((rows + 1, nsaved))
        out[0] = np.arange(nsaved) * self.saveSteps / self.sampleRate
        out[1:] = traj[:nsaved * rows].reshape(nsaved, rows).T
        return out

    def getGradient(self, save: int = 0):
        if not self.jacobianSet:
            raise ValueError("The jacobian must be set before computing the gradient.")
        return self._getGradient(save)

    def getMatrices(self):
        if not self.systemSet:
            raise ValueError("System is not set yet")
        return (self.system_B + self.system_K), self.system_Gamma, self.system_Lambda, self.system_forcePattern, \
            self.system_initialConditions
