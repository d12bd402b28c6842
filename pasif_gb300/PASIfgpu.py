"""Drop-in for the reference's compiled module `PASIfgpu` (src/PASIfgpu.cpp:22-105).

`from PASIfgpu import __GpuDriver` (PASIf.py:17) resolves to the class below
when this directory is on sys.path, or through `pasif_gb300.install_dropin()`.
Method names, argument names and defaults, return types and call order are
those of the pybind11 binding; the work is done by libpasif_gb300.so through
its C ABI.  Differences, on purpose:
  * CUDA failures raise RuntimeError instead of exit(0) (src/helpers.cuh:43-51);
  * an interpolation window that is not a power of two raises ValueError (the
    reference's kernel masks with W-1, src/kernels.cu:115-117);
  * an extra keyword `precision` ("fp64" default = reel double, "fp32",
    "fp32_kahan").
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from pasif_gb300 import _native as N

__all__ = ["__GpuDriver"]


def _signals(excitationSet_):
    rows = [np.ascontiguousarray(np.asarray(r, dtype=np.float64).reshape(-1)) for r in excitationSet_]
    ptrs = (N._dp * max(len(rows), 1))(*[N.dptr(r) for r in rows])
    lens = (C.c_longlong * max(len(rows), 1))(*[r.size for r in rows])
    return rows, ptrs, lens


def _uint(v, name):
    v = int(v)
    if v < 0:
        raise TypeError(f"{name} must be a non-negative integer")
    return v


class __GpuDriver:
    """src/__GpuDriver.cuh:18-83 / src/PASIfgpu.cpp:26-33."""

    def __init__(self, excitationSet_, sampleRate_, numsteps_, dCompute_=False, dSystem_=False, dSolver_=False,
                 GPUId_=0, precision="fp64"):
        rows, ptrs, lens = _signals(excitationSet_)
        h = C.c_void_p()
        N.check(N.lib.pasif_driver_create(C.byref(h), ptrs, lens, len(rows), _uint(sampleRate_, "sampleRate_"),
                                          _uint(numsteps_, "numsteps_"), int(bool(dCompute_)), int(bool(dSystem_)),
                                          int(bool(dSolver_)), _uint(GPUId_, "GPUId_")))
        self._pasif_handle = h
        if precision != "fp64":
            N.check(N.lib.pasif_driver_set_precision(h, N.PRECISIONS[precision]))

    def __del__(self):
        h = getattr(self, "_pasif_handle", None)
        if h:
            N.lib.pasif_driver_destroy(h)
            self._pasif_handle = None

    # ---- forward system interface (src/PASIfgpu.cpp:37-59) ----
    def _setK(self, fwd, n_, values_, indices_, indptr_):
        n = [int(x) for x in n_]
        v, ind, ptr = N.f64(values_).reshape(-1), N.u32(indices_).reshape(-1), N.u32(indptr_).reshape(-1)
        if len(n) != 2:
            raise TypeError("n_ must hold two dimensions")
        if ptr.size < n[0] + 1 or ind.size < v.size:
            raise ValueError("CSR arrays shorter than the declared shape")
        f = N.lib.pasif_driver_set_fwd_k if fwd else N.lib.pasif_driver_set_bwd_k
        N.check(f(self._pasif_handle, n[0], n[1], N.dptr(v), N.uptr(ind), N.uptr(ptr), v.size))

    def _setCoo(self, f, order, n_, values_, indices_):
        dims = N.u32([int(x) for x in n_])
        if dims.size != order:
            raise TypeError(f"n_ must hold {order} dimensions")
        v, ind = N.f64(values_).reshape(-1), N.u32(indices_).reshape(-1)
        if ind.size != order * v.size:
            raise ValueError(f"indices_ must hold {order} entries per value")
        N.check(f(self._pasif_handle, N.uptr(dims), N.dptr(v), N.uptr(ind), v.size))

    def _setFwdK(self, n_, values_, indices_, indptr_):
        self._setK(True, n_, values_, indices_, indptr_)

    def _setFwdGamma(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_fwd_gamma, 3, n_, values_, indices_)

    def _setFwdLambda(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_fwd_lambda, 4, n_, values_, indices_)

    def _setFwdPsi(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_fwd_psi, 5, n_, values_, indices_)

    def _setFwdForcePattern(self, forcePattern_):
        v = N.f64(forcePattern_).reshape(-1)
        N.check(N.lib.pasif_driver_set_fwd_force_pattern(self._pasif_handle, N.dptr(v), v.size))

    def _setFwdInitialConditions(self, initialConditions_):
        v = N.f64(initialConditions_).reshape(-1)
        N.check(N.lib.pasif_driver_set_fwd_initial_conditions(self._pasif_handle, N.dptr(v), v.size))

    def _allocateSystemOnDevice(self):
        N.check(N.lib.pasif_driver_allocate_system(self._pasif_handle))

    # ---- backward system interface (src/PASIfgpu.cpp:62-84) ----
    def _setBwdK(self, n_, values_, indices_, indptr_):
        self._setK(False, n_, values_, indices_, indptr_)

    def _setBwdGamma(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_bwd_gamma, 3, n_, values_, indices_)

    def _setBwdLambda(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_bwd_lambda, 4, n_, values_, indices_)

    def _setBwdPsi(self, n_, values_, indices_):
        self._setCoo(N.lib.pasif_driver_set_bwd_psi, 5, n_, values_, indices_)

    def _setBwdForcePattern(self, forcePattern_):
        v = N.f64(forcePattern_).reshape(-1)
        N.check(N.lib.pasif_driver_set_bwd_force_pattern(self._pasif_handle, N.dptr(v), v.size))

    def _setBwdInitialConditions(self, initialConditions_):
        v = N.f64(initialConditions_).reshape(-1)
        N.check(N.lib.pasif_driver_set_bwd_initial_conditions(self._pasif_handle, N.dptr(v), v.size))

    def _allocateAdjointOnDevice(self):
        N.check(N.lib.pasif_driver_allocate_adjoint(self._pasif_handle))

    # ---- compute options interface (src/PASIfgpu.cpp:88-96) ----
    def _loadExcitationsSet(self, excitationSet_, sampleRate_):
        rows, ptrs, lens = _signals(excitationSet_)
        rc = N.lib.pasif_driver_load_excitations(self._pasif_handle, ptrs, lens, len(rows),
                                                 _uint(sampleRate_, "sampleRate_"))
        if rc == N.ERR_LENGTH:
            print("[Error] __GpuDriver: Excitations vectors are not of the same size")
            return 1
        N.check(rc)
        return 0

    def _setInterpolationMatrix(self, interpolationMatrix_, interpolationWindowSize_):
        m = N.f64(interpolationMatrix_).reshape(-1)
        w = _uint(interpolationWindowSize_, "interpolationWindowSize_")
        rc = N.lib.pasif_driver_set_interpolation_matrix(self._pasif_handle, N.dptr(m), m.size, w)
        if rc == N.ERR_INVALID:
            raise ValueError(N.last_error())
        N.check(rc)

    def _setModulationBuffer(self, modulationBuffer_):
        m = N.f64(modulationBuffer_).reshape(-1)
        N.check(N.lib.pasif_driver_set_modulation_buffer(self._pasif_handle, N.dptr(m), m.size))

    # ---- solvers interface (src/PASIfgpu.cpp:100-104) ----
    def _collect(self, f, *args):
        ln = C.c_longlong()
        N.check(f(self._pasif_handle, *args, None, 0, C.byref(ln)))
        out = np.empty(ln.value)
        N.check(f(self._pasif_handle, *args, N.dptr(out), out.size, C.byref(ln)))
        return out

    def _getAmplitudes(self):
        return self._collect(N.lib.pasif_driver_get_amplitudes).tolist()

    def _getTrajectory(self, saveSteps_=1):
        return self._collect(N.lib.pasif_driver_get_trajectory, _uint(saveSteps_, "saveSteps_")).tolist()

    def _getGradient(self, save):
        return self._collect(N.lib.pasif_driver_get_gradient, _uint(save, "save")).tolist()

    # ---- not in the reference ----
    def _lastKernel(self) -> str:
        k = C.c_int()
        N.check(N.lib.pasif_driver_last_kernel(self._pasif_handle, C.byref(k)))
        return {0: "none", 1: "generic", 2: "specialised"}[k.value]

    # ---- memory-bounded sweeps (no reference method: the reference always
    # splits by the free device memory, src/__GpuDriver.cu:420-449) ----
    def _setMemoryBudget(self, bytes_: int) -> None:
        """Device memory a solve may use (0: 90 % of what is free); sweeps
        beyond it run as sequential batches, each instance on its own signal."""
        N.check(N.lib.pasif_driver_set_memory_budget(self._pasif_handle, int(bytes_)))

    def _lastChunks(self) -> int:
        """Sequential batches the last solve ran."""
        k = C.c_int()
        N.check(N.lib.pasif_driver_last_chunks(self._pasif_handle, C.byref(k)))
        return k.value
