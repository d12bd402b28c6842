"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module; it is the checker, never part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class OrcSys(C.Structure):
    _fields_ = [("n", C.c_int), ("n_sp", C.c_int),
                ("k_nnz", C.c_int), ("k_ptr", _ip), ("k_col", _ip), ("k_val", _dp),
                ("g_nnz", C.c_int), ("g_idx", _ip), ("g_val", _dp),
                ("l_nnz", C.c_int), ("l_idx", _ip), ("l_val", _dp),
                ("p_nnz", C.c_int), ("p_idx", _ip), ("p_val", _dp),
                ("f_nnz", C.c_int), ("f_idx", _ip), ("f_val", _dp)]


class OrcExc(C.Structure):
    _fields_ = [("x", _dp), ("n_exc", C.c_int), ("len", C.c_int), ("w", C.c_int), ("im", _dp)]


class OrcRed(C.Structure):
    _fields_ = [("n_max", C.c_int), ("max_comp", _ip), ("max_start", C.c_int),
                ("n_sq", C.c_int), ("sq_comp", _ip), ("sq_start", C.c_int)]


def _load():
    if not os.path.exists(LIB_PATH):
        import subprocess
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    lib = C.CDLL(LIB_PATH)
    sp, ep, rp = C.POINTER(OrcSys), C.POINTER(OrcExc), C.POINTER(OrcRed)
    for sfx in ("_d", "_f"):
        getattr(lib, "orc_batch_forward" + sfx).argtypes = [sp, C.c_int, _dp, _dp, _ip, ep, C.c_double, C.c_int,
                                                            C.c_int, C.c_int, rp, _dp, _dp, _dp, C.c_int]
        getattr(lib, "orc_integrate" + sfx).argtypes = [sp, _dp, C.c_int, ep, C.c_double, C.c_int, C.c_int, C.c_int,
                                                        rp, _dp, _dp, _dp]
    lib.orc_get_amplitudes_d.argtypes = [sp, _dp, ep, C.c_double, C.c_int, _dp, C.c_int]
    lib.orc_get_trajectory_d.argtypes = [sp, _dp, ep, C.c_double, C.c_int, C.c_int, _dp, C.c_longlong, C.c_int]
    lib.orc_get_gradient_d.argtypes = [sp, _dp, sp, _dp, ep, C.c_double, C.c_int, C.c_int, _dp, C.c_int]
    lib.orc_batch_adjoint_d.argtypes = [sp, C.c_int, _dp, _dp, _ip, ep, C.c_double, C.c_int, rp, _dp, _dp, _dp,
                                        _dp, C.c_int]
    return lib


lib = _load()


def _d(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _i(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def make_sys(pattern, values=None):
    """OrcSys for a pasif_gb300.system.Pattern and (optional) value vector."""
    keep = []
    s = OrcSys()
    s.n, s.n_sp = pattern.n, pattern.n_sp
    arrs = {}
    for name in ("k_ptr", "k_col", "g_idx", "l_idx", "p_idx", "f_idx"):
        arrs[name] = _i(getattr(pattern, name)).reshape(-1)
        keep.append(arrs[name])
    s.k_nnz, s.k_ptr, s.k_col = pattern.k_nnz, arrs["k_ptr"].ctypes.data_as(_ip), arrs["k_col"].ctypes.data_as(_ip)
    s.g_nnz, s.g_idx = len(pattern.g_idx), arrs["g_idx"].ctypes.data_as(_ip)
    s.l_nnz, s.l_idx = len(pattern.l_idx), arrs["l_idx"].ctypes.data_as(_ip)
    s.p_nnz, s.p_idx = len(pattern.p_idx), arrs["p_idx"].ctypes.data_as(_ip)
    s.f_nnz, s.f_idx = len(pattern.f_idx), arrs["f_idx"].ctypes.data_as(_ip)
    if values is not None:
        v = _d(values).reshape(-1)
        keep.append(v)
        o = pattern.offsets()
        base = v.ctypes.data
        s.k_val = C.cast(base + 8 * o["K"], _dp)
        s.g_val = C.cast(base + 8 * o["Gamma"], _dp)
        s.l_val = C.cast(base + 8 * o["Lambda"], _dp)
        s.p_val = C.cast(base + 8 * o["Psi"], _dp)
        s.f_val = C.cast(base + 8 * o["F"], _dp)
    s._keep = keep
    return s


def make_exc(x, window=0, im=None):
    x = _d(x)
    if x.ndim == 1:
        x = x[None, :]
    e = OrcExc()
    e.x, e.n_exc, e.len, e.w = x.ctypes.data_as(_dp), x.shape[0], x.shape[1], int(window)
    keep = [x]
    if window:
        im = _d(im).reshape(-1)
        keep.append(im)
        e.im = im.ctypes.data_as(_dp)
    e._keep = keep
    return e


def make_red(max_comp=(), max_start=0, sq_comp=(), sq_start=0):
    mc = _i(np.unique(np.asarray(max_comp, dtype=np.int32)))
    sc = _i(np.unique(np.asarray(sq_comp, dtype=np.int32)))
    r = OrcRed()
    r.n_max, r.max_comp, r.max_start = mc.size, mc.ctypes.data_as(_ip), int(max_start)
    r.n_sq, r.sq_comp, r.sq_start = sc.size, sc.ctypes.data_as(_ip), int(sq_start)
    r._keep = (mc, sc)
    return r


def batch_forward(pattern, values, x0, exc_index, x, h, nsteps, window=0, im=None, precision="fp64", step0=0,
                  max_comp=(), max_start=0, sq_comp=(), sq_start=0, threads=0):
    """Oracle of pasif_gb300.batch: returns (state, max, sq).
    precision: "fp64", "fp32", "fp32_kahan" or "fp32_ext" (float build of the oracle)."""
    v = _d(values).reshape(-1, pattern.P)
    B = v.shape[0]
    x0 = _d(x0).reshape(B, pattern.n)
    e = _i(exc_index).reshape(B)
    s = make_sys(pattern)
    ex = make_exc(x, window, im)
    red = make_red(max_comp, max_start, sq_comp, sq_start)
    st = np.empty((B, pattern.n))
    mx = np.empty((B, max(red.n_max, 1)))
    sq = np.empty(B)
    f = lib.orc_batch_forward_d if precision == "fp64" else lib.orc_batch_forward_f
    mode = {"fp32_kahan": 1, "fp32_ext": 2}.get(precision, 0)
    f(C.byref(s), B, v.ctypes.data_as(_dp), x0.ctypes.data_as(_dp), e.ctypes.data_as(_ip), C.byref(ex), float(h),
      int(step0), int(nsteps), mode, C.byref(red), st.ctypes.data_as(_dp), mx.ctypes.data_as(_dp),
      sq.ctypes.data_as(_dp), int(threads))
    return st, mx[:, :red.n_max], sq


def batch_adjoint(pattern, values, x0, exc_index, x, h, nsteps, window=0, im=None, g_final=None, g_sq=None,
                  sq_comp=(), sq_start=0, threads=0):
    v = _d(values).reshape(-1, pattern.P)
    B = v.shape[0]
    x0 = _d(x0).reshape(B, pattern.n)
    e = _i(exc_index).reshape(B)
    s = make_sys(pattern)
    ex = make_exc(x, window, im)
    red = make_red((), 0, sq_comp, sq_start)
    gf = _d(g_final).reshape(B, pattern.n) if g_final is not None else None
    gs = _d(g_sq).reshape(B) if g_sq is not None else None
    dv = np.empty((B, pattern.P))
    dx = np.empty((B, pattern.n))
    lib.orc_batch_adjoint_d(C.byref(s), B, v.ctypes.data_as(_dp), x0.ctypes.data_as(_dp), e.ctypes.data_as(_ip),
                            C.byref(ex), float(h), int(nsteps), C.byref(red),
                            gf.ctypes.data_as(_dp) if gf is not None else None,
                            gs.ctypes.data_as(_dp) if gs is not None else None,
                            dv.ctypes.data_as(_dp), dx.ctypes.data_as(_dp), int(threads))
    return dv, dx


def get_amplitudes(pattern, values, x0, x, h, nsteps, window=0, im=None, threads=0):
    s = make_sys(pattern, values)
    ex = make_exc(x, window, im)
    x0 = _d(x0)
    out = np.empty(ex.n_exc * pattern.n)
    lib.orc_get_amplitudes_d(C.byref(s), x0.ctypes.data_as(_dp), C.byref(ex), float(h), int(nsteps),
                             out.ctypes.data_as(_dp), int(threads))
    return out


def get_trajectory(pattern, values, x0, x, h, nsteps, save, window=0, im=None, threads=0):
    s = make_sys(pattern, values)
    ex = make_exc(x, window, im)
    x0 = _d(x0)
    n_out = (pattern.n * ex.n_exc * int(nsteps)) // int(save)
    out = np.empty(n_out)
    lib.orc_get_trajectory_d(C.byref(s), x0.ctypes.data_as(_dp), C.byref(ex), float(h), int(nsteps), int(save),
                             out.ctypes.data_as(_dp), n_out, int(threads))
    return out


def get_gradient(fpattern, fvalues, x0, bpattern, bvalues, a0, x, h, nsteps, save=0, window=0, im=None, threads=0):
    fs = make_sys(fpattern, fvalues)
    bs = make_sys(bpattern, bvalues)
    ex = make_exc(x, window, im)
    x0, a0 = _d(x0), _d(a0)
    out = np.empty(ex.n_exc * bpattern.n)
    lib.orc_get_gradient_d(C.byref(fs), x0.ctypes.data_as(_dp), C.byref(bs), a0.ctypes.data_as(_dp), C.byref(ex),
                           float(h), int(nsteps), int(save), out.ctypes.data_as(_dp), int(threads))
    return out
