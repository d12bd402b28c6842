"""Native batch interface: many instances of one pattern on the GPU.

    plan = Plan(pattern, "fp32_kahan")
    sig = Signals(x, window=8, im=weights, precision="fp32_kahan")
    b = Batch(plan, values, x0, exc_index)        # uploads once
    b.forward(sig, h, nsteps, sq_comp=[4])         # one persistent kernel
    state, mx, sq = b.get()
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .system import Pattern, reducers_c


def _prec(p) -> int:
    return N.PRECISIONS[p] if isinstance(p, str) else int(p)


def _stream(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Plan:
    def __init__(self, pattern: Pattern, precision="fp64", generic_only: bool = False, literals: bool = True,
                 slicing=None, fast: bool = False):
        """literals=False: the specialised kernels load every value, so one
        compiled kernel serves every batch of the plan (serving).
        slicing: None = warp-sliced kernels where they are faster on GB300
        (forward: FP32 from n >= 28, FP64 from n >= 8, or n >= 3 for batches
        up to 8192 systems; adjoint: FP32 from n >= 5, FP64 from n >= 2),
        True = always, False = never (thread per system).
        fast=True: the fast thread-per-system forward kernels (shared state
        products, folded RK sum): results differ from the oracle's bits and
        are checked against FP64 instead."""
        self.pattern = pattern
        self.precision = _prec(precision)
        self._c = pattern.to_c()
        h = C.c_void_p()
        flags = (N.PLAN_GENERIC_ONLY if generic_only else 0) | (0 if literals else N.PLAN_NO_LITERALS)
        if slicing is not None:
            flags |= N.PLAN_WARP_SLICED if slicing else N.PLAN_NO_WARP_SLICED
        if fast:
            flags |= N.PLAN_FAST
        N.check(N.lib.pasif_plan_create(C.byref(h), C.byref(self._c), self.precision, flags))
        self.handle = h

    def jit_report(self, values=None, max_mask: int = 0, sq_mask: int = 0, window: int = 0, im=None) -> str:
        """Compiler resource report of the specialised forward kernel, then its
        source after "// ---- source ----" (NVRTC only: no GPU needed)."""
        v = N.f64(values) if values is not None else None
        n_sys = int(v.shape[0]) if v is not None else 0
        w = N.f64(im).reshape(-1) if im is not None else None
        args = (self.handle, N.dptr(v) if v is not None else None, n_sys, max_mask, sq_mask, int(window),
                N.dptr(w) if w is not None else None)
        ln = C.c_longlong()
        N.check(N.lib.pasif_plan_jit_report(*args, None, 0, C.byref(ln)))
        buf = C.create_string_buffer(ln.value + 1)
        N.check(N.lib.pasif_plan_jit_report(*args, buf, ln.value + 1, C.byref(ln)))
        return buf.value.decode()

    def jit_report_pool(self, window: int = 0, im=None, max_comp=(), sq_comp=()) -> str:
        """Same as jit_report for the serving-pool chunk kernel."""
        w = N.f64(im).reshape(-1) if im is not None else None
        red = reducers_c(max_comp, 0, sq_comp, 0)
        args = (self.handle, int(window), N.dptr(w) if w is not None else None, C.byref(red))
        ln = C.c_longlong()
        N.check(N.lib.pasif_plan_jit_report_pool(*args, None, 0, C.byref(ln)))
        buf = C.create_string_buffer(ln.value + 1)
        N.check(N.lib.pasif_plan_jit_report_pool(*args, buf, ln.value + 1, C.byref(ln)))
        return buf.value.decode()

    def jit_report_adjoint(self, values=None, sq_mask: int = 0) -> str:
        """Same as jit_report for the specialised exact-adjoint kernel."""
        v = N.f64(values) if values is not None else None
        args = (self.handle, N.dptr(v) if v is not None else None, int(v.shape[0]) if v is not None else 0, sq_mask)
        ln = C.c_longlong()
        N.check(N.lib.pasif_plan_jit_report_adjoint(*args, None, 0, C.byref(ln)))
        buf = C.create_string_buffer(ln.value + 1)
        N.check(N.lib.pasif_plan_jit_report_adjoint(*args, buf, ln.value + 1, C.byref(ln)))
        return buf.value.decode()

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            N.lib.pasif_plan_destroy(h)
            self.handle = None


class Signals:
    """Excitation table (n_exc signals x len samples) in the plan precision.
    window 0: sample and hold; window W: linear weights im (2W values)."""

    def __init__(self, x, window: int = 0, im=None, precision="fp64", stream=None):
        x = N.f64(x)
        if x.ndim == 1:
            x = x[None, :]
        self.n_exc, self.len = x.shape
        self.window = int(window)
        im_a = N.f64(im).reshape(-1) if im is not None else None
        h = C.c_void_p()
        N.check(N.lib.pasif_signals_create(C.byref(h), N.dptr(x), self.n_exc, self.len, self.window,
                                           N.dptr(im_a) if im_a is not None else None, _prec(precision), N.HOST,
                                           _stream(stream)))
        self.handle = h

    def update(self, x, stream=None):
        """New table (same window, weights, precision) in the existing device
        buffers: no allocation once they are large enough."""
        x = N.f64(x)
        if x.ndim == 1:
            x = x[None, :]
        N.check(N.lib.pasif_signals_update(self.handle, C.c_void_p(x.ctypes.data), x.shape[0], x.shape[1], N.HOST,
                                           _stream(stream)))
        self.n_exc, self.len = x.shape

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            N.lib.pasif_signals_destroy(h)
            self.handle = None


class Batch:
    """n_sys instances: values[n_sys][P], x0[n_sys][n], exc_index[n_sys].
    Arrays are numpy (host) or torch CUDA tensors (device, float64, contiguous)."""

    def __init__(self, plan: Plan, values, x0, exc_index, stream=None):
        self.plan = plan
        p = plan.pattern
        self.n_sys = int(len(exc_index))
        h = C.c_void_p()
        N.check(N.lib.pasif_batch_create(C.byref(h), plan.handle, self.n_sys))
        self.handle = h
        self._h = 0.0
        self.set(values, x0, exc_index, stream)

    def reserve(self, n_sys: int, nsteps: int):
        """Size the device buffers for forward / adjoint solves of up to n_sys
        instances and nsteps steps (later calls then allocate nothing)."""
        N.check(N.lib.pasif_batch_reserve(self.handle, int(n_sys), int(nsteps)))

    def adjoint_storage(self, nbytes: int):
        """Device memory the exact adjoint may hold for the whole forward
        trajectory (default 16 GiB; 0 always recomputes from checkpoints).
        Results do not depend on it; set it before reserve()."""
        N.check(N.lib.pasif_batch_set_adjoint_storage(self.handle, int(nbytes)))

    def set(self, values, x0, exc_index, stream=None):
        """New inputs; a different instance count resizes the batch (its
        device buffers are kept, and grown only when too small)."""
        p = self.plan.pattern
        m = int(len(exc_index))
        if m != self.n_sys:
            N.check(N.lib.pasif_batch_resize(self.handle, m))
            self.n_sys = m
        if _is_device(values):
            mem = N.DEVICE
            ptrs = [C.c_void_p(t.data_ptr()) for t in (values, x0, exc_index)]
            self._keep = (values, x0, exc_index)
        else:
            mem = N.HOST
            v = N.f64(values).reshape(self.n_sys, p.P)
            x = N.f64(x0).reshape(self.n_sys, p.n)
            e = N.i32(exc_index).reshape(self.n_sys)
            self._keep = (v, x, e)
            ptrs = [C.c_void_p(a.ctypes.data) for a in (v, x, e)]
        N.check(N.lib.pasif_batch_set(self.handle, *ptrs, mem, _stream(stream)))

    def forward(self, signals: Signals, h: float, nsteps: int, step0: int = 0, max_comp=(), max_start: int = 0,
                sq_comp=(), sq_start: int = 0, stream=None):
        self._red = reducers_c(max_comp, max_start, sq_comp, sq_start)
        self._h = float(h)
        N.check(N.lib.pasif_batch_forward(self.handle, signals.handle, float(h), int(step0), int(nsteps),
                                          C.byref(self._red), _stream(stream)))

    def get(self, stream=None):
        """(state[n_sys][n], max[n_sys][n_max], sq[n_sys]) as numpy float64."""
        p = self.plan.pattern
        nmax = int(self._red.n_max) if hasattr(self, "_red") else 0
        st = np.empty((self.n_sys, p.n))
        mx = np.empty((self.n_sys, max(nmax, 1)))
        sq = np.empty(self.n_sys)
        N.check(N.lib.pasif_batch_get(self.handle, C.c_void_p(st.ctypes.data), C.c_void_p(mx.ctypes.data),
                                      C.c_void_p(sq.ctypes.data), N.HOST, _stream(stream)))
        return st, mx[:, :nmax], sq

    def get_device(self, state, mx=None, sq=None, stream=None):
        """Write results into CUDA tensors (float64, contiguous)."""
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)
        N.check(N.lib.pasif_batch_get(self.handle, ptr(state), ptr(mx), ptr(sq), N.DEVICE, _stream(stream)))

    def adjoint(self, signals: Signals, h: float, nsteps: int, g_final=None, g_sq=None, sq_comp=(),
                sq_start: int = 0, stream=None):
        """Exact discrete adjoint: returns (d_values[n_sys][P], d_x0[n_sys][n])."""
        p = self.plan.pattern
        red = reducers_c((), 0, sq_comp, sq_start)
        gf = N.f64(g_final).reshape(self.n_sys, p.n) if g_final is not None else None
        gs = N.f64(g_sq).reshape(self.n_sys) if g_sq is not None else None
        dv = np.empty((self.n_sys, p.P))
        dx = np.empty((self.n_sys, p.n))
        vp = lambda a: C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)
        N.check(N.lib.pasif_batch_adjoint(self.handle, signals.handle, float(h), int(nsteps), C.byref(red), vp(gf),
                                          vp(gs), vp(dv), vp(dx), N.HOST, _stream(stream)))
        return dv, dx

    def adjoint_device(self, signals: Signals, h: float, nsteps: int, g_final, g_sq, d_values, d_x0, sq_comp=(),
                       sq_start: int = 0, stream=None):
        red = reducers_c((), 0, sq_comp, sq_start)
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)
        N.check(N.lib.pasif_batch_adjoint(self.handle, signals.handle, float(h), int(nsteps), C.byref(red),
                                          ptr(g_final), ptr(g_sq), ptr(d_values), ptr(d_x0), N.DEVICE,
                                          _stream(stream)))

    def kernel_info(self):
        k, r, a = C.c_int(), C.c_int(), C.c_int()
        N.check(N.lib.pasif_batch_kernel_info(self.handle, C.byref(k), C.byref(r)))
        N.check(N.lib.pasif_batch_adjoint_kernel(self.handle, C.byref(a)))
        names = {0: "none", 1: "generic", 2: "specialised"}
        return {"kind": names[k.value], "registers": r.value, "adjoint": names[a.value]}

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            N.lib.pasif_batch_destroy(h)
            self.handle = None


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def forward(pattern: Pattern, values, x0, exc_index, x, h: float, nsteps: int, window: int = 0, im=None,
            precision="fp64", step0: int = 0, max_comp=(), max_start: int = 0, sq_comp=(), sq_start: int = 0):
    """One-shot forward from host arrays through pasif_forward (upload,
    integrate, download).  Returns (state, max, sq)."""
    v = N.f64(values).reshape(-1, pattern.P)
    n_sys = v.shape[0]
    x0a = N.f64(x0).reshape(n_sys, pattern.n)
    e = N.i32(exc_index).reshape(n_sys)
    xa = N.f64(x)
    if xa.ndim == 1:
        xa = xa[None, :]
    im_a = N.f64(im).reshape(-1) if im is not None else None
    red = reducers_c(max_comp, max_start, sq_comp, sq_start)
    c = pattern.to_c()
    st = np.empty((n_sys, pattern.n))
    mx = np.empty((n_sys, max(int(red.n_max), 1)))
    sq = np.empty(n_sys)
    N.check(N.lib.pasif_forward(C.byref(c), _prec(precision), n_sys, N.dptr(v), N.dptr(x0a), N.iptr(e), N.dptr(xa),
                                xa.shape[0], xa.shape[1], int(window), N.dptr(im_a) if im_a is not None else None,
                                float(h), int(step0), int(nsteps), C.byref(red), N.dptr(st), N.dptr(mx), N.dptr(sq)))
    return st, mx[:, :int(red.n_max)], sq


def verified_adjoint(pattern: Pattern, values, x0, exc_index, x, h: float, nsteps: int, window: int = 0, im=None,
                     g_final=None, g_sq=None, sq_comp=(), sq_start: int = 0, tol: float = 5e-6,
                     adjoint_storage=None, stream=None):
    """Gradients for every system within about 1e-5 of FP64, at FP32 speed
    for the systems FP32 stage arithmetic can serve.

    The extended-state adjoint ("fp32_ext") of every system is cross-checked
    against the compensated-FP32 adjoint ("fp32_kahan"): both carry the
    FP32 rounding of the stages, through different update arithmetic, so on
    a system whose trajectory amplifies rounding (chaotic or near-resonant
    over the horizon) they disagree.  Systems whose gradients differ by more
    than `tol` (per system, max|g_ext - g_kahan| / max|g_ext|) are recomputed
    with the FP64 adjoint.  On the 8-DOF chain configuration (4096 systems x
    5e4 steps) tol = 5e-6 flags 2 % of the systems, every one whose
    extended-state error exceeds 1e-5 among them (GB300 measurement).

    Returns (d_values[n_sys][P], d_x0[n_sys][n], recomputed indices)."""
    v = N.f64(values).reshape(-1, pattern.P)
    n_sys = v.shape[0]
    x0a = N.f64(x0).reshape(n_sys, pattern.n)
    e = N.i32(exc_index).reshape(n_sys)
    gf = N.f64(g_final).reshape(n_sys, pattern.n) if g_final is not None else None
    gs = N.f64(g_sq).reshape(n_sys) if g_sq is not None else None
    out = {}
    for prec in ("fp32_ext", "fp32_kahan"):
        b = Batch(Plan(pattern, prec), v, x0a, e, stream=stream)
        if adjoint_storage is not None:
            b.adjoint_storage(adjoint_storage)
        out[prec] = b.adjoint(Signals(x, window, im, prec, stream=stream), h, nsteps, gf, gs, sq_comp, sq_start,
                              stream=stream)
        del b
    dv, dx = out["fp32_ext"]
    dk = out["fp32_kahan"][0]
    scale = np.maximum(np.max(np.abs(dv), axis=1), 1e-300)
    redo = np.where(np.max(np.abs(dv - dk), axis=1) / scale > tol)[0]
    if redo.size:
        b = Batch(Plan(pattern, "fp64"), v[redo], x0a[redo], e[redo], stream=stream)
        if adjoint_storage is not None:
            b.adjoint_storage(adjoint_storage)
        rv, rx = b.adjoint(Signals(x, window, im, "fp64", stream=stream), h, nsteps,
                           gf[redo] if gf is not None else None, gs[redo] if gs is not None else None, sq_comp,
                           sq_start, stream=stream)
        dv = dv.copy()
        dx = dx.copy()
        dv[redo] = rv
        dx[redo] = rx
    return dv, dx, redo
