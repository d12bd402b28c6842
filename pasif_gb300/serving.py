"""Serving: continuous batching of forward and adjoint sweep requests.

A forward request (n systems of one pattern class, its signal table, a step
count) is admitted into a serving pool of its class as soon as the pool has
n free slots and room for the table in its signal arena (both device memory
allocated once, when the pool is made).  Each pool is driven by its own host
thread: one chunk launch (a CUDA-graph replay of the pattern-specialised
pk_pool kernel on the pool's stream) advances every busy slot by up to
`chunk` steps; between chunks finished requests are harvested and queued
ones admitted, so requests join and leave while others are in flight, and
the pools of different classes run concurrently on their own streams.

An adjoint request runs the exact discrete adjoint (pasif_batch_adjoint) in
one of a few worker threads, each on its own stream; it is admitted when its
device memory (checkpoints, chunk buffer, signal table, gradients) fits in
what is left of the adjoint memory budget.  A request that can never fit
(more systems than a pool has slots, a table larger than the arena, an
adjoint larger than the whole budget) is refused at once with an error
result instead of waiting forever.

A slot computes exactly what a one-request batch computes, so every result
is the same alone and in the mix, bit for bit (tests/test_gpu_serving.py).

The reference has no serving mode; the operator semantics follow its
forward and gradient calls (PASIf.py:469 getAmplitudes, PASIf.py:520
getGradient, src/__GpuDriver.cu:404, :451).
"""
from __future__ import annotations

import collections
import ctypes as C
import math
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .system import Pattern, reducers_c


class Pool:
    """Serving pool of one pattern class (pasif_pool_* of the C ABI)."""

    def __init__(self, pattern: Pattern, precision="fp32_kahan", window: int = 0, im=None, h: float = 1e-3,
                 max_comp=(), sq_comp=(), capacity: int = 4096, arena_samples: int = 1 << 22, chunk: int = 1024,
                 slicing=None):
        """slicing: None = by state size, True = warp-sliced kernel, False =
        thread per system."""
        self.pattern = pattern
        self.capacity = int(capacity)
        self.arena_samples = int(arena_samples)
        self.chunk = int(chunk)
        self.max_comp = tuple(max_comp)
        self.sq_comp = tuple(sq_comp)
        self.h = float(h)
        prec = N.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self._c = pattern.to_c()
        w = N.f64(im).reshape(-1) if (window and im is not None) else None
        red = reducers_c(self.max_comp, 0, self.sq_comp, 0)
        hdl = C.c_void_p()
        flags = 0 if slicing is None else (N.PLAN_WARP_SLICED if slicing else N.PLAN_NO_WARP_SLICED)
        N.check(N.lib.pasif_pool_create(C.byref(hdl), C.byref(self._c), prec, int(window),
                                        N.dptr(w) if w is not None else None, self.h, C.byref(red), self.capacity,
                                        self.arena_samples, self.chunk, flags))
        self.handle = hdl
        self._fin = np.zeros(self.capacity, np.int32)

    def admit(self, values, x0, exc_index, signals, nsteps: int, max_start: int = 0, sq_start: int = 0):
        """Request id, or None when slots or arena space are short now."""
        v = N.f64(values).reshape(-1, self.pattern.P)
        m = v.shape[0]
        x = N.f64(x0).reshape(m, self.pattern.n)
        e = N.i32(exc_index).reshape(m)
        s = N.f64(signals)
        s = s.reshape(1, -1) if s.ndim == 1 else s
        rid = C.c_int()
        rc = N.lib.pasif_pool_admit(self.handle, m, N.dptr(v), N.dptr(x), N.iptr(e), N.dptr(s), int(s.shape[0]),
                                    int(s.shape[1]), int(nsteps), int(max_start), int(sq_start), C.byref(rid))
        if rc == N.ERR_STATE:
            return None
        N.check(rc)
        return rid.value

    def launch(self) -> None:
        N.check(N.lib.pasif_pool_launch(self.handle))

    def poll(self) -> list:
        n = C.c_int()
        N.check(N.lib.pasif_pool_poll(self.handle, N.iptr(self._fin), self.capacity, C.byref(n)))
        return [int(r) for r in self._fin[:n.value]]

    def harvest(self, rid: int, n_sys: int):
        """(state[n_sys][n], max[n_sys][n_max], sq[n_sys]) of a finished request."""
        st = np.empty((n_sys, self.pattern.n))
        mx = np.empty((n_sys, max(len(self.max_comp), 1)))
        sq = np.empty(n_sys)
        N.check(N.lib.pasif_pool_harvest(self.handle, int(rid), N.dptr(st), N.dptr(mx), N.dptr(sq)))
        return st, mx[:, :len(self.max_comp)], sq

    def info(self) -> dict:
        fs, fa, ac = C.c_int(), C.c_longlong(), C.c_int()
        N.check(N.lib.pasif_pool_info(self.handle, C.byref(fs), C.byref(fa), C.byref(ac)))
        return {"free_slots": fs.value, "free_arena": fa.value, "active": ac.value}

    def close(self) -> None:
        h = getattr(self, "handle", None)
        if h:
            N.lib.pasif_pool_destroy(h)
            self.handle = None

    def __del__(self):
        self.close()


# ---- requests and results -------------------------------------------------

@dataclass
class ClassSpec:
    """What requests of one class share: pattern, time step, forcing window
    and weights, output components, chunk length of its pool."""
    pattern: Pattern
    h: float
    window: int = 0
    im: np.ndarray | None = None
    positions: tuple = ()
    chunk: int = 1024


@dataclass
class Request:
    """A sweep: values[n_sys][P], x0[n_sys][n], exc_index[n_sys] into
    signals[rows][len], nsteps RK4 steps from step 0.  forward -> state, max
    |x_i| (i in the class positions, steps >= max_start) and sum x_i^2 h;
    adjoint -> d loss / d values and d x0 for loss = h sum_{s >= sq_start}
    sum_i x_i(s+1)^2."""
    rid: int
    kind: str
    cls: object
    values: np.ndarray
    x0: np.ndarray
    exc_index: np.ndarray
    signals: np.ndarray
    nsteps: int
    max_start: int = 0
    sq_start: int = 0

    @property
    def n_sys(self) -> int:
        return int(self.values.shape[0])


@dataclass
class Result:
    rid: int
    kind: str
    t_arrival: float
    t_admit: float = math.nan
    t_done: float = math.nan
    state: np.ndarray | None = None
    amplitude: np.ndarray | None = None
    sq: np.ndarray | None = None
    d_values: np.ndarray | None = None
    d_x0: np.ndarray | None = None
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


def adjoint_bytes(pattern: Pattern, n_sys: int, nsteps: int, table: int, precision: str, storage: int = 0) -> int:
    """Device memory one adjoint request holds (the buffers pasif_batch_adjoint
    sizes: values, x0, state, FP64 gradients, scratch of the generic kernel,
    the signal table, and either the stored trajectory, when it fits in
    `storage` bytes (Batch.adjoint_storage), or checkpoints of state +
    compensation every ceil(sqrt(N)) steps and the recomputed chunk).  A
    trajectory slot is the state, and in FP64 also the stage inputs."""
    rs = 8 if precision == "fp64" else 4
    n, P = pattern.n, pattern.P
    sv = 4 if precision == "fp64" else 1
    full = (sv * nsteps + 1) * n
    if nsteps > 0 and n_sys * full * rs <= storage:
        traj = full
    else:
        c = max(1, math.ceil(math.sqrt(max(nsteps, 1))))
        nck = max(1, -(-nsteps // c))
        traj = 2 * n * nck + (sv * c + 1) * n + n   # checkpoints, a chunk's slots, the replay state
    per_sys = rs * (P + 3 * n + traj + 16 * n + 2) + 8 * (P + n)
    return int(n_sys * per_sys + rs * table + 4 * n_sys)


class Server:
    """Continuous-batching server over one GPU.

    specs: class key -> ClassSpec.  Pools (one per class) are made on first
    use or by warm().  Adjoint requests queue per class and each class has
    `adjoint_workers` workers, so cheap classes are not held behind long
    adjoints of large systems (head-of-line blocking); the memory budget is
    shared.  pool_factory(spec) and adjoint_runner(spec, request, stream) can
    be replaced (the host-only tests drive the scheduler with fakes); the
    defaults run the CUDA kernels."""

    def __init__(self, specs: dict, precision: str = "fp32_kahan", capacity: int = 8192,
                 arena_samples: int = 1 << 24, adjoint_budget: int = 8 << 30, adjoint_workers: int = 2,
                 pool_factory=None, adjoint_runner=None, stream_factory=None, clock=time.perf_counter,
                 reserve=None, adjoint_storage: int = 0):
        """reserve = (max systems, max steps, max signal samples) of an adjoint
        request: each worker sizes its batch and signal table for it on its
        first request, so later ones allocate nothing.  adjoint_storage:
        device bytes per adjoint worker batch for stored forward trajectories
        (a request whose trajectory fits skips the checkpoint recompute, about
        one forward pass; 0: always checkpointed)."""
        self.specs = dict(specs)
        self.reserve = reserve
        self.adjoint_storage = int(adjoint_storage)
        self.precision = precision
        self.capacity = int(capacity)
        self.arena_samples = int(arena_samples)
        self.adjoint_budget = int(adjoint_budget)
        self.clock = clock
        self._pool_factory = pool_factory or self._make_pool
        self._adjoint_runner = adjoint_runner or self._run_adjoint
        self._stream_factory = stream_factory or _torch_stream
        # adjoint stream priority per class: the cheaper a system-step, the
        # higher; their blocks then take SMs ahead of queued blocks of long
        # large-system adjoints (the pools' streams have the highest priority)
        cost = sorted(self.specs, key=lambda k: self.specs[k].pattern.flops_per_step())
        self._prio = {k: -max(0, 4 - (4 * i) // max(1, len(cost) - 1)) if len(cost) > 1 else 0
                      for i, k in enumerate(cost)}
        self._cv = threading.Condition()
        self._pools = {}
        self._fwd_q = collections.defaultdict(collections.deque)
        self._adj_q = collections.defaultdict(collections.deque)   # per class
        self._adj_used = 0
        self._results = {}
        self._outstanding = 0
        self._stop = False
        self._threads = []
        # adjoint workers per class: an int, or a dict class -> int (long adjoints of
        # large systems each run latency-bound on a few SMs: more of them at once)
        self._adj_workers = (dict(adjoint_workers) if isinstance(adjoint_workers, dict)
                             else {k: int(adjoint_workers) for k in self.specs})
        self._plans = {}
        self._tls = threading.local()     # per adjoint worker: reused batch and signal table per class
        self._worker_objs = {}            # (class, worker) -> (signals, batch) reserved by warm()
        self._errors = []
        self.t0 = self.clock()
        self.chunks = collections.Counter()

    # -- set-up ----------------------------------------------------------------
    def _make_pool(self, spec: ClassSpec):
        return Pool(spec.pattern, self.precision, spec.window, spec.im, spec.h, max_comp=spec.positions,
                    capacity=self.capacity, arena_samples=self.arena_samples, chunk=spec.chunk)

    def _pool(self, key):
        with self._cv:
            p = self._pools.get(key)
            if p is not None:
                return p
        p = self._pool_factory(self.specs[key])   # compiles outside the lock
        with self._cv:
            if key not in self._pools:
                self._pools[key] = p
                t = threading.Thread(target=self._pool_loop, args=(key,), daemon=True, name=f"pool-{key}")
                self._threads.append(t)
                t.start()
            return self._pools[key]

    def warm(self, keys=None, adjoint: bool = True) -> None:
        """Make the pools, compile the kernels of the given classes and (with
        `reserve`) size every adjoint worker's batch and signal table now:
        compilation and device allocation (which synchronises the device)
        are otherwise paid while requests are in flight."""
        for k in (self.specs if keys is None else keys):
            self._pool(k)
            if adjoint:
                spec = self.specs[k]
                n, P = spec.pattern.n, spec.pattern.P
                rq = Request(-1, "adjoint", k, np.zeros((1, P)), np.zeros((1, n)), np.zeros(1, np.int32),
                             np.zeros((1, 8)), 4, 0, 0)
                nw = self._adj_workers.get(k, 0)
                if nw == 0:
                    continue
                if self.reserve and self._adjoint_runner == self._run_adjoint:
                    for i in range(nw):
                        self._worker_objs[(k, i)] = self._adjoint_objects(spec, rq, None)
                    sig, b = self._worker_objs[(k, 0)]   # compile the adjoint kernel
                    b.adjoint(sig, spec.h, rq.nsteps, g_sq=np.ones(1), sq_comp=spec.positions, sq_start=0)
                    # and the forward kernels that replay the checkpoints of large requests
                    m = min(int(self.reserve[0]), 4096)
                    b.adjoint_storage(0)
                    b.set(np.zeros((m, P)), np.zeros((m, n)), np.zeros(m, np.int32))
                    b.adjoint(sig, spec.h, 8, g_sq=np.ones(m), sq_comp=spec.positions, sq_start=0)
                    b.adjoint_storage(self.adjoint_storage)
                else:
                    self._adjoint_runner(spec, rq, None)

    def start(self) -> None:
        self.t0 = self.clock()
        for key in self.specs:
            for i in range(self._adj_workers.get(key, 0)):
                t = threading.Thread(target=self._adj_loop, args=(key, i), daemon=True, name=f"adjoint-{key}-{i}")
                self._threads.append(t)
                t.start()

    def stop(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        self._threads = []
        for p in self._pools.values():
            close = getattr(p, "close", None)
            if close:
                close()
        self._pools = {}

    # -- requests --------------------------------------------------------------
    def now(self) -> float:
        return self.clock() - self.t0

    def submit(self, req: Request) -> None:
        n_sys = req.n_sys   # a malformed request raises here, before it is registered
        table = int(np.asarray(req.signals).size)
        res = Result(req.rid, req.kind, self.now())
        with self._cv:
            self._results[req.rid] = res
            self._outstanding += 1
        if req.kind in ("forward", "adjoint") and req.cls not in self.specs:
            return self._finish(res, error=f"unknown request class {req.cls!r}")
        if req.kind == "forward":
            if n_sys > self.capacity or table > self.arena_samples:
                return self._finish(res, error="request larger than a serving pool (slots or signal arena)")
            try:
                self._pool(req.cls)
            except Exception as exc:   # pool creation failed: this request fails, the server goes on
                return self._finish(res, error=f"serving pool for class {req.cls!r} unavailable: {exc}")
            with self._cv:
                self._fwd_q[req.cls].append((req, res))
                self._cv.notify_all()
        elif req.kind == "adjoint":
            spec = self.specs[req.cls]
            need = adjoint_bytes(spec.pattern, n_sys, req.nsteps, table, self.precision, self.adjoint_storage)
            if need > self.adjoint_budget:
                return self._finish(res, error=f"adjoint needs {need} bytes, budget {self.adjoint_budget}")
            with self._cv:
                self._adj_q[req.cls].append((req, res, need))
                self._cv.notify_all()
        else:
            self._finish(res, error=f"unknown request kind {req.kind!r}")

    def _finish(self, res: Result, error: str | None = None) -> None:
        res.t_done = self.now()
        res.error = error
        with self._cv:
            self._outstanding -= 1
            self._cv.notify_all()

    def wait(self, timeout: float | None = None) -> bool:
        """Block until every submitted request has a result."""
        end = None if timeout is None else self.clock() + timeout
        with self._cv:
            while self._outstanding > 0:
                if self._errors:
                    raise self._errors[0]
                left = None if end is None else end - self.clock()
                if left is not None and left <= 0:
                    return False
                self._cv.wait(0.05 if left is None else min(left, 0.05))
            if self._errors:
                raise self._errors[0]
        return True

    def results(self) -> dict:
        return dict(self._results)

    # -- pool threads ----------------------------------------------------------
    def _pool_loop(self, key) -> None:
        try:
            pool = self._pools[key]
            q = self._fwd_q[key]
            running = {}
            while True:
                with self._cv:
                    while not q and not running and not self._stop:
                        self._cv.wait()
                    if self._stop:
                        return
                    pending = list(q)
                consumed, refused = 0, []
                for req, res in pending:      # first come, first served; stop at the first that does not fit
                    try:
                        rid = pool.admit(req.values, req.x0, req.exc_index, req.signals, req.nsteps,
                                         req.max_start, req.sq_start)
                    except (N.PasifError, ValueError, TypeError) as e:   # invalid request; the pool goes on
                        refused.append((res, f"forward refused: {e}"))
                        consumed += 1
                        continue
                    if rid is None:
                        if not running and consumed == 0:   # does not fit an idle pool: never will
                            refused.append((res, "request does not fit an idle serving pool"))
                            consumed += 1
                        break
                    res.t_admit = self.now()
                    running[rid] = (req, res)
                    consumed += 1
                if consumed:
                    with self._cv:
                        for _ in range(consumed):
                            q.popleft()
                for res, err in refused:
                    self._finish(res, error=err)
                if not running:
                    continue
                pool.launch()
                self.chunks[key] += 1
                for rid in pool.poll():
                    req, res = running.pop(rid)
                    res.state, res.amplitude, res.sq = pool.harvest(rid, req.n_sys)
                    self._finish(res)
        except Exception as e:   # surfaced by wait()
            with self._cv:
                self._errors.append(e)
                self._cv.notify_all()

    # -- adjoint workers -------------------------------------------------------
    def _adj_loop(self, key, index: int = 0) -> None:
        try:
            objs = self._worker_objs.get((key, index))
            if objs is not None:   # reserved by warm()
                self._tls.__dict__.setdefault("objs", {})[id(self.specs[key])] = objs
            stream = self._stream_factory(self._prio.get(key, 0))
            q = self._adj_q[key]
            while True:
                with self._cv:
                    while not self._stop and not (q and q[0][2] <= self.adjoint_budget - self._adj_used):
                        self._cv.wait()
                    if self._stop:
                        return
                    req, res, need = q.popleft()
                    self._adj_used += need
                res.t_admit = self.now()
                err = None
                try:
                    res.d_values, res.d_x0 = self._adjoint_runner(self.specs[req.cls], req, stream)
                except (N.PasifError, ValueError, TypeError) as e:   # this request failed; the worker goes on
                    err = f"adjoint failed: {e}"
                finally:
                    with self._cv:
                        self._adj_used -= need
                        self._cv.notify_all()
                self._finish(res, error=err)
        except Exception as e:
            with self._cv:
                self._errors.append(e)
                self._cv.notify_all()

    def _run_adjoint(self, spec: ClassSpec, req: Request, stream):
        """One adjoint request on this worker's stream.  Each worker keeps one
        batch and one signal table per class and reuses their device buffers:
        a device allocation or free per request would synchronise the whole
        device and stall every other request in flight."""
        cache = self._tls.__dict__.setdefault("objs", {})
        objs = cache.get(id(spec))
        if objs is None:
            sig, b = cache[id(spec)] = self._adjoint_objects(spec, req, stream)
        else:
            sig, b = objs
            sig.update(req.signals, stream=stream)
            b.set(req.values, req.x0, req.exc_index, stream=stream)
        return b.adjoint(sig, spec.h, req.nsteps, g_sq=np.ones(req.n_sys), sq_comp=spec.positions,
                         sq_start=req.sq_start, stream=stream)

    def _adjoint_objects(self, spec: ClassSpec, req: Request, stream):
        """A signal table and a batch of the class (plan shared, no literals),
        holding `req`, with buffers reserved for the largest request."""
        from .batch import Batch, Plan, Signals
        with self._cv:
            plan = self._plans.get(id(spec))
        if plan is None:
            plan = Plan(spec.pattern, self.precision, literals=False)
            with self._cv:
                plan = self._plans.setdefault(id(spec), plan)
        sig = Signals(req.signals, spec.window, spec.im, self.precision, stream=stream)
        b = Batch(plan, req.values, req.x0, req.exc_index, stream=stream)
        b.adjoint_storage(self.adjoint_storage)   # the memory adjoint_bytes() books
        if self.reserve:   # grown buffers are fresh: upload the request again afterwards
            max_sys, max_steps, max_samples = self.reserve
            b.reserve(max_sys, max_steps)
            b.set(req.values, req.x0, req.exc_index, stream=stream)
            sig.update(np.zeros((1, int(max_samples))), stream=stream)
            sig.update(req.signals, stream=stream)
        return sig, b


def _torch_stream(priority: int = 0):
    """A CUDA stream; lower priority numbers are scheduled first (torch clamps
    to the device's range)."""
    import torch
    return torch.cuda.Stream(priority=priority)


# ---- the served mixed stream ------------------------------------------------

def chunk_for(pattern: Pattern) -> int:
    """Steps per chunk launch: shorter for larger systems, so that one chunk
    takes about a millisecond."""
    n = pattern.n
    return 4096 if n <= 8 else 2048 if n <= 16 else 1024 if n <= 32 else 512


def served_specs(dofs=None) -> dict:
    from . import synth
    out = {}
    for d in (synth.SERVED_DOFS if dofs is None else dofs):
        c = synth.served_class(d)
        out[d] = ClassSpec(c.pattern, c.h, c.window, c.im, c.positions, chunk_for(c.pattern))
    return out


def make_request(sr, spec: ClassSpec, rows: int = 4) -> Request:
    """Request of a ServedRequest (synth.served_stream): values of the class
    family, zero initial state, `rows` forcing signals."""
    from . import synth
    cls = synth.served_class(sr.dof)
    vals = cls.sample(sr.n_sys, sr.seed)
    sig = synth.served_signals(sr.seed + 1, sr.nsteps, spec.window, spec.h, rows)
    exc = (np.arange(sr.n_sys) % rows).astype(np.int32)
    half = sr.nsteps // 2
    return Request(sr.rid, sr.kind, sr.dof, vals, np.zeros((sr.n_sys, spec.pattern.n)), exc, sig, sr.nsteps,
                   max_start=half, sq_start=half)


def percentile(xs, q) -> float:
    xs = sorted(xs)
    if not xs:
        return math.nan
    k = (len(xs) - 1) * q / 100.0
    lo, hi = int(math.floor(k)), int(math.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def serve_stream(server: Server, requests, realtime: bool = True, timeout: float | None = None) -> dict:
    """Submit requests at their arrival times (realtime) or all at once,
    wait for every result; returns the per-request results and a summary."""
    server.start()
    t_start = server.now()
    for r in requests:
        if realtime:
            delay = r[0] - (server.now() - t_start)
            if delay > 0:
                time.sleep(delay)
        server.submit(r[1])
    ok = server.wait(timeout)
    t_end = server.now()
    res = server.results()
    done = [x for x in res.values() if x.error is None and not math.isnan(x.t_done)]
    lat = [x.latency * 1e3 for x in done]
    return {"results": res, "complete": ok, "wall_s": t_end - t_start,
            "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99),
            "refused": sum(1 for x in res.values() if x.error is not None)}
