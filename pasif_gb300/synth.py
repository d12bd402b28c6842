"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved: every value and excitation is drawn from a seeded
numpy Generator.  Systems are built directly in first-order form, i.e. with
the values the driver receives after PASIf.py's -M^-1 preprocessing
(PASIf.py:607-618) with M = I:  x' = v,  v' = -K x - C v + nonlinear + F u.

Mapping to the reference's tensor slots: quadratic terms go to the 3-D
`Gamma` slot and cubic terms to the 4-D `Lambda` slot (src/kernels.cu:52,56),
whatever the prose of a configuration calls them.

Choices recorded here (the configuration text leaves them open):
  * config 2: coupled springs K = [[k1+kc, -kc], [-kc, k2+kc]], Rayleigh
    C = a I + b K with a ~ U[0.01, 0.05] (a strictly positive floor keeps every
    draw damped) and b ~ U[0, 0.05]; the two self-cubic terms are restoring
    (-|N(0, 0.5^2)|), the two cross-cubic terms N(0, 0.5^2); quadratic
    x1 x2 -> v1, x1^2 -> v2, x2^2 -> v2 ~ N(0, 0.2^2); force 0.05 on DOF 1;
    8 noises band-limited to [0.05, 1] by a Gaussian-edged mask, unit RMS,
    stored as float32 values; one sample per 4 steps (window W = 8, linear
    weights); probe p' = x2^2, output sqrt(p(T)/T).
  * config 3: undamped chain, restoring cubic x_i^3 with g ~ U[0, 2], quadratic
    x_i x_{i+1} -> v_i for i = 0, 2, 4, 6 with N(0, 0.2^2); sine of frequency
    f ~ U[0.1, 1] per system (one signal per system), one sample per step.
  * config 4: 7-diagonal (|i-j| <= 3) stiffness, off-diagonals -U[0.5, 4]/8,
    diagonal sum|off| + U[0.5, 4]; light damping c_i ~ U[0.02, 0.1] (the
    configuration names none; undamped, some forced systems grew without
    bound over the 500 time units in FP64 too, leaving no reference value
    for the precision comparison); 96 cubic terms (x_i^3 restoring, x_i^2 x_j
    and x_i x_j^2 with |i-j| = 1, N(0, 0.3^2)); 8 multisines of 16 tones.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .system import Pattern


@dataclass
class Workload:
    name: str
    pattern: Pattern
    values: np.ndarray          # [B][P]
    x0: np.ndarray              # [B][n]
    exc_index: np.ndarray       # [B]
    signals: np.ndarray         # [E][L]
    window: int
    im: np.ndarray | None
    h: float
    nsteps: int
    sample_rate: int
    max_comp: tuple = ()
    max_start: int = 0
    sq_comp: tuple = ()
    sq_start: int = 0
    notes: dict = field(default_factory=dict)

    @property
    def n_sys(self) -> int:
        return int(self.values.shape[0])

    def flops_per_system_step(self) -> int:
        return self.pattern.flops_per_step(len(self.max_comp) + len(self.sq_comp))

    def forward_kwargs(self) -> dict:
        return dict(max_comp=self.max_comp, max_start=self.max_start, sq_comp=self.sq_comp, sq_start=self.sq_start)


def linear_weights(window: int) -> np.ndarray:
    """Rows (next-sample, current-sample) of a W-window linear interpolation,
    the layout src/kernels.cu:123 reads: u = IM[W+idx] x[j] + IM[idx] x[j+1]."""
    k = np.arange(window, dtype=np.float64) / window
    return np.stack([k, 1.0 - k])


class _Builder:
    """Collects first-order terms of one system in declaration order."""

    def __init__(self, n):
        self.n = n
        self.k = []      # (row, col)
        self.g = []      # (i, j, k)
        self.l = []      # (i, j, k, l)
        self.f = []      # i

    def pattern(self):
        pat, order = Pattern.from_dense_lists(self.n, [r for r, _ in self.k], [c for _, c in self.k], self.g, self.l,
                                              (), self.f)
        return pat, order


def _assemble(b: _Builder, kvals: np.ndarray, gvals: np.ndarray, lvals: np.ndarray, fvals: np.ndarray):
    """values [B][P] from per-term value columns (kvals in declaration order)."""
    pat, order = b.pattern()
    cols = [kvals[:, order]]
    if gvals.size:
        cols.append(gvals)
    if lvals.size:
        cols.append(lvals)
    cols.append(fvals)
    return pat, np.ascontiguousarray(np.concatenate(cols, axis=1))


def duffing(n_sys: int = 1024, nsteps: int = 100_000, seed: int = 1) -> Workload:
    """Config 1: x'' + c x' + k x + g x^3 = a u(t), u = sin(2 pi f t) sampled
    at 1e4 per unit time, RK4 at h = 1e-4, max |x| over the last half."""
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.5, 2.0, n_sys)
    c = rng.uniform(0.01, 0.1, n_sys)
    g = rng.uniform(0.0, 1.0, n_sys)
    a = rng.uniform(0.1, 1.0, n_sys)
    f = rng.uniform(0.05, 0.5, n_sys)
    b = _Builder(2)
    b.k = [(0, 1), (1, 0), (1, 1)]
    b.l = [(1, 0, 0, 0)]
    b.f = [1]
    kv = np.stack([np.ones(n_sys), -k, -c], axis=1)
    pat, vals = _assemble(b, kv, np.zeros((n_sys, 0)), (-g)[:, None], a[:, None])
    L = nsteps + 2
    t = np.arange(L) * 1e-4
    sig = np.sin(2 * np.pi * f[:, None] * t[None, :])
    return Workload("duffing_1dof_fp64", pat, vals, np.zeros((n_sys, 2)), np.arange(n_sys, dtype=np.int32), sig, 2,
                    linear_weights(2), 1e-4, nsteps, 10_000, max_comp=(0,), max_start=nsteps // 2,
                    notes={"output": "max |x| over steps >= N/2"})


def band_noise(n_sig: int, length: int, dt: float, lo: float, hi: float, rng) -> np.ndarray:
    """Unit-RMS noise band-limited to [lo, hi] by a Gaussian-edged mask, float32 values."""
    w = rng.standard_normal((n_sig, length))
    spec = np.fft.rfft(w, axis=1)
    fr = np.fft.rfftfreq(length, dt)
    edge = 0.1 * (hi - lo)
    mask = np.ones_like(fr)
    mask[fr < lo] = np.exp(-0.5 * ((fr[fr < lo] - lo) / (0.2 * lo)) ** 2)
    mask[fr > hi] = np.exp(-0.5 * ((fr[fr > hi] - hi) / edge) ** 2)
    x = np.fft.irfft(spec * mask[None, :], n=length, axis=1)
    x /= np.sqrt(np.mean(x * x, axis=1, keepdims=True))
    return x.astype(np.float32).astype(np.float64)


def coupled2(n_sys: int = 16384, nsteps: int = 200_000, seed: int = 2, n_sig: int = 8,
             sig_len: int = 65536) -> Workload:
    """Config 2: 2-DOF coupled Duffing-type systems, quadratic + cubic
    coupling, band-limited noise forcing, RMS of DOF 2 via a probe state."""
    rng = np.random.default_rng(seed)
    k1 = rng.uniform(0.5, 2.0, n_sys)
    k2 = rng.uniform(0.5, 2.0, n_sys)
    kc = rng.uniform(0.0, 0.3, n_sys)
    al = rng.uniform(0.01, 0.05, n_sys)
    be = rng.uniform(0.0, 0.05, n_sys)
    K11, K12, K22 = k1 + kc, -kc, k2 + kc
    C11, C12, C22 = al + be * K11, be * K12, al + be * K22
    b = _Builder(5)   # x1 x2 v1 v2 p
    b.k = [(0, 2), (1, 3), (2, 0), (2, 1), (2, 2), (2, 3), (3, 0), (3, 1), (3, 2), (3, 3)]
    kv = np.stack([np.ones(n_sys), np.ones(n_sys), -K11, -K12, -C11, -C12, -K12, -K22, -C12, -C22], axis=1)
    b.g = [(2, 0, 1), (3, 0, 0), (3, 1, 1), (4, 1, 1)]
    gv = np.concatenate([rng.normal(0.0, 0.2, (n_sys, 3)), np.ones((n_sys, 1))], axis=1)
    b.l = [(2, 0, 0, 0), (3, 1, 1, 1), (2, 0, 1, 1), (3, 0, 0, 1)]
    lv = np.concatenate([-np.abs(rng.normal(0.0, 0.5, (n_sys, 2))), rng.normal(0.0, 0.5, (n_sys, 2))], axis=1)
    b.f = [2]
    fv = np.full((n_sys, 1), 0.05)
    pat, vals = _assemble(b, kv, gv, lv, fv)
    window = 8
    h = 1e-3
    sig = band_noise(n_sig, sig_len, h * window / 2, 0.05, 1.0, rng)
    exc = (np.arange(n_sys) % n_sig).astype(np.int32)
    return Workload("coupled_2dof_fp32_kahan", pat, vals, np.zeros((n_sys, 5)), exc, sig, window,
                    linear_weights(window), h, nsteps, 1000,
                    notes={"output": "sqrt(p(T)/T), p' = x2^2 (state 4)", "T": nsteps * h})


def chain8(n_sys: int = 4096, nsteps: int = 50_000, seed: int = 3, nd: int = 8) -> Workload:
    """Config 3: 8-DOF spring chain, tridiagonal K, restoring cubic, 4
    quadratic couplings, sine forcing on DOF 1; loss = h sum of squared
    positions over the final half (sum-of-squares reducer).  `nd` gives the
    same chain with another number of DOFs (quadratic couplings on every
    second link)."""
    rng = np.random.default_rng(seed)
    n = 2 * nd
    b = _Builder(n)
    cols = []
    for i in range(nd):
        b.k.append((i, nd + i))
        cols.append(np.ones(n_sys))
    diag = rng.uniform(1.0, 3.0, (n_sys, nd))
    off = rng.uniform(-0.5, 0.0, (n_sys, nd - 1))
    for i in range(nd):
        b.k.append((nd + i, i))
        cols.append(-diag[:, i])
        if i > 0:
            b.k.append((nd + i, i - 1))
            cols.append(-off[:, i - 1])
        if i < nd - 1:
            b.k.append((nd + i, i + 1))
            cols.append(-off[:, i])
    kv = np.stack(cols, axis=1)
    b.g = [(nd + i, i, i + 1) for i in range(0, nd - 1, 2)]
    gv = rng.normal(0.0, 0.2, (n_sys, len(b.g)))
    b.l = [(nd + i, i, i, i) for i in range(nd)]
    lv = -rng.uniform(0.0, 2.0, (n_sys, nd))
    b.f = [nd]
    fv = np.ones((n_sys, 1))
    pat, vals = _assemble(b, kv, gv, lv, fv)
    f = rng.uniform(0.1, 1.0, n_sys)
    h = 1e-3
    t = np.arange(nsteps + 2) * h
    sig = np.sin(2 * np.pi * f[:, None] * t[None, :])
    return Workload(f"chain_{nd}dof_adjoint", pat, vals, np.zeros((n_sys, n)), np.arange(n_sys, dtype=np.int32), sig,
                    2, linear_weights(2), h, nsteps, 1000, sq_comp=tuple(range(min(nd, 64))), sq_start=nsteps // 2,
                    notes={"loss": "h * sum_{s >= N/2} sum_i x_i(s+1)^2"})


def banded32(n_sys: int = 2048, nsteps: int = 1_000_000, seed: int = 4, n_sig: int = 8,
             sig_len: int = 1 << 20) -> Workload:
    """Config 4: 32-DOF banded systems, 96 cubic terms, multisine forcing,
    long horizon; outputs the final state and max |x_0| over the last half."""
    rng = np.random.default_rng(seed)
    nd = 32
    n = 2 * nd
    b = _Builder(n)
    cols = []
    for i in range(nd):
        b.k.append((i, nd + i))
        cols.append(np.ones(n_sys))
    offs = {}
    for i in range(nd):
        for j in range(max(0, i - 3), min(nd, i + 4)):
            if j != i and (j, i) not in offs:
                offs[(i, j)] = offs[(j, i)] = -rng.uniform(0.5, 4.0, n_sys) / 8.0
    for i in range(nd):
        s = np.zeros(n_sys)
        row = []
        for j in range(max(0, i - 3), min(nd, i + 4)):
            if j != i:
                row.append((j, offs[(i, j)]))
                s += np.abs(offs[(i, j)])
        dval = s + rng.uniform(0.5, 4.0, n_sys)
        for j in range(max(0, i - 3), min(nd, i + 4)):
            b.k.append((nd + i, j))
            cols.append(-(dval if j == i else offs[(i, j)]))
    damp = rng.uniform(0.02, 0.1, (n_sys, nd))
    for i in range(nd):
        b.k.append((nd + i, nd + i))
        cols.append(-damp[:, i])
    kv = np.stack(cols, axis=1)
    terms = []
    vals_l = []
    for i in range(nd):
        terms.append((nd + i, i, i, i))
        vals_l.append(-np.abs(rng.normal(0.0, 0.3, n_sys)))
        j = i + 1 if i + 1 < nd else i - 1
        terms.append((nd + i, i, i, j))
        vals_l.append(rng.normal(0.0, 0.3, n_sys))
        terms.append((nd + i, i, j, j))
        vals_l.append(rng.normal(0.0, 0.3, n_sys))
    b.l = terms
    lv = np.stack(vals_l, axis=1)
    b.f = [nd]
    fv = np.full((n_sys, 1), 0.5)
    pat, vals = _assemble(b, kv, np.zeros((n_sys, 0)), lv, fv)
    h = 5e-4
    t = np.arange(sig_len) * h
    sig = np.zeros((n_sig, sig_len))
    for e in range(n_sig):
        fr = rng.uniform(0.05, 2.0, 16)
        ph = rng.uniform(0.0, 2 * np.pi, 16)
        sig[e] = np.sin(2 * np.pi * fr[:, None] * t[None, :] + ph[:, None]).sum(axis=0) / 4.0
    exc = (np.arange(n_sys) % n_sig).astype(np.int32)
    return Workload("banded_32dof_long", pat, vals, np.zeros((n_sys, n)), exc, sig, 2, linear_weights(2), h, nsteps,
                    2000, max_comp=(0,), max_start=nsteps // 2,
                    notes={"output": "final state and max |x_0| over steps >= N/2"})


CONFIGS = {"duffing": duffing, "coupled2": coupled2, "chain8": chain8, "banded32": banded32}


# ---- served mixed stream (config 5) -----------------------------------------

SERVED_DOFS = (1, 2, 4, 8, 16, 32, 64)


@dataclass
class ServedClass:
    """One request class of the served stream: a pattern with its time step
    and forcing interpolation; `positions` are the displacement components
    (amplitudes of a forward sweep, loss of an adjoint sweep)."""
    dof: int
    pattern: Pattern
    h: float
    window: int
    im: np.ndarray
    positions: tuple
    family: str

    def sample(self, n_sys: int, seed: int) -> np.ndarray:
        """values[n_sys][P] drawn as by the family's generator."""
        if self.family == "duffing":
            return duffing(n_sys=n_sys, nsteps=10, seed=seed).values
        if self.family == "coupled2":
            return coupled2(n_sys=n_sys, nsteps=10, seed=seed, sig_len=64).values
        if self.family == "banded32":
            return banded32(n_sys=n_sys, nsteps=10, seed=seed, sig_len=64).values
        return chain8(n_sys=n_sys, nsteps=10, seed=seed, nd=self.dof).values


def served_class(dof: int) -> ServedClass:
    """Request class with `dof` degrees of freedom: the Duffing oscillator
    (1), the coupled pair (2), the banded system (32) and the spring chain of
    that length otherwise."""
    if dof == 1:
        w = duffing(n_sys=1, nsteps=10)
        return ServedClass(1, w.pattern, 1e-4, 2, linear_weights(2), (0,), "duffing")
    if dof == 2:
        w = coupled2(n_sys=1, nsteps=10, sig_len=64)
        return ServedClass(2, w.pattern, 1e-3, 8, linear_weights(8), (0, 1), "coupled2")
    if dof == 32:
        w = banded32(n_sys=1, nsteps=10, sig_len=64)
        return ServedClass(32, w.pattern, 5e-4, 2, linear_weights(2), tuple(range(32)), "banded32")
    w = chain8(n_sys=1, nsteps=10, nd=dof)
    return ServedClass(dof, w.pattern, 1e-3, 2, linear_weights(2), tuple(range(min(dof, 64))), "chain")


@dataclass
class ServedRequest:
    rid: int
    kind: str              # "forward" or "adjoint"
    dof: int
    arrival: float         # seconds after the start of the stream
    n_sys: int
    nsteps: int
    seed: int


def served_stream(rate: float = 200.0, duration: float = 1.0, seed: int = 5, max_systems: int = 4096,
                  min_steps: int = 10_000, max_steps: int = 200_000, adjoint_fraction: float = 0.3,
                  dofs=SERVED_DOFS):
    """Poisson arrivals at `rate` per second for `duration` seconds: forward or
    adjoint (70/30) sweeps of log-uniform 1..max_systems systems of a DOF drawn
    from `dofs`, log-uniform min_steps..max_steps RK4 steps."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        n = int(np.exp(rng.uniform(0.0, np.log(max_systems))))
        steps = int(np.exp(rng.uniform(np.log(min_steps), np.log(max_steps))))
        kind = "adjoint" if rng.random() < adjoint_fraction else "forward"
        out.append(ServedRequest(len(out), kind, int(rng.choice(dofs)), t, max(1, n), steps,
                                 int(rng.integers(1 << 30))))
    return out


def served_signals(seed: int, nsteps: int, window: int, h: float, rows: int = 4) -> np.ndarray:
    """`rows` random-phase multisines long enough for nsteps steps (one sample
    per window/2 steps, float32 values)."""
    rng = np.random.default_rng(seed)
    spacing = max(1, window // 2)
    length = nsteps // spacing + 3
    t = np.arange(length) * h * spacing
    sig = np.zeros((rows, length))
    for r in range(rows):
        fr = rng.uniform(0.05, 1.0, 4)
        ph = rng.uniform(0.0, 2 * np.pi, 4)
        sig[r] = np.sin(2 * np.pi * fr[:, None] * t[None, :] + ph[:, None]).sum(axis=0) / 2.0
    return sig.astype(np.float32).astype(np.float64)
