"""Pure-Python loops restating the reference's semantics for tiny cases.

A second, independent restatement used to cross-check the C oracle (it
cannot reproduce fma rounding, so comparisons use a 1e-12 tolerance).
Follows src/kernels.cu:22-126,163-229 and src/__GpuDriver.cu:502-587,642-783.
"""
import math

import numpy as np


def force(x, e, L, total, W, im, step, off, half):
    if W == 0:
        st = step + off
        return x[e * L + st] if 0 < st < L else 0.0
    s2 = 2 * (step + off) + half
    idx = s2 & (W - 1)
    j = s2 >> int(math.log2(W))
    if 0 < j < L:
        base = e * L + j
        x1 = x[base + 1] if base + 1 < total else 0.0
        return im[W + idx] * x[base] + im[idx] * x1
    return 0.0


def rhs(sysd, xs, xp, u, use_force=True):
    n = sysd["n"]
    f = [0.0] * n
    for i in range(n):
        for p in range(sysd["k_ptr"][i], sysd["k_ptr"][i + 1]):
            f[i] += sysd["k_val"][p] * xs[sysd["k_col"][p]]
    for (i, j, k), v in zip(sysd["g_idx"], sysd["g_val"]):
        f[i] += v * xs[j] * xp[k]
    for (i, j, k, l), v in zip(sysd["l_idx"], sysd["l_val"]):
        f[i] += v * xs[j] * xp[k] * xp[l]
    for (i, j, k, l, m), v in zip(sysd["p_idx"], sysd["p_val"]):
        f[i] += v * xs[j] * xp[k] * xp[l] * xp[m]
    if use_force:
        for i, v in zip(sysd["f_idx"], sysd["f_val"]):
            f[i] += v * u
    return f


def step(sysd, Q, e, exc, h, t):
    x, L, W, im = exc["x"], exc["L"], exc["W"], exc["im"]
    total = len(x)
    h2, h6 = h / 2.0, h / 6.0
    ua = force(x, e, L, total, W, im, t, 0, 0)
    ub = force(x, e, L, total, W, im, t, 0, 1)
    uc = force(x, e, L, total, W, im, t, 1, 0)
    m1 = rhs(sysd, Q, Q, ua)
    mi = [q + h2 * m for q, m in zip(Q, m1)]
    m2 = rhs(sysd, mi, mi, ub)
    mi = [q + h2 * m for q, m in zip(Q, m2)]
    m3 = rhs(sysd, mi, mi, ub)
    mi = [q + h * m for q, m in zip(Q, m3)]
    m4 = rhs(sysd, mi, mi, uc)
    return [q + h6 * (a + 2 * b + 2 * c + d) for q, a, b, c, d in zip(Q, m1, m2, m3, m4)]


def amplitudes(sysd, x0, exc, h, N):
    out = []
    for e in range(exc["E"]):
        Q = list(x0)
        for t in range(N):
            Q = step(sysd, Q, e, exc, h, t)
        out.extend(Q)
    return np.array(out)


def gradient(fsys, x0, bsys, a0, exc, h, N, save=0):
    """_getGradient for a fresh driver, one excitation copy at a time."""
    nf, na = fsys["n"], bsys["n"]
    S = int(math.sqrt(N))
    C = int(math.ceil(N / S))
    lastC = C - (S * C) % N
    out = []
    for e in range(exc["E"]):
        traj = [[0.0] * nf for _ in range(S + C - 1)]
        Q = list(x0)
        idx = 0
        for t in range(N):
            Q = step(fsys, Q, e, exc, h, t)
            if t % C == 0:
                traj[idx] = list(Q)
                idx += 1
        A = list(a0)
        T = None
        for sp in range(S - 1, 0, -1):
            start = sp * C
            if sp == S - 1:
                end, sb = N, sp + lastC - 1
            else:
                end, sb = start + C, sp + C - 1
            Q = list(traj[sp])
            for i, t in enumerate(range(start, end)):
                Q = step(fsys, Q, e, exc, h, t)
                traj[sp + i] = list(Q)
            if T is None:
                T = sb
            spc = sb
            for _ in range(end - start):
                traj[T] = list(traj[spc])
                m1 = rhs(bsys, A, traj[T], 0.0, False)
                mi = [a + h / 2 * m for a, m in zip(A, m1)]
                traj[T] = [0.5 * (c + p) for c, p in zip(traj[spc], traj[spc - 1])]
                m2 = rhs(bsys, mi, traj[T], 0.0, False)
                mi = [a + h / 2 * m for a, m in zip(A, m2)]
                m3 = rhs(bsys, mi, traj[T], 0.0, False)
                mi = [a + h * m for a, m in zip(A, m3)]
                traj[T] = list(traj[spc - 1])
                m4 = rhs(bsys, mi, traj[T], 0.0, False)
                A = [a + h / 6 * (p + 2 * q + 2 * r + s) for a, p, q, r, s in zip(A, m1, m2, m3, m4)]
                spc -= 1
            if sp == save:
                break
        out.extend(A)
    return np.array(out)


def sysdict(pattern, values):
    o = pattern.offsets()
    v = np.asarray(values, dtype=np.float64)
    return {"n": pattern.n, "k_ptr": list(pattern.k_ptr), "k_col": list(pattern.k_col), "k_val": list(v[:o["Gamma"]]),
            "g_idx": [tuple(r) for r in pattern.g_idx], "g_val": list(v[o["Gamma"]:o["Lambda"]]),
            "l_idx": [tuple(r) for r in pattern.l_idx], "l_val": list(v[o["Lambda"]:o["Psi"]]),
            "p_idx": [tuple(r) for r in pattern.p_idx], "p_val": list(v[o["Psi"]:o["F"]]),
            "f_idx": list(pattern.f_idx), "f_val": list(v[o["F"]:o["end"]])}


def excdict(x, W=0, im=None):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[None, :]
    return {"x": list(x.reshape(-1)), "L": x.shape[1], "E": x.shape[0], "W": W,
            "im": list(np.asarray(im, dtype=np.float64).reshape(-1)) if W else []}
