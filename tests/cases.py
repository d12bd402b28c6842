"""Small seeded systems shared by the CPU and GPU tests."""
import numpy as np

from pasif_gb300.system import Pattern


def random_system(rng, n=None, with_psi=True, scale=0.3):
    """Random pattern + values: a damped linear part (stable) plus sparse
    quadratic / cubic / quartic terms in COO order that is NOT sorted by
    destination (exercises the canonical per-destination order)."""
    n = int(n or rng.integers(1, 7))
    rows, cols, vals = [], [], []
    for i in range(n):
        rows.append(i); cols.append(i); vals.append(-rng.uniform(0.5, 1.5))
        for j in rng.choice(n, size=min(n, 2), replace=False):
            if j != i:
                rows.append(i); cols.append(int(j)); vals.append(rng.normal(0, scale))
    ng = int(rng.integers(0, 5))
    g = [(int(rng.integers(n)), int(rng.integers(n)), int(rng.integers(n))) for _ in range(ng)]
    nl = int(rng.integers(0, 4))
    l = [(int(rng.integers(n)), int(rng.integers(n)), int(rng.integers(n)), int(rng.integers(n))) for _ in range(nl)]
    npsi = int(rng.integers(0, 3)) if with_psi else 0
    p = [tuple(int(rng.integers(n)) for _ in range(5)) for _ in range(npsi)]
    nf = int(rng.integers(1, min(n, 2) + 1))
    f = sorted(rng.choice(n, size=nf, replace=False).tolist())
    pat, order = Pattern.from_dense_lists(n, rows, cols, g, l, p, f)
    kv = np.asarray(vals)[order]
    v = np.concatenate([kv, rng.normal(0, scale, ng), rng.normal(0, scale, nl), rng.normal(0, scale, npsi),
                        rng.uniform(0.5, 1.5, nf)])
    return pat, v


def random_batch(rng, pat, v0, n_sys, spread=0.1):
    """n_sys instances of one pattern: values perturbed around v0, a few of
    them kept identical across instances (exercises literal folding)."""
    vals = np.repeat(v0[None, :], n_sys, axis=0)
    mask = rng.random(v0.size) < 0.7
    vals[:, mask] *= 1.0 + spread * rng.standard_normal((n_sys, int(mask.sum())))
    x0 = rng.normal(0, 0.2, (n_sys, pat.n))
    return vals, x0


def signals(rng, n_exc, length):
    t = np.arange(length)
    x = np.stack([np.sin(0.01 * (e + 1) * t) + 0.3 * rng.standard_normal(length) for e in range(n_exc)])
    return x


def one_dof_probe():
    """The 1-DOF probed system of examples/FullInterfaceTesting_1dof.py after
    PASIf's -M^-1 preprocessing (M = I): x' = v ... as the driver receives it.
    States (x, p?, v, probe) follow the example's 4x4 layout."""
    # forward: K_pre = -(B+K) with B (0,2)=-1,(1,3)=-1 and K (2,0)=k,(2,2)=b, k=b=1
    fk_rows, fk_cols, fk_vals = [0, 1, 2, 2], [2, 3, 0, 2], [1.0, 1.0, -1.0, -1.0]
    fg = [(3, 0, 0)]
    fg_vals = [1.0]          # -(-1)
    fl = [(0, 0, 0, 0)]
    fl_vals = [0.0]
    force = np.array([0.0, 0.0, 1.0, 0.0])
    # adjoint (6 states): K_pre = -(B) with B (1,4)=-1,(2,5)=-1; Lambda -(-1)
    bk_rows, bk_cols, bk_vals = [1, 2], [4, 5], [1.0, 1.0]
    bl = [(4, 0, 0, 0), (5, 0, 1, 1)]
    bl_vals = [1.0, 1.0]
    bpsi = [(1, 1, 1, 1, 1)]
    bpsi_vals = [0.0]
    a0 = np.array([1.0, 0, 0, 0, 0, 0])
    return dict(fk=(fk_rows, fk_cols, fk_vals), fg=(fg, fg_vals), fl=(fl, fl_vals), force=force,
                bk=(bk_rows, bk_cols, bk_vals), bl=(bl, bl_vals), bpsi=(bpsi, bpsi_vals), a0=a0, nf=4, na=6)
