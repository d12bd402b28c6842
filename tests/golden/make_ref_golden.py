"""Generate golden vectors from the REFERENCE's own CUDA driver.

Run once on a GPU machine, from the repository root, after building the
reference driver from the PASIf sources:

    REF_SRC=<dir holding PASIf's src/> bash oracle/ref/build_ref.sh
    python tests/golden/make_ref_golden.py

Every case is a seeded concatenated system in the reference's input format,
solved by oracle/_ref/ref_driver (the reference's __GpuDriver, reel =
double).  Inputs and the reference's outputs are stored in
tests/golden/ref_<case>.npz; tests/test_golden.py checks the CPU oracle
against them.  Cases stay inside what the reference computes correctly:
total tensor entries <= 128 (its SpTdV Lambda indexing is wrong beyond one
block of 128 threads), no interpolation read past the last signal, no full
last chunk in _getGradient (it writes one slot past its buffer), numsteps a
multiple of saveSteps for _getTrajectory.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from pasif_gb300.system import Pattern  # noqa: E402
from tests import cases  # noqa: E402

OUT = os.environ.get("GOLDEN_OUT", os.path.join(ROOT, "tests", "golden"))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def concat(blocks, sp_sizes=None):
    """Block-diagonal concatenation of (Pattern, values) blocks.  Tensor
    setpoint indices (positions 2.. of an entry) are offset by the blocks'
    setpoint sizes sp_sizes (the forward sizes, for adjoint systems)."""
    n_tot = sum(p.n for p, _ in blocks)
    sp_sizes = sp_sizes or [p.n for p, _ in blocks]
    ptr, col, g, l, ps, f = [0], [], [], [], [], []
    kv, gv, lv, pv, fv = [], [], [], [], []
    off = soff = 0
    for (p, v), spn in zip(blocks, sp_sizes):
        o = p.offsets()
        for i in range(p.n):
            for q in range(p.k_ptr[i], p.k_ptr[i + 1]):
                col.append(p.k_col[q] + off)
                kv.append(v[q])
            ptr.append(len(col))
        for idx, dst in ((p.g_idx, g), (p.l_idx, l), (p.p_idx, ps)):
            shift = np.array([off, off] + [soff] * (idx.shape[1] - 2))
            dst += (idx + shift).tolist()
        gv += list(v[o["Gamma"]:o["Lambda"]])
        lv += list(v[o["Lambda"]:o["Psi"]])
        pv += list(v[o["Psi"]:o["F"]])
        f += (p.f_idx + off).tolist()
        fv += list(v[o["F"]:o["end"]])
        off += p.n
        soff += spn
    pat = Pattern(n=n_tot, k_ptr=ptr, k_col=col, g_idx=np.asarray(g).reshape(-1, 3),
                  l_idx=np.asarray(l).reshape(-1, 4), p_idx=np.asarray(ps).reshape(-1, 5), f_idx=f, n_sp=soff)
    return pat, np.concatenate([kv, gv, lv, pv, fv]).astype(float)


def sys_block(pat, vals, n_sp=None, dims_sp=None):
    """Reference text block: K, Gamma, Lambda, Psi, dense F, IC placeholder."""
    o = pat.offsets()
    n = pat.n
    sp = n_sp or n
    lines = [f"{n} {n} {pat.k_nnz}", " ".join(repr(float(x)) for x in vals[:o['Gamma']]),
             " ".join(str(int(c)) for c in pat.k_col), " ".join(str(int(c)) for c in pat.k_ptr)]
    for name, w, a, b, idx in (("G", 3, "Gamma", "Lambda", pat.g_idx), ("L", 4, "Lambda", "Psi", pat.l_idx),
                               ("P", 5, "Psi", "F", pat.p_idx)):
        dims = [n, n] + [sp] * (w - 2)
        vv = vals[o[a]:o[b]]
        lines.append(" ".join(str(d) for d in dims) + f" {len(vv)}")
        lines.append(" ".join(repr(float(x)) for x in vv))
        lines.append(" ".join(str(int(x)) for x in idx.reshape(-1)))
    dense = np.zeros(n)
    dense[pat.f_idx] = vals[o["F"]:o["end"]]
    lines.append(f"{n} " + " ".join(repr(float(x)) for x in dense))
    return "\n".join(lines), dense


def run_case(name, fpat, fvals, x0, x, sr, N, W=0, im=None, task=0, save=0, bpat=None, bvals=None, a0=None):
    x = np.asarray(x, float)
    parts = [f"{x.shape[0]} {x.shape[1]}", " ".join(repr(float(v)) for v in x.reshape(-1)), f"{sr} {N}"]
    imf = np.asarray(im, float).reshape(-1) if W else np.zeros(0)
    parts.append(f"{W} {imf.size} " + " ".join(repr(float(v)) for v in imf))
    fb, fdense = sys_block(fpat, fvals)
    parts += [fb, f"{fpat.n} " + " ".join(repr(float(v)) for v in x0)]
    if bpat is not None:
        bb, bdense = sys_block(bpat, bvals, n_sp=fpat.n)
        parts += ["1", bb, f"{bpat.n} " + " ".join(repr(float(v)) for v in a0)]
    else:
        parts.append("0")
    parts.append(f"{task} {save}" if task else "0")
    with tempfile.TemporaryDirectory() as d:
        cf, of = os.path.join(d, "case.txt"), os.path.join(d, "out.txt")
        open(cf, "w").write("\n".join(parts) + "\n")
        r = subprocess.run([DRIVER, cf, of], capture_output=True, text=True, timeout=600)
        if r.returncode != 0 or not os.path.exists(of):
            raise RuntimeError(f"{name}: reference driver failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
        lines = open(of).read().split()
        err, count = int(lines[0]), int(lines[1])
        out = np.array([float(v) for v in lines[2:2 + count]])
        if err != 0:
            raise RuntimeError(f"{name}: CUDA error {err}")
    rec = dict(f_n=fpat.n, f_k_ptr=fpat.k_ptr, f_k_col=fpat.k_col, f_g=fpat.g_idx, f_l=fpat.l_idx, f_p=fpat.p_idx,
               f_f=fpat.f_idx, f_vals=fvals, x0=np.asarray(x0, float), x=x, h=1.0 / sr, N=N, W=W, im=imf,
               task=task, save=save, out=out)
    if bpat is not None:
        rec.update(b_n=bpat.n, b_k_ptr=bpat.k_ptr, b_k_col=bpat.k_col, b_g=bpat.g_idx, b_l=bpat.l_idx,
                   b_p=bpat.p_idx, b_f=bpat.f_idx, b_vals=bvals, a0=np.asarray(a0, float))
    np.savez_compressed(os.path.join(OUT, f"ref_{name}.npz"), **rec)
    print(name, "ok", out.size, "values")
    return out


def random_adjoint(rng, na, nf):
    """Random adjoint-shaped system: K over the adjoint state, Gamma/Lambda/Psi
    with setpoint (forward) trailing indices."""
    rows, cols, vals = [], [], []
    for i in range(na):
        for j in rng.choice(na, size=min(na, 2), replace=False):
            rows.append(i); cols.append(int(j)); vals.append(rng.normal(0, 0.3))
    g = [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf))) for _ in range(3)]
    l = [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf)), int(rng.integers(nf))) for _ in range(3)]
    p = [(int(rng.integers(na)), int(rng.integers(na)), int(rng.integers(nf)), int(rng.integers(nf)),
          int(rng.integers(nf))) for _ in range(2)]
    pat, order = Pattern.from_dense_lists(na, rows, cols, g, l, p, [], n_sp=nf)
    v = np.concatenate([np.asarray(vals)[order], rng.normal(0, 0.3, 3), rng.normal(0, 0.3, 3), rng.normal(0, 0.2, 2)])
    return pat, v


def main():
    if not os.path.exists(DRIVER):
        raise SystemExit("build the reference driver first: bash oracle/ref/build_ref.sh")
    rng = np.random.default_rng(2024)
    # A: sample and hold, 3 different systems, 3 signals, run past the signal end
    blocks = [cases.random_system(rng, n) for n in (3, 4, 2)]
    fp, fv = concat(blocks)
    x = cases.signals(rng, 3, 260)
    run_case("sah_mixed", fp, fv, rng.normal(0, 0.2, fp.n), x, 64, 300)
    # B: interpolation window 4 (j+1 stays inside the table)
    blocks = [cases.random_system(rng, n) for n in (2, 3)]
    fp, fv = concat(blocks)
    x = cases.signals(rng, 2, 200)
    W = 4
    im = np.stack([np.arange(W) / W, 1 - np.arange(W) / W])
    run_case("interp_w4", fp, fv, rng.normal(0, 0.2, fp.n), x, 100, 300, W=W, im=im)
    # C: config-2 shaped systems, W = 8
    from pasif_gb300 import synth
    w = synth.coupled2(n_sys=6, nsteps=2000, sig_len=2048)
    blocks = [(w.pattern, w.values[b]) for b in range(6)]
    fp, fv = concat(blocks)
    run_case("coupled2_w8", fp, fv, np.zeros(fp.n), w.signals[:3], 1000, 2000, W=8, im=w.im)
    # D: Duffing (config 1 shape), W = 2
    d = synth.duffing(n_sys=8, nsteps=1500)
    fp, fv = concat([(d.pattern, d.values[b]) for b in range(8)])
    run_case("duffing_w2", fp, fv, np.zeros(fp.n), d.signals[:2, :1600], 10000, 1500, W=2, im=d.im)
    # E: trajectory every 5 steps
    blocks = [cases.random_system(rng, n) for n in (3, 2)]
    fp, fv = concat(blocks)
    run_case("trajectory_s5", fp, fv, rng.normal(0, 0.2, fp.n), cases.signals(rng, 2, 150), 50, 100, task=1,
             save=5)
    # F: _getGradient, the 1-DOF probe system twice with its adjoint (N = 117: last chunk not full)
    c = cases.one_dof_probe()
    fpat1, fo = Pattern.from_dense_lists(4, c["fk"][0], c["fk"][1], g=c["fg"][0], l=c["fl"][0], f=[2])
    fv1 = np.concatenate([np.asarray(c["fk"][2])[fo], c["fg"][1], c["fl"][1], [1.0]])
    bpat1, bo = Pattern.from_dense_lists(6, c["bk"][0], c["bk"][1], l=c["bl"][0], p=c["bpsi"][0], n_sp=4)
    bv1 = np.concatenate([np.asarray(c["bk"][2])[bo], c["bl"][1], c["bpsi"][1]])
    fp, fv = concat([(fpat1, fv1), (fpat1, fv1)])
    bp, bv = concat([(bpat1, bv1), (bpat1, bv1)], sp_sizes=[4, 4])
    x = 1.0 + 0.1 * rng.standard_normal((2, 140))
    run_case("gradient_probe", fp, fv, np.zeros(8), x, 16, 117, task=2, save=0, bpat=bp, bvals=bv,
             a0=np.concatenate([c["a0"], c["a0"]]))
    # G: _getGradient with random adjoint tensors (N = 150: S = 12, C = 13, last chunk 7)
    fpat2, fv2 = cases.random_system(rng, 3)
    bpat2, bv2 = random_adjoint(rng, 5, 3)
    run_case("gradient_random", fpat2, fv2, rng.normal(0, 0.2, 3), cases.signals(rng, 2, 200), 40, 150, task=2,
             save=0, bpat=bpat2, bvals=bv2, a0=rng.normal(0, 1.0, 5))


if __name__ == "__main__":
    main()
