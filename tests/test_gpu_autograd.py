"""torch.autograd.Function: gradients through the adjoint kernel equal the
oracle's exact discrete adjoint (FP64, bit for bit) and match finite
differences of the forward; FP32-Kahan and extended-state gradients within
1e-5 of FP64 (per system, relative to its largest gradient)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pasif_gb300 import synth

pytestmark = pytest.mark.gpu


def test_autograd_chain8(gpu):
    torch = pytest.importorskip("torch")
    from pasif_gb300.autograd import RK4Solver
    w = synth.chain8(n_sys=32, nsteps=1500)
    values = torch.tensor(w.values, device="cuda", requires_grad=True)
    x0 = torch.tensor(w.x0 + 0.01, device="cuda", requires_grad=True)
    solver = RK4Solver(w.pattern, w.signals, w.window, w.im, w.h, w.nsteps, w.exc_index, "fp64", w.sq_comp,
                       w.sq_start)
    state, sq = solver(values, x0)
    wts = torch.linspace(0.5, 1.5, w.n_sys, device="cuda", dtype=torch.float64)
    loss = (sq * wts).sum() + 0.3 * state[:, 0].sum()
    loss.backward()
    gf = np.zeros((w.n_sys, w.pattern.n))
    gf[:, 0] = 0.3
    odv, odx = O.batch_adjoint(w.pattern, w.values, w.x0 + 0.01, w.exc_index, w.signals, w.h, w.nsteps, w.window,
                               w.im, g_final=gf, g_sq=wts.cpu().numpy(), sq_comp=w.sq_comp, sq_start=w.sq_start)
    np.testing.assert_array_equal(values.grad.cpu().numpy(), odv)
    np.testing.assert_array_equal(x0.grad.cpu().numpy(), odx)
    # FP32 with compensated update, and the extended-state mode
    g64 = values.grad.cpu().numpy()
    for prec in ("fp32_kahan", "fp32_ext"):
        v32 = torch.tensor(w.values, device="cuda", requires_grad=True)
        s32 = RK4Solver(w.pattern, w.signals, w.window, w.im, w.h, w.nsteps, w.exc_index, prec, w.sq_comp,
                        w.sq_start)
        st32, sq32 = s32(v32, torch.tensor(w.x0 + 0.01, device="cuda"))
        ((sq32 * wts).sum() + 0.3 * st32[:, 0].sum()).backward()
        g32 = v32.grad.cpu().numpy()
        rel = np.max(np.abs(g32 - g64), axis=1) / np.max(np.abs(g64), axis=1)
        assert rel.max() <= 1e-5, (prec, rel.max())
