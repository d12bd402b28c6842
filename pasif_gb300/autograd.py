"""torch.autograd.Function over the forward kernel and the exact adjoint kernel.

    from pasif_gb300.autograd import RK4Solver
    solver = RK4Solver(pattern, signals, window, im, h, nsteps, exc_index,
                       precision="fp32_kahan", sq_comp=(0, 1), sq_start=nsteps // 2)
    state, sq = solver(values, x0)          # values[B][P], x0[B][n]: CUDA float64
    loss = sq.sum() + state[:, 0].pow(2).sum()
    loss.backward()                          # values.grad, x0.grad from the adjoint kernel

Outputs: the final state Q_N [B][n] and the reducer h * sum_{s >= sq_start}
sum_{c in sq_comp} Q_{s+1}[c]^2 [B].  The backward pass is the exact discrete
adjoint of the RK4 map (sqrt(N) checkpoints, recomputed segments, FP64
accumulation of parameter gradients), not a finite-difference or
continuous-adjoint approximation.
"""
from __future__ import annotations

import numpy as np
import torch

from .batch import Batch, Plan, Signals
from .system import Pattern


class _RK4Function(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, x0, solver):
        B = values.shape[0]
        p = solver.pattern
        values = values.detach().to(torch.float64).contiguous()
        x0 = x0.detach().to(torch.float64).contiguous()
        exc = solver.exc_index_dev(values.device)
        batch = Batch(solver.plan, values, x0, exc)
        batch.forward(solver.signals, solver.h, solver.nsteps, sq_comp=solver.sq_comp, sq_start=solver.sq_start)
        state = torch.empty((B, p.n), dtype=torch.float64, device=values.device)
        sq = torch.empty((B,), dtype=torch.float64, device=values.device)
        batch.get_device(state, None, sq)
        ctx.batch = batch
        ctx.solver = solver
        return state, sq

    @staticmethod
    def backward(ctx, g_state, g_sq):
        batch, solver = ctx.batch, ctx.solver
        B, p = batch.n_sys, solver.pattern
        dev = torch.device("cuda", torch.cuda.current_device())
        gf = g_state.to(torch.float64).contiguous() if g_state is not None else None
        gs = g_sq.to(torch.float64).contiguous() if g_sq is not None else None
        dv = torch.empty((B, p.P), dtype=torch.float64, device=dev)
        dx = torch.empty((B, p.n), dtype=torch.float64, device=dev)
        batch.adjoint_device(solver.signals, solver.h, solver.nsteps, gf, gs, dv, dx, sq_comp=solver.sq_comp,
                             sq_start=solver.sq_start)
        ctx.batch = None
        return dv, dx, None


class RK4Solver:
    """A pattern, an excitation table and a horizon; call with (values, x0)."""

    def __init__(self, pattern: Pattern, signals, window: int, im, h: float, nsteps: int, exc_index,
                 precision: str = "fp64", sq_comp=(), sq_start: int = 0):
        self.pattern = pattern
        self.precision = precision
        self.plan = Plan(pattern, precision)
        self.signals = Signals(signals, window, im, precision)
        self.h = float(h)
        self.nsteps = int(nsteps)
        self.exc_index = np.ascontiguousarray(np.asarray(exc_index, dtype=np.int32))
        self.sq_comp = tuple(int(c) for c in sq_comp)
        self.sq_start = int(sq_start)
        self._exc_dev = None

    def exc_index_dev(self, device):
        if self._exc_dev is None or self._exc_dev.device != device:
            self._exc_dev = torch.as_tensor(self.exc_index, device=device)
        return self._exc_dev

    def __call__(self, values: torch.Tensor, x0: torch.Tensor):
        if not values.is_cuda or not x0.is_cuda:
            raise ValueError("values and x0 must be CUDA tensors")
        return _RK4Function.apply(values, x0, self)
