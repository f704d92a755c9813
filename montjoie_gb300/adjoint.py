"""Receiver-misfit gradient with respect to the per-element wave speed.

The reference has no time-domain adjoint; this module adds one on top of the
many-source leap-frog.
- Forward: S sources from rest, traces of K receivers for U^0..U^N.
- Backward: the exact discrete adjoint of the leap-frog, a time-reversed
  leap-frog with the same symmetric operator.  Its adjoint sources are the
  trace residuals.  Forward states are checkpointed every ~sqrt(N) steps and
  replayed segment by segment.
- Gradient: dJ/dc_e = -2 dt^2 / c_e sum_n lambda^{n+1}^T A_e U^n.
All of it runs on the GPU through the C ABI (FP32 states, FP64 gradient
accumulation).  ``misfit`` exposes J(c) as a ``torch.autograd.Function``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .leapfrog import BatchLeapFrog
from .operator import FemMatrixFreeOperator


class AcousticAdjoint:
    """J(c) = 1/2 sum_{k,s,n} (r_{k,s}^n(c) - d_{k,s}^n)^2 and dJ/dc."""

    def __init__(self, order: int, nodle: np.ndarray, unit_factors: np.ndarray, n_dof: int, mass: np.ndarray,
                 dt: float, nsteps: int, n_runs: int, src_idx, src_rhs, src_val, pulse, rec_idx, rec_w,
                 checkpoint_every: int = 0):
        L = _lib.load()
        self.dt, self.N, self.S = float(dt), int(nsteps), int(n_runs)
        self.op = FemMatrixFreeOperator(order, nodle, unit_factors, n_dof, "fp32")
        self.n_elt = self.op.n_elt
        self.batch = BatchLeapFrog(self.op, dt, n_runs, mass, None, src_idx, src_rhs, src_val, pulse, rec_idx, rec_w)
        self.n_rec = int(np.asarray(rec_idx).shape[0])
        h = ctypes.c_void_p()
        _lib.check(L.mj_adj_create(self.batch.handle, self.N, int(checkpoint_every), ctypes.byref(h)))
        self._h = h
        self._c = None

    def set_speed(self, c: np.ndarray) -> None:
        c = np.ascontiguousarray(c, dtype=np.float64)
        if c.size != self.n_elt or np.any(c <= 0):
            raise ValueError("one positive wave speed per element")
        self.op.set_element_scale(c * c)  # mu = c^2 on unit-mu factors
        self._c = c.copy()

    def forward(self, c: np.ndarray) -> np.ndarray:
        """Traces (n_rec, S, N+1) of U^0..U^N for wave speed c."""
        self.set_speed(c)
        tr = np.zeros((self.n_rec, self.S, self.N + 1))
        _lib.check(_lib.load().mj_adj_forward(self._h, _lib.dptr(tr)))
        return tr

    def backward(self, residual: np.ndarray) -> np.ndarray:
        """dJ/dc for J with trace gradient `residual` (r - d), after forward()."""
        res = np.ascontiguousarray(residual, dtype=np.float64).reshape(self.n_rec, self.S, self.N + 1)
        coef = -2.0 * self.dt * self.dt / self._c
        grad = np.zeros(self.n_elt)
        _lib.check(_lib.load().mj_adj_backward(self._h, _lib.dptr(res), _lib.dptr(coef), _lib.dptr(grad)))
        return grad

    def loss_and_grad(self, c: np.ndarray, data: np.ndarray):
        tr = self.forward(c)
        res = tr - data
        return 0.5 * float((res * res).sum()), self.backward(res)

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().mj_adj_destroy(self._h)
            self._h = None
        self.batch.close()
        self.op.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _torch_function():
    import torch

    class MisfitFunction(torch.autograd.Function):
        """J(c) with the adjoint gradient; c is a 1-D tensor of per-element speeds."""

        @staticmethod
        def forward(ctx, c, model: AcousticAdjoint, data):
            c_np = c.detach().to("cpu", torch.float64).numpy()
            tr = model.forward(c_np)
            res = tr - data
            ctx.model, ctx.res = model, res
            ctx.dtype, ctx.device = c.dtype, c.device
            return torch.tensor(0.5 * float((res * res).sum()), dtype=c.dtype, device=c.device)

        @staticmethod
        def backward(ctx, grad_out):
            g = ctx.model.backward(ctx.res)
            g = torch.from_numpy(g).to(device=ctx.device, dtype=ctx.dtype) * grad_out
            return g, None, None

    return MisfitFunction


_MISFIT = None


def misfit(c, model: AcousticAdjoint, data: np.ndarray):
    """Differentiable J(c) (torch.autograd.Function over the C ABI)."""
    global _MISFIT
    if _MISFIT is None:
        _MISFIT = _torch_function()
    return _MISFIT.apply(c, model, data)
