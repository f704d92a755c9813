"""Receiver-misfit gradient with respect to the per-element wave speed.

The reference has no time-domain adjoint; this module adds one on top of the
many-source leap-frog.
- Forward: S sources from rest, traces of K receivers for U^0..U^N.
- Backward: the exact discrete adjoint of the leap-frog, a time-reversed
  leap-frog with the same symmetric operator.  Its adjoint sources are the
  trace residuals.  Forward states are checkpointed either every ~sqrt(N)
  steps and replayed segment by segment, or by a binomial (revolve) schedule
  under a budget of stored states, which recomputes the fewest forward steps
  for that budget; both give the same gradient bit for bit.
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
                 checkpoint_every: int = 0, snapshots: int | None = None):
        L = _lib.load()
        self.dt, self.N, self.S = float(dt), int(nsteps), int(n_runs)
        self.op = FemMatrixFreeOperator(order, nodle, unit_factors, n_dof, "fp32")
        self.n_elt = self.op.n_elt
        self.batch = BatchLeapFrog(self.op, dt, n_runs, mass, None, src_idx, src_rhs, src_val, pulse, rec_idx, rec_w)
        self.n_rec = int(np.asarray(rec_idx).shape[0])
        h = ctypes.c_void_p()
        if snapshots:
            _lib.check(L.mj_adj_create_revolve(self.batch.handle, self.N, int(snapshots), ctypes.byref(h)))
        else:
            _lib.check(L.mj_adj_create(self.batch.handle, self.N, int(checkpoint_every), ctypes.byref(h)))
        self._h = h
        self._c = None

    def schedule(self) -> dict:
        """Checkpoint schedule: revolve or uniform, stored state pairs, forward
        steps of one forward + backward pass, checkpoint bytes on the device."""
        rv, sn, fs, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_size_t()
        _lib.check(_lib.load().mj_adj_info(self._h, ctypes.byref(rv), ctypes.byref(sn), ctypes.byref(fs),
                                           ctypes.byref(nb)))
        return {"revolve": bool(rv.value), "snapshots": sn.value, "forward_steps": fs.value,
                "checkpoint_bytes": nb.value}

    def set_speed(self, c: np.ndarray) -> None:
        c = np.ascontiguousarray(c, dtype=np.float64)
        if c.size != self.n_elt or np.any(c <= 0):
            raise ValueError("one positive wave speed per element")
        self.op.set_element_scale(c * c)  # mu = c^2 on unit-mu factors
        self._c = c.copy()

    def forward(self, c: np.ndarray) -> np.ndarray:
        """Traces (n_rec, S, N+1) of U^0..U^N for wave speed c."""
        self.set_speed(c)
        S_dev = self.batch.S_dev  # runs padded to a multiple of 8 (no source, zero state)
        tr = np.zeros((self.n_rec, S_dev, self.N + 1))
        _lib.check(_lib.load().mj_adj_forward(self._h, _lib.dptr(tr)))
        return np.ascontiguousarray(tr[:, :self.S, :])

    def backward(self, residual: np.ndarray) -> np.ndarray:
        """dJ/dc for J with trace gradient `residual` (r - d), after forward()."""
        res = np.zeros((self.n_rec, self.batch.S_dev, self.N + 1))  # padding runs: no residual
        res[:, :self.S, :] = np.asarray(residual, dtype=np.float64).reshape(self.n_rec, self.S, self.N + 1)
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


class Fp64Misfit:
    """J(c) of AcousticAdjoint computed by the FP64 plain form: one FP64
    single-source integrator run per source (mj_lf_run with receivers), on
    unit-mu factors scaled by c^2 (mj_op_set_element_scale).  Slower than the
    FP32 batch; it serves as the reference of finite-difference checks of the
    adjoint gradient."""

    def __init__(self, order, nodle, unit_factors, n_dof, mass, dt, nsteps, n_runs, src_idx, src_rhs, src_val,
                 pulse, rec_idx, rec_w):
        from .leapfrog import LeapFrogIterator
        self.N, self.S, self.n_dof = int(nsteps), int(n_runs), int(n_dof)
        self.op = FemMatrixFreeOperator(order, nodle, unit_factors, n_dof, "fp64")
        src_idx, src_rhs, src_val = np.asarray(src_idx), np.asarray(src_rhs), np.asarray(src_val)
        self.runs = []
        for s in range(self.S):
            m = src_rhs == s
            self.runs.append(LeapFrogIterator(self.op, dt, mass, None, src_idx[m], src_val[m], pulse, None,
                                              rec_idx, rec_w))

    def traces(self, c: np.ndarray) -> np.ndarray:
        """(n_rec, S, N+1) traces of U^0..U^N for wave speed c."""
        c = np.ascontiguousarray(c, dtype=np.float64)
        self.op.set_element_scale(c * c)
        out = [lf.Run(np.zeros(self.n_dof), None, self.N)[2] for lf in self.runs]
        return np.stack(out, axis=1)

    def __call__(self, c: np.ndarray, data: np.ndarray) -> float:
        res = self.traces(c) - data
        return 0.5 * float((res * res).sum())

    def close(self) -> None:
        for lf in self.runs:
            lf.close()
        self.runs = []
        self.op.close()


def central_differences(J, c: np.ndarray, elements, rel_step: float = 1e-4) -> np.ndarray:
    """(J(c + h e_k) - J(c - h e_k)) / 2h, h = rel_step * c_k, for k in elements."""
    out = []
    for e in elements:
        h = rel_step * c[e]
        cp, cm = c.copy(), c.copy()
        cp[e] += h
        cm[e] -= h
        out.append((J(cp) - J(cm)) / (2.0 * h))
    return np.array(out)


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
