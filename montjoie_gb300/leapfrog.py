"""Python mirror of the reference's order-2 leap-frog driver.

``LeapFrogIterator`` follows ``ModifiedEquationIterator<double>`` of order 2
(``MONTJOIE/src/Instationary/ModifiedEquation.hxx:78-114``):
``SetInitialConditionS`` (``ModifiedEquation.cxx:92-124``), ``Advance``
(``:290-345``) and ``GetIterate`` (``:230-236``), with the ODE-system operators
of the acoustic problem (stiffness ``Kh``, lumped mass ``Dh``, sparse source
``F`` times the pulse) bound at construction.  ``RunSecondOrderScheme``
mirrors ``MONTJOIE/src/Instationary/ModifiedEquation.cxx:16-53``.
The loop runs on the GPU through the C ABI.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .operator import FemMatrixFreeOperator


class LeapFrogIterator:
    def __init__(self, op: FemMatrixFreeOperator, dt: float, mass: np.ndarray, inv_mass: np.ndarray | None = None,
                 src_idx=None, src_val=None, pulse=None, norm_weight=None, rec_idx=None, rec_w=None,
                 time_order: int = 2, pulse_d2=None):
        """time_order = 4 selects the modified-equation leap-frog of order 4
        (ModifiedEquation.cxx:125-175, 346-408); pulse_d2 is then the second
        time derivative of the pulse at t_n + dt."""
        L = _lib.load()
        self.op = op
        self.dt = float(dt)
        n = op.n_dof
        self._keep = []

        def f(a, size=None):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            if size is not None and a.size != size:
                raise ValueError("array size mismatch")
            self._keep.append(a)
            return a

        def i(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int32)
            self._keep.append(a)
            return a

        mass = f(mass, n)
        inv_mass = f(inv_mass, n)
        src_idx, src_val = i(src_idx), f(src_val)
        pulse = f(pulse)
        norm_weight = f(norm_weight, n)
        rec_idx, rec_w = i(rec_idx), f(rec_w)
        n_src = 0 if src_idx is None else int(src_idx.size)
        n_rec = 0 if rec_idx is None else int(rec_idx.shape[0])
        n_rec_w = 0 if rec_idx is None else int(rec_idx.shape[1])
        self.n_rec = n_rec
        self.has_norm = norm_weight is not None
        desc = _lib.LfDesc(self.dt, _lib.dptr(mass), _lib.dptr(inv_mass), n_src, _lib.iptr(src_idx),
                           _lib.dptr(src_val), 0 if pulse is None else int(pulse.size), _lib.dptr(pulse),
                           _lib.dptr(norm_weight), n_rec, n_rec_w, _lib.iptr(rec_idx), _lib.dptr(rec_w))
        handle = ctypes.c_void_p()
        _lib.check(L.mj_lf_create(op.handle, ctypes.byref(desc), ctypes.byref(handle)))
        self._h = handle
        self.n_time = 0
        self.time_order = int(time_order)
        if self.time_order != 2:
            p2 = f(pulse_d2)
            _lib.check(L.mj_lf_set_scheme(self._h, self.time_order, 0 if p2 is None else int(p2.size), _lib.dptr(p2)))

    @property
    def handle(self):
        return self._h

    def SetInitialConditionS(self, u0: np.ndarray, du0: np.ndarray | None = None) -> None:
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        du0 = None if du0 is None else np.ascontiguousarray(du0, dtype=np.float64)
        _lib.check(_lib.load().mj_lf_init(self._h, _lib.dptr(u0), _lib.dptr(du0)))
        self.n_time = 0

    def Advance(self, nsteps: int = 1):
        """Advances nsteps; returns (norms, traces) of the iterates handed out before each step."""
        norms = np.zeros(nsteps) if self.has_norm else None
        traces = np.zeros((self.n_rec, nsteps)) if self.n_rec else None
        _lib.check(_lib.load().mj_lf_advance(self._h, int(nsteps), _lib.dptr(norms), _lib.dptr(traces),
                                             int(nsteps)))
        self.n_time += nsteps
        return norms, traces

    def set_stream_gather(self, enable: bool) -> None:
        """FP32: streaming gather + update + source kernel (default) or the
        gather kernel followed by the source kernel (bitwise the same states)."""
        _lib.check(_lib.load().mj_lf_set_stream_gather(self._h, int(bool(enable))))

    def SetNormeMaxSolution(self, norm_max: float) -> None:
        """Divergence guard (NormeMaxSolution, VarInstationary.cxx:362-374,2741-2745):
        Advance / Run raise MontjoieError (MJ_ERR_NONFINITE) when a recorded
        norm exceeds norm_max (default 1e30, as in the reference)."""
        _lib.check(_lib.load().mj_lf_set_norm_max(self._h, float(norm_max)))

    def set_graph(self, enable: bool) -> None:
        """Replay captured CUDA graphs of 20 steps when no diagnostics are asked (default on)."""
        _lib.check(_lib.load().mj_lf_set_graph(self._h, int(bool(enable))))

    def GetIterate(self) -> np.ndarray:
        u = np.zeros(self.op.n_dof)
        _lib.check(_lib.load().mj_lf_get_state(self._h, _lib.dptr(u), None))
        return u

    def GetState(self):
        u, v = np.zeros(self.op.n_dof), np.zeros(self.op.n_dof)
        _lib.check(_lib.load().mj_lf_get_state(self._h, _lib.dptr(u), _lib.dptr(v)))
        return u, v

    def Run(self, u0, du0, nsteps: int, out=None):
        """Whole RunSecondOrderScheme in one C-ABI call: returns (u_final, norms, traces)
        with nsteps+1 diagnostic columns (iterates 0..nsteps).  out: an optional
        float64 array of n_dof (e.g. in pinned host memory) that receives u_final."""
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        du0 = None if du0 is None else np.ascontiguousarray(du0, dtype=np.float64)
        if out is not None and (out.dtype != np.float64 or out.size != self.op.n_dof or not out.flags.c_contiguous):
            raise ValueError("Run: out must be a contiguous float64 array of n_dof values")
        uf = np.zeros(self.op.n_dof) if out is None else out
        norms = np.zeros(nsteps + 1) if self.has_norm else None
        traces = np.zeros((self.n_rec, nsteps + 1)) if self.n_rec else None
        _lib.check(_lib.load().mj_lf_run(self._h, _lib.dptr(u0), _lib.dptr(du0), int(nsteps), _lib.dptr(uf),
                                         _lib.dptr(norms), _lib.dptr(traces), int(nsteps + 1)))
        self.n_time = nsteps
        return uf, norms, traces

    def device_state(self):
        a, b, s = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_int()
        _lib.check(_lib.load().mj_lf_device_state(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(s)))
        return a.value, b.value, s.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().mj_lf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchLeapFrog:
    """S leap-frog runs sharing one mesh and operator (FP32), each with its own
    sources and state: the reference's order-2 ModifiedEquationIterator run
    S times, advanced together on the GPU (state n_dof x S, row-major).  The
    C ABI takes S in multiples of 8; any other S >= 1 is padded to the next
    multiple with runs that have no source and stay zero (``S_dev``), and
    every array handed in or out has the caller's S."""

    def __init__(self, op: FemMatrixFreeOperator, dt: float, n_rhs: int, mass, inv_mass=None, src_idx=None,
                 src_rhs=None, src_val=None, pulse=None, rec_idx=None, rec_w=None):
        L = _lib.load()
        self.op, self.S, self.dt = op, int(n_rhs), float(dt)
        if self.S < 1:
            raise ValueError("at least one run")
        self.S_dev = (self.S + 7) // 8 * 8
        n = op.n_dof
        keep = self._keep = []

        def f(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a

        def i(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return a

        mass, inv_mass, pulse = f(mass), f(inv_mass), f(pulse)
        src_idx, src_rhs, src_val = i(src_idx), i(src_rhs), f(src_val)
        rec_idx, rec_w = i(rec_idx), f(rec_w)
        if mass.size != n:
            raise ValueError("mass size differs from the operator size")
        if src_rhs is not None and src_rhs.size and (src_rhs.min() < 0 or src_rhs.max() >= self.S):
            raise ValueError("source run index outside [0, n_rhs)")
        n_src = 0 if src_idx is None else int(src_idx.size)
        self.n_rec = 0 if rec_idx is None else int(rec_idx.shape[0])
        n_rec_w = 0 if rec_idx is None else int(rec_idx.shape[1])
        desc = _lib.LfbDesc(self.dt, self.S_dev, _lib.dptr(mass), _lib.dptr(inv_mass), n_src, _lib.iptr(src_idx),
                            _lib.iptr(src_rhs), _lib.dptr(src_val), 0 if pulse is None else int(pulse.size),
                            _lib.dptr(pulse), self.n_rec, n_rec_w, _lib.iptr(rec_idx), _lib.dptr(rec_w))
        h = ctypes.c_void_p()
        _lib.check(L.mj_lfb_create(op.handle, ctypes.byref(desc), ctypes.byref(h)))
        self._h = h

    def _pad(self, a):
        """(n_dof, S) -> (n_dof, S_dev), the padding runs zero."""
        n = self.op.n_dof
        a = np.asarray(a, dtype=np.float64).reshape(n, self.S)
        if self.S_dev == self.S:
            return np.ascontiguousarray(a)
        out = np.zeros((n, self.S_dev))
        out[:, :self.S] = a
        return out

    def init(self, u0=None, du0=None) -> None:
        u0 = None if u0 is None else self._pad(u0)
        du0 = None if du0 is None else self._pad(du0)
        _lib.check(_lib.load().mj_lfb_init(self._h, _lib.dptr(u0), _lib.dptr(du0)))

    def advance(self, nsteps: int, traces: bool = False, graph: bool = True):
        """Advances nsteps; with traces, returns the receiver values before each
        step as an (n_rec, S, nsteps) array."""
        tr = np.zeros((self.n_rec, self.S_dev, nsteps)) if (traces and self.n_rec) else None
        _lib.check(_lib.load().mj_lfb_advance(self._h, int(nsteps), _lib.dptr(tr), int(nsteps), int(bool(graph))))
        return None if tr is None else np.ascontiguousarray(tr[:, :self.S, :])

    def state(self):
        n = self.op.n_dof
        u, v = np.zeros((n, self.S_dev)), np.zeros((n, self.S_dev))
        _lib.check(_lib.load().mj_lfb_get_state(self._h, _lib.dptr(u), _lib.dptr(v)))
        return np.ascontiguousarray(u[:, :self.S]), np.ascontiguousarray(v[:, :self.S])

    def info(self):
        """n_rhs: the caller's runs; n_rhs_device: the runs stepped (a multiple of 8)."""
        vals = [ctypes.c_int() for _ in range(5)]
        _lib.check(_lib.load().mj_lfb_info(self._h, *[ctypes.byref(v) for v in vals]))
        out = dict(zip(["n_rhs_device", "tile_elems", "lanes", "grid", "step"], [v.value for v in vals]))
        out["n_rhs"] = self.S
        return out

    def set_fused(self, enable: bool) -> None:
        """One cooperative kernel per step (default) or two kernels per step."""
        _lib.check(_lib.load().mj_lfb_set_fused(self._h, int(bool(enable))))

    def profile(self, enable: bool) -> None:
        """Plain launches with per-CTA phase time stamps (no graph) while enabled."""
        _lib.check(_lib.load().mj_lfb_profile(self._h, int(bool(enable))))

    def phase_ms(self) -> dict:
        out = np.zeros(4)
        _lib.check(_lib.load().mj_lfb_phase_ms(self._h, _lib.dptr(out)))
        return dict(zip(["element_last", "element_mean", "barrier", "dof"], out.tolist()))

    def step_info(self) -> dict:
        vals = [ctypes.c_int() for _ in range(4)]
        ms = np.zeros(16)
        _lib.check(_lib.load().mj_lfb_step_info(self._h, *[ctypes.byref(v) for v in vals], _lib.dptr(ms)))
        fused, threads, grid, nc = (v.value for v in vals)
        return {"one_kernel": bool(fused), "threads": threads, "grid": grid, "candidate_ms": ms[:nc].tolist()}

    def set_step_variant(self, tile_elems: int, lanes: int, sources_per_thread: int) -> None:
        """Forces the one-kernel step's variant: tile_elems elements per tile,
        lanes thread lanes per z-line and sources_per_thread right-hand sides
        per thread; every variant gives the same states bit for bit."""
        _lib.check(_lib.load().mj_lfb_set_step_variant(self._h, int(tile_elems), int(lanes),
                                                       int(sources_per_thread)))

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().mj_lfb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def number_of_iterations(t_begin: float, t_end: float, dt: float) -> int:
    """nb_max_iter = ceil(|t_end - t_begin| / dt) (ModifiedEquation.cxx:23-24)."""
    return int(math.ceil(abs(t_end - t_begin) / dt))


def RunSecondOrderScheme(t_begin: float, t_end: float, dt: float, U0: np.ndarray, dU0_dt: np.ndarray | None,
                         scheme: LeapFrogIterator):
    """Runs the scheme from t_begin to t_end; returns (final iterate, norms, traces)."""
    nsteps = number_of_iterations(t_begin, t_end, dt)
    if nsteps < 1:
        return np.array(U0, dtype=np.float64), None, None
    return scheme.Run(U0, dU0_dt, nsteps)


class MeshBatch:
    """Leap-frog runs on meshes of different size and order (each a
    ``LeapFrogIterator`` on its own FP32 operator) advanced together by one
    cooperative persistent kernel per time step, or, when the autotuner finds
    it faster, one launch per order group, or the runs of one order stepped
    as one union operator (``union_info``).  The reference advances such
    runs one after the other (``ModifiedEquation.cxx:290-345`` per run).
    Each run stays usable on its own (``SetInitialConditionS``,
    ``GetIterate``, ``Advance``) between calls."""

    def __init__(self, runs):
        L = _lib.load()
        self.runs = list(runs)
        arr = (ctypes.c_void_p * len(self.runs))(*[r.handle.value for r in self.runs])
        h = ctypes.c_void_p()
        _lib.check(L.mj_mb_create(len(self.runs), arr, ctypes.byref(h)))
        self._h = h

    def advance(self, nsteps: int, graph: bool = True) -> None:
        _lib.check(_lib.load().mj_mb_advance(self._h, int(nsteps), int(bool(graph))))
        for r in self.runs:
            r.n_time += nsteps

    def info(self) -> dict:
        """Launch shape; single_order = n when every mesh has order n-1 (the
        batch runs that order's kernel instance), else 0."""
        vals = [ctypes.c_int() for _ in range(6)]
        _lib.check(_lib.load().mj_mb_info(self._h, *[ctypes.byref(v) for v in vals]))
        return dict(zip(["grid", "ctas_per_sm", "tiles", "chunks", "graph", "single_order"], [v.value for v in vals]))

    def n_dof(self) -> int:
        return sum(r.op.n_dof for r in self.runs)

    def tuning(self) -> dict:
        """Launch configuration picked at the first advance and the timings of both."""
        th = ctypes.c_int()
        ms = np.zeros(2)
        _lib.check(_lib.load().mj_mb_tuning(self._h, ctypes.byref(th), _lib.dptr(ms)))
        return {"threads": th.value, "candidate_ms": {"256": ms[0], "128": ms[1]}}

    def set_config(self, threads: int) -> None:
        """Forces the form of a step (128 or 256 threads per CTA: one kernel
        of all orders per step; -1: one launch per order group; -2: unions,
        of the whole batch when it has one order, else of every order group),
        or 0 to time them again at the next advance."""
        _lib.check(_lib.load().mj_mb_set_config(self._h, int(threads)))

    def union_info(self, group: int = -1) -> dict:
        """The union form (one operator over the disjoint union of the runs'
        meshes) of the batch (group -1) or of an order group: whether it steps
        the runs, its timed ms per step, its element kernel's tile size and
        its dofs (0: no union, the runs are too large for one)."""
        use, tile, nd, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), np.zeros(1)
        _lib.check(_lib.load().mj_mb_union_info(self._h, int(group), ctypes.byref(use), _lib.dptr(ms),
                                                ctypes.byref(tile), ctypes.byref(nd)))
        return {"in_use": bool(use.value), "union_ms": float(ms[0]), "tile_elems": tile.value, "n_dof": nd.value}

    def grouping(self) -> dict:
        """Whether steps run one launch per order group, the number of groups,
        the grouped form's timed ms per step and, per group, its form (batch
        kernel, its runs' own kernels, or its union) with the timings."""
        L = _lib.load()
        g, n, ms = ctypes.c_int(), ctypes.c_int(), np.zeros(1)
        _lib.check(L.mj_mb_grouping(self._h, ctypes.byref(g), ctypes.byref(n), _lib.dptr(ms)))
        groups = []
        for i in range(n.value):
            o, nr, own, bms, oms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), np.zeros(1), np.zeros(1)
            _lib.check(L.mj_mb_group_info(self._h, i, ctypes.byref(o), ctypes.byref(nr), ctypes.byref(own),
                                          _lib.dptr(bms), _lib.dptr(oms)))
            u = self.union_info(i)
            groups.append({"order": o.value, "runs": nr.value, "own_kernels": bool(own.value),
                           "union": u["in_use"], "batch_ms": float(bms[0]), "own_ms": float(oms[0]),
                           "union_ms": u["union_ms"]})
        return {"grouped": bool(g.value), "groups": n.value, "grouped_ms": float(ms[0]), "per_group": groups}

    def profile(self, enable: bool) -> None:
        """Plain launches with per-CTA time stamps (no graph) while enabled."""
        _lib.check(_lib.load().mj_mb_profile(self._h, int(bool(enable))))

    def phase_ms(self) -> dict:
        """Phase times of the last step (ms): element phase (last and mean CTA),
        barrier release, dof phase, and the mean time a CTA waited for the bulk
        copies of its element tiles and of its dof chunks."""
        out = np.zeros(6)
        _lib.check(_lib.load().mj_mb_phase_ms(self._h, _lib.dptr(out)))
        return dict(zip(["element_last", "element_mean", "barrier", "dof", "element_copy_wait", "dof_copy_wait"],
                        out.tolist()))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().mj_mb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
