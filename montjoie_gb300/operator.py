"""Python mirror of the reference's matrix-free stiffness operator interface.

``FemMatrixFreeOperator`` plays the role of
``FemMatrixFreeClass<double, LaplaceEquation<Dimension3> >``
(``MONTJOIE/src/Computation/FemMatrixFreeClass.hxx:74-300``) seen through
``Seldon::VirtualMatrix<double>`` (``SELDON/matrix/Matrix_Base.hxx:41-140``):
``MltAddVector(alpha, x, beta, y)`` computes ``y <- beta*y + alpha*A*x`` in place,
``MltVector(x, y)`` computes ``y <- A*x``.  ``A`` is the positive stiffness
operator of ``-div(mu grad u)``.  All the work runs in the CUDA library through
the C ABI; a missing library raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class FemMatrixFreeOperator:
    def __init__(self, order: int, nodle: np.ndarray, factors: np.ndarray | None, n_dof: int,
                 precision: str = "fp64", gradphi: np.ndarray | None = None, verts_e: np.ndarray | None = None,
                 mu: np.ndarray | None = None):
        """From the reference's arrays (Nodle and the stiffness factors), or,
        with factors = None, from the geometry (element vertices verts_e,
        n_elt x 8 x 3, and mu per element): the factors are then computed on
        the device (mj_op_create_geometry) and the operator can also assemble
        the lumped mass and Gaussian sources there."""
        L = _lib.load()
        self.order = int(order)
        self.n_dof = int(n_dof)
        nodle = np.ascontiguousarray(nodle, dtype=np.int32)
        Q = (self.order + 1) ** 3
        if nodle.ndim != 2 or nodle.shape[1] != Q:
            raise ValueError(f"nodle must be (n_elt, {Q})")
        self.n_elt = nodle.shape[0]
        self.precision = {"fp64": _lib.MJ_FP64, "fp32": _lib.MJ_FP32}[precision]
        self.dtype = np.float64 if self.precision == _lib.MJ_FP64 else np.float32
        mesh = _lib.MeshDesc(self.order, self.n_elt, self.n_dof, _lib.iptr(nodle))
        handle = ctypes.c_void_p()
        if factors is None:
            verts_e = np.ascontiguousarray(verts_e, dtype=np.float64)
            mu = np.ascontiguousarray(mu, dtype=np.float64)
            if verts_e.shape != (self.n_elt, 8, 3) or mu.shape != (self.n_elt,):
                raise ValueError("from geometry: verts_e (n_elt, 8, 3) and mu (n_elt,) are required")
            _lib.check(L.mj_op_create_geometry(ctypes.byref(mesh), _lib.dptr(verts_e), _lib.dptr(mu),
                                               self.precision, ctypes.byref(handle)))
        else:
            factors = np.ascontiguousarray(factors, dtype=np.float64)
            if factors.size != self.n_elt * Q * 6:
                raise ValueError(f"factors must hold n_elt*{Q}*6 values")
            g = None if gradphi is None else np.ascontiguousarray(gradphi, dtype=np.float64)
            geom = _lib.GeomDesc(_lib.dptr(factors), _lib.dptr(g))
            _lib.check(L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), self.precision, ctypes.byref(handle)))
        self._h = handle

    def lumped_mass(self, rho: np.ndarray | None = None) -> np.ndarray:
        """D_i = sum rho_e J w over the points on dof i, assembled on the device
        (operators built from geometry)."""
        out = np.zeros(self.n_dof)
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
        _lib.check(_lib.load().mj_op_lumped_mass(self._h, _lib.dptr(r), _lib.dptr(out)))
        return out

    def gaussian_source(self, center, radius: float):
        """(idx, val): the Gaussian volume source F_i = sum J w g(x), assembled
        on the device (operators built from geometry)."""
        L = _lib.load()
        c = np.ascontiguousarray(center, dtype=np.float64)
        n = ctypes.c_int()
        _lib.check(L.mj_op_gaussian_source(self._h, _lib.dptr(c), float(radius), 0, None, None, ctypes.byref(n)))
        idx, val = np.zeros(n.value, dtype=np.int32), np.zeros(n.value)
        _lib.check(L.mj_op_gaussian_source(self._h, _lib.dptr(c), float(radius), n.value, _lib.iptr(idx),
                                           _lib.dptr(val), ctypes.byref(n)))
        return idx, val

    def power_iteration(self, inv_mass: np.ndarray, x0: np.ndarray, iters: int) -> float:
        """lambda_max(D^-1 A) by power iteration on the device."""
        lam = ctypes.c_double()
        _lib.check(_lib.load().mj_op_power_iteration(self._h, _lib.dptr(np.ascontiguousarray(inv_mass, np.float64)),
                                                     _lib.dptr(np.ascontiguousarray(x0, np.float64)), int(iters),
                                                     ctypes.byref(lam)))
        return float(lam.value)

    @property
    def handle(self):
        return self._h

    def GetM(self) -> int:
        return self.n_dof

    def GetN(self) -> int:
        return self.n_dof

    def MltAddVector(self, alpha: float, x: np.ndarray, beta: float, y: np.ndarray) -> None:
        """y <- beta*y + alpha*A*x (host vectors, y updated in place)."""
        if x.shape != (self.n_dof,) or y.shape != (self.n_dof,):
            raise ValueError("vector size differs from the operator size")
        if y.dtype != np.float64 or not y.flags.c_contiguous:
            raise TypeError("y must be a contiguous float64 vector")
        xc = np.ascontiguousarray(x, dtype=np.float64)
        _lib.check(_lib.load().mj_op_mltadd(self._h, float(alpha), _lib.dptr(xc), float(beta), _lib.dptr(y)))

    def MltVector(self, x: np.ndarray, y: np.ndarray) -> None:
        self.MltAddVector(1.0, x, 0.0, y)

    def mltadd_device(self, alpha: float, x_ptr: int, beta: float, y_ptr: int, stream: int = 0) -> None:
        """Same product on device vectors (operator precision), ordered on ``stream``."""
        _lib.check(_lib.load().mj_op_mltadd_device(self._h, float(alpha), ctypes.c_void_p(x_ptr), float(beta),
                                                   ctypes.c_void_p(y_ptr), ctypes.c_void_p(stream)))

    def set_element_scale(self, scale: np.ndarray) -> None:
        """factors(e) <- scale[e] * factors given at creation (media update)."""
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        if sc.size != self.n_elt:
            raise ValueError("one scale per element")
        _lib.check(_lib.load().mj_op_set_element_scale(self._h, _lib.dptr(sc)))

    def tuning(self) -> dict:
        """Element-kernel variant picked by the autotuner at creation."""
        vals = [ctypes.c_int() for _ in range(4)]
        ms = np.zeros(64)
        _lib.check(_lib.load().mj_op_tuning(self._h, *[ctypes.byref(v) for v in vals], _lib.dptr(ms)))
        E, lay, grid, nc = (v.value for v in vals)
        return {"tile_elems": E,
                "layout": ["compact", "vector_lines", "warp_per_element", "warp_per_element_packed",
                           "compact_one_factor_stage"][lay],
                "grid": grid, "candidate_ms": ms[:nc].tolist()}

    def set_variant(self, tile_elems: int, layout) -> None:
        """Forces the element-kernel variant (otherwise chosen by the autotuner):
        layout 0 / False compact, 1 / True vector lines, 2 one element per warp,
        3 one element per warp reading the packed connectivity, 4 compact with
        one factor stage."""
        _lib.check(_lib.load().mj_op_set_variant(self._h, int(tile_elems), int(layout)))

    def device_bytes(self) -> int:
        sz = ctypes.c_size_t()
        _lib.check(_lib.load().mj_op_info(self._h, None, None, None, None, ctypes.byref(sz)))
        return int(sz.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().mj_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
