"""Set-up of one acoustic leap-frog run on a hexahedral mesh (host side).

Builds, for a ``HexMesh`` and an ``AcousticSetup``:
  * the global numbering ``Nodle``          (``mj_number_hex_mesh``, C++),
  * the FP64 geometric factors and ``J w``  (``mj_geometry``, CUDA),
  * the lumped mass ``D``                   (``mj_lumped_mass``, C++),
  * the Gaussian spatial source ``F`` (``MONTJOIE/src/Source/SourceSpatiale.cxx:22-95``),
  * the interpolated Ricker pulse ``p(t_n + dt)`` (``MONTJOIE/src/Source/TimeSource.cxx:778-880``),
  * receiver interpolation weights (the role of ``SismoPoint``,
    ``MONTJOIE/src/Output/GridInterpolation.cxx:836``),
and the operator / integrator objects of the CUDA library.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .leapfrog import LeapFrogIterator
from .mesh import AcousticSetup, HexMesh
from .operator import FemMatrixFreeOperator

# ----------------------------------------------------------------- 1-D rules


def gauss_lobatto(r: int):
    """Gauss-Lobatto points and weights on [0,1] (r+1 points): Newton on P_r'."""
    x = -np.cos(np.pi * np.arange(r + 1) / r)

    def leg(xv):
        p0, p1 = np.ones_like(xv), xv.copy()
        d0, d1 = np.zeros_like(xv), np.ones_like(xv)
        for k in range(1, r):
            p2 = ((2 * k + 1) * xv * p1 - k * p0) / (k + 1)
            d2 = d0 + (2 * k + 1) * p1
            p0, p1, d0, d1 = p1, p2, d1, d2
        return p1, d1

    xi = x[1:-1].copy()
    for _ in range(100):
        p, dp = leg(xi)
        d2 = (2 * xi * dp - r * (r + 1) * p) / (1 - xi * xi)
        step = dp / d2
        xi -= step
        if np.max(np.abs(step), initial=0.0) < 1e-17:
            break
    x[1:-1] = xi
    p, _ = leg(x)
    pts = 0.5 * (x + 1.0)
    pts[0], pts[-1] = 0.0, 1.0
    return pts, 1.0 / (r * (r + 1) * p * p)


def derivative_matrix(pts: np.ndarray) -> np.ndarray:
    """G[a, b] = phi_a'(x_b) with the barycentric formula (GaussLobatto.cxx:175-191)."""
    n = pts.size
    diff = pts[:, None] - pts[None, :]
    np.fill_diagonal(diff, 1.0)
    c = 1.0 / diff.prod(axis=1)
    G = np.zeros((n, n))
    for b in range(n):
        s = 0.0
        for a in range(n):
            if a != b:
                G[a, b] = c[a] / (c[b] * (pts[b] - pts[a]))
                s += G[a, b]
        G[b, b] = -s if abs(s) > 1e3 * np.finfo(float).eps else 0.0
    return G


def lagrange_values(pts: np.ndarray, x: float) -> np.ndarray:
    n = pts.size
    out = np.ones(n)
    for a in range(n):
        for b in range(n):
            if b != a:
                out[a] *= (x - pts[b]) / (pts[a] - pts[b])
    return out


def local_numbering(r: int) -> np.ndarray:
    """NumDofs3D as an (r+1)^3 array num[i,j,k] (HexahedronQuadrature.cxx:51-171)."""
    n = r + 1
    num = -np.ones((n, n, n), dtype=np.int64)
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    edges = [(0, 1), (1, 2), (3, 2), (0, 3), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (5, 6), (7, 6), (4, 7)]
    node = 0
    for c in corner:
        num[c[0] * r, c[1] * r, c[2] * r] = node
        node += 1
    for a, b in edges:
        A, B = np.array(corner[a]), np.array(corner[b])
        for l in range(1, r):
            p = A * r + l * (B - A)
            num[p[0], p[1], p[2]] = node
            node += 1
    for fix in ((0, 0), (1, 0), (2, 0), (2, r), (1, r), (0, r)):
        for p in range(1, r):
            for q in range(1, r):
                idx = [0, 0, 0]
                idx[fix[0]] = fix[1]
                other = [d for d in range(3) if d != fix[0]]
                idx[other[0]], idx[other[1]] = p, q
                num[tuple(idx)] = node
                node += 1
    for i in range(1, r):
        for j in range(1, r):
            for k in range(1, r):
                num[i, j, k] = node
                node += 1
    return num


# ----------------------------------------------------------------- sources


def ricker_primitive(f0: float, t: np.ndarray) -> np.ndarray:
    """-(f0 t - 1) exp(-pi^2 (f0 t - 1)^2) / f0 on (-0.9/f0, 2.9/f0) (TimeSource.cxx:33-50)."""
    t = np.asarray(t, dtype=np.float64)
    tmp = f0 * t - 1.0
    v = -tmp * np.exp(-tmp * tmp * np.pi * np.pi) / f0
    return np.where((t <= -0.9 / f0) | (t >= 2.9 / f0), 0.0, v)


def ricker_pulse(f0: float, t_init: float, dt: float, nsteps: int, eps_time: float, tlimit: float | None = None,
                 nb_deriv: int = 1):
    """Derivative nb_deriv of the source primitive at t_n + dt for
    n = 0..nsteps-1 (1: the pulse p; 3: its second derivative p''): spectral
    derivative of the degree-24 Gauss-Lobatto interpolant of the Ricker
    primitive on windows of length 0.5/f0, the derivative matrix applied
    nb_deriv times (TimeSourceHyperbolic, TimeSource.cxx:826-880); zero from
    tlimit = 2.5/f0 on (VarInstationary.cxx:2392-2396)."""
    if tlimit is None:
        tlimit = 2.5 / f0
    pts, _ = gauss_lobatto(24)
    G = derivative_matrix(pts)
    n = pts.size
    # the window of every step (a window covers [t0, t1] and moves on when
    # t > t1 + eps_time), then each window's steps at once
    times = t_init + np.arange(nsteps) * dt + dt
    win = np.zeros(nsteps, dtype=np.int64)
    starts = [(t_init, t_init + 0.5 / f0)]
    t0, t1 = starts[0]
    for s in range(nsteps):
        t = times[s]
        if t > t1 + eps_time and t1 > t0:
            while t > t1 + eps_time:
                t0, t1 = t1, t1 + (t1 - t0)
            starts.append((t0, t1))
        win[s] = len(starts) - 1
    out = np.zeros(nsteps)
    for w, (t0, t1) in enumerate(starts):
        sel = np.nonzero(win == w)[0]
        if sel.size == 0:
            continue
        der = ricker_primitive(f0, (1.0 - pts) * t0 + pts * t1)
        for _ in range(nb_deriv):
            der = (G.T @ der) * (1.0 / (t1 - t0))
        x = (times[sel] - t0) / (t1 - t0)
        L = np.ones((sel.size, n))  # Lagrange values, factors multiplied in the order of lagrange_values
        with np.errstate(divide="ignore", invalid="ignore"):
            for b in range(n):
                f = (x[:, None] - pts[b]) / (pts[None, :] - pts[b])
                f[:, b] = 1.0
                L *= f
        out[sel] = L @ der
    out[times >= tlimit] = 0.0
    return out


def gaussian_source(nodle: np.ndarray, jw: np.ndarray, xq: np.ndarray, n_dof: int, center, radius: float):
    """F_i = sum over points on dof i of (J w) g(x), g = beta exp(-alpha r^2) for
    r < R, alpha = -ln(1e-6)/R^2, beta = sqrt(alpha/pi) (SourceSpatiale.cxx:33-90).
    Returns the sparse (index, value) pairs in increasing dof order."""
    c = np.asarray(center, dtype=np.float64)
    alpha = -math.log(1e-6) / (radius * radius)
    beta = math.sqrt(alpha / math.pi)
    d = xq.reshape(-1, 3) - c
    rr = np.sqrt((d * d).sum(axis=1))
    mask = rr < radius
    F = np.zeros(n_dof)
    np.add.at(F, nodle.reshape(-1)[mask], jw.reshape(-1)[mask] * beta * np.exp(-alpha * rr[mask] ** 2))
    idx = np.nonzero(F)[0].astype(np.int32)
    return idx, F[idx]


# ----------------------------------------------------------------- receivers


def _trilinear(v: np.ndarray, xi: np.ndarray):
    x, y, z = xi
    cx, cy, cz = (1 - x, x), (1 - y, y), (1 - z, z)
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    F = np.zeros(3)
    DF = np.zeros((3, 3))
    for c, (a, b, g) in enumerate(corner):
        N = cx[a] * cy[b] * cz[g]
        dN = np.array([(-1, 1)[a] * cy[b] * cz[g], cx[a] * (-1, 1)[b] * cz[g], cx[a] * cy[b] * (-1, 1)[g]])
        F += N * v[c]
        DF += np.outer(v[c], dN)
    return F, DF


def locate_point(verts_e: np.ndarray, p: np.ndarray, candidates: np.ndarray, tol: float = 1e-10):
    """Element containing p among candidates and its reference coordinates."""
    for e in candidates:
        xi = np.full(3, 0.5)
        for _ in range(50):
            F, DF = _trilinear(verts_e[e], xi)
            step = np.linalg.solve(DF, p - F)
            xi += step
            if np.abs(step).sum() < 1e-15:
                break
        if np.all(xi >= -tol) and np.all(xi <= 1 + tol):
            return int(e), xi
    raise ValueError(f"point {p} is outside the mesh")


def receiver_weights(order: int, verts_e: np.ndarray, nodle: np.ndarray, points: np.ndarray):
    """(rec_idx, rec_w): per receiver the Q dofs of its element and the tensor
    Lagrange weights at its reference coordinates."""
    pts1d, _ = gauss_lobatto(order)
    num = local_numbering(order)
    lo, hi = verts_e.min(axis=1), verts_e.max(axis=1)
    Q = (order + 1) ** 3
    idx = np.zeros((len(points), Q), dtype=np.int32)
    w = np.zeros((len(points), Q))
    for k, p in enumerate(np.asarray(points, dtype=np.float64)):
        cand = np.nonzero(np.all((lo <= p + 1e-12) & (hi >= p - 1e-12), axis=1))[0]
        e, xi = locate_point(verts_e, p, cand)
        px, py, pz = (lagrange_values(pts1d, xi[a]) for a in range(3))
        wl = np.einsum("i,j,k->ijk", px, py, pz)
        w[k, num.ravel()] = wl.ravel()
        idx[k] = nodle[e]
    return idx, w


# ----------------------------------------------------------------- problem


def number_mesh(order: int, hexes: np.ndarray, n_vert: int):
    L = _lib.load()
    hexes = np.ascontiguousarray(hexes, dtype=np.int32)
    ne = hexes.shape[0]
    nodle = np.zeros((ne, (order + 1) ** 3), dtype=np.int32)
    ndof = ctypes.c_int()
    _lib.check(L.mj_number_hex_mesh(order, ne, n_vert, _lib.iptr(hexes), _lib.iptr(nodle), ctypes.byref(ndof)))
    return nodle, int(ndof.value)


def geometry(order: int, verts_e: np.ndarray, mu: np.ndarray, want_positions: bool = True):
    L = _lib.load()
    verts_e = np.ascontiguousarray(verts_e, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    ne = verts_e.shape[0]
    Q = (order + 1) ** 3
    fac = np.zeros((ne, Q, 6))
    jw = np.zeros((ne, Q))
    xq = np.zeros((ne, Q, 3)) if want_positions else None
    _lib.check(L.mj_geometry(order, ne, _lib.dptr(verts_e), _lib.dptr(mu), _lib.dptr(fac), _lib.dptr(jw),
                             _lib.dptr(xq)))
    return fac, jw, xq


def lumped_mass(order: int, nodle: np.ndarray, jw: np.ndarray, n_dof: int, rho=None):
    L = _lib.load()
    D = np.zeros(n_dof)
    rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
    _lib.check(L.mj_lumped_mass(order, nodle.shape[0], n_dof, _lib.iptr(np.ascontiguousarray(nodle, np.int32)),
                                _lib.dptr(np.ascontiguousarray(jw, np.float64)), _lib.dptr(rho), _lib.dptr(D)))
    return D


class AcousticProblem:
    """All arrays of one leap-frog run, built by this library from a mesh.

    The medium of element e is rho_e = 1, mu_e = c_e^2 (``mesh.elem_c``)
    unless per-element ``rho`` and ``mu`` are given (``from_deck`` passes the
    deck's ``MateriauDielec`` values): mass D_i = sum rho J w
    (TimeAcoustic.cxx:889-965), factors B = (J w) DF^-1 mu DF^-T
    (VarHelmholtz.cxx:95-123), norm weight sum J w (VarInstationary.cxx:2696-2745)."""

    def __init__(self, mesh: HexMesh, setup: AcousticSetup, receivers=None, defer_time: bool = False, rho=None,
                 mu=None):
        r = setup.order
        self.mesh, self.setup, self.order = mesh, setup, r
        self.verts_e = mesh.verts[mesh.hexes]
        self.nodle, self.n_dof = number_mesh(r, mesh.hexes, mesh.verts.shape[0])
        self.mu = mesh.elem_c ** 2 if mu is None else np.asarray(mu, dtype=np.float64)
        self.rho = None if rho is None else np.asarray(rho, dtype=np.float64)
        # On the device: the FP32 operator's factors from the geometry, then the
        # lumped mass, the norm weights and the Gaussian source, each assembled
        # in element order (the host arrays of the reference layout, factors,
        # jw and xq, are computed only when asked for)
        self._op = self._make_operator("fp32")
        self.norm_weight = self._op.lumped_mass(None)  # sum of J w (GetNormeSolution)
        self.mass = self.norm_weight.copy() if self.rho is None else self._op.lumped_mass(self.rho)
        self.norm_max = 1e30
        self.src_idx, self.src_val = self._op.gaussian_source(setup.src_center, setup.src_radius)
        self._geom = None
        self.pulse = None
        if not defer_time:
            self.set_time_step(setup.dt, setup.nsteps)
        if receivers is not None and len(receivers):
            self.rec_idx, self.rec_w = receiver_weights(r, self.verts_e, self.nodle, np.asarray(receivers))
        else:
            self.rec_idx, self.rec_w = None, None

    def set_time_step(self, dt: float, nsteps: int) -> None:
        """Fixes dt and the run length and builds the pulse of every step
        (epsilon_time = (tf - t0) 1e-15, VarInstationary.cxx:993)."""
        self.setup.dt, self.setup.nsteps = float(dt), int(nsteps)
        eps_time = (self.setup.tf - self.setup.t0) * 1e-15
        self.pulse = ricker_pulse(self.setup.f0, self.setup.t0, self.setup.dt, self.setup.nsteps, eps_time)
        self.pulse_d2 = None
        if self.setup.time_order == 4:
            self.pulse_d2 = ricker_pulse(self.setup.f0, self.setup.t0, self.setup.dt, self.setup.nsteps, eps_time,
                                         nb_deriv=3)

    @classmethod
    def from_deck(cls, deck_path: str, defer_time: bool = False) -> "AcousticProblem":
        """The run a reference data deck describes, read from disk with its
        Medit mesh (the subset of keywords this path has; anything else in the
        deck, such as output settings, is ignored):

        - ``TypeElement = HEXAHEDRON_LOBATTO``, ``OrderDiscretization = r``;
        - ``MeshPath`` (optional) and ``FileMesh``: the Medit ``.mesh`` file;
        - ``MateriauDielec = ref ISOTROPE rho mu sigma`` per medium reference
          (VarHelmholtz.cxx:1179-1197; sigma must be 0);
        - ``ConditionReference = ref NEUMANN`` (the only condition of this path);
        - ``TypeSource = SRC_VOLUME GAUSSIAN x y z R``, ``Frequency = f0``,
          ``TemporalSource = RICKER``;
        - ``TimeStep = dt`` (explicit: ``AUTO`` needs an eigensolver),
          ``TimeInterval = t0 tf`` (ceil((tf - t0)/dt) steps,
          ModifiedEquation.cxx:23-24), ``OrderTimeScheme = 2|4 LEAP_FROG``;
        - ``SismoPoint = x y z`` receivers (GridInterpolation.cxx:836-850);
        - ``NormeMaxSolution = value`` (VarInstationary.cxx:362-374).
        Unsupported values raise ValueError naming the keyword."""
        import os

        from .mesh import read_deck, read_medit
        kw = read_deck(deck_path)

        def one(key, default=None):
            if key not in kw:
                if default is None:
                    raise ValueError(f"{deck_path}: keyword {key} missing")
                return default
            return kw[key][-1]

        if one("TypeElement")[0] != "HEXAHEDRON_LOBATTO":
            raise ValueError(f"TypeElement {one('TypeElement')[0]}: only HEXAHEDRON_LOBATTO is on this path")
        order = int(one("OrderDiscretization")[0])
        mesh_dir = one("MeshPath", [os.path.dirname(os.path.abspath(deck_path))])[0]
        mesh_file = one("FileMesh")[0]
        if not os.path.isabs(mesh_file):
            mesh_file = os.path.join(mesh_dir, mesh_file)
        if not os.path.exists(mesh_file):  # a deck moved with its mesh
            mesh_file = os.path.join(os.path.dirname(os.path.abspath(deck_path)), os.path.basename(mesh_file))
        mesh = read_medit(mesh_file)
        media = {}
        for p in kw.get("MateriauDielec", []):
            if p[1] != "ISOTROPE" or float(p[4] if len(p) > 4 else 0.0) != 0.0:
                raise ValueError(f"MateriauDielec {' '.join(p)}: only ISOTROPE media without damping")
            media[int(p[0])] = (float(p[2]), float(p[3]))
        missing = sorted(set(np.unique(mesh.elem_ref).tolist()) - set(media))
        if missing:
            raise ValueError(f"MateriauDielec missing for references {missing}")
        for p in kw.get("ConditionReference", []):
            if p[1] != "NEUMANN":
                raise ValueError(f"ConditionReference {' '.join(p)}: only NEUMANN is on this path")
        rho = np.array([media[int(r_)][0] for r_ in mesh.elem_ref])
        mu = np.array([media[int(r_)][1] for r_ in mesh.elem_ref])
        refs = sorted(media)
        mesh.media_c = np.array([np.sqrt(media[r_][1] / media[r_][0]) for r_ in refs])
        mesh.elem_ref = np.searchsorted(refs, mesh.elem_ref).astype(np.int32) + 1
        src = one("TypeSource")
        if src[0] != "SRC_VOLUME" or src[1] != "GAUSSIAN":
            raise ValueError(f"TypeSource {' '.join(src)}: only SRC_VOLUME GAUSSIAN is on this path")
        if one("TemporalSource", ["RICKER"])[0] != "RICKER":
            raise ValueError("TemporalSource: only RICKER is on this path")
        if one("TimeStep")[0] == "AUTO":
            raise ValueError("TimeStep = AUTO needs an eigensolver; give an explicit time step")
        dt = float(one("TimeStep")[0])
        t0, tf = (float(v) for v in one("TimeInterval")[:2])
        scheme = one("OrderTimeScheme", ["2", "LEAP_FROG"])
        if len(scheme) > 1 and scheme[1] != "LEAP_FROG":
            raise ValueError(f"OrderTimeScheme {' '.join(scheme)}: only LEAP_FROG is on this path")
        setup = AcousticSetup(order=order, f0=float(one("Frequency")[0]),
                              src_center=tuple(float(v) for v in src[2:5]), src_radius=float(src[5]), dt=dt, t0=t0,
                              nsteps=int(math.ceil((tf - t0) / dt)), time_order=int(scheme[0]), t_end=tf)
        receivers = np.array([[float(v) for v in p[:3]] for p in kw.get("SismoPoint", [])]).reshape(-1, 3)
        pb = cls(mesh, setup, receivers=receivers if len(receivers) else None, defer_time=True,
                 rho=None if np.all(rho == 1.0) else rho, mu=mu)
        pb.norm_max = float(one("NormeMaxSolution", ["1e30"])[0])
        if not defer_time:
            pb.set_time_step(dt, setup.nsteps)
        return pb

    def _make_operator(self, precision: str) -> FemMatrixFreeOperator:
        return FemMatrixFreeOperator(self.order, self.nodle, None, self.n_dof, precision, verts_e=self.verts_e,
                                     mu=self.mu)

    def _geometry(self):
        if self._geom is None:
            self._geom = geometry(self.order, self.verts_e, self.mu)
        return self._geom

    @property
    def factors(self) -> np.ndarray:
        """Stiffness factors in the reference layout (n_elt, Q, 6), host (computed on first use)."""
        return self._geometry()[0]

    @property
    def jw(self) -> np.ndarray:
        """J w of every quadrature point (n_elt, Q), host (computed on first use)."""
        return self._geometry()[1]

    @property
    def xq(self) -> np.ndarray:
        """Physical quadrature points (n_elt, Q, 3), host (computed on first use)."""
        return self._geometry()[2]

    def operator(self, precision: str = "fp64") -> FemMatrixFreeOperator:
        """A new operator owned by the caller; the first FP32 one is the
        operator the set-up already built."""
        if precision == "fp32" and self._op is not None:
            op, self._op = self._op, None
            return op
        return self._make_operator(precision)

    def close(self) -> None:
        if getattr(self, "_op", None) is not None:
            self._op.close()
            self._op = None

    def integrator(self, op: FemMatrixFreeOperator, diagnostics: bool = True) -> LeapFrogIterator:
        lf = LeapFrogIterator(op, self.setup.dt, self.mass, None, self.src_idx, self.src_val, self.pulse,
                              self.norm_weight if diagnostics else None,
                              self.rec_idx if diagnostics else None, self.rec_w if diagnostics else None,
                              time_order=self.setup.time_order, pulse_d2=self.pulse_d2)
        if self.norm_max != 1e30:
            lf.SetNormeMaxSolution(self.norm_max)
        return lf


def cfl_time_step(pb: AcousticProblem, safety: float = 0.5, iters: int = 40, seed: int = 0) -> float:
    """dt = safety * C / sqrt(lambda_max(D^-1 A)) with the scheme's CFL
    constant C = 2 (order 2) or 2 sqrt(3) (order 4) (ModifiedEquation.cxx:217-225);
    lambda_max by power iteration on the device with the FP32 operator (the
    reference needs ARPACK/SLEPc for TimeStep = AUTO)."""
    op = pb._op if pb._op is not None else pb.operator("fp32")
    x0 = np.random.default_rng(seed).uniform(-1.0, 1.0, pb.n_dof)
    lam = op.power_iteration(1.0 / pb.mass, x0, iters)
    if op is not pb._op:
        op.close()
    c = 2.0 if pb.setup.time_order == 2 else 2.0 * math.sqrt(3.0)
    return safety * c / math.sqrt(lam * 1.05)
