"""Hexahedral meshes of the unit cube, Medit ``.mesh`` files and acoustic decks.

The reference reads meshes in the Medit ``.mesh`` format (vertices, hexahedra,
boundary quadrilaterals, each with an integer reference;
``Mesh<Dimension3>::Read``, ``MONTJOIE/src/Mesh/Mesh3D.cxx:1027-1054,3561-3638``)
and data decks of ``Keyword = values`` lines (``ReadInputFile``,
``MONTJOIE/src/Output/CommonInputOutput.cxx:1793-1858``; the acoustic keywords
in ``MONTJOIE/src/Instationary/VarInstationary.cxx:79-378``).  This module
writes and reads both, so that one seeded mesh and deck drive the reference
solver and this library alike.

Vertex order of a hexahedron is the reference cube's
(``MONTJOIE/src/Quadrature/HexahedronQuadrature.cxx:78-86``):
``(0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1)``.

A structured ``N x N x N`` cube keeps elements in lexicographic order
``e = (ez*N + ey)*N + ex`` and vertices ``v = (iz*(N+1) + iy)*(N+1) + ix``.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

HEX_CORNERS = np.array(
    [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int64)


@dataclasses.dataclass
class HexMesh:
    """A conforming hexahedral mesh.

    ``verts``  (nv, 3) float64 vertex coordinates.
    ``hexes``  (ne, 8) int32 vertex indices in reference-cube order.
    ``elem_ref`` (ne,) int32 medium reference of each element (1-based).
    ``media_c``  (n_media,) float64 wave speed of medium ``ref`` at index ``ref-1``.
    ``bfaces`` (nb, 4) int32 boundary quadrilaterals (reference 1: Neumann).
    ``n`` cells per axis when the mesh is a structured cube, else 0.
    """

    verts: np.ndarray
    hexes: np.ndarray
    elem_ref: np.ndarray
    media_c: np.ndarray
    bfaces: np.ndarray
    n: int = 0

    @property
    def n_elt(self) -> int:
        return int(self.hexes.shape[0])

    @property
    def elem_c(self) -> np.ndarray:
        return self.media_c[self.elem_ref - 1]


def _structured_topology(n: int):
    idx = np.arange(n + 1)
    iz, iy, ix = np.meshgrid(idx, idx, idx, indexing="ij")
    grid = np.stack([ix, iy, iz], axis=-1).reshape(-1, 3).astype(np.float64) / n
    vid = lambda x, y, z: (z * (n + 1) + y) * (n + 1) + x  # noqa: E731
    e = np.arange(n)
    ez, ey, ex = np.meshgrid(e, e, e, indexing="ij")
    ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
    hexes = np.stack([vid(ex + c[0], ey + c[1], ez + c[2]) for c in HEX_CORNERS], axis=1)
    # boundary quads, outward orientation irrelevant for Neumann
    faces = []
    a = np.arange(n)
    p, q = np.meshgrid(a, a, indexing="ij")
    p, q = p.ravel(), q.ravel()
    for side in (0, n):
        faces.append(np.stack([vid(side, p, q), vid(side, p + 1, q), vid(side, p + 1, q + 1), vid(side, p, q + 1)], 1))
        faces.append(np.stack([vid(p, side, q), vid(p + 1, side, q), vid(p + 1, side, q + 1), vid(p, side, q + 1)], 1))
        faces.append(np.stack([vid(p, q, side), vid(p + 1, q, side), vid(p + 1, q + 1, side), vid(p, q + 1, side)], 1))
    return grid, hexes.astype(np.int32), np.concatenate(faces).astype(np.int32)


def _tangential_mask(grid: np.ndarray) -> np.ndarray:
    """1 where a coordinate may move: a vertex on x=0/1 keeps its x, etc."""
    on_bnd = (np.abs(grid) < 1e-12) | (np.abs(grid - 1.0) < 1e-12)
    return (~on_bnd).astype(np.float64)


def perturbed_cube(n: int, seed: int = 0, amplitude: float = 0.05, kind: str = "random",
                   c_mode: str = "element", c_range=(1.0, 3.0), c_blocks: int = 8) -> HexMesh:
    """Unit cube with ``n^3`` hexahedra and seeded vertex perturbation.

    kind="random": every coordinate of an interior vertex moves by
      ``U[-amplitude*h, amplitude*h]``; boundary vertices move only
      tangentially, so the domain stays the unit cube.
    kind="sin": smooth displacement ``amplitude*h*sin(2 pi x) sin(2 pi y) sin(2 pi z)``
      applied to each coordinate (zero on the cube faces).
    kind="none": regular grid.

    Wave speed: c_mode="element" draws ``c ~ U[c_range]`` per element;
    c_mode="blocks" draws one value per cell of a ``c_blocks^3`` block grid;
    c_mode="smooth" samples ``2 + 0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z)`` at each
    element centre; c_mode="constant" uses ``c_range[0]``.
    Each distinct value becomes one medium reference.
    """
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    grid, hexes, bfaces = _structured_topology(n)
    if kind == "random":
        disp = rng.uniform(-amplitude * h, amplitude * h, size=grid.shape)
        verts = grid + disp * _tangential_mask(grid)
    elif kind == "sin":
        s = np.sin(2 * np.pi * grid[:, 0]) * np.sin(2 * np.pi * grid[:, 1]) * np.sin(2 * np.pi * grid[:, 2])
        verts = grid + amplitude * h * s[:, None] * _tangential_mask(grid)
    elif kind == "none":
        verts = grid.copy()
    else:
        raise ValueError(f"unknown perturbation kind {kind!r}")
    # exact boundary coordinates
    verts[np.abs(grid) < 1e-12] = 0.0
    verts[np.abs(grid - 1.0) < 1e-12] = 1.0

    ne = n ** 3
    if c_mode == "element":
        media_c = rng.uniform(c_range[0], c_range[1], size=ne)
        elem_ref = np.arange(1, ne + 1, dtype=np.int32)
    elif c_mode == "blocks":
        nb = c_blocks
        media_c = rng.uniform(c_range[0], c_range[1], size=nb ** 3)
        e = np.arange(n)
        ez, ey, ex = np.meshgrid(e, e, e, indexing="ij")
        bx, by, bz = (ex.ravel() * nb) // n, (ey.ravel() * nb) // n, (ez.ravel() * nb) // n
        elem_ref = ((bz * nb + by) * nb + bx + 1).astype(np.int32)
    elif c_mode == "smooth":
        ctr = verts[hexes].mean(axis=1)
        media_c = 2.0 + 0.5 * np.sin(2 * np.pi * ctr[:, 0]) * np.sin(2 * np.pi * ctr[:, 1]) * np.sin(2 * np.pi * ctr[:, 2])
        elem_ref = np.arange(1, ne + 1, dtype=np.int32)
    elif c_mode == "constant":
        media_c = np.array([float(c_range[0])])
        elem_ref = np.ones(ne, dtype=np.int32)
    else:
        raise ValueError(f"unknown c_mode {c_mode!r}")
    return HexMesh(verts=verts, hexes=hexes, elem_ref=elem_ref,
                   media_c=np.asarray(media_c, dtype=np.float64), bfaces=bfaces, n=n)


def write_medit(path: str, mesh: HexMesh) -> None:
    """Medit ``.mesh`` (1-based indices) with hexahedra and boundary quadrilaterals."""
    with open(path, "w") as f:
        f.write("MeshVersionFormatted 2\n\nDimension 3\n\n")
        f.write(f"Vertices\n{mesh.verts.shape[0]}\n")
        np.savetxt(f, np.column_stack([mesh.verts, np.zeros(len(mesh.verts))]),
                   fmt=["%.17g", "%.17g", "%.17g", "%d"])
        f.write(f"\nQuadrilaterals\n{mesh.bfaces.shape[0]}\n")
        np.savetxt(f, np.column_stack([mesh.bfaces + 1, np.ones(len(mesh.bfaces), dtype=np.int64)]), fmt="%d")
        f.write(f"\nHexahedra\n{mesh.hexes.shape[0]}\n")
        np.savetxt(f, np.column_stack([mesh.hexes + 1, mesh.elem_ref]), fmt="%d")
        f.write("\nEnd\n")


@dataclasses.dataclass
class AcousticSetup:
    """Physical and time parameters of one acoustic leap-frog run."""

    order: int = 4
    f0: float = 5.0
    src_center: tuple = (0.5, 0.5, 0.5)
    src_radius: float = 0.125
    dt: float = 1e-3
    t0: float = 0.0
    nsteps: int = 200
    print_level: int = 0
    time_order: int = 2   # 2: leap-frog; 4: modified-equation leap-frog (OrderTimeScheme = 4 LEAP_FROG)
    t_end: float | None = None  # the deck's final time when read from one

    @property
    def tf(self) -> float:
        if self.t_end is not None:
            return self.t_end
        # ceil((tf - t0)/dt) must give exactly nsteps
        return self.t0 + (self.nsteps - 0.5) * self.dt


def write_deck(path: str, mesh_file: str, mesh: HexMesh, setup: AcousticSetup, receivers=None) -> None:
    """Data deck for the reference's ``acous3D`` solver on ``mesh_file``.

    ``rho = 1`` and ``mu = c^2`` per medium (``MateriauDielec = ref ISOTROPE rho mu sigma``,
    ``MONTJOIE/src/Elliptic/Helmholtz/VarHelmholtz.cxx:1179-1197``); Neumann on all
    faces; Gaussian volume source with a Ricker pulse; explicit time step;
    optional ``SismoPoint`` receivers.
    """
    lines = [
        "TypeElement = HEXAHEDRON_LOBATTO",
        "TypeEquation = ACOUSTIC",
        f"MeshPath = {os.path.dirname(os.path.abspath(mesh_file))}/",
        f"FileMesh = {os.path.basename(mesh_file)}",
        "TypeMesh = HEXA",
        f"OrderDiscretization = {setup.order}",
        f"NumberPhysicalMedia = {len(mesh.media_c) + 2}",
        "ConditionReference = 1 NEUMANN",
    ]
    for ref, c in enumerate(mesh.media_c, start=1):
        lines.append(f"MateriauDielec = {ref} ISOTROPE 1.0 {c * c:.17g} 0.0")
    cx, cy, cz = setup.src_center
    lines += [
        f"TypeSource = SRC_VOLUME GAUSSIAN {cx:.17g} {cy:.17g} {cz:.17g} {setup.src_radius:.17g}",
        f"Frequency = {setup.f0:.17g} 0.0",
        "TemporalSource = RICKER",
        "OutputFormat = BINARY DOUBLE",
        "ElectricOrMagnetic = 0",
        f"TimeStep = {setup.dt:.17g}",
        f"TimeInterval = {setup.t0:.17g} {setup.tf:.17g}",
        f"OrderTimeScheme = {setup.time_order} LEAP_FROG",
        f"PrintLevel = {setup.print_level}",
    ]
    for p in receivers if receivers is not None else ():
        lines.append(f"SismoPoint = {p[0]:.17g} {p[1]:.17g} {p[2]:.17g}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_medit(path: str) -> HexMesh:
    """Reads a Medit ``.mesh`` file the way the reference does
    (Mesh3D.cxx:3561-3638): a line holding a section keyword (``Vertices``,
    ``Edges``, ``Triangles``, ``Quadrilaterals``, ``Tetrahedra``,
    ``Hexahedra``) is followed by a count and that many whitespace-separated
    records, 1-based vertex numbers and an integer reference last; lines
    starting with ``#`` are comments.  Returns the hexahedra (reference-cube
    vertex order, as the file gives them) with their references, and the
    boundary quadrilaterals.  Meshes of other elements (tetrahedra, or
    degenerate hexahedra: pyramids and wedges) are outside the hexahedral
    Gauss-Lobatto path and raise ValueError.  ``media_c`` is left empty: the
    media come from the deck (``MateriauDielec``)."""
    with open(path) as f:
        lines = f.read().splitlines()
    verts = hexes = elem_ref = None
    quads = []
    i = 0

    def records(start, count, width):
        toks = []
        j = start
        while len(toks) < count * width:
            if j >= len(lines):
                raise ValueError(f"{path}: truncated section")
            toks.extend(lines[j].split())
            j += 1
        return np.array(toks[:count * width], dtype=np.float64).reshape(count, width), j

    while i < len(lines):
        line = lines[i]
        i += 1
        if not line or line[0] == "#":
            continue
        key = next((k for k in ("Vertices", "Edges", "Triangles", "Quadrilaterals", "Tetrahedra", "Hexahedra")
                    if k in line), None)
        if key is None:
            continue
        while not lines[i].split():
            i += 1
        count = int(lines[i].split()[0])
        rest = lines[i].split()[1:]
        if rest:  # records start on the count's line
            lines[i] = " ".join(rest)
        else:
            i += 1
        width = {"Vertices": 4, "Edges": 3, "Triangles": 4, "Quadrilaterals": 5, "Tetrahedra": 5, "Hexahedra": 9}[key]
        rec, i = records(i, count, width)
        if key == "Vertices":
            verts = rec[:, :3].copy()
        elif key == "Quadrilaterals":
            quads.append(rec[:, :4].astype(np.int64) - 1)
        elif key == "Tetrahedra" and count:
            raise ValueError(f"{path}: tetrahedra are not supported (hexahedral Gauss-Lobatto elements only)")
        elif key == "Hexahedra":
            h = rec[:, :8].astype(np.int64)
            if np.any(h[:, 7] == h[:, 6]):
                raise ValueError(f"{path}: degenerate hexahedra (pyramids or wedges) are not supported")
            hexes = (h - 1).astype(np.int32)
            elem_ref = rec[:, 8].astype(np.int32)
    if verts is None or hexes is None:
        raise ValueError(f"{path}: no Vertices or no Hexahedra section")
    if hexes.min() < 0 or hexes.max() >= verts.shape[0]:
        raise ValueError(f"{path}: vertex number out of range")
    bfaces = np.concatenate(quads).astype(np.int32) if quads else np.zeros((0, 4), dtype=np.int32)
    return HexMesh(verts=verts, hexes=hexes, elem_ref=elem_ref, media_c=np.zeros(0), bfaces=bfaces, n=0)


def _tokens(line: str):
    """Words of a deck line: split on blanks and tabs outside parentheses,
    empty words dropped (StringTokenize, MONTJOIE/src/Share/CommonMontjoie.cxx:70-97)."""
    out, cur, level = [], "", 0
    for ch in line:
        level += (ch == "(") - (ch == ")")
        if ch in " \t" and level == 0:
            if cur:
                out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur:
        out.append(cur)
    return out


def read_deck(path: str) -> dict:
    """Reads a data deck as ``ReadInputFile`` does (CommonInputOutput.cxx:1793-1858):
    lines starting with ``#`` are comments; a line is split on blanks and tabs,
    its first word is the keyword and the words after the second (``=``) its
    parameters (parenthesised groups stay one word); a last word ending in a
    backslash continues the parameters on
    the next line; a keyword without parameters is ignored.  Returns
    ``{keyword: [parameters of each occurrence]}`` in file order (keywords
    such as ``MateriauDielec`` and ``SismoPoint`` repeat)."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = {}
    n = 0
    while n < len(lines):
        line = lines[n]
        n += 1
        if not line or line[0] == "#":
            continue
        words = _tokens(line)
        if len(words) <= 2:
            continue
        params = words[2:]
        while params and params[-1].endswith("\\") and n < len(lines):
            params[-1] = params[-1][:-1]
            if not params[-1]:
                params.pop()
            params += _tokens(lines[n])
            n += 1
        out.setdefault(words[0], []).append(params)
    return out
