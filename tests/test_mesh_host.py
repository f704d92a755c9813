"""Host side of the mesh generator and of the files written for the
reference's solver (no GPU): the perturbed unit cube keeps its faces, moves
vertices within the stated amplitude, assigns wave speeds as asked; the
Medit file and the data deck say what the mesh and the set-up are."""
import numpy as np
import pytest

from montjoie_gb300 import mesh as M


@pytest.mark.parametrize("kind,amp", [("random", 0.05), ("sin", 0.1), ("none", 0.0)])
def test_perturbed_cube_geometry(kind, amp):
    n = 6
    m = M.perturbed_cube(n, seed=3, amplitude=amp, kind=kind)
    grid = M.perturbed_cube(n, kind="none").verts
    assert m.verts.shape == ((n + 1) ** 3, 3) and m.hexes.shape == (n ** 3, 8)
    assert m.n_elt == n ** 3 and m.n == n
    d = np.abs(m.verts - grid)
    assert d.max() <= amp / n + 1e-15
    # the domain stays the unit cube: face vertices keep their normal coordinate
    for ax in range(3):
        for face in (0.0, 1.0):
            on = np.abs(grid[:, ax] - face) < 1e-12
            assert np.all(m.verts[on, ax] == face)
    # every hexahedron keeps a positive volume (corner 0 to the far corner 6 along +x+y+z)
    v = m.verts[m.hexes]
    assert np.all((v[:, 6] - v[:, 0]).min(axis=1) > 0)
    # boundary quadrilaterals: 6 faces of n^2 each, all on the cube's faces
    assert m.bfaces.shape == (6 * n * n, 4)
    fv = grid[m.bfaces]
    assert np.all(np.any(np.all((np.abs(fv) < 1e-12) | (np.abs(fv - 1) < 1e-12), axis=1), axis=1))


def test_perturbation_is_seeded():
    a = M.perturbed_cube(5, seed=11, kind="random")
    b = M.perturbed_cube(5, seed=11, kind="random")
    c = M.perturbed_cube(5, seed=12, kind="random")
    assert np.array_equal(a.verts, b.verts) and np.array_equal(a.media_c, b.media_c)
    assert not np.array_equal(a.verts, c.verts)


@pytest.mark.parametrize("c_mode", ["element", "blocks", "smooth", "constant"])
def test_wave_speed_modes(c_mode):
    n, nb = 8, 4
    m = M.perturbed_cube(n, seed=5, c_mode=c_mode, c_blocks=nb, c_range=(1.0, 3.0))
    c = m.elem_c
    assert c.shape == (n ** 3,) and m.elem_ref.min() >= 1 and m.elem_ref.max() <= len(m.media_c)
    if c_mode == "element":
        assert len(m.media_c) == n ** 3 and c.min() >= 1.0 and c.max() <= 3.0
    elif c_mode == "blocks":
        assert len(m.media_c) == nb ** 3
        # each block of (n/nb)^3 elements shares one medium
        e = np.arange(n)
        ez, ey, ex = np.meshgrid(e, e, e, indexing="ij")
        blk = ((ez // (n // nb)) * nb + ey // (n // nb)) * nb + ex // (n // nb)
        for b in range(nb ** 3):
            assert len(np.unique(c[blk.ravel() == b])) == 1
    elif c_mode == "smooth":
        assert c.min() >= 1.5 - 1e-12 and c.max() <= 2.5 + 1e-12
    else:
        assert np.all(c == 1.0)


def test_medit_and_deck(tmp_path):
    m = M.perturbed_cube(3, seed=2, kind="random", c_mode="blocks", c_blocks=3)
    mf = tmp_path / "cube.mesh"
    M.write_medit(str(mf), m)
    text = mf.read_text().split()
    i = text.index("Vertices")
    assert int(text[i + 1]) == len(m.verts)
    first = np.array(text[i + 2:i + 5], dtype=float)
    assert np.array_equal(first, m.verts[0])
    j = text.index("Hexahedra")
    assert int(text[j + 1]) == m.n_elt
    h0 = np.array(text[j + 2:j + 11], dtype=int)
    assert np.array_equal(h0[:8], m.hexes[0] + 1) and h0[8] == m.elem_ref[0]  # 1-based, then the reference
    k = text.index("Quadrilaterals")
    assert int(text[k + 1]) == len(m.bfaces)
    s = M.AcousticSetup(order=6, dt=2e-3, nsteps=50, time_order=4)
    df = tmp_path / "cube.ini"
    M.write_deck(str(df), str(mf), m, s)
    deck = df.read_text().splitlines()
    assert "OrderDiscretization = 6" in deck and "OrderTimeScheme = 4 LEAP_FROG" in deck
    assert "FileMesh = cube.mesh" in deck and "TimeStep = 0.002" in deck
    media = [ln for ln in deck if ln.startswith("MateriauDielec")]
    assert len(media) == len(m.media_c)
    mu = np.array([float(ln.split()[5]) for ln in media])  # "= ref ISOTROPE rho mu sigma"
    assert np.allclose(mu, m.media_c ** 2, rtol=1e-15)
    # ceil((tf - t0) / dt) is the step count the reference will run
    t0, tf = (float(x) for x in [ln for ln in deck if ln.startswith("TimeInterval")][0].split()[2:4])
    assert int(np.ceil((tf - t0) / s.dt)) == s.nsteps


def test_medit_round_trip(tmp_path):
    """write_medit then read_medit gives back the mesh exactly (17 digits)."""
    m = M.perturbed_cube(5, seed=9, amplitude=0.1, kind="sin", c_mode="blocks", c_blocks=2)
    path = str(tmp_path / "m.mesh")
    M.write_medit(path, m)
    r = M.read_medit(path)
    assert np.array_equal(r.verts, m.verts)
    assert np.array_equal(r.hexes, m.hexes) and np.array_equal(r.elem_ref, m.elem_ref)
    assert np.array_equal(r.bfaces, m.bfaces)


def test_medit_reader_follows_the_reference_layout(tmp_path):
    """Comments, blank lines, records spread over lines, sections in any
    order and unknown sections, as the reference's stream reader accepts."""
    path = tmp_path / "hand.mesh"
    path.write_text("""MeshVersionFormatted 2
# a comment
Dimension 3

Hexahedra
1
1 2 3 4
5 6 7 8 7

Corners
0

Vertices
8
0 0 0 0   1 0 0 0
1 1 0 0
0 1 0 0
0 0 1 0
1 0 1 0
1 1 1 0
0 1 1 0
Quadrilaterals
1
1 4 3 2 1
End
""")
    r = M.read_medit(str(path))
    assert r.verts.shape == (8, 3) and np.array_equal(r.verts[6], [1.0, 1.0, 1.0])
    assert np.array_equal(r.hexes, [[0, 1, 2, 3, 4, 5, 6, 7]]) and np.array_equal(r.elem_ref, [7])
    assert np.array_equal(r.bfaces, [[0, 3, 2, 1]])
    tet = tmp_path / "tet.mesh"
    tet.write_text("Vertices\n4\n0 0 0 0\n1 0 0 0\n0 1 0 0\n0 0 1 0\nTetrahedra\n1\n1 2 3 4 1\n")
    with pytest.raises(ValueError, match="tetrahedra"):
        M.read_medit(str(tet))


def test_deck_reader_follows_the_reference_rules(tmp_path):
    """ReadInputFile's rules: # comments, words after '=' as parameters, a
    trailing backslash continues the line, repeated keywords kept in order,
    keywords without parameters ignored, blanks inside parentheses kept."""
    path = tmp_path / "d.ini"
    path.write_text("""# deck
TypeElement = HEXAHEDRON_LOBATTO
OrderDiscretization = 4
MateriauDielec = 1 ISOTROPE 1.0 4.0 0.0
MateriauDielec = 2 ISOTROPE 2.0 \\
   8.0 0.0
SismoPoint = 0.1 0.2 0.3
SismoPoint = 0.4 0.5 0.6
Empty =
\tTimeStep\t=\t0.001
Function = (a b) c
""")
    d = M.read_deck(str(path))
    assert d["TypeElement"] == [["HEXAHEDRON_LOBATTO"]] and d["OrderDiscretization"] == [["4"]]
    assert d["MateriauDielec"] == [["1", "ISOTROPE", "1.0", "4.0", "0.0"], ["2", "ISOTROPE", "2.0", "8.0", "0.0"]]
    assert d["SismoPoint"] == [["0.1", "0.2", "0.3"], ["0.4", "0.5", "0.6"]]
    assert "Empty" not in d
    assert d["TimeStep"] == [["0.001"]]  # empty words (leading tab) are dropped
    assert d["Function"] == [["(a b)", "c"]]


def test_written_deck_reads_back(tmp_path):
    m = M.perturbed_cube(3, seed=2, amplitude=0.05, kind="random", c_mode="element")
    s = M.AcousticSetup(order=3, dt=1.25e-3, nsteps=40, src_radius=0.3, time_order=4)
    rec = np.array([[0.2, 0.3, 0.4], [0.6, 0.5, 0.7]])
    M.write_medit(str(tmp_path / "c.mesh"), m)
    M.write_deck(str(tmp_path / "c.ini"), str(tmp_path / "c.mesh"), m, s, receivers=rec)
    d = M.read_deck(str(tmp_path / "c.ini"))
    assert float(d["TimeStep"][0][0]) == s.dt
    assert [float(v) for v in d["TimeInterval"][0]] == [s.t0, s.tf]
    assert d["OrderTimeScheme"] == [["4", "LEAP_FROG"]]
    assert np.array_equal(np.array(d["SismoPoint"], dtype=float), rec)
    mu = np.array([float(p[3]) for p in d["MateriauDielec"]])
    assert np.array_equal(mu, m.media_c ** 2)


@pytest.mark.parametrize("edit,match", [
    (("TimeStep = ", "TimeStep = AUTO"), "AUTO"),
    (("ConditionReference = 1 NEUMANN", "ConditionReference = 1 DIRICHLET"), "NEUMANN"),
    (("TypeElement = HEXAHEDRON_LOBATTO", "TypeElement = TETRAHEDRON_CLASSICAL"), "HEXAHEDRON_LOBATTO"),
    (("TemporalSource = RICKER", "TemporalSource = GAUSSIAN"), "RICKER"),
])
def test_deck_outside_the_path_is_refused(tmp_path, edit, match):
    """Keywords this path does not cover raise before any GPU work."""
    from montjoie_gb300.problem import AcousticProblem
    m = M.perturbed_cube(2, seed=2, amplitude=0.05, kind="random", c_mode="element")
    M.write_medit(str(tmp_path / "c.mesh"), m)
    M.write_deck(str(tmp_path / "c.ini"), str(tmp_path / "c.mesh"), m, M.AcousticSetup(order=2))
    text = (tmp_path / "c.ini").read_text().splitlines()
    text = [edit[1] if line.startswith(edit[0]) else line for line in text]
    (tmp_path / "c.ini").write_text("\n".join(text) + "\n")
    with pytest.raises(ValueError, match=match):
        AcousticProblem.from_deck(str(tmp_path / "c.ini"))
