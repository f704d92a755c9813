"""Runs read from disk: a reference data deck and its Medit mesh, parsed by
this library (mesh.read_deck, mesh.read_medit) into AcousticProblem.from_deck
and advanced on the GPU, against what the reference computed from the same
files.

The deck and the mesh are rewritten here, byte for byte as the fixtures'
generator wrote them for the reference (same writer, seed and time step), then
read back from disk.  Parity: FP64 norm history, receiver traces and final
state within 1e-10 of the reference (configuration 1: 16^3 Q4, 200 steps;
the golden Q8 case on a sinusoidally displaced mesh with smooth c)."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _by_position(pb, u, pos_ref):
    """Values of u (this library's numbering) at the reference's dof positions."""
    pos = np.zeros((pb.n_dof, 3))
    pos[pb.nodle.ravel()] = pb.xq.reshape(-1, 3)
    key = lambda p: np.round(p * 1e9).astype(np.int64)  # noqa: E731
    table = {tuple(k): i for i, k in enumerate(key(pos))}
    return u[np.array([table[tuple(k)] for k in key(pos_ref)])]


def test_config1_deck_from_disk(tmp_path):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem
    g = load_golden("config1_16q4")
    m = M.perturbed_cube(16, seed=int(g["seed"]), amplitude=0.05, kind="random", c_mode="element")
    s = M.AcousticSetup(order=4, dt=float(g["dt"]), nsteps=int(g["nsteps"]), src_radius=float(g["src_radius"]))
    M.write_medit(str(tmp_path / "config1.mesh"), m)
    M.write_deck(str(tmp_path / "config1.ini"), str(tmp_path / "config1.mesh"), m, s, receivers=g["receivers"])
    del m, s
    pb = AcousticProblem.from_deck(str(tmp_path / "config1.ini"))
    assert pb.setup.nsteps == int(g["nsteps"]) and pb.setup.dt == float(g["dt"])
    assert rel_l2(pb.pulse, g["pulse"]) < 1e-12 and pb.src_idx.size == int(g["n_src"])
    assert abs(pb.mass.sum() - float(g["massD_sum"])) < 1e-12 * float(g["massD_sum"])
    op = pb.operator("fp64")
    lf = pb.integrator(op)
    uf, norms, traces = lf.Run(np.zeros(pb.n_dof), None, pb.setup.nsteps)
    assert rel_l2(norms, g["norms"]) < FP64_TOL
    assert np.abs(traces - g["traces"]).max() < FP64_TOL * np.abs(g["traces"]).max()
    assert rel_l2(_by_position(pb, uf, g["probe_pos"]), g["probe_u"]) < FP64_TOL
    lf.close()
    op.close()


def test_golden_q8_deck_from_disk(tmp_path):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem
    from oracle import oracle as oc
    g = load_golden("cube2_q8")
    m = M.HexMesh(verts=g["verts"], hexes=g["hexes"], elem_ref=g["elem_ref"], media_c=g["media_c"],
                  bfaces=M.perturbed_cube(int(g["n"]), kind="none").bfaces, n=int(g["n"]))
    s = M.AcousticSetup(order=8, dt=float(g["dt"]), nsteps=int(g["nsteps"]), src_radius=float(g["src_radius"]))
    M.write_medit(str(tmp_path / "q8.mesh"), m)
    M.write_deck(str(tmp_path / "q8.ini"), str(tmp_path / "q8.mesh"), m, s)
    pb = AcousticProblem.from_deck(str(tmp_path / "q8.ini"))
    op = pb.operator("fp64")
    lf = pb.integrator(op)
    uf, norms, _ = lf.Run(np.zeros(pb.n_dof), None, pb.setup.nsteps)
    assert rel_l2(norms, g["norms"]) < FP64_TOL
    # final state at the reference's dof positions
    _, _, xq_ref = oc.geometry(8, g["verts_e"], np.ones(g["verts_e"].shape[0]))
    pos_ref = np.zeros((g["massD"].size, 3))
    pos_ref[g["nodle"].ravel()] = xq_ref.reshape(-1, 3)
    assert rel_l2(_by_position(pb, uf, pos_ref), g["u_final"]) < FP64_TOL
    lf.close()
    op.close()
