"""GPU parity of the order-4 modified-equation leap-frog
(ModifiedEquationIterator with order 4, MONTJOIE/src/Instationary/ModifiedEquation.cxx:125-175, 346-408)
against the reference's own order-4 runs (golden fixtures) and the oracle.

FP64 plain form: relative L2 <= 1e-10 of the final iterate, the snapshots and
the norm history; FP32 chosen form <= 1e-4.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def integrator4(g, precision, norms=True):
    from montjoie_gb300.leapfrog import LeapFrogIterator
    from montjoie_gb300.operator import FemMatrixFreeOperator
    op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, precision,
                               gradphi=g["gradphi"])
    jwsum = np.zeros(g["massD"].size)
    np.add.at(jwsum, g["nodle"].ravel(), g["jw"].ravel())
    lf = LeapFrogIterator(op, float(g["dt"]), g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"],
                          jwsum if norms else None, time_order=4, pulse_d2=g["pulse3"])
    return op, lf


def test_order4_fp64_matches_reference(golden_case4):
    name, g = golden_case4
    op, lf = integrator4(g, "fp64")
    n = int(g["nsteps"])
    uf, norms, _ = lf.Run(np.zeros(g["massD"].size), None, n)
    assert rel_l2(uf, g["u_final"]) < FP64_TOL
    assert rel_l2(norms, g["norms"]) < FP64_TOL
    lf.close(); op.close()


def test_order4_snapshots_chunked_and_graph(golden_case4):
    """Chunked Advance (graph replays and odd chunks) reaches the reference's snapshots."""
    name, g = golden_case4
    op, lf = integrator4(g, "fp64", norms=False)
    lf.SetInitialConditionS(np.zeros(g["massD"].size))
    done = 0
    for k, snap in zip(g["snap_steps"].tolist(), g["snaps"]):
        if k > done:
            lf.Advance(k - done)
            done = k
        assert rel_l2(lf.GetIterate(), snap) < FP64_TOL if k else np.allclose(lf.GetIterate(), snap)
    lf.close(); op.close()


def test_order4_fp32_error(golden_case4):
    name, g = golden_case4
    op, lf = integrator4(g, "fp32")
    n = int(g["nsteps"])
    uf, norms, _ = lf.Run(np.zeros(g["massD"].size), None, n)
    assert rel_l2(uf, g["u_final"]) < 1e-4
    assert rel_l2(norms, g["norms"]) < 1e-4
    lf.close(); op.close()


def test_order4_initial_conditions_match_oracle():
    """Non-zero u0 and du0 (the Taylor start with all four derivatives)."""
    from oracle import oracle as oc
    g = load_golden("cube3_q4_o4")
    rng = np.random.default_rng(13)
    u0 = rng.uniform(-1, 1, g["massD"].size)
    du0 = rng.uniform(-1, 1, g["massD"].size)
    op, lf = integrator4(g, "fp64")
    n = 50
    uf, norms, _ = lf.Run(u0, du0, n)
    uo, _, no, _ = oc.leapfrog4(int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"],
                                g["src_val"], g["pulse"], g["pulse3"], float(g["dt"]), n, u0, du0=du0, jw=g["jw"])
    assert rel_l2(uf, uo) < 1e-12
    assert rel_l2(norms, no) < 1e-12
    lf.close(); op.close()


def test_order4_graph_equals_plain():
    g = load_golden("cube3_q4_o4")
    op1, a = integrator4(g, "fp32", norms=False)
    op2, b = integrator4(g, "fp32", norms=False)
    b.set_graph(False)
    a.SetInitialConditionS(np.zeros(g["massD"].size)); b.SetInitialConditionS(np.zeros(g["massD"].size))
    a.Advance(3); b.Advance(3)
    a.Advance(61); b.Advance(61)
    ua, va = a.GetState()
    ub, vb = b.GetState()
    assert np.array_equal(ua, ub) and np.array_equal(va, vb)
    a.close(); b.close(); op1.close(); op2.close()


def test_order4_problem_setup_matches_oracle():
    """Our own set-up (mesh, numbering, geometry, source, pulse and p'', CFL of
    order 4) through AcousticProblem against the oracle's order-4 run."""
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem, cfl_time_step
    from oracle import oracle as oc
    m = M.perturbed_cube(4, seed=7, amplitude=0.05, kind="random", c_mode="element")
    s = M.AcousticSetup(order=3, dt=1.0, nsteps=60, src_radius=0.5, time_order=4)
    pb = AcousticProblem(m, s, defer_time=True)
    dt = cfl_time_step(pb, safety=0.5)
    pb.set_time_step(dt, 60)
    assert pb.pulse_d2 is not None and np.abs(pb.pulse_d2).max() > 0
    op = pb.operator("fp64")
    lf = pb.integrator(op, diagnostics=False)
    uf, _, _ = lf.Run(np.zeros(pb.n_dof), None, 60)
    uo, _, _, _ = oc.leapfrog4(3, pb.nodle, pb.factors, pb.mass, 1.0 / pb.mass, pb.src_idx, pb.src_val, pb.pulse,
                               pb.pulse_d2, dt, 60, np.zeros(pb.n_dof))
    assert np.linalg.norm(uo) > 0
    assert rel_l2(uf, uo) < 1e-10
    lf.close(); op.close()
