"""Failure paths, made to happen on purpose without faulting or hanging the GPU.

- Bounded waits.  mj_debug_set_wait_limits makes waits run out: the element
  kernel's bulk-copy waits (two variants switched to instances compiled with
  a wait limit of 0; the variant is forced here) and the grid barrier of the
  cooperative steps (its limits lowered to 0).  The kernels report through
  their error flag after letting their own copies in flight land, the entry
  point returns an error status with a message, and the next call (limits
  restored) gives the same result as before.
- Divergence guard.  An unstable time step (well above the CFL limit) makes
  the norm grow past NormeMaxSolution (1e30 by default, as in the reference,
  MONTJOIE/src/Instationary/VarInstationary.cxx:2741-2745) and, with no limit,
  overflow: both return MJ_ERR_NONFINITE.
- Geometry.  An inverted hexahedron (negative Jacobian) makes mj_geometry
  return MJ_ERR_GEOMETRY (the reference aborts on a non-positive Jacobian,
  MONTJOIE/src/Harmonic/VarGeometryProblem.cxx:716-750).
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture
def lowered_waits():
    """Lowers the wait limits for the test body; restores them whatever happens."""
    from montjoie_gb300 import _lib
    L = _lib.load()

    def lower(mbar_polls=-1, barrier_polls=-1, barrier_ns=-1):
        _lib.check(L.mj_debug_set_wait_limits(mbar_polls, barrier_polls, barrier_ns))

    yield lower
    _lib.check(L.mj_debug_set_wait_limits(-1, -1, -1))


def _problem(cells=12, order=4, seed=3):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem, cfl_time_step
    m = M.perturbed_cube(cells, seed=seed, amplitude=0.05, kind="random", c_mode="element")
    s = M.AcousticSetup(order=order, dt=1.0, nsteps=60, src_radius=2.0 / cells)
    pb = AcousticProblem(m, s, defer_time=True)
    pb.set_time_step(cfl_time_step(pb, safety=0.5), 60)
    return pb


# the element-kernel variants that have instances with a wait limit of 0:
# (elements per CTA, layout) for each precision
WAITS_OUT_VARIANT = {"fp32": (2, 2), "fp64": (4, 0)}


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_element_kernel_wait_runs_out_and_next_call_works(lowered_waits, precision):
    from montjoie_gb300._lib import MJ_ERR_CUDA, MontjoieError
    pb = _problem()
    op = pb.operator(precision)
    op.set_variant(*WAITS_OUT_VARIANT[precision])
    x = np.random.default_rng(0).uniform(-1, 1, pb.n_dof)
    y_ok = np.zeros(pb.n_dof)
    op.MltAddVector(1.0, x, 0.0, y_ok)
    lowered_waits(mbar_polls=0)
    y = np.zeros(pb.n_dof)
    with pytest.raises(MontjoieError) as exc:
        op.MltAddVector(1.0, x, 0.0, y)
    assert exc.value.code == MJ_ERR_CUDA and "bounded wait" in str(exc.value)
    lowered_waits()
    op.MltAddVector(1.0, x, 0.0, y)
    assert rel_l2(y, y_ok) == 0.0  # same kernels, same sums: bitwise
    op.close()


def test_leapfrog_waits_run_out_and_next_run_works(lowered_waits):
    """FP32 order-2 steps launched one by one (a captured graph keeps its kernels)."""
    from montjoie_gb300._lib import MJ_ERR_CUDA, MontjoieError
    pb = _problem()
    op = pb.operator("fp32")
    op.set_variant(*WAITS_OUT_VARIANT["fp32"])
    lf = pb.integrator(op, diagnostics=False)
    lf.set_graph(False)
    zeros = np.zeros(pb.n_dof)
    lf.SetInitialConditionS(zeros)
    lf.Advance(45)
    u_ok = lf.GetIterate()
    lf.SetInitialConditionS(zeros)
    lowered_waits(mbar_polls=0)
    with pytest.raises(MontjoieError) as exc:
        lf.Advance(45)
    assert exc.value.code == MJ_ERR_CUDA and "bounded wait" in str(exc.value)
    lowered_waits()
    lf.SetInitialConditionS(zeros)
    lf.Advance(45)
    assert rel_l2(lf.GetIterate(), u_ok) == 0.0
    lf.close()
    op.close()


def _batch_runs():
    from montjoie_gb300.leapfrog import LeapFrogIterator
    from montjoie_gb300.operator import FemMatrixFreeOperator
    runs = []
    for c in ["cube2_q2", "cube3_q4", "cube2_q8"]:
        g = load_golden(c)
        op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, "fp32",
                                   gradphi=g["gradphi"])
        lf = LeapFrogIterator(op, float(g["dt"]), g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"])
        lf.SetInitialConditionS(np.zeros(g["massD"].size))
        runs.append((op, lf))
    return runs


def test_mesh_batch_waits_run_out_and_next_advance_works(lowered_waits):
    from montjoie_gb300._lib import MJ_ERR_STATE, MontjoieError
    from montjoie_gb300.leapfrog import MeshBatch
    runs = _batch_runs()
    mb = MeshBatch([lf for _, lf in runs])
    mb.set_config(256)  # the one-kernel form, whose grid barrier the lowered limits make run out
    mb.advance(25)
    u_ok = [lf.GetIterate() for _, lf in runs]
    for _, lf in runs:
        lf.SetInitialConditionS(np.zeros(lf.op.n_dof))
    lowered_waits(barrier_polls=0, barrier_ns=0)
    with pytest.raises(MontjoieError) as exc:
        mb.advance(25)
    assert exc.value.code == MJ_ERR_STATE and "timed out" in str(exc.value)
    lowered_waits()
    for _, lf in runs:
        lf.SetInitialConditionS(np.zeros(lf.op.n_dof))
    mb.advance(25)
    for (_, lf), u in zip(runs, u_ok):
        assert rel_l2(lf.GetIterate(), u) == 0.0
    mb.close()
    for op, lf in runs:
        lf.close()
        op.close()


def test_many_source_step_waits_run_out_and_next_advance_works(lowered_waits):
    from montjoie_gb300._lib import MJ_ERR_STATE, MontjoieError
    from montjoie_gb300.leapfrog import BatchLeapFrog
    g = load_golden("cube3_q4")
    from montjoie_gb300.operator import FemMatrixFreeOperator
    op = FemMatrixFreeOperator(4, g["nodle"], g["bh"], g["massD"].size, "fp32", gradphi=g["gradphi"])
    S = 8
    idx = np.concatenate([g["src_idx"]] * S)
    rhs = np.repeat(np.arange(S), g["src_idx"].size)
    val = np.concatenate([g["src_val"] * (1.0 + 0.1 * s) for s in range(S)])
    b = BatchLeapFrog(op, float(g["dt"]), S, g["massD"], g["invD"], idx, rhs, val, g["pulse"])
    assert b.step_info()["one_kernel"]
    b.init()
    b.advance(25)
    u_ok, _ = b.state()
    b.init()
    lowered_waits(barrier_polls=0, barrier_ns=0)
    with pytest.raises(MontjoieError) as exc:
        b.advance(25)
    assert exc.value.code == MJ_ERR_STATE and "timed out" in str(exc.value)
    lowered_waits()
    b.init()
    b.advance(25)
    u, _ = b.state()
    assert rel_l2(u, u_ok) == 0.0
    b.close()
    op.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_unstable_run_hits_the_norm_limit(precision):
    """dt = 3 x the stable step: the norm passes NormeMaxSolution (1e30)."""
    from montjoie_gb300._lib import MJ_ERR_NONFINITE, MontjoieError
    pb = _problem(cells=4, order=3)
    pb.set_time_step(pb.setup.dt * 6.0, 400)  # 0.5 CFL x 6 = 3 CFL
    op = pb.operator(precision)
    lf = pb.integrator(op)
    with pytest.raises(MontjoieError) as exc:
        lf.Run(np.zeros(pb.n_dof), None, 400)
    assert exc.value.code == MJ_ERR_NONFINITE and "above the limit" in str(exc.value)
    lf.close()
    op.close()


def test_unstable_run_without_limit_overflows_to_nonfinite():
    """With no norm limit the same run overflows; the device flag reports it."""
    from montjoie_gb300._lib import MJ_ERR_NONFINITE, MontjoieError
    pb = _problem(cells=4, order=3)
    pb.set_time_step(pb.setup.dt * 6.0, 600)
    op = pb.operator("fp64")
    lf = pb.integrator(op)
    lf.SetNormeMaxSolution(float("inf"))
    lf.SetInitialConditionS(np.zeros(pb.n_dof))
    with pytest.raises(MontjoieError) as exc:
        lf.Advance(600)
    assert exc.value.code == MJ_ERR_NONFINITE and "non-finite" in str(exc.value)
    lf.close()
    op.close()


def test_norm_limit_is_a_threshold_on_stable_runs():
    """A stable run passes with the default limit and trips a limit below its norms."""
    from montjoie_gb300._lib import MJ_ERR_NONFINITE, MontjoieError
    pb = _problem(cells=4, order=3)
    op = pb.operator("fp64")
    lf = pb.integrator(op)
    _, norms, _ = lf.Run(np.zeros(pb.n_dof), None, 60)
    peak = float(np.max(norms))
    assert 0.0 < peak < 1e30
    lf.SetNormeMaxSolution(0.5 * peak)
    with pytest.raises(MontjoieError) as exc:
        lf.Run(np.zeros(pb.n_dof), None, 60)
    assert exc.value.code == MJ_ERR_NONFINITE
    lf.SetNormeMaxSolution(2.0 * peak)
    lf.Run(np.zeros(pb.n_dof), None, 60)
    lf.close()
    op.close()


def test_inverted_element_is_a_geometry_error():
    from montjoie_gb300 import mesh as M
    from montjoie_gb300._lib import MJ_ERR_GEOMETRY, MontjoieError
    from montjoie_gb300.problem import geometry
    m = M.perturbed_cube(3, seed=1, amplitude=0.05, kind="random", c_mode="element")
    verts_e = m.verts[m.hexes].copy()
    fac, jw, _ = geometry(2, verts_e, m.elem_c ** 2)
    assert (jw > 0).all()
    verts_e[13] = verts_e[13][[4, 5, 6, 7, 0, 1, 2, 3]]  # element 13 turned inside out (z reversed)
    with pytest.raises(MontjoieError) as exc:
        geometry(2, verts_e, m.elem_c ** 2)
    assert exc.value.code == MJ_ERR_GEOMETRY
    fac2, jw2, _ = geometry(2, m.verts[m.hexes], m.elem_c ** 2)  # the next call works
    assert np.array_equal(fac2, fac) and np.array_equal(jw2, jw)
