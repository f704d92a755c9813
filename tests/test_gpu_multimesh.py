"""Heterogeneous batch of meshes (orders 1..8, one cooperative kernel per
step) against the reference's trajectories and against the same runs
advanced one by one.

- Reference: the golden snapshots of u at 30 and 40 steps, within the FP32
  chosen-form tolerance (relative L2 <= 1e-4, as for single FP32 runs).
- Single runs: every batched run equals the same run advanced alone through
  mj_lf_advance (same FP32 arithmetic; relative L2 <= 1e-6).
- The batch keeps each run's state, step counter and pulse index consistent
  across graph replays, odd step counts and a run advanced on its own.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

CASES = ["cube2_q1", "cube2_q2", "cube2_q3", "regular2_q4", "cube3_q4", "cube2_q6", "cube2_q8", "cube4_q4"]
FP32_TOL = 1e-4
SAME_TOL = 1e-6


def run_fp32(g):
    from montjoie_gb300.leapfrog import LeapFrogIterator
    from montjoie_gb300.operator import FemMatrixFreeOperator
    op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, "fp32", gradphi=g["gradphi"])
    lf = LeapFrogIterator(op, float(g["dt"]), g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"])
    lf.SetInitialConditionS(np.zeros(g["massD"].size))
    return op, lf


def snapshot(g, step):
    steps = g["snap_steps"].tolist()
    return g["snaps"][steps.index(step)] if step in steps else None


@pytest.mark.parametrize("threads", [0, 128, 256, -1, -2])
def test_batch_matches_reference_and_single_runs(threads):
    """threads = 0: the autotuned launch configuration; 128 / 256: one kernel
    of all orders per step, forced; -1: one launch per order group, forced;
    -2: every order group stepped as its union, forced."""
    from montjoie_gb300.leapfrog import MeshBatch
    gs = [load_golden(c) for c in CASES]
    batch_runs = [run_fp32(g) for g in gs]
    single_runs = [run_fp32(g) for g in gs]
    mb = MeshBatch([lf for _, lf in batch_runs])
    if threads:
        mb.set_config(threads)
    info = mb.info()
    assert info["tiles"] > 0 and info["chunks"] >= len(CASES) and info["grid"] >= 1
    assert info["single_order"] == 0  # several orders: the all-orders kernel
    mb.advance(30)  # one 20-step graph + 10 launches
    assert mb.info()["graph"] == 1
    assert mb.grouping()["groups"] == len({int(g["order"]) for g in gs})
    if threads in (-1, -2):
        assert mb.grouping()["grouped"]
        if threads == -2:
            assert all(g["union"] for g in mb.grouping()["per_group"])
    elif threads:
        assert mb.tuning()["threads"] == threads and not mb.grouping()["grouped"]
    assert mb.tuning()["threads"] in (128, 256)
    for g, (_, lf), (_, ls) in zip(gs, batch_runs, single_runs):
        ls.Advance(30)
        u = lf.GetIterate()
        assert rel_l2(u, ls.GetIterate()) < SAME_TOL
        ref = snapshot(g, 30)
        if ref is not None:
            assert rel_l2(u, ref) < FP32_TOL
    mb.advance(10, graph=False)
    for g, (_, lf), (_, ls) in zip(gs, batch_runs, single_runs):
        ls.Advance(10)
        u = lf.GetIterate()
        assert rel_l2(u, ls.GetIterate()) < SAME_TOL
        ref = snapshot(g, 40)
        if ref is not None:
            assert rel_l2(u, ref) < FP32_TOL
    # odd counts: the graph starting at an odd offset, then a run advanced alone
    mb.advance(21)
    mb.advance(25)
    batch_runs[3][1].Advance(3)
    mb.advance(22)
    for k, ((_, lf), (_, ls)) in enumerate(zip(batch_runs, single_runs)):
        ls.Advance(68 + (3 if k == 3 else 0))
        u0, u1 = lf.GetState()
        v0, v1 = ls.GetState()
        assert rel_l2(u0, v0) < SAME_TOL and rel_l2(u1, v1) < SAME_TOL
        assert lf.n_time == ls.n_time
    mb.close()
    for op, lf in batch_runs + single_runs:
        lf.close()
        op.close()


@pytest.mark.parametrize("threads", [128, 256, -2])
@pytest.mark.parametrize("cases,n", [(["regular2_q4", "cube3_q4", "cube4_q4"], 5), (["cube2_q8", "cube2_q8"], 9)])
def test_single_order_batch(cases, n, threads):
    """Meshes of one order run that order's kernel instance: the same states
    as the runs advanced one by one, and the reference's snapshots."""
    from montjoie_gb300.leapfrog import MeshBatch
    gs = [load_golden(c) for c in cases]
    batch_runs = [run_fp32(g) for g in gs]
    single_runs = [run_fp32(g) for g in gs]
    mb = MeshBatch([lf for _, lf in batch_runs])
    mb.set_config(threads)
    assert mb.info()["single_order"] == n
    for steps, kw in ((30, {}), (9, {"graph": False}), (1, {})):
        mb.advance(steps, **kw)
        for g, (_, lf), (_, ls) in zip(gs, batch_runs, single_runs):
            ls.Advance(steps)
            u = lf.GetIterate()
            assert rel_l2(u, ls.GetIterate()) < SAME_TOL
            ref = snapshot(g, lf.n_time)
            if ref is not None:
                assert rel_l2(u, ref) < FP32_TOL
    mb.close()
    for op, lf in batch_runs + single_runs:
        lf.close()
        op.close()


def test_union_is_bitwise_the_runs_own_kernels():
    """Runs of every order stepped as unions (forced) give bit for bit the
    states of the same runs advanced alone, through graph replays, plain
    steps, odd counts and a run advanced on its own in between; the factors
    of one run scaled after the batch was made are taken up at the next
    advance."""
    from montjoie_gb300.leapfrog import MeshBatch
    gs = [load_golden(c) for c in CASES]
    batch_runs = [run_fp32(g) for g in gs]
    single_runs = [run_fp32(g) for g in gs]
    mb = MeshBatch([lf for _, lf in batch_runs])
    mb.set_config(-2)

    def same():
        for (_, lf), (_, ls) in zip(batch_runs, single_runs):
            u0, u1 = lf.GetState()
            v0, v1 = ls.GetState()
            assert np.array_equal(u0, v0) and np.array_equal(u1, v1)
            assert lf.n_time == ls.n_time

    for steps, kw in ((40, {}), (7, {"graph": False}), (21, {})):
        mb.advance(steps, **kw)
        for _, ls in single_runs:
            ls.Advance(steps)
        same()
    for k in (2, 5):  # runs advanced on their own: the batch re-reads their states
        batch_runs[k][1].Advance(3)
        single_runs[k][1].Advance(3)
    mb.advance(20)
    for _, ls in single_runs:
        ls.Advance(20)
    same()
    for op, _ in (batch_runs[4], single_runs[4]):
        op.set_element_scale(np.full(op.n_elt, 1.25))
    mb.advance(20)
    for _, ls in single_runs:
        ls.Advance(20)
    same()
    per_group = mb.grouping()["per_group"]
    assert all(g["union"] for g in per_group)
    assert sum(mb.union_info(i)["n_dof"] for i in range(len(per_group))) == mb.n_dof()
    mb.close()
    for op, lf in batch_runs + single_runs:
        lf.close()
        op.close()


def test_batch_long_run_matches_reference():
    """cube4_q4 (200 steps) and cube3_q4 (120 steps) batched with a Q8 mesh:
    final iterates against the reference's."""
    from montjoie_gb300.leapfrog import MeshBatch
    gs = [load_golden("cube4_q4"), load_golden("cube3_q4"), load_golden("cube2_q8")]
    runs = [run_fp32(g) for g in gs]
    mb = MeshBatch([lf for _, lf in runs])
    mb.advance(120)
    assert rel_l2(runs[1][1].GetIterate(), gs[1]["u_final"]) < FP32_TOL
    mb.advance(80)
    assert rel_l2(runs[0][1].GetIterate(), gs[0]["u_final"]) < FP32_TOL
    mb.close()
    for op, lf in runs:
        lf.close()
        op.close()


def test_batch_rejects_bad_runs():
    from montjoie_gb300 import _lib
    from montjoie_gb300.leapfrog import LeapFrogIterator, MeshBatch
    from montjoie_gb300.operator import FemMatrixFreeOperator
    g = load_golden("cube2_q2")
    op64 = FemMatrixFreeOperator(2, g["nodle"], g["bh"], g["massD"].size, "fp64")
    lf64 = LeapFrogIterator(op64, float(g["dt"]), g["massD"])
    with pytest.raises(_lib.MontjoieError):
        MeshBatch([lf64])
    op, lf = run_fp32(g)
    lf2 = LeapFrogIterator(op, float(g["dt"]), g["massD"])
    with pytest.raises(_lib.MontjoieError):
        MeshBatch([lf, lf2])  # shared operator
    lf3 = LeapFrogIterator(op, float(g["dt"]), g["massD"])
    mb = MeshBatch([lf3])
    with pytest.raises(_lib.MontjoieError):
        mb.advance(1)  # not initialised
    mb.close()
    for x in (lf64, lf, lf2, lf3, op64, op):
        x.close()
