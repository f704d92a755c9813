"""Many sources on one mesh (64 Ricker sources on 32^3 Q4 at full size): S leap-frog
runs advanced together in FP32 must match S separate runs of the reference's
scheme (the FP64 oracle) within the FP32 tolerance, 1e-4 relative L2 over
the run; the captured-graph path must equal the plain launch path bit for bit."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu


def _batch(g, S, graph_src_scale=None, receivers=None):
    from montjoie_gb300.leapfrog import BatchLeapFrog
    from montjoie_gb300.operator import FemMatrixFreeOperator
    op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, "fp32", gradphi=g["gradphi"])
    idx, rhs, val = [], [], []
    for s in range(S):
        idx.append(g["src_idx"])
        rhs.append(np.full(g["src_idx"].size, s))
        val.append(g["src_val"] * (1.0 + 0.25 * s))
    kw = {}
    if receivers is not None:
        kw = dict(rec_idx=receivers[0], rec_w=receivers[1])
    b = BatchLeapFrog(op, float(g["dt"]), S, g["massD"], g["invD"], np.concatenate(idx), np.concatenate(rhs),
                      np.concatenate(val), g["pulse"], **kw)
    return op, b


@pytest.mark.parametrize("case", ["cube3_q4", "cube2_q2", "cube2_q8"])
def test_batched_sources_match_separate_runs(case):
    from oracle import oracle as oc
    g = load_golden(case)
    S = 16
    op, b = _batch(g, S)
    n = int(g["nsteps"])
    b.init()
    b.advance(n, graph=False)
    u, _ = b.state()
    for s in (0, 5, S - 1):
        uo, _, _, _ = oc.leapfrog(int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"],
                                  g["src_val"] * (1.0 + 0.25 * s), g["pulse"], float(g["dt"]), n,
                                  np.zeros(g["massD"].size))
        assert rel_l2(u[:, s], uo) < 1e-4
    assert rel_l2(u[:, 0] * 1.25, u[:, 1]) < 1e-4  # linearity in the source amplitude
    b.close(); op.close()


@pytest.mark.parametrize("S", [1, 3, 13])
def test_any_number_of_runs(S):
    """S not a multiple of 8: the runs are padded to the next multiple with
    runs that have no source; the caller's runs match separate oracle runs
    and the arrays handed out have S columns."""
    from oracle import oracle as oc
    from montjoie_gb300.problem import receiver_weights
    g = load_golden("cube3_q4")
    rng = np.random.default_rng(S)
    rec = receiver_weights(int(g["order"]), g["verts_e"], g["nodle"], rng.uniform(0.1, 0.9, size=(2, 3)))
    op, b = _batch(g, S, receivers=rec)
    info = b.info()
    assert info["n_rhs"] == S and info["n_rhs_device"] == (S + 7) // 8 * 8
    u0 = rng.uniform(-1, 1, (g["massD"].size, S))
    n = 30
    b.init(u0)
    tr = b.advance(n, traces=True)
    u, v = b.state()
    assert u.shape == (g["massD"].size, S) and v.shape == u.shape and tr.shape == (2, S, n)
    for s in sorted({0, S - 1}):
        uo, _, _, to = oc.leapfrog(int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"],
                                   g["src_val"] * (1.0 + 0.25 * s), g["pulse"], float(g["dt"]), n, u0[:, s],
                                   rec_idx=rec[0], rec_w=rec[1])
        assert rel_l2(u[:, s], uo) < 1e-4
        assert np.abs(tr[:, s, :] - to[:, :n]).max() < 1e-4 * np.abs(to).max()
    b.close(); op.close()


def test_graph_replay_equals_plain_launches():
    g = load_golden("cube4_q4")
    S = 32
    op1, b1 = _batch(g, S)
    op2, b2 = _batch(g, S)
    b1.init(); b2.init()
    b1.advance(3, graph=False); b2.advance(3, graph=False)      # odd start: realignment path
    b1.advance(61, graph=True); b2.advance(61, graph=False)
    u1, v1 = b1.state()
    u2, v2 = b2.state()
    assert np.array_equal(u1, u2) and np.array_equal(v1, v2)
    assert b1.info()["step"] == 64
    b1.close(); b2.close(); op1.close(); op2.close()


def test_batched_initial_conditions_and_traces():
    from oracle import oracle as oc
    from montjoie_gb300.problem import receiver_weights
    g = load_golden("cube3_q4")
    S = 8
    rng = np.random.default_rng(11)
    pts = rng.uniform(0.1, 0.9, size=(3, 3))
    rec = receiver_weights(int(g["order"]), g["verts_e"], g["nodle"], pts)
    op, b = _batch(g, S, receivers=rec)
    u0 = rng.uniform(-1, 1, (g["massD"].size, S))
    n = 40
    b.init(u0)
    tr = b.advance(n, traces=True)
    u, _ = b.state()
    for s in (0, S - 1):
        uo, _, _, to = oc.leapfrog(int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"],
                                   g["src_val"] * (1.0 + 0.25 * s), g["pulse"], float(g["dt"]), n, u0[:, s],
                                   rec_idx=rec[0], rec_w=rec[1])
        assert rel_l2(u[:, s], uo) < 1e-4
        assert np.abs(tr[:, s, :] - to[:, :n]).max() < 1e-4 * np.abs(to).max()
    b.close(); op.close()


@pytest.mark.parametrize("case,S", [("cube3_q4", 64), ("cube2_q2", 16), ("cube2_q8", 8), ("cube2_q1", 24),
                                    ("cube2_q6", 32), ("cube4_q4", 40)])
def test_one_kernel_step_equals_two_kernel_step(case, S):
    """The default step (one cooperative kernel: element products, grid
    barrier, gather + update + sources) against the two-kernel step on the same
    integrator set-up: same FP32 arithmetic per (dof, source), relative L2
    <= 1e-6 (measured: bitwise equal), including odd step counts and the graph."""
    g = load_golden(case)
    op1, b1 = _batch(g, S)
    op2, b2 = _batch(g, S)
    info = b1.step_info()
    assert info["one_kernel"] and info["threads"] > 0 and info["grid"] > 0 and len(info["candidate_ms"]) >= 1
    b2.set_fused(False)
    assert not b2.step_info()["one_kernel"]
    b1.init(); b2.init()
    for k, gr in ((3, False), (45, True), (20, True), (7, False)):
        b1.advance(k, graph=gr)
        b2.advance(k, graph=gr)
    u1, v1 = b1.state()
    u2, v2 = b2.state()
    assert rel_l2(u1, u2) < 1e-6 and rel_l2(v1, v2) < 1e-6
    assert b1.info()["step"] == b2.info()["step"] == 75
    b1.close(); b2.close(); op1.close(); op2.close()


# every one-kernel step variant of order 4 (n = 5): (elements per tile, lanes
# per z-line, sources per thread)
Q4_STEP_VARIANTS = [(1, 4, 4), (1, 8, 4), (2, 4, 4), (1, 8, 2), (2, 2, 4)]


@pytest.mark.parametrize("variant", Q4_STEP_VARIANTS)
def test_every_q4_step_variant_equals_two_kernel_step(variant):
    """Each one-kernel step variant of order 4, forced, against the two-kernel
    step: bitwise the same states (the element products' operation order does
    not depend on how threads and lanes are laid out)."""
    g = load_golden("cube4_q4")
    S = 32
    op1, b1 = _batch(g, S)
    op2, b2 = _batch(g, S)
    b1.set_step_variant(*variant)
    b2.set_fused(False)
    b1.init(); b2.init()
    for k, gr in ((3, False), (40, True), (5, False)):
        b1.advance(k, graph=gr)
        b2.advance(k, graph=gr)
    u1, v1 = b1.state()
    u2, v2 = b2.state()
    assert np.array_equal(u1, u2) and np.array_equal(v1, v2)
    b1.close(); b2.close(); op1.close(); op2.close()


def test_one_kernel_step_traces_match_two_kernel_step():
    from montjoie_gb300.problem import receiver_weights
    g = load_golden("cube3_q4")
    S = 16
    rng = np.random.default_rng(5)
    rec = receiver_weights(int(g["order"]), g["verts_e"], g["nodle"], rng.uniform(0.1, 0.9, size=(4, 3)))
    op1, b1 = _batch(g, S, receivers=rec)
    op2, b2 = _batch(g, S, receivers=rec)
    b2.set_fused(False)
    u0 = rng.uniform(-1, 1, (g["massD"].size, S))
    b1.init(u0); b2.init(u0)
    t1 = b1.advance(30, traces=True)
    t2 = b2.advance(30, traces=True)
    assert np.abs(t1 - t2).max() <= 1e-6 * np.abs(t2).max()
    b1.close(); b2.close(); op1.close(); op2.close()
