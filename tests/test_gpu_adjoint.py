"""GPU discrete adjoint (the 32^3 Q4 inverse problem's pattern on small meshes).

- FP32 forward traces against the FP64 oracle (1e-4).
- The FP32 adjoint gradient against the FP64 CPU adjoint of the oracle and,
  on 20 random elements, against central differences of the oracle's FP64
  forward misfit: relative L2 <= 1e-4, the spec bar (measured
  ~1.5e-5).  The torch.autograd.Function wrapper gives the same gradient.
- On an 8^3 Q4 mesh (8 sources x 16 receivers, 60 steps): the gradient
  against central differences of the GPU's FP64 plain-form misfit on the 20
  elements with the largest gradient, <= 1e-4.
- Checkpointing does not change the result: uniform intervals and binomial
  (revolve) schedules of any budget give the same gradient bit for bit.
"""
import numpy as np
import pytest

from adjoint_case import build_case, oracle_adjoint
from conftest import rel_l2

pytestmark = pytest.mark.gpu


GRAD_TOL = 1e-4


def make_model(case, checkpoint_every=0, snapshots=None):
    from montjoie_gb300.adjoint import AcousticAdjoint
    g = case["g"]
    return AcousticAdjoint(case["r"], g["nodle"], case["bh_unit"], g["massD"].size, g["massD"], case["dt"], case["N"],
                           case["S"], case["src_idx"], case["src_rhs"], case["src_val"], case["pulse"],
                           case["rec_idx"], case["rec_w"], checkpoint_every=checkpoint_every, snapshots=snapshots)


@pytest.fixture(scope="module")
def case():
    return build_case(S=8, nsteps=80)


def test_forward_traces_match_oracle(case):
    model = make_model(case)
    tr = model.forward(case["c_true"])
    assert rel_l2(tr, case["data"]) < 1e-4
    model.close()


def test_adjoint_gradient_matches_fp64_adjoint(case):
    J_ref, _, g_ref = oracle_adjoint(case, case["c0"], case["data"])
    model = make_model(case)
    J, g = model.loss_and_grad(case["c0"], case["data"])
    assert abs(J - J_ref) < 1e-4 * J_ref
    assert rel_l2(g, g_ref) < GRAD_TOL
    model.close()


def test_adjoint_gradient_matches_central_differences(case):
    from montjoie_gb300.adjoint import central_differences
    model = make_model(case)
    _, g = model.loss_and_grad(case["c0"], case["data"])
    model.close()
    els = np.random.default_rng(7).choice(case["c0"].size, size=20, replace=False)
    fd = central_differences(lambda c: oracle_adjoint(case, c, case["data"], want_grad=False)[0], case["c0"], els)
    assert rel_l2(g[els], fd) < GRAD_TOL


def test_adjoint_gradient_matches_fp64_gpu_differences_8cube():
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.adjoint import AcousticAdjoint, Fp64Misfit, central_differences
    from montjoie_gb300.problem import AcousticProblem, cfl_time_step, gaussian_source, receiver_weights
    cells, r, S, nrec, N = 8, 4, 8, 16, 60
    rng = np.random.default_rng(11)
    m = M.perturbed_cube(cells, seed=11, amplitude=0.05, kind="random", c_mode="constant", c_range=(1.0, 1.0))
    pb = AcousticProblem(m, M.AcousticSetup(order=r, dt=1.0, nsteps=N + 2, src_radius=2.0 / cells), defer_time=True)
    c0 = rng.uniform(1.5, 2.5, pb.nodle.shape[0])
    c_true = c0 * (1.0 + 0.1 * rng.uniform(-1, 1, c0.size))
    pb.set_time_step(cfl_time_step(pb, safety=0.5) / c_true.max(), N + 2)
    idx, rhs, val = [], [], []
    for s_, c in enumerate(rng.uniform(0.2, 0.8, size=(S, 3))):
        i_, v_ = gaussian_source(pb.nodle, pb.jw, pb.xq, pb.n_dof, c, 2.0 / cells)
        idx.append(i_); val.append(v_); rhs.append(np.full(i_.size, s_))
    rec_idx, rec_w = receiver_weights(r, pb.verts_e, pb.nodle, rng.uniform(0.1, 0.9, size=(nrec, 3)))
    args = (r, pb.nodle, pb.factors, pb.n_dof, pb.mass, pb.setup.dt, N, S, np.concatenate(idx),
            np.concatenate(rhs), np.concatenate(val), pb.pulse, rec_idx, rec_w)
    model = AcousticAdjoint(*args)
    data = model.forward(c_true)
    _, g = model.loss_and_grad(c0, data)
    model.close()
    J64 = Fp64Misfit(*args)
    els = np.argsort(-np.abs(g))[:20]
    fd = central_differences(lambda c: J64(c, data), c0, els)
    J64.close()
    assert rel_l2(g[els], fd) < GRAD_TOL


def test_checkpoint_interval_does_not_change_gradient(case):
    """sqrt(N), 3, and N or more (every forward state kept, nothing
    recomputed): bitwise the same gradient."""
    grads = []
    N = case["N"]
    for K in (0, 3, N, 10 * N):
        model = make_model(case, checkpoint_every=K)
        if K >= N:
            sch = model.schedule()
            assert sch["snapshots"] == N and sch["forward_steps"] == N
        grads.append(model.loss_and_grad(case["c0"], case["data"])[1])
        model.close()
    for g in grads[1:]:
        assert np.array_equal(grads[0], g)


def test_revolve_schedules_give_the_same_gradient(case):
    """Binomial checkpointing with 1, 3 and 12 stored states against the
    uniform sqrt(N) schedule: bitwise the same gradient; fewer snapshots,
    more recomputed steps."""
    model = make_model(case)
    ref = model.loss_and_grad(case["c0"], case["data"])[1]
    model.close()
    steps = []
    for snaps in (1, 3, 12):
        model = make_model(case, snapshots=snaps)
        sch = model.schedule()
        assert sch["revolve"] and sch["snapshots"] == snaps
        steps.append(sch["forward_steps"])
        g = model.loss_and_grad(case["c0"], case["data"])[1]
        model.close()
        assert np.array_equal(g, ref), snaps
    assert steps[0] > steps[1] > steps[2] >= case["N"]


def test_three_runs_padded_to_eight():
    """3 sources: the runs are padded to 8 on the device (no source, zero
    state, no residual); the gradient matches the FP64 CPU adjoint."""
    case3 = build_case(S=3, nsteps=60)
    _, _, g_ref = oracle_adjoint(case3, case3["c0"], case3["data"])
    m = make_model(case3)
    J, g = m.loss_and_grad(case3["c0"], case3["data"])
    m.close()
    assert rel_l2(g, g_ref) < GRAD_TOL


def test_torch_autograd_function(case):
    torch = pytest.importorskip("torch")
    from montjoie_gb300.adjoint import misfit
    _, _, g_ref = oracle_adjoint(case, case["c0"], case["data"])
    model = make_model(case)
    c = torch.tensor(case["c0"], dtype=torch.float64, requires_grad=True)
    J = misfit(c, model, case["data"])
    J.backward()
    assert rel_l2(c.grad.numpy(), g_ref) < GRAD_TOL
    model.close()


def test_one_kernel_and_two_kernel_steps_give_the_same_gradient(case):
    """Forward, checkpoint replays and adjoint steps run on the one-kernel
    step by default, the adjoint steps with the gradient term inside; the
    two-kernel form (element kernel, gather, and the separate gradient
    kernel) gives the same traces and gradient bit for bit."""
    m1 = make_model(case, checkpoint_every=5)
    m2 = make_model(case, checkpoint_every=5)
    assert m1.batch.step_info()["one_kernel"]
    m2.batch.set_fused(False)
    J1, g1 = m1.loss_and_grad(case["c0"], case["data"])
    J2, g2 = m2.loss_and_grad(case["c0"], case["data"])
    assert J1 == J2
    assert np.array_equal(g1, g2)
    m1.close(); m2.close()


def test_every_step_variant_gives_the_same_gradient():
    """16 sources: every order-4 one-kernel step variant whose pass divides
    16, each with the gradient term inside its adjoint steps, gives the
    gradient of the two-kernel form bit for bit, under the uniform and the
    binomial schedules."""
    case16 = build_case(S=16, nsteps=40)
    ref = make_model(case16, checkpoint_every=7)
    ref.batch.set_fused(False)
    J0, g0 = ref.loss_and_grad(case16["c0"], case16["data"])
    ref.close()
    for E, LB, V in [(1, 4, 4), (2, 4, 4), (1, 8, 2), (2, 2, 4)]:
        for kw in (dict(checkpoint_every=7), dict(snapshots=3)):
            m = make_model(case16, **kw)
            m.batch.set_step_variant(E, LB, V)
            J, g = m.loss_and_grad(case16["c0"], case16["data"])
            m.close()
            assert J == J0, (E, LB, V, kw)
            assert np.array_equal(g, g0), (E, LB, V, kw)
