"""GPU discrete adjoint (the 32^3 Q4 inverse problem's pattern on a small mesh):
FP32 forward traces and the adjoint gradient against the FP64 CPU adjoint of
the oracle, the torch.autograd.Function wrapper, and checkpointing that does
not change the result."""
import numpy as np
import pytest

from adjoint_case import build_case, oracle_adjoint
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def make_model(case, checkpoint_every=0):
    from montjoie_gb300.adjoint import AcousticAdjoint
    g = case["g"]
    return AcousticAdjoint(case["r"], g["nodle"], case["bh_unit"], g["massD"].size, g["massD"], case["dt"], case["N"],
                           case["S"], case["src_idx"], case["src_rhs"], case["src_val"], case["pulse"],
                           case["rec_idx"], case["rec_w"], checkpoint_every=checkpoint_every)


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
    assert abs(J - J_ref) < 1e-3 * J_ref
    assert rel_l2(g, g_ref) < 1e-3
    model.close()


def test_checkpoint_interval_does_not_change_gradient(case):
    grads = []
    for K in (0, 3, 80):
        model = make_model(case, checkpoint_every=K)
        grads.append(model.loss_and_grad(case["c0"], case["data"])[1])
        model.close()
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


def test_torch_autograd_function(case):
    torch = pytest.importorskip("torch")
    from montjoie_gb300.adjoint import misfit
    _, _, g_ref = oracle_adjoint(case, case["c0"], case["data"])
    model = make_model(case)
    c = torch.tensor(case["c0"], dtype=torch.float64, requires_grad=True)
    J = misfit(c, model, case["data"])
    J.backward()
    assert rel_l2(c.grad.numpy(), g_ref) < 1e-3
    model.close()


def test_one_kernel_and_two_kernel_steps_give_the_same_gradient(case):
    """Forward, checkpoint replays and adjoint steps run on the one-kernel
    step by default; the two-kernel form gives the same traces and gradient
    (same FP32 arithmetic: bitwise, asserted at 1e-12)."""
    m1 = make_model(case, checkpoint_every=5)
    m2 = make_model(case, checkpoint_every=5)
    assert m1.batch.step_info()["one_kernel"]
    m2.batch.set_fused(False)
    J1, g1 = m1.loss_and_grad(case["c0"], case["data"])
    J2, g2 = m2.loss_and_grad(case["c0"], case["data"])
    assert abs(J1 - J2) <= 1e-12 * abs(J2)
    assert rel_l2(g1, g2) <= 1e-12
    m1.close(); m2.close()
