"""The FP64 CPU adjoint of the oracle against central finite differences of
its own misfit (the reference has no adjoint to compare with)."""
import numpy as np

from adjoint_case import build_case, oracle_adjoint


def test_oracle_adjoint_matches_central_differences():
    case = build_case(S=2, nsteps=60)
    c0 = case["c0"]
    J, _, grad = oracle_adjoint(case, c0, case["data"])
    assert J > 0 and np.abs(grad).max() > 0
    rng = np.random.default_rng(2)
    for e in rng.choice(c0.size, size=5, replace=False):
        h = 1e-5 * c0[e]
        cp, cm = c0.copy(), c0.copy()
        cp[e] += h
        cm[e] -= h
        Jp, _, _ = oracle_adjoint(case, cp, case["data"], want_grad=False)
        Jm, _, _ = oracle_adjoint(case, cm, case["data"], want_grad=False)
        fd = (Jp - Jm) / (2 * h)
        assert abs(fd - grad[e]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(grad).max()), (e, fd, grad[e])
