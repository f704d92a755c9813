"""The oracle (C restatement) against the reference's own outputs (golden
fixtures made by tests/golden/make_golden.py from the compiled reference)."""
import numpy as np
import pytest

from conftest import SMALL_CASES, load_golden, rel_l2
from oracle import oracle as oc


@pytest.mark.parametrize("r", range(1, 9))
def test_gauss_lobatto_rule(r):
    pts, wts = oc.gauss_lobatto(r)
    assert abs(wts.sum() - 1.0) < 1e-14
    # exact for polynomials of degree 2r-1
    for d in range(2 * r):
        assert abs((wts * pts ** d).sum() - 1.0 / (d + 1)) < 1e-13
    num = oc.hex_numbering(r)
    assert sorted(num.tolist()) == list(range((r + 1) ** 3))


def test_rule_matches_reference(golden_case):
    name, g = golden_case
    r = int(g["order"])
    pts, wts = oc.gauss_lobatto(r)
    assert np.abs(pts - g["points1d"]).max() < 1e-15
    assert np.abs(oc.grad_matrix(r) - g["gradphi"]).max() < 1e-12 * max(1.0, np.abs(g["gradphi"]).max())
    assert (oc.hex_numbering(r) == g["numdofs3d"]).all()


def test_geometry_and_mass(golden_case):
    name, g = golden_case
    r = int(g["order"])
    mu = g["media_c"][g["elem_ref"] - 1] ** 2
    bh, jw, xq = oc.geometry(r, g["verts_e"], mu)
    assert rel_l2(bh, g["bh"]) < 1e-14
    assert rel_l2(jw, g["jw"]) < 1e-14
    D = oc.lumped_mass(g["nodle"], g["jw"], g["massD"].size)
    assert rel_l2(D, g["massD"]) < 1e-15
    assert rel_l2(1.0 / g["massD"], g["invD"]) < 1e-15
    F = oc.gaussian_source(g["nodle"], g["jw"], xq, g["massD"].size, g["src_center"], float(g["src_radius"]))
    Fr = np.zeros_like(F)
    Fr[g["src_idx"]] = g["src_val"]
    assert set(np.nonzero(F)[0]) == set(g["src_idx"].tolist())
    assert rel_l2(F, Fr) < 1e-14


def test_pulse(golden_case):
    name, g = golden_case
    p = oc.ricker_pulse(float(g["f0"]), float(g["t0"]), float(g["dt"]), int(g["nsteps"]), float(g["eps_time"]),
                        float(g["tlimit"]))
    assert rel_l2(p, g["pulse"]) < 1e-12


def test_operator_mltadd(golden_case):
    name, g = golden_case
    r = int(g["order"])
    y = g["y0"].copy()
    oc.stiffness_mltadd(r, g["nodle"], g["bh"], float(g["alpha"]), g["x"], float(g["beta"]), y)
    assert rel_l2(y, g["kh_y"]) < 1e-13
    y = np.zeros_like(g["x"])
    oc.stiffness_mltadd(r, g["nodle"], g["bh"], 1.0, g["x"], 0.0, y)
    assert rel_l2(y, g["kh_ax"]) < 1e-13


def test_trajectory(golden_case):
    name, g = golden_case
    r = int(g["order"])
    n = int(g["nsteps"])
    u0 = np.zeros(g["massD"].size)
    uN, _, norms, _ = oc.leapfrog(r, g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"], g["src_val"],
                                  g["pulse"], float(g["dt"]), n, u0, jw=g["jw"])
    assert norms.size == g["norms"].size == n + 1
    assert rel_l2(norms, g["norms"]) < 1e-11
    assert rel_l2(uN, g["u_final"]) < 1e-11


def test_config1_pulse_and_norm_history():
    g = load_golden("config1_16q4")
    p = oc.ricker_pulse(float(g["f0"]), float(g["t0"]), float(g["dt"]), int(g["nsteps"]), float(g["eps_time"]),
                        float(g["tlimit"]))
    assert rel_l2(p, g["pulse"]) < 1e-12
    assert g["norms"].size == int(g["nsteps"]) + 1
    assert np.all(np.isfinite(g["norms"])) and g["norms"][-1] > 0


# ---- order-4 modified-equation leap-frog (ModifiedEquation.cxx:125-175, 346-408)

def test_order4_pulse_derivatives(golden_case4):
    """p and p'' (derivative orders 1 and 3 of the interpolated primitive)
    against the reference's own TimeSourceHyperbolic: <= 1e-12 / 1e-9 relative
    (p'' amplifies rounding of the 25-point interpolant)."""
    from montjoie_gb300.problem import ricker_pulse
    name, g = golden_case4
    n = int(g["nsteps"])
    eps = (float(g["tf"]) - float(g["t0"])) * 1e-15
    for fn in (oc.ricker_pulse, ricker_pulse):
        p1 = fn(float(g["f0"]), float(g["t0"]), float(g["dt"]), n, eps, float(g["tlimit"]))
        p3 = fn(float(g["f0"]), float(g["t0"]), float(g["dt"]), n, eps, float(g["tlimit"]), nb_deriv=3)
        assert np.abs(p1 - g["pulse"]).max() <= 1e-12 * np.abs(g["pulse"]).max()
        assert np.abs(p3 - g["pulse3"]).max() <= 1e-9 * np.abs(g["pulse3"]).max()


def test_order4_trajectory(golden_case4):
    """The C restatement of the order-4 scheme against the reference's run:
    final iterate, snapshots and norm history <= 1e-11 relative."""
    name, g = golden_case4
    n = int(g["nsteps"])
    args = (int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"],
            g["pulse3"], float(g["dt"]))
    uf, _, norms, _ = oc.leapfrog4(*args, n, np.zeros(g["massD"].size), jw=g["jw"])
    assert rel_l2(uf, g["u_final"]) < 1e-11
    assert rel_l2(norms, g["norms"]) < 1e-11
    for k, snap in zip(g["snap_steps"].tolist(), g["snaps"]):
        if k:
            uk, _, _, _ = oc.leapfrog4(*args, k, np.zeros(g["massD"].size))
            assert rel_l2(uk, snap) < 1e-11


def test_order4_differs_from_order2():
    """The order-4 and order-2 schemes give different iterates on the same
    inputs (the d^4u/dt^4 correction is active)."""
    g = load_golden("cube3_q4_o4")
    n = 40
    args = (int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"])
    u4, _, _, _ = oc.leapfrog4(*args, g["pulse3"], float(g["dt"]), n, np.zeros(g["massD"].size))
    u2, _, _, _ = oc.leapfrog(*args, float(g["dt"]), n, np.zeros(g["massD"].size))
    assert rel_l2(u2, u4) > 1e-6
