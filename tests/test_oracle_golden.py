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
