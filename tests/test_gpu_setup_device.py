"""Set-up on the device against the host set-up.

mj_op_create_geometry computes the stiffness factors on the device in the
operator's layout, with the arithmetic of mj_geometry: its products equal those
of an operator built from mj_geometry's host factors bit for bit (FP64 and
FP32).  mj_op_lumped_mass and mj_op_gaussian_source assemble D and F on the
device in element order (the reference's assembly order): D is the host loop's
bit for bit (rho = 1) and F matches the host assembly to rounding (the device
exp may differ from the host's by an ulp); both match the reference's own
arrays (golden fixtures) to 1e-14.  mj_op_power_iteration gives the
eigenvalue of the host power iteration."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu


def _mesh(cells, order, kind="random"):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import number_mesh
    m = M.perturbed_cube(cells, seed=cells + order, amplitude=0.1 if kind == "sin" else 0.05, kind=kind,
                         c_mode="element")
    nodle, ndof = number_mesh(order, m.hexes, m.verts.shape[0])
    return m, nodle, ndof


@pytest.mark.parametrize("cells,order,kind", [(4, 2, "random"), (5, 4, "random"), (3, 8, "sin"), (3, 5, "random")])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_operator_from_geometry_equals_host_factors(cells, order, kind, precision):
    from montjoie_gb300.operator import FemMatrixFreeOperator
    from montjoie_gb300.problem import geometry
    m, nodle, ndof = _mesh(cells, order, kind)
    ve, mu = m.verts[m.hexes], m.elem_c ** 2
    fac, _, _ = geometry(order, ve, mu)
    a = FemMatrixFreeOperator(order, nodle, fac, ndof, precision)
    b = FemMatrixFreeOperator(order, nodle, None, ndof, precision, verts_e=ve, mu=mu)
    x = np.random.default_rng(order).uniform(-1, 1, ndof)
    ya, yb = np.zeros(ndof), np.zeros(ndof)
    a.MltVector(x, ya)
    b.MltVector(x, yb)
    assert np.array_equal(ya, yb)
    a.close(); b.close()


@pytest.mark.parametrize("cells,order", [(4, 2), (5, 4), (3, 8)])
def test_mass_and_source_on_device_equal_host(cells, order):
    from montjoie_gb300.operator import FemMatrixFreeOperator
    from montjoie_gb300.problem import gaussian_source, geometry, lumped_mass
    m, nodle, ndof = _mesh(cells, order)
    ve, mu = m.verts[m.hexes], m.elem_c ** 2
    _, jw, xq = geometry(order, ve, mu)
    op = FemMatrixFreeOperator(order, nodle, None, ndof, "fp32", verts_e=ve, mu=mu)
    assert np.array_equal(op.lumped_mass(), lumped_mass(order, nodle, jw, ndof))
    rho = np.random.default_rng(1).uniform(0.5, 2.0, nodle.shape[0])
    assert rel_l2(op.lumped_mass(rho), lumped_mass(order, nodle, jw, ndof, rho)) < 1e-15
    for c, R in (((0.5, 0.5, 0.5), 0.3), ((0.21, 0.7, 0.4), 0.25), ((0.0, 0.0, 0.0), 0.4)):
        i_d, v_d = op.gaussian_source(c, R)
        i_h, v_h = gaussian_source(nodle, jw, xq, ndof, c, R)
        assert np.array_equal(i_d, i_h)
        assert np.abs(v_d - v_h).max() <= 1e-14 * np.abs(v_h).max()
    op.close()


@pytest.mark.parametrize("case", ["cube3_q4", "cube2_q8", "cube2_q3"])
def test_device_assembly_matches_reference_arrays(case):
    """Against the reference's own mass and source, on its own numbering and geometry."""
    from montjoie_gb300.operator import FemMatrixFreeOperator
    g = load_golden(case)
    r = int(g["order"])
    mu = g["media_c"][g["elem_ref"] - 1] ** 2
    op = FemMatrixFreeOperator(r, g["nodle"], None, g["massD"].size, "fp64", verts_e=g["verts_e"], mu=mu)
    assert rel_l2(op.lumped_mass(), g["massD"]) < 1e-14
    idx, val = op.gaussian_source(g["src_center"], float(g["src_radius"]))
    F = np.zeros(g["massD"].size)
    F[idx] = val
    Fr = np.zeros(g["massD"].size)
    Fr[g["src_idx"]] = g["src_val"]
    assert rel_l2(F, Fr) < 1e-14
    op.close()


def test_power_iteration_on_device_equals_host_loop():
    from montjoie_gb300.operator import FemMatrixFreeOperator
    m, nodle, ndof = _mesh(6, 4)
    op = FemMatrixFreeOperator(4, nodle, None, ndof, "fp32", verts_e=m.verts[m.hexes], mu=m.elem_c ** 2)
    inv = 1.0 / op.lumped_mass()
    x0 = np.random.default_rng(0).uniform(-1, 1, ndof)
    lam_dev = op.power_iteration(inv, x0, 30)
    x, y, lam = x0.copy(), np.zeros(ndof), 0.0
    for _ in range(30):  # the host loop the device one replaces
        op.MltVector(x, y)
        y *= inv
        lam = np.linalg.norm(y) / np.linalg.norm(x)
        x = y / np.linalg.norm(y)
    assert abs(lam_dev - lam) < 1e-12 * lam
    op.close()
