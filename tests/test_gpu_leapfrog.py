"""GPU parity of the leap-frog time loop (C ABI) against the reference.

FP64 plain form: relative L2 of the final iterate and of the norm history
<= 1e-10 against the reference's own run (golden fixtures; 30-200 steps).
The 16^3 Q4 parity case (200 steps) runs our whole
set-up (numbering, geometry, mass, source, pulse, receivers) and compares
the norm history, the 8 receiver traces and 512 probe values of u^200 with
the reference's, <= 1e-10 relative.  FP32 errors are stated per test.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def integrator(g, precision, norms=True):
    from montjoie_gb300.leapfrog import LeapFrogIterator
    from montjoie_gb300.operator import FemMatrixFreeOperator
    op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, precision,
                               gradphi=g["gradphi"])
    jwsum = np.zeros(g["massD"].size)
    np.add.at(jwsum, g["nodle"].ravel(), g["jw"].ravel())
    lf = LeapFrogIterator(op, float(g["dt"]), g["massD"], g["invD"], g["src_idx"], g["src_val"], g["pulse"],
                          jwsum if norms else None)
    return op, lf


def test_trajectory_fp64_matches_reference(golden_case):
    name, g = golden_case
    op, lf = integrator(g, "fp64")
    n = int(g["nsteps"])
    uf, norms, _ = lf.Run(np.zeros(g["massD"].size), None, n)
    assert rel_l2(uf, g["u_final"]) < FP64_TOL
    assert rel_l2(norms, g["norms"]) < FP64_TOL
    lf.close(); op.close()


def test_chunked_advance_equals_run(golden_case):
    name, g = golden_case
    op, lf = integrator(g, "fp64")
    n = int(g["nsteps"])
    lf.SetInitialConditionS(np.zeros(g["massD"].size))
    k = n // 3
    n1, _ = lf.Advance(k)
    n2, _ = lf.Advance(n - k)
    u = lf.GetIterate()
    assert rel_l2(u, g["u_final"]) < FP64_TOL
    assert rel_l2(np.concatenate([n1, n2]), g["norms"][:n]) < FP64_TOL
    snaps = dict(zip(g["snap_steps"].tolist(), g["snaps"]))
    if k in snaps:
        pass
    lf.close(); op.close()


def test_trajectory_fp32_error(golden_case):
    name, g = golden_case
    op, lf = integrator(g, "fp32")
    n = int(g["nsteps"])
    uf, norms, _ = lf.Run(np.zeros(g["massD"].size), None, n)
    assert rel_l2(uf, g["u_final"]) < 1e-4
    assert rel_l2(norms, g["norms"]) < 1e-4
    lf.close(); op.close()


def test_nonzero_initial_conditions_match_oracle():
    from oracle import oracle as oc
    g = load_golden("cube3_q4")
    rng = np.random.default_rng(3)
    u0 = rng.uniform(-1, 1, g["massD"].size)
    du0 = rng.uniform(-1, 1, g["massD"].size)
    op, lf = integrator(g, "fp64")
    uf, norms, _ = lf.Run(u0, du0, 50)
    uo, _, no, _ = oc.leapfrog(int(g["order"]), g["nodle"], g["bh"], g["massD"], g["invD"], g["src_idx"],
                               g["src_val"], g["pulse"], float(g["dt"]), 50, u0, du0=du0, jw=g["jw"])
    assert rel_l2(uf, uo) < 1e-12
    assert rel_l2(norms, no) < 1e-12


@pytest.fixture(scope="module")
def config1():
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem
    g = load_golden("config1_16q4")
    m = M.perturbed_cube(16, seed=int(g["seed"]), amplitude=0.05, kind="random", c_mode="element")
    s = M.AcousticSetup(order=4, dt=float(g["dt"]), nsteps=int(g["nsteps"]), src_radius=float(g["src_radius"]))
    pb = AcousticProblem(m, s, receivers=g["receivers"])
    return g, pb


def _probe_values(pb, g, u):
    pos = np.zeros((pb.n_dof, 3))
    pos[pb.nodle.ravel()] = pb.xq.reshape(-1, 3)
    key = lambda p: np.round(p * 1e9).astype(np.int64)  # noqa: E731
    table = {tuple(k): i for i, k in enumerate(key(pos))}
    idx = np.array([table[tuple(k)] for k in key(g["probe_pos"])])
    return u[idx]


def test_config1_fp64_end_to_end(config1):
    g, pb = config1
    assert rel_l2(pb.pulse, g["pulse"]) < 1e-12
    assert pb.src_idx.size == int(g["n_src"])
    op = pb.operator("fp64")
    lf = pb.integrator(op)
    n = int(g["nsteps"])
    uf, norms, traces = lf.Run(np.zeros(pb.n_dof), None, n)
    assert rel_l2(norms, g["norms"]) < FP64_TOL
    assert np.abs(traces - g["traces"]).max() < FP64_TOL * np.abs(g["traces"]).max()
    assert rel_l2(_probe_values(pb, g, uf), g["probe_u"]) < FP64_TOL
    assert abs(np.linalg.norm(uf) - float(g["u_final_norm2"])) < FP64_TOL * float(g["u_final_norm2"])


def test_config1_fp32_error(config1):
    g, pb = config1
    op = pb.operator("fp32")
    lf = pb.integrator(op)
    n = int(g["nsteps"])
    uf, norms, traces = lf.Run(np.zeros(pb.n_dof), None, n)
    # chosen form: FP32 state and contractions; error stated against the FP64 reference
    assert rel_l2(norms, g["norms"]) < 1e-4
    assert np.abs(traces - g["traces"]).max() < 1e-4 * np.abs(g["traces"]).max()
    assert rel_l2(_probe_values(pb, g, uf), g["probe_u"]) < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_diagnosed_graph_replay_equals_plain_launches(config1, precision):
    """Steps with the norm and the receivers every step: graph replays (from
    an odd step too) give the same norms, traces and states, bit for bit, as
    steps launched one by one (chunks too short for a graph)."""
    g, pb = config1
    runs = []
    for chunks in ((3, 45, 25), (7,) * 10 + (3,)):
        op = pb.operator(precision)
        lf = pb.integrator(op)
        lf.SetInitialConditionS(np.zeros(pb.n_dof))
        out = [lf.Advance(k) for k in chunks]
        runs.append((np.concatenate([o[0] for o in out]), np.concatenate([o[1] for o in out], axis=1),
                     lf.GetIterate()))
        lf.close(); op.close()
    (n1, t1, u1), (n2, t2, u2) = runs
    assert n1.shape == (73,) and t1.shape == (8, 73)
    assert np.array_equal(n1, n2) and np.array_equal(t1, t2) and np.array_equal(u1, u2)


@pytest.mark.parametrize("nsteps", [0, 1, 2, 21, 22])
def test_diagnosed_run_lengths_fp32_vs_fp64(config1, nsteps):
    """Short and odd runs through the fused FP32 diagnostics (iterates 0 and 1
    by their own launch, later ones by the steps): nsteps+1 columns, close to
    the FP64 plain form's; Advance(0) records nothing."""
    g, pb = config1
    out = {}
    for precision in ("fp64", "fp32"):
        op = pb.operator(precision)
        lf = pb.integrator(op)
        uf, norms, traces = lf.Run(np.zeros(pb.n_dof), None, nsteps)
        assert norms.shape == (nsteps + 1,) and traces.shape == (8, nsteps + 1)
        n0, t0 = lf.Advance(0)
        assert n0.shape == (0,) and t0.shape == (8, 0)
        out[precision] = (uf, norms, traces)
        lf.close(); op.close()
    (u64, n64, t64), (u32, n32, t32) = out["fp64"], out["fp32"]
    assert np.abs(n32 - n64).max() <= 1e-5 * max(np.abs(n64).max(), 1e-300)
    assert np.abs(t32 - t64).max() <= 1e-5 * max(np.abs(t64).max(), 1e-300)


def test_graph_replay_equals_plain_launches_single_source():
    g = load_golden("cube4_q4")
    for precision in ("fp64", "fp32"):
        op1, lf1 = integrator(g, precision, norms=False)
        op2, lf2 = integrator(g, precision, norms=False)
        lf2.set_graph(False)
        for lf in (lf1, lf2):
            lf.SetInitialConditionS(np.zeros(g["massD"].size))
            lf.Advance(1)       # odd start: realignment path
            lf.Advance(63)
        u1, v1 = lf1.GetState()
        u2, v2 = lf2.GetState()
        assert np.array_equal(u1, u2) and np.array_equal(v1, v2)
        for o in (lf1, lf2, op1, op2):
            o.close()


@pytest.mark.parametrize("case", ["cube3_q4", "cube2_q1", "cube2_q8", "cube4_q4"])
def test_fp32_streaming_gather_equals_two_kernels(case):
    """The FP32 default step (streaming gather + update + source in one
    kernel) against the gather kernel followed by the source kernel: the same
    arithmetic, so the states agree bit for bit (graph replays and odd counts)."""
    g = load_golden(case)
    op1, a = integrator(g, "fp32", norms=False)
    op2, b = integrator(g, "fp32", norms=False)
    b.set_stream_gather(False)
    a.SetInitialConditionS(np.zeros(g["massD"].size)); b.SetInitialConditionS(np.zeros(g["massD"].size))
    for k in (3, 41, 20, 5):
        a.Advance(k); b.Advance(k)
    ua, va = a.GetState()
    ub, vb = b.GetState()
    assert np.array_equal(ua, ub) and np.array_equal(va, vb)
    assert np.abs(ua).max() > 0
    a.close(); b.close(); op1.close(); op2.close()


def test_fp32_norm_with_weights_equal_to_the_mass():
    """The fused FP32 norm takes norm weights equal to the mass from the
    dt^2/D it stages (dt^2 / (dt^2/D)), other weights from their own FP32
    array: both agree with the FP64 plain form's norm to 1e-6, and with each
    other to the FP32 rounding of the weights."""
    from montjoie_gb300.leapfrog import LeapFrogIterator
    from montjoie_gb300.operator import FemMatrixFreeOperator
    g = load_golden("cube4_q4")
    n = g["massD"].size
    mass = g["massD"]
    other = mass.copy()
    other[n // 2] = np.nextafter(other[n // 2], np.inf)  # not equal to the mass: its own weight array
    norms = {}
    for name, precision, w in (("fp64", "fp64", mass), ("from_mass", "fp32", mass), ("own", "fp32", other)):
        op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], n, precision, gradphi=g["gradphi"])
        lf = LeapFrogIterator(op, float(g["dt"]), mass, g["invD"], g["src_idx"], g["src_val"], g["pulse"], w)
        _, norms[name], _ = lf.Run(np.zeros(n), None, 120)
        lf.close()
        op.close()
    ref = norms["fp64"]
    assert rel_l2(norms["from_mass"], ref) < 1e-6 and rel_l2(norms["own"], ref) < 1e-6
    assert rel_l2(norms["from_mass"], norms["own"]) < 1e-6
