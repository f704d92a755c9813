"""The operator and the time loop at the benchmark's full sizes, through
properties that hold at any size (the oracle's element loop is too slow to
run there as a whole):

- 64^3 Q4 (16,974,593 dofs; c on 8^3 random blocks) and 32^3 Q8 (16,974,593
  dofs; smooth sinusoidal displacement and c): the FP64 product is
  deterministic, linear and symmetric (x.A y = y.A x), annihilates constants
  (Neumann: A 1 = 0), and its rows agree with the oracle's element loop on a
  sample of dofs; the FP32 product stays within 1e-5 relative L2 of FP64.
- 64^3 Q4 leap-frog without source: the discrete energy of the order-2
  scheme, (u^{n+1}-u^n).D(u^{n+1}-u^n)/dt^2 + u^{n+1}.A u^n, is conserved
  from step to step (FP64, relative 1e-9 over 50 steps).
- The benchmark's own workload (64^3 Q4, c on 8^3 random blocks, Ricker
  source, dt = 0.5 CFL, 8 receivers) run 200 steps by the FP64 plain form
  against the FP64 oracle (the C restatement of the reference loop, run on
  the host cores on the same arrays): final state within 1e-10 relative L2
  (the reference trajectory bar), norm history and traces within 1e-10; the
  FP32 chosen form within 1e-5 (its traces relative to the field amplitude).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _problem(cells, order, kind, c_mode):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem
    amp = 0.05 if kind == "random" else 0.1
    m = M.perturbed_cube(cells, seed=7, amplitude=amp, kind=kind, c_mode=c_mode, c_blocks=8)
    s = M.AcousticSetup(order=order, dt=1e-4, nsteps=60, src_radius=2.0 / cells)
    return AcousticProblem(m, s)


@pytest.mark.parametrize("cells,order,kind,c_mode", [(64, 4, "random", "blocks"), (32, 8, "sin", "smooth")])
def test_operator_properties_full_size(cells, order, kind, c_mode):
    pb = _problem(cells, order, kind, c_mode)
    n = pb.n_dof
    assert n == (cells * order + 1) ** 3
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    op = pb.operator("fp64")
    ax, ay, t = np.zeros(n), np.zeros(n), np.zeros(n)
    op.MltVector(x, ax)
    op.MltVector(x, t)
    assert np.array_equal(ax, t)  # owner-computes gather: bitwise repeatable
    op.MltVector(y, ay)
    op.MltVector(2.0 * x - 0.5 * y, t)
    assert rel_l2(t, 2.0 * ax - 0.5 * ay) < 1e-13
    assert abs(y @ ax - x @ ay) < 1e-11 * abs(x @ ay)
    op.MltVector(np.ones(n), t)
    assert np.abs(t).max() < 1e-10 * np.abs(ax).max()
    # rows of a sample of dofs against the oracle's element loop on the
    # elements that touch them
    from oracle import oracle as oc
    nod = pb.nodle
    sample = rng.choice(n, 64, replace=False)
    touch = np.unique(np.nonzero(np.isin(nod, sample))[0])
    sub = nod[touch]
    yo = oc.stiffness_mltadd(order, sub, pb.factors[touch], 1.0, x, 0.0, np.zeros(n))
    assert rel_l2(ax[sample], yo[sample]) < 1e-12
    op32 = pb.operator("fp32")
    t32 = np.zeros(n)
    op32.MltVector(x, t32)
    assert rel_l2(t32, ax) < 1e-5
    op32.close()
    op.close()


def test_leapfrog_energy_conserved_full_size():
    from montjoie_gb300.leapfrog import LeapFrogIterator
    pb = _problem(64, 4, "random", "blocks")
    n = pb.n_dof
    op = pb.operator("fp64")
    dt = 0.5 * 2.0 / np.sqrt(_lambda_max(op, pb.mass))
    lf = LeapFrogIterator(op, dt, pb.mass)  # no source
    rng = np.random.default_rng(5)
    # a smooth start: a Gaussian bump, zero velocity
    xq = np.zeros((n, 3))
    xq[pb.nodle.ravel()] = pb.xq.reshape(-1, 3)
    u0 = np.exp(-40.0 * ((xq - 0.5) ** 2).sum(axis=1)) * (1.0 + 1e-3 * rng.uniform(-1, 1, n))
    lf.SetInitialConditionS(u0)
    energies = []
    au = np.zeros(n)
    for _ in range(5):
        lf.Advance(10)
        un, un1 = lf.GetState()
        op.MltVector(un, au)
        dv = un1 - un
        energies.append(dv @ (pb.mass * dv) / dt ** 2 + un1 @ au)
    e = np.array(energies)
    assert e[0] > 0
    assert np.abs(e - e[0]).max() < 1e-9 * e[0]
    lf.close()
    op.close()


def _lambda_max(op, mass, iters=30):
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, mass.size)
    y = np.zeros_like(x)
    lam = 0.0
    for _ in range(iters):
        op.MltVector(x, y)
        y /= mass
        lam = np.linalg.norm(y) / np.linalg.norm(x)
        x = y / np.linalg.norm(y)
    return lam * 1.05


def test_leapfrog_matches_oracle_on_benchmark_workload():
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem, cfl_time_step
    from oracle import oracle as oc
    cells, order, steps = 64, 4, 200
    m = M.perturbed_cube(cells, seed=20251203, amplitude=0.05, kind="random", c_mode="blocks", c_blocks=8)
    s = M.AcousticSetup(order=order, dt=1.0, nsteps=steps, src_radius=2.0 / cells)
    rec = np.random.default_rng(20251206).uniform(0.1, 0.9, size=(8, 3))
    pb = AcousticProblem(m, s, receivers=rec, defer_time=True)
    pb.set_time_step(cfl_time_step(pb, safety=0.5), steps)
    zeros = np.zeros(pb.n_dof)
    o = oc.trajectory(order, pb.nodle, pb.factors, pb.mass, 1.0 / pb.mass, pb.src_idx, pb.src_val, pb.pulse,
                      pb.setup.dt, steps, zeros, jw=pb.jw, rec_idx=pb.rec_idx, rec_w=pb.rec_w,
                      colors=oc.structured_colors(cells))
    uo, no, to = o["u"], o["norms"], o["traces"]
    assert np.linalg.norm(uo) > 0
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-5)):
        op = pb.operator(precision)
        lf = pb.integrator(op)
        u, norms, traces = lf.Run(zeros, None, steps)
        assert rel_l2(u, uo) < tol, precision
        assert rel_l2(norms, no) < tol, precision
        # FP64: relative to the traces themselves; FP32: relative to the field's
        # amplitude (after 200 steps the wave has not reached every receiver,
        # whose values then sit far below FP32's range)
        scale = np.abs(to).max() if precision == "fp64" else np.abs(uo).max()
        assert np.abs(traces - to).max() < tol * scale, precision
        lf.close()
        op.close()
