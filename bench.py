#!/usr/bin/env python
"""Benchmark: DOF-updates/s of the Q4 hexahedral acoustic leap-frog on one GB300.

Workload: unit cube, 64^3 hexahedra, vertices
perturbed uniformly by +-5% h (seeded), Q4 Gauss-Lobatto, c piecewise
constant on 8^3 random blocks in [1,3], Ricker f0 = 5 at the centre (Gaussian
R = 2h), Neumann, dt = 0.5 CFL.  One bench step = one leap-frog time step over
all 16,974,593 dofs.  ``value`` is the FP32 chosen form with everything
resident in HBM; the FP64 plain form is timed beside it; ``e2e`` is the whole
run through the C ABI (``mj_lf_run``) with host buffers.  The CPU baseline is
the oracle's C restatement on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--cells 64] [--order 4]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-updates/s (Q4/Q8 hex acoustic leap-frog), FP32 vs FP64 at stated L2 error"
ORACLE_REF = "FP64 oracle (port): the C restatement of the reference loop, run on the host cores on the same arrays"
UNIT = "DOF-updates/s"
SEED = 20251203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--order", type=int, default=4)
    ap.add_argument("--fp64-steps", type=int, default=200)
    ap.add_argument("--error-steps", type=int, default=1000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-oracle", action="store_true",
                    help="skip the full-size comparisons with the FP64 oracle (about 1.5 min of host time)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other workloads (Q8, sources, meshes, adjoint, order-4 scheme)")
    ap.add_argument("--extra-steps", type=int, default=500)
    ap.add_argument("--adjoint-steps", type=int, default=1000)
    ap.add_argument("--mb-orders", default="2,3,4,6,8",
                    help="orders cycled over the heterogeneous batch (default 2,3,4,6,8)")
    ap.add_argument("--mb-max-cells", type=int, default=40,
                    help="largest mesh of the heterogeneous batch (default 40; smaller for profiling)")
    ap.add_argument("--fp32-only", action="store_true",
                    help="profiling aid: only the FP32 set-up and timed steps of the workload (no JSON line contract)")
    ap.add_argument("--k1-variant", default=None,
                    help="profiling aid with --fp32-only: force the element-kernel variant E,layout (the one the "
                         "autotuner picks unprofiled), since under a profiler its timings are distorted")
    ap.add_argument("--e2e-only", action="store_true",
                    help="profiling aid: only the FP32 set-up and the end-to-end run (diagnostics every step, "
                         "--error-steps steps; no JSON line contract)")
    ap.add_argument("--leg", default="all", choices=["all", "q8", "sources", "meshes", "adjoint", "order4"],
                    help="profiling aid: run one extra leg alone (no JSON line contract)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x, dist, device):
    """Largest x over the ranks of the default process group (the slowest
    replica's time)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, ms_max):
    """Units all replicas processed per second, timed by the slowest one."""
    return units_per_rank * world / (ms_max / 1e3)


def workload_mesh(cells):
    from montjoie_gb300 import mesh as M
    return M.perturbed_cube(cells, seed=SEED, amplitude=0.05, kind="random", c_mode="blocks", c_blocks=8)


def workload_name(cells, order):
    return (f"unit cube {cells}^3 hex Q{order}, +-5% h random vertex perturbation, c on 8^3 random blocks in [1,3], "
            f"Ricker f0=5 Gaussian R=2h at centre, Neumann, leap-frog dt=0.5 CFL")


def workload_config(cells, order, n_dof):
    """The `config` record, the same in both arms."""
    return {"workload": workload_name(cells, order), "cells": cells, "order": order, "n_dof": n_dof,
            "l2_flush": "none: inputs larger than L2 (the factors alone are %.2f GB or more per step)"
                        % (cells ** 3 * (order + 1) ** 3 * 24 / 1e9)}


def receivers():
    return np.random.default_rng(SEED + 3).uniform(0.1, 0.9, size=(8, 3))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_element(name):
    """DRAM bytes per element of the element kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("dram_bytes_per_element"):
            return float(line.split("=")[1].split()[0])
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def build_problem(cells, order, nsteps, mesh=None, time_order=2):
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.problem import AcousticProblem, cfl_time_step
    m = workload_mesh(cells) if mesh is None else mesh
    s = M.AcousticSetup(order=order, dt=1.0, nsteps=nsteps, src_radius=2.0 / cells, time_order=time_order)
    pb = AcousticProblem(m, s, receivers=receivers(), defer_time=True)
    dt = cfl_time_step(pb, safety=0.5)
    pb.set_time_step(dt, nsteps)
    return pb


def oracle_run(pb, nsteps, snap_every=None, diag=False, src=None):
    """The FP64 oracle (the C restatement of the reference loop, colour-
    parallel on the host cores) on the problem's own arrays, from rest:
    returns {"snaps": {step: u}, "u": U^nsteps} and, with diag, the norms and
    receiver traces of iterates 0..nsteps.  src: (idx, val) instead of the
    problem's source."""
    from oracle import oracle as oc
    idx, val = (pb.src_idx, pb.src_val) if src is None else src
    rec = (pb.rec_idx, pb.rec_w) if (diag and pb.rec_idx is not None) else (None, None)
    return oc.trajectory(pb.order, pb.nodle, pb.factors, pb.mass, 1.0 / pb.mass, idx, val, pb.pulse, pb.setup.dt,
                         nsteps, np.zeros(pb.n_dof), jw=pb.jw if diag else None, rec_idx=rec[0], rec_w=rec[1],
                         colors=oc.structured_colors(pb.mesh.n), snap_every=snap_every)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def timed_steps(torch, step_fn, steps):
    """Device time (ms) of step_fn(steps) with CUDA events on the legacy default stream."""
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    step_fn(steps)
    end.record()
    torch.cuda.synchronize()
    return start.elapsed_time(end)


def leg_q8(args, torch, _lib):
    """32^3 hexahedra, smooth sinusoidal vertex
    displacement 0.1h, Q8, c = 2 + 0.5 sin sin sin, FP32 state (factors stored
    FP64, cast to FP32), error stated against the FP64 plain path."""
    from montjoie_gb300 import mesh as M
    cells, order, K = 32, 8, args.extra_steps
    m = M.perturbed_cube(cells, seed=SEED + 30, amplitude=0.1, kind="sin", c_mode="smooth")
    t0 = time.perf_counter()
    pb = build_problem(cells, order, K + 20, mesh=m)
    setup_s = time.perf_counter() - t0
    zeros = np.zeros(pb.n_dof)
    op32 = pb.operator("fp32")
    lf = pb.integrator(op32, diagnostics=False)
    lf.SetInitialConditionS(zeros)
    lf.Advance(5)
    ms32 = timed_steps(torch, lf.Advance, K)
    lf.close()
    op64 = pb.operator("fp64")
    lf = pb.integrator(op64, diagnostics=False)
    lf.SetInitialConditionS(zeros)
    lf.Advance(3)
    K64 = min(K, 100)
    ms64 = timed_steps(torch, lf.Advance, K64)
    lf.close()
    d64 = pb.integrator(op64)
    u64, n64, _ = d64.Run(zeros, None, K)
    d32 = pb.integrator(op32)
    u32, n32, _ = d32.Run(zeros, None, K)
    d64.close(); d32.close(); op32.close(); op64.close()
    err = {"steps": K, "reference": ORACLE_REF}
    if not args.no_oracle:
        t0 = time.perf_counter()
        o = oracle_run(pb, K, diag=True)
        err.update({"fp32_u_rel_l2": rel(u32, o["u"]), "fp64_u_rel_l2": rel(u64, o["u"]),
                    "fp32_norm_history_rel_l2": rel(n32, o["norms"]), "fp64_norm_history_rel_l2": rel(n64, o["norms"]),
                    "oracle_seconds": time.perf_counter() - t0})
    return {"workload": f"unit cube 32^3 hex Q8, 0.1h sinusoidal vertex displacement, c = 2 + 0.5 sin(2 pi x) sin(2 pi y) "
                        f"sin(2 pi z) per element, Ricker f0=5, Neumann, dt=0.5 CFL, FP32 state, {K} steps",
            "n_dof": pb.n_dof, "steps": K, "value": pb.n_dof * K / (ms32 / 1e3), "unit": UNIT,
            "ms_per_step": ms32 / K, "fp64_value": pb.n_dof * K64 / (ms64 / 1e3), "fp64_ms_per_step": ms64 / K64,
            "error_vs_oracle": err, "u_rel_l2_fp32_vs_fp64": rel(u32, u64), "setup_seconds": setup_s}


def leg_sources(args, torch, _lib):
    """64 independent Ricker sources at
    seeded random positions on one 32^3 Q4 mesh (c per element in [1,3]),
    FP32, advanced together, CUDA-graph replay."""
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.leapfrog import BatchLeapFrog
    from montjoie_gb300.problem import gaussian_source
    cells, order, S, K = 32, 4, 64, args.extra_steps
    m = M.perturbed_cube(cells, seed=SEED + 40, amplitude=0.05, kind="random", c_mode="element")
    NE = max(K + 20, args.error_steps)
    pb = build_problem(cells, order, max(K, NE) + 40, mesh=m)
    pos = np.random.default_rng(SEED + 41).uniform(0.1, 0.9, size=(S, 3))
    op = pb.operator("fp32")
    idx, rhs, val = [], [], []
    for s_, c in enumerate(pos):  # each source assembled on the device
        i_, v_ = op.gaussian_source(c, 2.0 / cells)
        idx.append(i_); val.append(v_); rhs.append(np.full(i_.size, s_))
    b = BatchLeapFrog(op, pb.setup.dt, S, pb.mass, None, np.concatenate(idx), np.concatenate(rhs),
                      np.concatenate(val), pb.pulse)
    b.init()
    b.advance(20)
    l0 = _lib.kernel_launches()
    ms = timed_steps(torch, b.advance, K)
    launches = _lib.kernel_launches() - l0
    u, _ = b.state()
    info = b.info()
    info["one_kernel_step"] = b.step_info()
    b.profile(True)  # phase times of one extra step (per-CTA time stamps)
    b.advance(1)
    info["phase_ms_one_step"] = b.phase_ms()
    b.profile(False)
    # run 0 after NE steps, against the FP64 oracle and a single-source run
    b.init()
    b.advance(NE)
    u_ne, _ = b.state()
    # the same runs with two kernels per step (element kernel, then gather + update)
    b.set_fused(False)
    b.init()
    b.advance(20)
    ms_two = timed_steps(torch, b.advance, K)
    u_two, _ = b.state()
    b.close()
    lf = LeapFrogIteratorFor(pb, op, idx[0], val[0])
    lf.SetInitialConditionS(np.zeros(pb.n_dof))
    lf.Advance(K + 20)
    u0 = lf.GetIterate()
    lf.close(); op.close()
    err = {"steps": NE, "run": 0, "reference": ORACLE_REF}
    if not args.no_oracle:
        t0 = time.perf_counter()
        o = oracle_run(pb, NE, src=(idx[0], val[0]))
        err.update({"fp32_u_rel_l2": rel(u_ne[:, 0], o["u"]), "oracle_seconds": time.perf_counter() - t0})
    n_elt, Q = pb.nodle.shape
    # batched bytes per right-hand side and step: factors and Nodle shared by the
    # S runs, R written and read, the state rows; divided by the dofs
    bytes_step = (n_elt * Q * (6 * 4 + 4) / S + pb.n_dof * (3 * 4 + 4 / S)) / pb.n_dof
    value = pb.n_dof * S * K / (ms / 1e3)
    peak, _ = measured_peaks()
    return {"workload": f"64 Ricker sources (Gaussian R=2h, seeded positions in [0.1,0.9]^3) on one 32^3 Q4 mesh, "
                        f"+-5% h perturbation, c per element in [1,3], FP32, {K} steps, state [dof][64], "
                        f"one cooperative kernel per step",
            "n_dof": pb.n_dof, "n_rhs": S, "steps": K, "value": value, "unit": UNIT, "ms_per_step": ms / K,
            "variant": info, "gpu_launches": launches,
            "two_kernel_ms_per_step": ms_two / K,
            "one_vs_two_kernel_rel_l2": float(np.linalg.norm(u - u_two) / max(np.linalg.norm(u_two), 1e-300)),
            "run0_rel_l2_vs_single_source_run_after_%d_steps" % (K + 20): rel(u[:, 0], u0),
            "error_vs_oracle": err,
            "algorithmic_bytes_per_dof_update": bytes_step,
            "step_frac_of_hbm": value * bytes_step / 1e9 / peak}


def leg_meshes(args, torch, _lib):
    """24 meshes from 8^3 to 40^3
    hexahedra (+-5% h perturbation, c per element in [1,3]) with orders
    cycling 2,3,4,6,8, each with its own Ricker source at the centre and its
    own dt = 0.5 CFL, FP32, all advanced by one cooperative kernel per step
    under a CUDA graph.  The same runs advanced one after the other (each
    with its own graph-replayed step kernels) are timed beside it, and their
    final states must agree with the batch's."""
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.leapfrog import MeshBatch
    K = args.extra_steps
    orders = [int(o) for o in args.mb_orders.split(",")]
    t0 = time.perf_counter()
    runs = []
    for i in range(24):
        cells, r = 8 + round((args.mb_max_cells - 8) * i / 23), orders[i % len(orders)]
        m = M.perturbed_cube(cells, seed=SEED + 60 + i, amplitude=0.05, kind="random", c_mode="element")
        pb = build_problem(cells, r, K + 40, mesh=m)
        op = pb.operator("fp32")
        lf = pb.integrator(op, diagnostics=False)
        lf.SetInitialConditionS(np.zeros(pb.n_dof))
        runs.append((cells, r, pb, op, lf))
    setup_s = time.perf_counter() - t0
    mb = MeshBatch([x[4] for x in runs])
    mb.advance(20)
    l0 = _lib.kernel_launches()
    ms = timed_steps(torch, mb.advance, K)
    launches = _lib.kernel_launches() - l0
    info = mb.info()
    info["tuning"] = mb.tuning()
    info["grouping"] = mb.grouping()
    u_batch = [x[4].GetIterate() for x in runs]
    mb.profile(True)  # phase times of one extra step (per-CTA time stamps)
    mb.advance(1)
    phases = mb.phase_ms()
    mb.close()
    # the same runs one after the other
    for x in runs:
        x[4].SetInitialConditionS(np.zeros(x[2].n_dof))
        x[4].Advance(20)
    torch.cuda.synchronize()

    def sequential(k):
        for x in runs:
            x[4].Advance(k)
    ms_seq = timed_steps(torch, sequential, K)
    diff = 0.0
    for x, ub in zip(runs, u_batch):
        us = x[4].GetIterate()
        diff = max(diff, float(np.linalg.norm(ub - us) / max(np.linalg.norm(us), 1e-300)))
    n_dof = sum(x[2].n_dof for x in runs)
    step_bytes = sum(x[2].nodle.shape[0] * x[2].nodle.shape[1] * (6 * 4 + 4) + x[2].n_dof * (3 * 4 + 4)
                     for x in runs)
    for x in runs:
        x[4].close(); x[3].close()
    value = n_dof * K / (ms / 1e3)
    peak, _ = measured_peaks()
    return {"workload": f"24 meshes 8^3..{args.mb_max_cells}^3 hex, orders {args.mb_orders} cycling, +-5% h perturbation, c per element in "
                        f"[1,3], own Ricker source and dt each, FP32, {K} steps, one cooperative kernel per step",
            "meshes": [[x[0], x[1], x[2].n_dof] for x in runs], "n_dof": n_dof, "steps": K,
            "value": value, "unit": UNIT, "ms_per_step": ms / K, "gpu_launches": launches, "launch": info,
            "phase_ms_one_step": phases,
            "sequential_value": n_dof * K / (ms_seq / 1e3), "sequential_ms_per_step": ms_seq / K,
            "batch_over_sequential": ms_seq / ms,
            "max_rel_l2_batch_vs_sequential": diff,
            "algorithmic_bytes_per_step": step_bytes,
            "step_frac_of_hbm": step_bytes / (ms / K / 1e3) / 1e9 / peak,
            "setup_seconds": setup_s}


def leg_order4(args, torch, _lib):
    """The order-4 modified-equation leap-frog (two stiffness products per
    step, CFL constant 2 sqrt(3)) on the 64^3 Q4 mesh of the headline workload, at
    dt = 0.5 CFL of that scheme: FP32 and FP64 step rates, FP32 error against
    FP64, and simulated time per second against the order-2 leap-frog."""
    cells, order, K = args.cells, args.order, args.extra_steps
    pb = build_problem(cells, order, K + 40, time_order=4)
    zeros = np.zeros(pb.n_dof)
    op32 = pb.operator("fp32")
    lf = pb.integrator(op32, diagnostics=False)
    lf.SetInitialConditionS(zeros)
    lf.Advance(20)
    l0 = _lib.kernel_launches()
    ms32 = timed_steps(torch, lf.Advance, K)
    launches = _lib.kernel_launches() - l0
    lf.close()
    op64 = pb.operator("fp64")
    lf = pb.integrator(op64, diagnostics=False)
    lf.SetInitialConditionS(zeros)
    lf.Advance(3)
    K64 = min(K, 100)
    ms64 = timed_steps(torch, lf.Advance, K64)
    lf.close()
    KE = min(K, 200)
    d64 = pb.integrator(op64)
    u64, n64, _ = d64.Run(zeros, None, KE)
    d32 = pb.integrator(op32)
    u32, n32, _ = d32.Run(zeros, None, KE)
    d64.close(); d32.close(); op32.close(); op64.close()
    err = {"steps": KE, "reference": ORACLE_REF.replace("reference loop", "reference's order-4 loop")}
    if not args.no_oracle:
        from oracle import oracle as oc
        t0 = time.perf_counter()
        uo, _, _, _ = oc.leapfrog4(order, pb.nodle, pb.factors, pb.mass, 1.0 / pb.mass, pb.src_idx, pb.src_val,
                                   pb.pulse, pb.pulse_d2, pb.setup.dt, KE, zeros, colors=oc.structured_colors(cells))
        err.update({"fp32_u_rel_l2": rel(u32, uo), "fp64_u_rel_l2": rel(u64, uo),
                    "oracle_seconds": time.perf_counter() - t0})
    return {"workload": workload_name(cells, order).replace("leap-frog dt=0.5 CFL",
                                                           "order-4 modified-equation leap-frog dt=0.5 CFL(2 sqrt 3)")
            + f", FP32 state, {K} steps",
            "n_dof": pb.n_dof, "dt": pb.setup.dt, "steps": K, "value": pb.n_dof * K / (ms32 / 1e3), "unit": UNIT,
            "ms_per_step": ms32 / K, "gpu_launches": launches,
            "fp64_value": pb.n_dof * K64 / (ms64 / 1e3), "fp64_ms_per_step": ms64 / K64,
            "simulated_time_per_second_fp32": pb.setup.dt * K / (ms32 / 1e3),
            "error_vs_oracle": err, "u_rel_l2_fp32_vs_fp64": rel(u32, u64)}


def leg_adjoint(args, torch, _lib):
    """32^3 Q4, per-element c as parameter (start
    U[1.5,2.5]), 16 sources x 64 receivers, FP32 steps, L2 misfit against
    traces of a seeded perturbed true c; gradient by the discrete adjoint with
    every forward state kept (or sqrt(N) checkpoints when they do not fit);
    the sqrt(N) and binomial schedules are timed beside it and must give the
    same gradient bit for bit.  Timed at full size; the gradient is checked on a
    small case against central differences (20 elements) and the FP64 CPU adjoint."""
    from montjoie_gb300 import mesh as M
    from montjoie_gb300.adjoint import AcousticAdjoint
    from montjoie_gb300.problem import gaussian_source, geometry, receiver_weights
    cells, order, S, nrec, N = 32, 4, 16, 64, args.adjoint_steps
    rng = np.random.default_rng(SEED + 50)
    m = M.perturbed_cube(cells, seed=SEED + 50, amplitude=0.05, kind="random", c_mode="constant", c_range=(1.0, 1.0))
    pb = build_problem(cells, order, N + 2, mesh=m)   # unit mu (c = 1) factors
    c0 = rng.uniform(1.5, 2.5, pb.nodle.shape[0])
    c_true = c0 * (1.0 + 0.1 * rng.uniform(-1, 1, c0.size))
    # CFL of the fastest medium: scale the c = 1 step by 1/max c
    dt = pb.setup.dt / c_true.max()
    pb.set_time_step(dt, N + 2)
    idx, rhs, val = [], [], []
    for s_, c in enumerate(rng.uniform(0.1, 0.9, size=(S, 3))):
        i_, v_ = gaussian_source(pb.nodle, pb.jw, pb.xq, pb.n_dof, c, 2.0 / cells)
        idx.append(i_); val.append(v_); rhs.append(np.full(i_.size, s_))
    rec_idx, rec_w = receiver_weights(order, pb.verts_e, pb.nodle, rng.uniform(0.1, 0.9, size=(nrec, 3)))
    # every forward state kept when it fits in device memory (N x n_dof x S
    # floats: 137 GB here), else sqrt(N) checkpoints
    adj_args = (order, pb.nodle, pb.factors, pb.n_dof, pb.mass, dt, N, S, np.concatenate(idx), np.concatenate(rhs),
                np.concatenate(val), pb.pulse, rec_idx, rec_w)
    free_bytes = torch.cuda.mem_get_info()[0]
    keep_all = 4.0 * pb.n_dof * S * (N + 2) < 0.8 * free_bytes
    model = AcousticAdjoint(*adj_args, checkpoint_every=N if keep_all else 0)
    data = model.forward(c_true)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tr = model.forward(c0)
    t1 = time.perf_counter()
    res = tr - data
    grad = model.backward(res)
    t2 = time.perf_counter()
    J = 0.5 * float((res * res).sum())
    sched = dict(model.schedule(), kind="every state kept" if keep_all else "sqrt(N) checkpoints")
    model.close()
    uniform = None
    if keep_all:  # the sqrt(N) schedule beside it
        model_u = AcousticAdjoint(*adj_args)
        model_u.forward(c0)
        torch.cuda.synchronize()
        t5 = time.perf_counter()
        grad_u = model_u.backward(res)
        t6 = time.perf_counter()
        uniform = dict(model_u.schedule(), backward_seconds=t6 - t5,
                       grad_bitwise_equal=bool(np.array_equal(grad_u, grad)))
        model_u.close()
    # the same model with binomial checkpointing under a budget of 16 stored states
    model_rv = AcousticAdjoint(order, pb.nodle, pb.factors, pb.n_dof, pb.mass, dt, N, S, np.concatenate(idx),
                               np.concatenate(rhs), np.concatenate(val), pb.pulse, rec_idx, rec_w, snapshots=16)
    model_rv.forward(c0)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    grad_rv = model_rv.backward(res)
    t4 = time.perf_counter()
    sched_rv = model_rv.schedule()
    model_rv.close()
    fd = adjoint_fd_check_32(pb, order, dt, rng, idx, rhs, val, rec_idx, rec_w, c0, c_true)
    # forward N steps + backward (replay ~N steps, N adjoint steps, N gradient kernels)
    dof_updates = pb.n_dof * S * N
    return {"workload": f"32^3 Q4, per-element c (start U[1.5,2.5], true c perturbed by U[-10%,10%]), {S} sources x "
                        f"{nrec} receivers, {N} FP32 steps, L2 trace misfit, discrete adjoint",
            "n_dof": pb.n_dof, "steps": N, "loss": J, "grad_norm": float(np.linalg.norm(grad)),
            "forward_seconds": t1 - t0, "backward_seconds": t2 - t1,
            "forward_value": dof_updates / (t1 - t0), "gradient_value": dof_updates / (t2 - t0), "unit": UNIT,
            "schedule": sched,
            "checkpoints_uniform": uniform,
            "checkpoints_revolve_16": dict(sched_rv, backward_seconds=t4 - t3,
                                           grad_bitwise_equal=bool(np.array_equal(grad_rv, grad))),
            "fd_check_32": fd,
            "small_case_check": adjoint_small_check()}


def adjoint_fd_check_32(pb, order, dt, rng, idx, rhs, val, rec_idx, rec_w, c0, c_true):
    """The adjoint gradient on the 32^3 mesh against central differences of
    the FP64 plain-form misfit (one FP64 integrator run per source), on 20
    elements drawn from the 1,000 with the largest gradient.  Reduced to the
    first 8 sources and 100 steps (the FP64 misfit is evaluated 40 times)."""
    from montjoie_gb300.adjoint import AcousticAdjoint, Fp64Misfit, central_differences
    S, N = 8, 100
    keep = [i for i in range(len(idx)) if i < S]
    args = (order, pb.nodle, pb.factors, pb.n_dof, pb.mass, dt, N, S, np.concatenate([idx[i] for i in keep]),
            np.concatenate([rhs[i] for i in keep]), np.concatenate([val[i] for i in keep]), pb.pulse, rec_idx, rec_w)
    t0 = time.perf_counter()
    model = AcousticAdjoint(*args)
    data = model.forward(c_true)
    _, g = model.loss_and_grad(c0, data)
    model.close()
    els = rng.choice(np.argsort(-np.abs(g))[:1000], size=20, replace=False)
    J64 = Fp64Misfit(*args)
    fd = central_differences(lambda c: J64(c, data), c0, els)
    J64.close()
    return {"mesh": "the 32^3 Q4 mesh of this workload", "sources": S, "receivers": int(rec_idx.shape[0]),
            "steps": N, "elements": "20 drawn from the 1000 with the largest |gradient|",
            "fd_rel_l2_20_elements": float(np.linalg.norm(g[els] - fd) / np.linalg.norm(fd)),
            "reference": "central differences (h = 1e-4 c_e) of the FP64 plain-form misfit on the GPU",
            "seconds": time.perf_counter() - t0}


def adjoint_small_check():
    """GPU FP32 adjoint vs FP64 CPU adjoint vs central differences on 20 elements (small mesh)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from adjoint_case import build_case, oracle_adjoint
    from montjoie_gb300.adjoint import AcousticAdjoint
    case = build_case(S=8, nsteps=80)
    g = case["g"]
    model = AcousticAdjoint(case["r"], g["nodle"], case["bh_unit"], g["massD"].size, g["massD"], case["dt"],
                            case["N"], case["S"], case["src_idx"], case["src_rhs"], case["src_val"], case["pulse"],
                            case["rec_idx"], case["rec_w"])
    J, grad = model.loss_and_grad(case["c0"], case["data"])
    model.close()
    J64, _, g64 = oracle_adjoint(case, case["c0"], case["data"])
    rng = np.random.default_rng(7)
    els = rng.choice(case["c0"].size, size=min(20, case["c0"].size), replace=False)
    fd = []
    for e in els:
        h = 1e-5 * case["c0"][e]
        cp, cm = case["c0"].copy(), case["c0"].copy()
        cp[e] += h
        cm[e] -= h
        fd.append((oracle_adjoint(case, cp, case["data"], False)[0] - oracle_adjoint(case, cm, case["data"], False)[0])
                  / (2 * h))
    fd = np.array(fd)
    return {"mesh": "3^3 Q4 golden mesh, 8 sources x 4 receivers, 80 steps",
            "gpu_fp32_vs_fp64_adjoint_rel_l2": float(np.linalg.norm(grad - g64) / np.linalg.norm(g64)),
            "gpu_fp32_vs_fd_rel_l2_20_elements": float(np.linalg.norm(grad[els] - fd) / np.linalg.norm(fd)),
            "fp64_adjoint_vs_fd_rel_l2_20_elements": float(np.linalg.norm(g64[els] - fd) / np.linalg.norm(fd)),
            "loss_rel_diff": abs(J - J64) / J64}


def LeapFrogIteratorFor(pb, op, src_idx, src_val):
    from montjoie_gb300.leapfrog import LeapFrogIterator
    return LeapFrogIterator(op, pb.setup.dt, pb.mass, None, src_idx, src_val, pb.pulse)


def time_advance(torch, lf, steps, lib, prof_steps=100, barrier=None):
    """Times `steps` leap-frog steps (already initialised) with CUDA events on the
    library's stream (the legacy default stream; CUDA-graph replay), bracketed
    by `barrier` (the replicas' barrier, if any) and a device synchronisation
    on both sides; then `prof_steps` more steps launched one by one with events
    around each kernel for the per-kernel times."""
    import ctypes
    L = lib.load()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if barrier:
        barrier()
    l0 = lib.kernel_launches()
    start.record()
    lf.Advance(steps)
    end.record()
    torch.cuda.synchronize()
    if barrier:
        barrier()
    launches = lib.kernel_launches() - l0
    L.mj_lf_profile(lf.handle, 1, None, None, None)
    lf.Advance(min(steps, prof_steps))
    e_ms, u_ms, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    L.mj_lf_profile(lf.handle, 0, ctypes.byref(e_ms), ctypes.byref(u_ms), ctypes.byref(n))
    return start.elapsed_time(end), e_ms.value / max(1, n.value), u_ms.value / max(1, n.value), launches


def run_ours(args):
    import torch
    import torch.distributed as dist
    from montjoie_gb300 import _lib
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    _lib.load(build_if_missing=False)
    K, W = args.steps, args.warmup
    nsteps_pulse = max(K + W, args.error_steps) + 10
    t_setup = time.perf_counter()
    pb = build_problem(args.cells, args.order, nsteps_pulse)
    setup_s = time.perf_counter() - t_setup
    n_dof, n_elt, Q = pb.n_dof, pb.nodle.shape[0], (args.order + 1) ** 3
    zeros = np.zeros(n_dof)

    # ---- FP32 chosen form, resident (value)
    op32 = pb.operator("fp32")
    if args.e2e_only:
        lfd = pb.integrator(op32, diagnostics=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, nd, _ = lfd.Run(zeros, None, args.error_steps)
        print(json.dumps({"e2e_only": True, "steps": args.error_steps, "seconds": time.perf_counter() - t0,
                          "last_norm": float(nd[-1])}))
        return
    if args.k1_variant and args.fp32_only:
        e_, lay_ = (int(v) for v in args.k1_variant.split(","))
        op32.set_variant(e_, lay_)
    tuning32 = op32.tuning()
    lf32 = pb.integrator(op32, diagnostics=False)
    lf32.SetInitialConditionS(zeros)
    lf32.Advance(W)
    clocks = ClockSampler(local)
    clocks.start()
    ms32, k1_ms, k2_ms, launches = time_advance(torch, lf32, K, _lib, barrier=dist.barrier if world > 1 else None)
    if args.fp32_only:
        clocks.stop()
        print(json.dumps({"fp32_only": True, "cells": args.cells, "order": args.order, "ms_per_step": ms32 / K,
                          "element_kernel_ms": k1_ms, "update_kernel_ms": k2_ms, "tuning": tuning32,
                          "setup_seconds": setup_s}))
        return
    # ---- FP64 plain form, resident (its own step count, after one graph's worth of warm-up)
    op64 = pb.operator("fp64")
    lf64 = pb.integrator(op64, diagnostics=False)
    lf64.SetInitialConditionS(zeros)
    lf64.Advance(21)
    K64 = args.fp64_steps
    ms64, k1_64, k2_64, _ = time_advance(torch, lf64, K64, _lib)
    clk = clocks.stop()
    if world > 1:
        ms32 = max_over_ranks(ms32, dist, "cuda")
    value = whole_job_rate(n_dof * K, world, ms32)
    value64 = n_dof * K64 / (ms64 / 1e3)
    lf32.close(); lf64.close()

    # ---- error of the FP32 form against the FP64 form (same run, error_steps steps)
    lf64d = pb.integrator(op64, diagnostics=True)
    u64, n64, tr64 = lf64d.Run(zeros, None, args.error_steps)
    lf64d.close()
    e2e = None
    lf32d = pb.integrator(op32, diagnostics=True)
    # host side of the call in pinned memory: u0 in, u_final out
    u0_pin = torch.zeros(n_dof, dtype=torch.float64, pin_memory=True).numpy()
    uf_pin = torch.empty(n_dof, dtype=torch.float64, pin_memory=True).numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u32, n32, tr32 = lf32d.Run(u0_pin, None, args.error_steps, out=uf_pin)
    e2e_s = time.perf_counter() - t0
    lf32d.close()
    # the FP32 and FP64 states every 100 steps (Advance in chunks; states read back)
    NE = args.error_steps
    snaps32, snaps64 = {}, {}
    a64, a32 = pb.integrator(op64, diagnostics=False), pb.integrator(op32, diagnostics=False)
    a64.SetInitialConditionS(zeros); a32.SetInitialConditionS(zeros)
    for k in range(0, NE, 100):
        a64.Advance(min(100, NE - k)); a32.Advance(min(100, NE - k))
        snaps64[a64.n_time], snaps32[a32.n_time] = a64.GetIterate(), a32.GetIterate()
    a64.close(); a32.close()
    err = {"steps": NE, "reference": ORACLE_REF,
           "fp32_vs_fp64_gpu_u_rel_l2": rel(u32, u64)}
    if not args.no_oracle:
        t0 = time.perf_counter()
        o = oracle_run(pb, NE, snap_every=100, diag=True)
        err.update({
            "fp32_u_rel_l2_every_100_steps": [[k, rel(snaps32[k], o["snaps"][k])] for k in sorted(o["snaps"])],
            "fp64_u_rel_l2_every_100_steps": [[k, rel(snaps64[k], o["snaps"][k])] for k in sorted(o["snaps"])],
            "fp32_u_rel_l2": rel(u32, o["u"]), "fp64_u_rel_l2": rel(u64, o["u"]),
            "fp32_norm_history_rel_l2": rel(n32, o["norms"]), "fp64_norm_history_rel_l2": rel(n64, o["norms"]),
            "fp32_traces_rel_max": float(np.abs(tr32 - o["traces"]).max() / np.abs(o["traces"]).max()),
            "fp64_traces_rel_max": float(np.abs(tr64 - o["traces"]).max() / np.abs(o["traces"]).max()),
            "oracle_seconds": time.perf_counter() - t0})
    if not args.no_e2e:
        h2d = n_dof * 8  # u0 (du0 = NULL)
        d2h = n_dof * 8 + 8 * (args.error_steps + 1) * (1 + 8)  # u_final, norms, 8 traces
        e2e = {"value": n_dof * args.error_steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.error_steps, "d2h_bytes_per_step": d2h / args.error_steps,
               "call": "mj_lf_run: host u0 in, FP32 run with norm and 8 receiver traces every step, host u out "
                       "(u0 and u in pinned host memory)",
               "seconds": e2e_s}

    # ---- roofline of the dominant kernel (element kernel, FP32)
    peak, peak_kind = measured_peaks()
    bytes_k1 = n_elt * Q * (6 * 4 + 4) + n_dof * 4   # factors + connectivity + input state, read once
    achieved = bytes_k1 / (k1_ms / 1e3) / 1e9
    per_elt = ncu_traffic_per_element(f"k_local_stiffness_fp32_q{args.order}.md")
    step_bytes = n_elt * Q * (6 * 4 + 4) + n_dof * (3 * 4 + 4)
    kname = ("k_local_stiffness_w<float,%d,%d%s>" % (args.order + 1, tuning32["tile_elems"],
                                                    ",packed" if tuning32["layout"].endswith("packed") else "")
             if tuning32["layout"].startswith("warp_per_element") else
             "k_local_stiffness<float,%d,%d,%s>" % (args.order + 1, tuning32["tile_elems"],
                                                   "vec" if tuning32["layout"] == "vector_lines" else "compact"))
    roofline = {"bound": "hbm", "kernel": kname + " (element kernel, autotuned)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
                "traffic": None if per_elt is None else per_elt * n_elt,
                "algorithmic_bytes_per_launch": bytes_k1,
                "kernel_ms": k1_ms, "update_kernel_ms": k2_ms,
                "step_frac": (step_bytes / (ms32 / K / 1e3) / 1e9) / peak, "autotuned": tuning32,
                "step_algorithmic_bytes": step_bytes}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
           "ms_per_step": ms32 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded perturbed 64^3 Q4 mesh, c on 8^3 random blocks)",
           "config": workload_config(args.cells, args.order, n_dof),
           "parallelism": f"replicas x{world}", "n_elt": n_elt, "dt": pb.setup.dt, "setup_seconds": setup_s,
           "fp64": {"value": value64, "ms_per_step": ms64 / K64, "steps": K64, "elem_kernel_ms": k1_64,
                    "update_kernel_ms": k2_64, "fp32_over_fp64": value / world / value64},
           "error_vs_oracle": err,
           "roofline": roofline, "clocks": clk, "gpu_launches": launches, "e2e": e2e}
    if not args.no_extras:
        op32.close(); op64.close()
        out["q8_curved_32"] = leg_q8(args, torch, _lib)
        out["sources64_32"] = leg_sources(args, torch, _lib)
        out["meshes24"] = leg_meshes(args, torch, _lib)
        out["adjoint_32"] = leg_adjoint(args, torch, _lib)
        o4 = leg_order4(args, torch, _lib)
        o4["simulated_time_per_second_order2_fp32"] = pb.setup.dt * K / (ms32 / 1e3)
        out["order4_scheme"] = o4
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def port_workload(cells, order, nsteps, nodle=None):
    """The headline workload set up by the oracle alone (no GPU): the seeded
    mesh, FP64 factors and mass, the Gaussian source at the centre, dt from a
    power iteration on the oracle operator and the pulse of nsteps steps.
    `nodle` reuses a numbering made elsewhere (any numbering gives the same
    work); by default the lattice numbering."""
    from oracle import oracle as oc
    m = workload_mesh(cells)
    if nodle is None:
        nodle = oc.structured_nodle(cells, order)
    bh, jw, xq = oc.geometry(order, m.verts[m.hexes], m.elem_c ** 2)
    ndof = int(nodle.max()) + 1
    D = oc.lumped_mass(nodle, jw, ndof)
    invD = 1.0 / D
    colors = oc.structured_colors(cells)
    F = oc.gaussian_source(nodle, jw, xq, ndof, np.array([0.5, 0.5, 0.5]), 2.0 / cells)
    idx = np.nonzero(F)[0].astype(np.int32)
    lam = oc.power_iteration_lambda_max(order, nodle, bh, invD, iters=8, colors=colors)
    dt = 0.5 * 2.0 / np.sqrt(1.05 * lam)
    pulse = oc.ricker_pulse(5.0, 0.0, dt, nsteps, 1e-15 * nsteps * dt)
    return {"order": order, "nodle": nodle, "bh": bh, "D": D, "invD": invD, "colors": colors, "idx": idx,
            "val": F[idx], "dt": dt, "pulse": pulse, "n_dof": ndof}


def time_port_steps(w, steps, warmup=0, threads=None):
    """Wall time of `steps` whole leap-frog steps of the oracle's restatement
    in ONE call that continues from the state after `warmup` steps (no start
    step inside the timed call).  threads: host threads (None: all)."""
    from oracle import oracle as oc
    before = oc.threads()
    if threads:
        oc.threads(threads)
    u0, u1 = np.zeros(w["n_dof"]), np.zeros(w["n_dof"])
    a = (w["order"], w["nodle"], w["bh"], w["D"], w["invD"], w["idx"], w["val"])
    try:
        if warmup:
            oc.leapfrog_advance(*a, w["pulse"], w["dt"], warmup, u0, u1, colors=w["colors"])
        t0 = time.perf_counter()
        oc.leapfrog_advance(*a, w["pulse"][warmup:], w["dt"], steps, u0, u1, colors=w["colors"])
        el = time.perf_counter() - t0
    finally:
        oc.threads(before)
    return el


def steps_for(seconds, per_step, cap):
    return int(max(1, min(cap, seconds // max(per_step, 1e-9))))


def cpu_baseline(args, seconds=None):
    """The oracle's C restatement (element loop in the reference's order,
    colour-parallel over the host cores) on a bounded sample of the workload:
    whole leap-frog steps of the same mesh, timed as one call; also on one
    core, the reference's own mode."""
    seconds = args.cpu_seconds if seconds is None else seconds
    cells, order = args.cells, args.order
    w = port_workload(cells, order, 600)
    probe = time_port_steps(w, 1, warmup=2)
    steps = steps_for(seconds, probe, 500)
    el = time_port_steps(w, steps, warmup=2)
    probe1 = time_port_steps(w, 1, warmup=2, threads=1)
    steps1 = steps_for(seconds / 2, probe1, 100)
    el1 = time_port_steps(w, steps1, warmup=2, threads=1)
    nd = w["n_dof"]
    return {"value": nd * steps / el, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
            "sample": f"{steps} FP64 leap-frog steps of the same {cells}^3 Q{order} mesh ({nd} dofs, source on) in "
                      f"one call after 2 warm-up steps, oracle C restatement, colour-parallel OpenMP, {el:.1f} s",
            "seconds": el,
            "one_core": {"value": nd * steps1 / el1, "cores": 1, "steps": steps1, "seconds": el1}}


def run_reference(args):
    """The reference arm: the oracle's C restatement of the reference loop,
    all host threads, the headline workload; K steps timed as ONE call after
    W warm-up steps (capped to fit about two minutes), plus a one-core sample."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import oracle as oc
    oc.build()
    K, W = args.steps, args.warmup
    cells, order = args.cells, args.order
    w = port_workload(cells, order, K + W + 10)
    budget = 120.0
    probe = time_port_steps(w, 1, warmup=min(W, 3))
    steps = steps_for(budget, probe, K)
    el = time_port_steps(w, steps, warmup=W)
    value = w["n_dof"] * steps / el
    probe1 = time_port_steps(w, 1, warmup=2, threads=1)
    steps1 = steps_for(10.0, probe1, K)
    el1 = time_port_steps(w, steps1, warmup=2, threads=1)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
           "requested_steps": K, "warmup": W, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(cells, order, w["n_dof"]), "parallelism": "host cores",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
                            "sample": f"{steps} FP64 leap-frog steps of the {cells}^3 Q{order} mesh in one call after "
                                      f"{W} warm-up steps, oracle C restatement of the reference loop, "
                                      f"colour-parallel OpenMP",
                            "one_core": {"value": w["n_dof"] * steps1 / el1, "cores": 1, "steps": steps1,
                                         "seconds": el1}},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    if args.leg != "all":
        import torch
        from montjoie_gb300 import _lib
        _lib.load(build_if_missing=False)
        fn = {"q8": leg_q8, "sources": leg_sources, "meshes": leg_meshes, "adjoint": leg_adjoint,
              "order4": leg_order4}[args.leg]
        print(json.dumps({args.leg: fn(args, torch, _lib)}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
