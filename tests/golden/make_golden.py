"""Generates the golden fixtures of tests/golden/ by running the reference's own
solver (oracle/_ref/ref_dump, compiled from the Montjoie sources by
oracle/Makefile) on seeded meshes written by montjoie_gb300.mesh.

Run from the repository root:   python tests/golden/make_golden.py [case ...]

Every fixture is an .npz holding what the reference computed (connectivity,
factors, mass, source, pulse, operator products, trajectory norms,
snapshots or probe values) plus the inputs that produced it.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from montjoie_gb300 import mesh as M  # noqa: E402
from oracle import oracle as oc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name: (cells per axis, order, perturbation kind, amplitude, c_mode, steps, source radius, snaps[, time order])
CASES = {
    "regular2_q4": (2, 4, "none", 0.0, "constant", 30, 0.35, (0, 30)),
    "cube2_q1": (2, 1, "random", 0.1, "element", 40, 0.45, (0, 40)),
    "cube2_q2": (2, 2, "random", 0.1, "element", 60, 0.35, (0, 30, 60)),
    "cube2_q3": (2, 3, "random", 0.1, "element", 40, 0.35, (0, 40)),
    "cube3_q4": (3, 4, "random", 0.1, "element", 120, 0.3, (0, 60, 120)),
    "cube2_q6": (2, 6, "random", 0.1, "element", 40, 0.3, (0, 40)),
    "cube2_q8": (2, 8, "sin", 0.1, "smooth", 30, 0.3, (0, 30)),
    "cube4_q4": (4, 4, "random", 0.05, "element", 200, 0.25, (0, 100, 200)),
    # order-4 modified-equation leap-frog (OrderTimeScheme = 4 LEAP_FROG)
    "cube3_q4_o4": (3, 4, "random", 0.1, "element", 120, 0.3, (0, 60, 120), 4),
    "cube2_q2_o4": (2, 2, "random", 0.1, "element", 60, 0.35, (0, 30, 60), 4),
    "cube2_q8_o4": (2, 8, "sin", 0.1, "smooth", 30, 0.3, (0, 30), 4),
}

SEED = 20251203


def cfl_dt(r, ref, factor=0.5, time_order=2):
    """dt = factor * C / sqrt(lambda_max(D^-1 A)) with the scheme's CFL constant
    C = 2 (order 2) or 2 sqrt(3) (order 4) (ModifiedEquation.cxx:217-225),
    lambda_max by power iteration on the reference's own arrays."""
    lam = oc.power_iteration_lambda_max(r, ref["nodle"], ref["bh"], ref["invD"], iters=300)
    c = 2.0 if time_order == 2 else 2.0 * np.sqrt(3.0)
    return factor * c / np.sqrt(lam * 1.02)


def run_case(name, n, r, kind, amp, c_mode, steps, radius, snaps, time_order=2, work=None):
    m = M.perturbed_cube(n, seed=SEED + n * 10 + r, amplitude=amp, kind=kind, c_mode=c_mode)
    mesh_file = os.path.join(work, f"{name}.mesh")
    M.write_medit(mesh_file, m)
    # first pass: 1 step, to get the reference's arrays for the CFL estimate
    s = M.AcousticSetup(order=r, dt=1e-4, nsteps=1, src_radius=radius)
    deck = os.path.join(work, f"{name}.ini")
    M.write_deck(deck, mesh_file, m, s)
    probe = oc.run_reference(deck, os.path.join(work, name + "_probe"))
    dt = cfl_dt(r, probe, time_order=time_order)
    s = M.AcousticSetup(order=r, dt=dt, nsteps=steps, src_radius=radius, time_order=time_order)
    M.write_deck(deck, mesh_file, m, s)
    rng = np.random.default_rng(SEED + 7)
    ndof = probe["meta"]["n_dof"]
    x = rng.uniform(-1.0, 1.0, ndof)
    y0 = rng.uniform(-1.0, 1.0, ndof)
    alpha, beta = 0.7, -1.3
    ref = oc.run_reference(deck, os.path.join(work, name), x=x, y0=y0, alpha=alpha, beta=beta, snaps=snaps)
    meta = ref["meta"]
    assert meta["nsteps"] == steps, (meta["nsteps"], steps)
    out = dict(
        n=n, order=r, kind=kind, amplitude=amp, c_mode=c_mode, seed=SEED + n * 10 + r, nsteps=steps,
        dt=meta["dt"], t0=meta["t0"], tf=meta["tf"], f0=meta["frequency"], tlimit=meta["tlimit_source"],
        eps_time=meta["epsilon_time"], src_radius=radius, src_center=np.array([0.5, 0.5, 0.5]),
        verts=m.verts, hexes=m.hexes, elem_ref=m.elem_ref, media_c=m.media_c,
        nodle=ref["nodle"], verts_e=ref["verts"], bh=ref["bh"], jw=ref["jw"], affine=ref["affine"],
        massD=ref["massD"], invD=ref["invD"], src_idx=ref["src_idx"], src_val=ref["src_val"], pulse=ref["pulse"],
        points1d=ref["points1d"], gradphi=ref["gradphi"], numdofs3d=ref["numdofs3d"],
        x=x, y0=y0, alpha=alpha, beta=beta, kh_y=ref["kh_y"], kh_ax=ref["kh_ax"],
        norms=ref["norms"], times=ref["times"], u_final=ref["u_final"],
        snap_steps=np.array(sorted(ref["snaps"])), snaps=np.stack([ref["snaps"][k] for k in sorted(ref["snaps"])]),
        time_order=time_order, pulse3=ref["pulse3"],
    )
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    print(f"{name}: ndof={ndof} dt={dt:.3e} steps={steps} norm_final={ref['norms'][-1]:.6e}")


def run_config1(work):
    """16^3 Q4, +-5% h random perturbation, c ~ U[1,3] per element, Ricker f0 = 5
    at the centre (Gaussian R = 2h), Neumann, dt = 0.5 CFL, 200 steps: the
    reference's norms, 8 receiver traces and 512 probe values of the final u."""
    n, r, steps = 16, 4, 200
    seed = SEED + 1
    m = M.perturbed_cube(n, seed=seed, amplitude=0.05, kind="random", c_mode="element")
    mesh_file = os.path.join(work, "config1.mesh")
    M.write_medit(mesh_file, m)
    radius = 2.0 / n
    s = M.AcousticSetup(order=r, dt=1e-4, nsteps=1, src_radius=radius)
    deck = os.path.join(work, "config1.ini")
    M.write_deck(deck, mesh_file, m, s)
    probe = oc.run_reference(deck, os.path.join(work, "config1_probe"))
    colors = oc.structured_colors(n)
    lam = oc.power_iteration_lambda_max(r, probe["nodle"], probe["bh"], probe["invD"], iters=200, colors=colors)
    dt = 0.5 * 2.0 / np.sqrt(lam * 1.02)
    s = M.AcousticSetup(order=r, dt=dt, nsteps=steps, src_radius=radius)
    M.write_deck(deck, mesh_file, m, s)
    ref = oc.run_reference(deck, os.path.join(work, "config1"), snaps=tuple(range(steps + 1)))
    ndof = ref["meta"]["n_dof"]
    # dof positions from the reference's own connectivity and points
    _, _, xq = oc.geometry(r, ref["verts"], np.ones(ref["verts"].shape[0]))
    pos = np.zeros((ndof, 3))
    pos[ref["nodle"].reshape(-1)] = xq.reshape(-1, 3)
    rng = np.random.default_rng(seed + 3)
    rec = rng.uniform(0.1, 0.9, size=(8, 3))
    probes = rng.choice(ndof, size=512, replace=False)
    # receiver weights in the reference numbering (oracle point location)
    verts_e = ref["verts"]
    Q = (r + 1) ** 3
    rec_idx = np.zeros((8, Q), dtype=np.int32)
    rec_w = np.zeros((8, Q))
    for k, p in enumerate(rec):
        lo, hi = verts_e.min(axis=1), verts_e.max(axis=1)
        for e in np.nonzero(np.all((lo <= p) & (hi >= p), axis=1))[0]:
            w, xi, inside = oc.point_weights(r, verts_e[e], p)
            if inside:
                rec_idx[k], rec_w[k] = ref["nodle"][e], w
                break
        else:
            raise RuntimeError("receiver not located")
    U = np.stack([ref["snaps"][s_] for s_ in range(steps + 1)])
    traces = np.einsum("kq,skq->ks", rec_w, U[:, rec_idx])
    out = dict(n=n, order=r, seed=seed, nsteps=steps, dt=dt, f0=ref["meta"]["frequency"],
               t0=ref["meta"]["t0"], tf=ref["meta"]["tf"], eps_time=ref["meta"]["epsilon_time"],
               tlimit=ref["meta"]["tlimit_source"], src_radius=radius, src_center=np.array([0.5, 0.5, 0.5]),
               n_dof=ndof, n_src=ref["meta"]["n_src"], pulse=ref["pulse"], norms=ref["norms"], times=ref["times"],
               receivers=rec, traces=traces, probe_pos=pos[probes], probe_u=ref["u_final"][probes],
               u_final_norm2=float(np.linalg.norm(ref["u_final"])), massD_sum=float(ref["massD"].sum()),
               loop_seconds=ref["run"]["loop_seconds"])
    np.savez_compressed(os.path.join(OUT, "config1_16q4.npz"), **out)
    print(f"config1: ndof={ndof} dt={dt:.4e} norm_final={ref['norms'][-1]:.6e} loop={ref['run']['loop_seconds']:.2f}s")


def main(argv):
    if not os.path.exists(oc.REF_DUMP):
        raise SystemExit("oracle/_ref/ref_dump missing: run `make -C oracle ref` first")
    wanted = argv or list(CASES) + ["config1"]
    work = tempfile.mkdtemp(prefix="mj_golden_")
    try:
        for name in wanted:
            if name == "config1":
                run_config1(work)
            else:
                run_case(name, *CASES[name], work=work)
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main(sys.argv[1:])
