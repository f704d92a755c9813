"""Shared small inversion case for the adjoint tests (cube3_q4 golden mesh)."""
import numpy as np

from conftest import load_golden


def build_case(S=8, nrec=4, nsteps=80, seed=5):
    from oracle import oracle as oc
    g = load_golden("cube3_q4")
    r = int(g["order"])
    mu = g["media_c"][g["elem_ref"] - 1] ** 2
    bh_unit = g["bh"] / mu[:, None, None]
    _, jw, xq = oc.geometry(r, g["verts_e"], np.ones(g["verts_e"].shape[0]))
    rng = np.random.default_rng(seed)
    ndof = g["massD"].size
    idx, rhs, val = [], [], []
    for s, c in enumerate(rng.uniform(0.25, 0.75, size=(S, 3))):
        F = oc.gaussian_source(g["nodle"], jw, xq, ndof, c, 0.3)
        nz = np.nonzero(F)[0]
        idx.append(nz); val.append(F[nz]); rhs.append(np.full(nz.size, s))
    rec_pts = rng.uniform(0.1, 0.9, size=(nrec, 3))
    Q = (r + 1) ** 3
    rec_idx = np.zeros((nrec, Q), dtype=np.int32)
    rec_w = np.zeros((nrec, Q))
    lo, hi = g["verts_e"].min(axis=1), g["verts_e"].max(axis=1)
    for k, p in enumerate(rec_pts):
        for e in np.nonzero(np.all((lo <= p) & (hi >= p), axis=1))[0]:
            w, _, inside = oc.point_weights(r, g["verts_e"][e], p)
            if inside:
                rec_idx[k], rec_w[k] = g["nodle"][e], w
                break
    c_true = np.sqrt(mu)
    c0 = c_true * (1.0 + 0.1 * rng.uniform(-1, 1, c_true.size))
    case = dict(g=g, r=r, bh_unit=bh_unit, S=S, src_idx=np.concatenate(idx).astype(np.int32),
                src_rhs=np.concatenate(rhs).astype(np.int32), src_val=np.concatenate(val), rec_idx=rec_idx,
                rec_w=rec_w, N=nsteps, dt=float(g["dt"]), pulse=g["pulse"], c_true=c_true, c0=c0)
    _, data, _ = oracle_adjoint(case, c_true, None, want_grad=False)
    case["data"] = data
    return case


def oracle_adjoint(case, c, data, want_grad=True):
    from oracle import oracle as oc
    g = case["g"]
    pulse = np.zeros(case["N"])
    pulse[:min(case["N"], case["pulse"].size)] = case["pulse"][:case["N"]]
    return oc.adjoint(case["r"], g["nodle"], case["bh_unit"], c, g["massD"], g["invD"], case["S"], case["src_idx"],
                      case["src_rhs"], case["src_val"], pulse, case["dt"], case["N"], case["rec_idx"],
                      case["rec_w"], data=data, want_grad=want_grad)
