"""The allocation-free product mj_stiffness_mltadd_static, through the C ABI.

It is for callers that must not let a library allocate GPU memory: a solver
whose device memory all belongs to one arena, or a time loop that stages its
buffers up front and must not call cudaMalloc/cudaFree later.  Here the
caller's buffers come from torch; the entry point itself allocates nothing.
Its output must match the allocating entry point (mj_op_create + mj_op_mltadd)
within the FP64 operator tolerance, on two calls in a row that share the one
static scratch array, for every order 1..8 (the entry point has its own
closed-form local numbering, so each order's numbering is checked).  This file
runs last so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12

# golden cases of the reference for orders 1, 2, 3, 4, 6, 8; orders 5 and 7
# are built by the oracle on a perturbed 3^3 cube
CASES = ["cube2_q1", "cube2_q2", "cube2_q3", "cube3_q4", "cube2_q6", "cube2_q8", "oracle_q5", "oracle_q7"]


def _case(name):
    if not name.startswith("oracle_"):
        return load_golden(name)
    from montjoie_gb300 import mesh as M
    from oracle import oracle as oc
    r, n = int(name[-1]), 3
    m = M.perturbed_cube(n, seed=40 + r, amplitude=0.05, kind="random", c_mode="element")
    nodle = oc.structured_nodle(n, r)
    bh, jw, _ = oc.geometry(r, m.verts[m.hexes], m.elem_c ** 2)
    ndof = (n * r + 1) ** 3
    rng = np.random.default_rng(r)
    return {"order": r, "nodle": nodle, "bh": bh, "massD": oc.lumped_mass(nodle, jw, ndof),
            "x": rng.uniform(-1, 1, ndof), "y0": rng.uniform(-1, 1, ndof), "alpha": 0.75, "beta": -1.25,
            "gradphi": oc.grad_matrix(r)}


def _static_call(L, g, alpha, beta, y0, torch):
    dev = torch.device("cuda")
    nodle = torch.from_numpy(np.ascontiguousarray(g["nodle"], dtype=np.int32)).to(dev)
    fac = torch.from_numpy(np.ascontiguousarray(g["bh"], dtype=np.float64)).to(dev)
    x = torch.from_numpy(np.ascontiguousarray(g["x"], dtype=np.float64)).to(dev)
    y = torch.from_numpy(np.ascontiguousarray(y0, dtype=np.float64)).to(dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.mj_stiffness_mltadd_static(int(g["order"]), g["nodle"].shape[0], g["massD"].size,
                                      ctypes.c_void_p(nodle.data_ptr()), ctypes.c_void_p(fac.data_ptr()),
                                      float(alpha), ctypes.c_void_p(x.data_ptr()), float(beta),
                                      ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, L.mj_last_error()
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("case", CASES)
def test_static_entry_matches_allocating_entry(case):
    torch = pytest.importorskip("torch")
    from montjoie_gb300 import _lib
    from montjoie_gb300.operator import FemMatrixFreeOperator
    L = _lib.load()
    g = _case(case)
    op = FemMatrixFreeOperator(int(g["order"]), g["nodle"], g["bh"], g["massD"].size, "fp64", gradphi=g["gradphi"])
    calls = [(float(g["alpha"]), float(g["beta"]), g["y0"]), (-2.5, 0.0, np.full_like(g["y0"], np.nan))]
    for alpha, beta, y0 in calls:  # two calls in a row on the shared scratch
        y_ref = np.array(y0, copy=True)
        op.MltAddVector(alpha, g["x"], beta, y_ref)
        y = _static_call(L, g, alpha, beta, y0, torch)
        assert rel_l2(y, y_ref) < FP64_TOL
    op.close()


def test_static_entry_rejects_meshes_beyond_its_scratch():
    from montjoie_gb300 import _lib
    L = _lib.load()
    big = 4194304 // 125 + 1  # Q4 elements just past the static scratch
    rc = L.mj_stiffness_mltadd_static(4, big, 10, ctypes.c_void_p(8), ctypes.c_void_p(8), 1.0,
                                      ctypes.c_void_p(8), 0.0, ctypes.c_void_p(8), None)
    assert rc == _lib.MJ_ERR_ARG
    assert b"exceeds the static scratch" in L.mj_last_error()
