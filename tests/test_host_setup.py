"""Product host-side logic on the CPU: the C-ABI library loads and exports
every declared symbol, argument validation, the global numbering, the lumped
mass, the pulse, the source and the receivers, against the reference's
golden outputs.  No compute call here touches a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2
from montjoie_gb300 import _lib, problem
from oracle import oracle as oc


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "montjoie_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mj_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), f"{s} not exported"
    assert set(syms) <= set(_lib.EXPORTED) | set(syms)
    assert L.mj_version().decode().startswith("montjoie_gb300")


def test_create_rejects_bad_arguments():
    L = _lib.load()
    nodle = np.zeros((1, 8), dtype=np.int32)
    fac = np.zeros(8 * 6)
    h = ctypes.c_void_p()
    mesh = _lib.MeshDesc(0, 1, 8, _lib.iptr(nodle))
    geom = _lib.GeomDesc(_lib.dptr(fac), None)
    assert L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), _lib.MJ_FP64, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert b"order" in L.mj_last_error()
    mesh = _lib.MeshDesc(1, 1, 8, _lib.iptr(np.full((1, 8), 9, dtype=np.int32)))
    assert L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), _lib.MJ_FP64, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert b"out of" in L.mj_last_error()
    mesh = _lib.MeshDesc(1, 1, 9, _lib.iptr(np.arange(8, dtype=np.int32).reshape(1, 8)))
    assert L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), _lib.MJ_FP64, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert b"no element" in L.mj_last_error()
    mesh = _lib.MeshDesc(1, 1, 8, _lib.iptr(np.arange(8, dtype=np.int32).reshape(1, 8)))
    assert L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), 7, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    bad = fac.copy()
    bad[3] = np.nan
    geom = _lib.GeomDesc(_lib.dptr(bad), None)
    assert L.mj_op_create(ctypes.byref(mesh), ctypes.byref(geom), _lib.MJ_FP64, ctypes.byref(h)) == _lib.MJ_ERR_NONFINITE
    assert L.mj_lf_create(None, None, None) == _lib.MJ_ERR_ARG
    assert L.mj_lf_advance(None, 1, None, None, 0) == _lib.MJ_ERR_ARG


def test_batch_entry_points_reject_null_handles():
    """The batch, many-source and adjoint entry points check their handles
    before touching the device."""
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.mj_mb_create(0, None, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert L.mj_mb_create(1, None, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert L.mj_mb_advance(None, 1, 1) == _lib.MJ_ERR_ARG
    assert L.mj_mb_info(None, None, None, None, None, None, None) == _lib.MJ_ERR_ARG
    assert L.mj_mb_phase_ms(None, None) == _lib.MJ_ERR_ARG
    assert L.mj_mb_set_config(None, 128) == _lib.MJ_ERR_ARG
    assert L.mj_mb_tuning(None, None, None) == _lib.MJ_ERR_ARG
    assert L.mj_lfb_create(None, None, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert L.mj_adj_create(None, 10, 0, ctypes.byref(h)) == _lib.MJ_ERR_ARG
    assert b"null" in L.mj_last_error()


def test_numbering_is_the_reference_numbering_up_to_permutation(golden_case):
    name, g = golden_case
    r = int(g["order"])
    nodle, ndof = problem.number_mesh(r, g["hexes"], g["verts"].shape[0])
    assert ndof == g["massD"].size
    a, b = nodle.ravel(), g["nodle"].ravel()
    fwd = np.full(ndof, -1)
    fwd[a] = b
    assert (fwd[a] == b).all(), "one of our dofs maps to two reference dofs"
    assert np.unique(fwd).size == ndof, "not a bijection"


def test_numbering_rejects_bad_vertices():
    L = _lib.load()
    hexes = np.full((1, 8), 5, dtype=np.int32)
    nodle = np.zeros((1, 8), dtype=np.int32)
    nd = ctypes.c_int()
    assert L.mj_number_hex_mesh(1, 1, 4, _lib.iptr(hexes), _lib.iptr(nodle), ctypes.byref(nd)) == _lib.MJ_ERR_ARG


def test_lumped_mass_matches_reference(golden_case):
    name, g = golden_case
    D = problem.lumped_mass(int(g["order"]), g["nodle"], g["jw"], g["massD"].size)
    assert rel_l2(D, g["massD"]) < 1e-15


def test_pulse_and_source_match_reference(golden_case):
    name, g = golden_case
    p = problem.ricker_pulse(float(g["f0"]), float(g["t0"]), float(g["dt"]), int(g["nsteps"]), float(g["eps_time"]),
                             float(g["tlimit"]))
    assert rel_l2(p, g["pulse"]) < 1e-12
    r = int(g["order"])
    _, _, xq = oc.geometry(r, g["verts_e"], np.ones(g["verts_e"].shape[0]))
    idx, val = problem.gaussian_source(g["nodle"], g["jw"], xq, g["massD"].size, g["src_center"],
                                       float(g["src_radius"]))
    assert (idx == np.sort(g["src_idx"])).all()
    ref = dict(zip(g["src_idx"].tolist(), g["src_val"].tolist()))
    assert rel_l2(val, np.array([ref[i] for i in idx])) < 1e-14


def test_host_rules_match_oracle():
    for r in range(1, 9):
        p, w = problem.gauss_lobatto(r)
        po, wo = oc.gauss_lobatto(r)
        assert np.abs(p - po).max() < 1e-15 and np.abs(w - wo).max() < 1e-15
        assert np.abs(problem.derivative_matrix(p) - oc.grad_matrix(r)).max() < 1e-11
        assert (problem.local_numbering(r).ravel() == oc.hex_numbering(r)).all()


def test_receiver_weights_match_oracle():
    g = load_golden("cube3_q4")
    r = int(g["order"])
    rng = np.random.default_rng(5)
    pts = rng.uniform(0.05, 0.95, size=(6, 3))
    idx, w = problem.receiver_weights(r, g["verts_e"], g["nodle"], pts)
    assert np.allclose(w.sum(axis=1), 1.0, atol=1e-12)
    for k, p in enumerate(pts):
        e = int(np.nonzero((g["nodle"] == idx[k]).all(axis=1))[0][0])
        wo, xi, inside = oc.point_weights(r, g["verts_e"][e], p)
        assert inside and np.abs(wo - w[k]).max() < 1e-12


def _cpp_blocks(markdown):
    out, cur = [], None
    for line in markdown.splitlines():
        if line.startswith("```cpp"):
            cur = []
        elif line.startswith("```") and cur is not None:
            out.append(cur)
            cur = None
        elif cur is not None:
            cur.append(line)
    return out


def test_integration_code_is_the_compiled_dropin():
    """Every C++ block of INTEGRATION.md sections 1-2 (the operator subclass,
    its installation, the order-2 loop and its order-4 variant) appears line
    for line in oracle/dropin.cc, the file the drop-in build compiles."""
    md = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sections = md.split("## 2b.")[0]
    src = [l.strip() for l in open(os.path.join(ROOT, "oracle", "dropin.cc")).read().splitlines() if l.strip()]
    blocks = _cpp_blocks(sections)
    assert len(blocks) == 4
    for block in blocks:
        lines = [l.strip() for l in block if l.strip()]
        while lines and lines[0].startswith("//"):  # a context comment above the code
            lines.pop(0)
        starts = [i for i, l in enumerate(src) if l == lines[0]]
        assert any(src[i:i + len(lines)] == lines for i in starts), lines[0]


def test_dropin_links_with_the_library():
    """oracle/_ref/dropin (built by __graft_entry__.build() where the reference
    checkout is present): the binding compiled against the reference's
    headers, whose mj_ symbols all resolve from libmontjoie_gb300.so."""
    import shutil
    import subprocess
    exe = os.path.join(ROOT, "oracle", "_ref", "dropin")
    if not os.path.exists(exe):
        import __graft_entry__ as ge
        ref = ge.reference_root()
        if not os.path.isdir(os.path.join(ref, "MONTJOIE", "src")):
            pytest.skip("no reference checkout here: the drop-in is built where the reference is")
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin", f"REF={ref}"], check=True)
    if not shutil.which("nm") or not shutil.which("ldd"):
        pytest.skip("binutils absent")
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    lib_line = [l for l in ldd.splitlines() if "libmontjoie_gb300.so" in l]
    assert lib_line and "not found" not in lib_line[0]
    und = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    used = {l.split()[-1] for l in und.splitlines() if l.split() and l.split()[-1].startswith("mj_")}
    # mj_op_mltadd is called from the overriding MltAddFree, which the vtable keeps
    assert {"mj_op_create", "mj_op_mltadd", "mj_op_destroy", "mj_lf_create", "mj_lf_run", "mj_lf_destroy",
            "mj_lf_set_scheme", "mj_last_error"} <= used
    exported = subprocess.run(["nm", "-D", "--defined-only", _lib.library_path()], capture_output=True,
                              text=True).stdout
    assert used <= {l.split()[-1] for l in exported.splitlines() if l.split()}
