"""The oracle's FVM_TVD_IMPLICIT against the reference's own (golden fixtures, CPU only).

Pins the restatement of the implicit method: on every fixture (made by
tests/golden/make_golden_implicit.py from the reference's fvm_tvd_implicit.cpp, with
the oracle's GMRES standing in for HYPRE) the oracle reproduces the reference's
state, cTau, flags, CFL number and last solve bit for bit.
"""
import json

import numpy as np
import pytest

from conftest import implicit_golden_names, load_golden
from cfd2d import meshgen as mg


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def implicit_task(g):
    d = json.loads(str(g["task_json"]))
    d["regions"] = [mg.ImplicitRegion(**r) for r in d["regions"]]
    d["boundaries"] = [mg.ImplicitBoundary(**b) for b in d["boundaries"]]
    for k in ("cfl", "smoothing", "limits"):
        d[k] = tuple(d[k])
    d["materials"] = [tuple(m) for m in d["materials"]]
    return mg.ImplicitTask(**d)


def implicit_mesh(g):
    return mg.Mesh(g["nodes"], g["tris"], g["cell_region"], g["bsegs"], g["bseg_bnd"])


def oracle_of(oracle, g):
    t = implicit_task(g)
    U0 = g["U0"] if g["U0"].size else None
    return oracle.implicit_from_task(t, implicit_mesh(g), U0=U0)


def run_to(o, steps, cap=1000):
    """FVM_TVD_IMPLICIT::run's loop: passes until the step counter reaches STEP_MAX (a pass
    whose solve failed in a steady run does not count, :532)."""
    for _ in range(cap):
        if o.info()["step"] >= steps:
            return
        o.step(1)
    raise AssertionError("step counter did not reach STEP_MAX")


@pytest.mark.parametrize("name", implicit_golden_names())
def test_oracle_implicit_bit_exact_vs_reference(oracle, name):
    g = load_golden(name)
    o = oracle_of(oracle, g)
    U, ct, fl = o.state()
    assert bits_equal(U, g["ref_U_init"])
    run_to(o, int(g["steps"]))
    U, ct, fl = o.state()
    info = o.info()
    assert bits_equal(U, g["ref_U"])
    assert bits_equal(ct, g["ref_cTau"])
    assert np.array_equal(fl, g["ref_flags"])
    assert info["iters"] == int(g["ref_iters"])
    assert info["rel"] == float(g["ref_rel"])
    if implicit_task(g).steady:
        assert info["cfl"] == float(g["ref_cfl"])


def test_oracle_gmres_solves_block_system(oracle):
    """orc_gmres_block on a small diagonally dominant block system: the residual it reports
    is the true one and the solution matches a dense solve."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(7))
    nc = 40
    nbr = np.full((nc, 3), -1, np.int32)
    for c in range(nc):
        nbr[c, 0] = (c + 1) % nc
        nbr[c, 1] = (c - 1) % nc
    diag = rng.normal(size=(nc, 4, 4)) * 0.1 + np.eye(4) * 4.0
    off = np.zeros((nc, 3, 4, 4))
    off[:, :2] = rng.normal(size=(nc, 2, 4, 4)) * 0.3
    b = rng.normal(size=4 * nc)
    x = np.zeros(4 * nc)
    it, rel = C.c_int(), C.c_double()
    d = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.POINTER(C.c_double))
    st = oracle.lib().orc_gmres_block(nc, nbr.ctypes.data_as(C.POINTER(C.c_int)), d(diag), d(off), d(b), d(x),
                                      1e-10, 200, 30, C.byref(it), C.byref(rel))
    A = np.zeros((4 * nc, 4 * nc))
    for c in range(nc):
        A[4 * c:4 * c + 4, 4 * c:4 * c + 4] = diag[c]
        for k in range(3):
            if nbr[c, k] >= 0:
                A[4 * c:4 * c + 4, 4 * nbr[c, k]:4 * nbr[c, k] + 4] += off[c, k]
    assert st == 0
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) == pytest.approx(rel.value, rel=1e-6)
    assert rel.value < 1e-10
    assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-8, atol=1e-10)
