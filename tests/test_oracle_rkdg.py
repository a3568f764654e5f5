"""The oracle's FEM_RKDG against the reference's own (golden fixtures, CPU only).

Pins the restatement of the discontinuous Galerkin method: on every fixture (made by
tests/golden/make_golden_rkdg.py from the reference's fem_rkdg.cpp, with its getF made to
return a valid reference) the oracle reproduces the reference's initial coefficients,
cTau, the coefficients after the steps and the residuals bit for bit. Also: the mesh-part
writer and reader, and properties of the Heun variant.
"""
import numpy as np
import pytest

from conftest import load_golden, rkdg_golden_names, rkdg_task
from cfd2d import cases
from cfd2d import meshgen as mg


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def oracle_of(oracle, g, rk=None):
    t = rkdg_task(g)
    pm = mg.read_proc(str(g["proc"]))
    o = oracle.OracleDG(t, pm, rk=rk)
    if g["U0"].size:
        o.set_coeffs(g["U0"])
    if np.isfinite(g["impose_tau"]):
        o.set_tau(float(g["impose_tau"]))
    return o, t, pm


@pytest.mark.parametrize("name", rkdg_golden_names())
def test_oracle_rkdg_bit_exact_vs_reference(oracle, name):
    g = load_golden(name)
    o, t, pm = oracle_of(oracle, g)
    s0 = o.state()
    assert bits_equal(s0["U"], g["ref_U_init"])
    assert bits_equal(s0["cTau"], g["ref_cTau_init"])
    o.step(int(g["steps"]))
    s = o.state()
    assert bits_equal(s["U"], g["ref_U"])
    assert bits_equal(s["cTau"], g["ref_cTau"])
    assert bits_equal(s["res"], g["ref_res"])
    assert s["tau"] == float(g["ref_tau"])
    assert not np.array_equal(s["U"], s0["U"])  # the state moved


def test_rkdg_fixture_coverage():
    """The fixtures cover both fluxes, both cell and both edge quadratures, steady and
    unsteady runs, the four boundary kinds, two materials and P1 data with slopes."""
    seen = set()
    for name in rkdg_golden_names():
        g = load_golden(name)
        t = rkdg_task(g)
        seen |= {("flux", t.flux), ("gc", t.gp_cell), ("ge", t.gp_edge), ("steady", t.steady),
                 ("mats", len(t.materials)), ("slopes", bool(g["U0"].size))}
        seen |= {("bnd", b.kind) for b in t.boundaries}
    for item in [("flux", "GODUNOV"), ("flux", "LAX"), ("gc", 3), ("gc", 4), ("ge", 2), ("ge", 3), ("steady", 0),
                 ("steady", 1), ("mats", 2), ("slopes", True), ("bnd", "BOUND_INLET"), ("bnd", "BOUND_OUTLET"),
                 ("bnd", "BOUND_WALL_SLIP"), ("bnd", "BOUND_WALL_NO_SLIP")]:
        assert item in seen, item


def test_proc_writer_reader_round_trip():
    t, m, pm, _ = cases.rkdg_quadrants(5)
    txt = mg.write_proc(pm)
    back = mg.read_proc(txt)
    assert np.array_equal(back.nodes, pm.nodes) and np.array_equal(back.tris, pm.tris)
    assert np.array_equal(back.edges, pm.edges) and np.array_equal(back.edge_type, pm.edge_type)
    assert back.cell_names == pm.cell_names and back.edge_names == pm.edge_names
    # every side of every cell is an edge, each edge is on one or two cells
    key = lambda a, b: (min(a, b), max(a, b))
    edges = {key(a, b) for a, b in pm.edges}
    assert len(edges) == len(pm.edges)
    sides = [key(c[j], c[(j + 1) % 3]) for c in pm.tris for j in range(3)]
    assert set(sides) == edges
    nb = (pm.edge_type != 0).sum()
    assert nb == 4 * 5


def test_oracle_rkdg_heun_keeps_a_uniform_stream(oracle):
    """P1 DG keeps a uniform state uniform (Heun stages, inlet boundaries with the same state)."""
    t, m, pm, _ = cases.rkdg_vortex(6, rk="HEUN")
    o = oracle.OracleDG(t, pm)
    U0 = o.state()["U"]
    o.step(5)
    U = o.state()["U"]
    assert np.abs(U - U0).max() < 1e-12


def test_oracle_rkdg_heun_conserves_mass_with_walls(oracle):
    """With slip walls all round, Heun stages keep sum_i J_i ro_i[0] (the cell means) to rounding."""
    t, m, pm, U0 = cases.rkdg_vortex(8, rk="HEUN", kinds=("BOUND_WALL_SLIP",), tau=0.005)
    o = oracle.OracleDG(t, pm)
    o.set_coeffs(U0)
    J = o.geom()["cell6"][:, 5]
    m0 = float((J * o.state()["U"][:, 0]).sum())
    o.step(6)
    m1 = float((J * o.state()["U"][:, 0]).sum())
    assert abs(m1 - m0) <= 1e-12 * abs(m0)


def test_oracle_rkdg_reference_mode_differs_from_heun(oracle):
    """The reference's second stage (average with the first stage's result, shared ro_old for
    the first half of the cells) is not Heun's: the two modes part after one step."""
    t, m, pm, U0 = cases.rkdg_vortex(6)
    a = oracle.OracleDG(t, pm, rk="REFERENCE"); a.set_coeffs(U0); a.step(1)
    b = oracle.OracleDG(t, pm, rk="HEUN"); b.set_coeffs(U0); b.step(1)
    assert not np.array_equal(a.state()["U"], b.state()["U"])


def test_proc_part_with_numeric_edge_types_round_trip():
    t, m, pm, _ = cases.rkdg_quadrants(5)
    pm_num = mg.proc_mesh(m, [r.name for r in t.regions], bnd_types=[b.edge_type for b in t.boundaries])
    back = mg.read_proc(mg.write_proc(pm_num))
    assert np.array_equal(back.edge_type, pm_num.edge_type) and back.edge_names == pm_num.edge_names
    assert set(back.edge_type[back.edge_type != 0]) == {b.edge_type for b in t.boundaries}
