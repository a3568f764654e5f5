"""The C oracle against the reference's own FVM_TVD (golden fixtures, CPU only).

Pins the oracle: on every fixture the restatement must reproduce the
reference's Grid, TAU and final state bit for bit.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from cfd2d import meshgen as mg


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def task_of(g):
    """Rebuild the fixture's Task description from its XML (the fields the oracle needs)."""
    import xml.etree.ElementTree as ET
    root = ET.fromstring(str(g["task_xml"]))
    ctl = root.find("control")
    v = lambda n, a="value": float(n.get(a))
    mats = [("m", v(m.find("parameters/M")), v(m.find("parameters/Cp")), 0.0, 0.0)
            for m in root.find("materials").findall("material")]
    regs = [mg.Region(r.find("name").text, v(r.find("parameters/Vx")), v(r.find("parameters/Vy")),
                      v(r.find("parameters/T")), v(r.find("parameters/P")), int(r.find("material").get("id")))
            for r in root.find("regions").findall("region")]
    bnds = []
    for b in root.find("boundaries").findall("boundCond"):
        p = b.find("parameters")
        vals = [v(p.find(k)) for k in ("Vx", "Vy", "T", "P")] if p is not None else [0, 0, 1, 1]
        bnds.append(mg.Boundary(b.find("name").text, b.find("type").text, int(b.get("edgeType")), *vals))
    lim = root.find("limits")
    t = mg.Task(regions=regs, boundaries=bnds, steady=int(ctl.find("STEADY").get("value")),
                tau=v(ctl.find("TAU")), cfl=v(ctl.find("CFL")), step_max=int(ctl.find("STEP_MAX").get("value")),
                limits=(v(lim.find("ro"), "min"), v(lim.find("ro"), "max"), v(lim.find("p"), "min"),
                        v(lim.find("p"), "max"), v(lim.find("u"), "max")), materials=mats)
    return t


def mesh_of(g):
    return mg.Mesh(g["nodes"], g["tris"], g["cell_region"], g["bsegs"], g["bseg_bnd"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_mesh_matches_reference_grid(oracle, name):
    g = load_golden(name)
    om = oracle.OracleMesh.from_mesh(mesh_of(g)).export()
    for k in ("cell_edges", "cell_S", "cell_c", "edge_n12", "edge_c12", "edge_npts", "edge_n", "edge_l", "edge_pts"):
        assert bits_equal(om[k], g["grid_" + k]), k
    # boundary binding: the fixture's boundary index per edge
    assert np.array_equal(om["edge_bnd"], g["grid_edge_bnd"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_state_bit_exact_vs_reference(oracle, name):
    g = load_golden(name)
    t = task_of(g)
    U0 = g["U0"] if g["U0"].size else None
    s = oracle.solver_from_task(t, mesh_of(g), U0=U0)
    assert s.tau == g["ref_tau"]
    Ui, _, _ = s.state()
    assert bits_equal(Ui, g["ref_U_init"])
    s.step(int(g["steps"]))
    U, ct, fl = s.state()
    assert bits_equal(U, g["ref_U"])
    assert bits_equal(ct, g["ref_cTau"])
    assert np.array_equal(fl, g["ref_flags"])


def test_limits_fixture_exercises_remediation(oracle):
    """vortex_limits must flag cells, keep them 0x20 steps and release them."""
    g = load_golden("vortex_limits")
    t = task_of(g)
    s = oracle.solver_from_task(t, mesh_of(g), U0=g["U0"])
    s.step(1)
    _, _, fl = s.state()
    assert ((fl & 2) > 0).sum() > 0
    s.step(31)
    _, _, fl = s.state()
    assert ((fl & 2) > 0).sum() == 0
