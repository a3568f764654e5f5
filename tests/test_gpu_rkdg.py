"""FEM_RKDG (P1 discontinuous Galerkin) on the GPU against the reference's own runs and the oracle.

The initial coefficients and cTau equal the reference's bit for bit on every fixture; after
the steps the coefficients, cTau and residuals equal the reference's bit for bit with the LAX
flux, and within 1e-12 of the largest coefficient with the exact Godunov solver (whose exp/log
last bits differ between CUDA and the host libm). The step-0 VTU and PVTU files equal the
reference's byte for byte.
"""
import os

import numpy as np
import pytest

from conftest import load_golden, rkdg_golden_names, rkdg_task
from cfd2d import cases
from cfd2d import meshgen as mg

pytestmark = pytest.mark.gpu

GODUNOV_TOL = 1e-12


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def write_dg_case(tmp_path, task_xml, proc_text):
    (tmp_path / "task.xml").write_text(task_xml)
    (tmp_path / "mesh").mkdir(exist_ok=True)
    (tmp_path / "mesh" / "mesh.0000.proc").write_text(proc_text)
    return str(tmp_path / "task.xml")


def gpu_of(capi, tmp_path, g, inject=True):
    s = capi.Solver(write_dg_case(tmp_path, str(g["task_xml"]), str(g["proc"])))
    if inject and g["U0"].size:
        s.set_dg_coeffs(g["U0"])
    if inject and np.isfinite(g["impose_tau"]):
        s.dg_set_time_step(float(g["impose_tau"]))
    return s


def assert_near(got, ref, flux, what):
    if flux == "LAX":
        assert np.array_equal(bits(got), bits(ref)), what
    else:
        scale = max(float(np.max(np.abs(ref))), 1e-300)
        assert float(np.max(np.abs(got - ref))) <= GODUNOV_TOL * scale, what


@pytest.mark.parametrize("name", rkdg_golden_names())
def test_rkdg_matches_reference_fixture(capi, tmp_path, name):
    g = load_golden(name)
    t = rkdg_task(g)
    s = gpu_of(capi, tmp_path, g)
    assert np.array_equal(bits(s.dg_coeffs()), bits(g["ref_U_init"]))
    assert np.array_equal(bits(s.time_step()), bits(g["ref_cTau_init"]))
    s.step(int(g["steps"]), allow_warnings=False)
    assert_near(s.dg_coeffs(), g["ref_U"], t.flux, "coefficients")
    assert_near(s.time_step(), g["ref_cTau"], t.flux if t.steady else "LAX", "cTau")
    assert_near(s.dg_residuals(), g["ref_res"], t.flux, "residuals")
    assert s.tau == float(g["ref_tau"]) or t.steady


@pytest.mark.parametrize("name", rkdg_golden_names())
def test_rkdg_step0_vtu_equals_reference(capi, tmp_path, name, monkeypatch):
    g = load_golden(name)
    s = gpu_of(capi, tmp_path, g, inject=False)
    monkeypatch.chdir(tmp_path)
    s.save_vtk(0)
    assert (tmp_path / "res_0000000000.pvtu").read_text() == str(g["ref_pvtu0"])
    assert (tmp_path / "vtk_data" / "res_0000000000.0000.vtu").read_text() == str(g["ref_vtu0"])


@pytest.mark.parametrize("flux", ["LAX", "GODUNOV"])
@pytest.mark.parametrize("rk", ["REFERENCE", "HEUN"])
@pytest.mark.parametrize("quad", [(4, 3), (3, 2)])
def test_rkdg_matches_oracle(capi, oracle, tmp_path, flux, rk, quad):
    """A 7,200-triangle vortex with P1 data, 8 steps, every option against the oracle."""
    t, m, pm, U0 = cases.rkdg_vortex(60, flux=flux, rk=rk, gp_cell=quad[0], gp_edge=quad[1], tau=0.004,
                                     kinds=("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP"))
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    o = oracle.OracleDG(t, pm)
    s.set_dg_coeffs(U0)
    o.set_coeffs(U0)
    assert np.array_equal(bits(s.time_step()), bits(o.state()["cTau"]))
    s.step(8)
    o.step(8)
    so = o.state()
    assert_near(s.dg_coeffs(), so["U"], flux, "coefficients")
    assert_near(s.dg_residuals(), so["res"], flux, "residuals")
    assert s.get_info().step == 8 and abs(s.get_info().time - so["t"]) == 0.0


def test_rkdg_steady_time_step_matches_oracle(capi, oracle, tmp_path):
    t, m, pm, U0 = cases.rkdg_vortex(40, flux="LAX", steady=1, cfl=0.05)
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    o = oracle.OracleDG(t, pm)
    s.set_dg_coeffs(U0)
    o.set_coeffs(U0)
    s.step(3)
    o.step(3)
    assert np.array_equal(bits(s.time_step()), bits(o.state()["cTau"]))
    assert np.array_equal(bits(s.dg_coeffs()), bits(o.state()["U"]))


def test_rkdg_mesh_arrays_equal_mesh_part(capi, tmp_path):
    """cfd2d_create_with_mesh numbers edges as the part writer does: the same results."""
    t, m, pm, U0 = cases.rkdg_quadrants(12, flux="LAX")
    a = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    m2 = mg.Mesh(pm.nodes, pm.tris, m.cell_region, m.bsegs, m.bseg_bnd)  # the part's (rounded) coordinates
    b = capi.Solver(str(tmp_path / "task.xml"), mesh=m2)
    a.step(4)
    b.step(4)
    assert np.array_equal(bits(a.dg_coeffs()), bits(b.dg_coeffs()))


def test_rkdg_state_exchange(capi, tmp_path):
    t, m, pm, U0 = cases.rkdg_vortex(10, flux="LAX")
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    s.set_dg_coeffs(U0)
    assert np.array_equal(s.dg_coeffs(), U0)
    # cell-centre values: the polynomial at the centre is the first coefficient
    U = s.state()
    assert np.array_equal(U, U0[:, 0::3].T)
    # set_state: piecewise constant coefficients
    s.set_state(U * 1.01)
    C = s.dg_coeffs()
    assert np.array_equal(C[:, 0::3].T, U * 1.01) and not C[:, 1::3].any() and not C[:, 2::3].any()


def test_rkdg_errors(capi, tmp_path):
    t, m, pm, _ = cases.rkdg_quadrants(4)
    t.func_count = 6
    with pytest.raises(capi.CfdError) as e:
        capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    assert e.value.code == 2
    t.func_count = 3
    (tmp_path / "task.xml").write_text(mg.write_rkdg_task_xml(t))
    os.remove(tmp_path / "mesh" / "mesh.0000.proc")
    with pytest.raises(capi.CfdError) as e:
        capi.Solver(str(tmp_path / "task.xml"))
    assert e.value.code == 301
    pm.cell_names[3] = "nowhere"
    with pytest.raises(capi.CfdError) as e:
        capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    assert e.value.code == 3
    t.steady = 1
    pm.cell_names[3] = pm.cell_names[4]
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    with pytest.raises(capi.CfdError) as e:
        s.run()
    assert e.value.code == 6


def test_rkdg_run_loop_files_and_log(capi, tmp_path, monkeypatch, capfd):
    """run(): while t < TMAX with t += TAU, a VTU pair every FILE_OUTPUT_STEP, a log line every
    LOG_OUTPUT_STEP."""
    t, m, pm, _ = cases.rkdg_quadrants(6, flux="LAX", tau=1e-3)
    t.tmax = 0.0055
    t.file_output_step = 2
    t.log_output_step = 1
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    monkeypatch.chdir(tmp_path)
    capi.set_verbosity(1)
    try:
        s.run()
    finally:
        capi.set_verbosity(0)
    out = capfd.readouterr().out
    tt, n = 0.0, 0
    while tt < t.tmax:
        tt += 1e-3
        n += 1
    assert s.get_info().step == n == 6
    for k in (0, 2, 4, 6):
        assert (tmp_path / f"res_{k:010d}.pvtu").exists()
        assert (tmp_path / "vtk_data" / f"res_{k:010d}.0000.vtu").exists()
    lines = [ln for ln in out.splitlines() if ln.startswith("step:")]
    tt = 0.0
    want = []
    for k in range(1, n + 1):
        tt += 1e-3
        want.append("step: %d\t\ttime step: %.16f" % (k, tt))
    assert lines == want


def test_rkdg_half_million_cells_properties(capi, tmp_path):
    """524,288 triangles: Heun stages with slip walls keep the mass (sum of J ro0) to rounding."""
    t, m, pm, U0 = cases.rkdg_vortex(512, flux="LAX", rk="HEUN", kinds=("BOUND_WALL_SLIP",), tau=1e-4)
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    s.set_dg_coeffs(U0)
    p = pm.nodes[pm.tris]
    J = 0.5 * np.abs((p[:, 0, 0] - p[:, 2, 0]) * (p[:, 1, 1] - p[:, 2, 1]) -
                     (p[:, 0, 1] - p[:, 2, 1]) * (p[:, 1, 0] - p[:, 2, 0]))
    m0 = float((J * s.dg_coeffs()[:, 0]).sum())
    s.step(3)
    C = s.dg_coeffs()
    assert np.isfinite(C).all()
    assert abs(float((J * C[:, 0]).sum()) - m0) <= 1e-12 * abs(m0)


def test_rkdg_executable_writes_the_reference_files(capi, tmp_path):
    """The stand-alone executable (the reference's main) on a FEM_RKDG task: init's step-0
    files equal the reference's byte for byte, and run() ends with status 0."""
    import subprocess
    from conftest import PKG
    g = load_golden("rkdg_quadrants_lax_3pt")
    write_dg_case(tmp_path, str(g["task_xml"]), str(g["proc"]))
    r = subprocess.run([os.path.join(PKG, "lib", "cfd2d_gpu")], cwd=tmp_path, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "res_0000000000.pvtu").read_text() == str(g["ref_pvtu0"])
    assert (tmp_path / "vtk_data" / "res_0000000000.0000.vtu").read_text() == str(g["ref_vtu0"])
    assert "UNSTEADY. Proc =    0. Time step TAU = 1.000000e-03." in r.stdout


def test_rkdg_restart_resumes_bit_for_bit(capi, tmp_path):
    """cfd2d_save_state / cfd2d_load_state on a FEM_RKDG handle: 3 steps, save, 3 more; a new
    handle loading the file and taking 3 steps ends on the same coefficients, time and step."""
    t, m, pm, U0 = cases.rkdg_vortex(20, flux="GODUNOV", steady=1, cfl=0.05)
    task = write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm))
    a = capi.Solver(task)
    a.set_dg_coeffs(U0)
    a.step(3)
    a.save_state(str(tmp_path / "dg.state"))
    a.step(3)
    b = capi.Solver(task)
    b.load_state(str(tmp_path / "dg.state"))
    assert b.get_info().step == 3
    b.step(3)
    assert np.array_equal(bits(a.dg_coeffs()), bits(b.dg_coeffs()))
    assert np.array_equal(bits(a.time_step()), bits(b.time_step()))
    assert b.get_info().step == 6 and b.get_info().time == a.get_info().time


def test_rkdg_reports_a_nonphysical_state(capi, tmp_path):
    """A negative density injected into the coefficients: the step returns
    CFD2D_ERR_NONPHYSICAL (the state is still advanced) and the handle stays usable."""
    t, m, pm, U0 = cases.rkdg_vortex(10, flux="LAX")
    s = capi.Solver(write_dg_case(tmp_path, mg.write_rkdg_task_xml(t), mg.write_proc(pm)))
    bad = U0.copy()
    bad[7, 0] = -1.0
    s.set_dg_coeffs(bad)
    rc = s.step(1, allow_warnings=True)
    assert rc == capi.ERR_NONPHYSICAL
    s.set_dg_coeffs(U0)
    assert s.step(2) == 0
    assert np.isfinite(s.dg_coeffs()).all()


def test_rkdg_full_size_step_equals_oracle(capi, oracle, tmp_path):
    """The bench workload's mesh (1024 x 1024 x 2 = 2,097,152 triangles, P1 vortex, LAX): one
    step through cfd2d_create_with_mesh equals the oracle's bit for bit."""
    t, m, pm, U0 = cases.rkdg_vortex(1024, flux="LAX")
    (tmp_path / "task.xml").write_text(mg.write_rkdg_task_xml(t))
    mesh = mg.Mesh(pm.nodes, pm.tris, m.cell_region, m.bsegs, m.bseg_bnd)
    s = capi.Solver(str(tmp_path / "task.xml"), mesh=mesh)
    s.set_dg_coeffs(U0)
    s.step(1)
    o = oracle.OracleDG(t, pm)
    o.set_coeffs(U0)
    o.step(1)
    assert np.array_equal(bits(s.dg_coeffs()), bits(o.state()["U"]))


def test_rkdg_numeric_edge_types_bind_like_names(capi, oracle, tmp_path):
    """Boundary edges typed by number (bound to <boundCond edgeType>) and by name (TYPE_NAMED,
    bound by <name>) give the same run; both equal the oracle."""
    t, m, pm, U0 = cases.rkdg_vortex(16, flux="LAX",
                                     kinds=("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP"))
    pm_num = mg.proc_mesh(m, [r.name for r in t.regions], bnd_types=[b.edge_type for b in t.boundaries])
    assert set(pm_num.edge_type[pm_num.edge_type != 0]) == {1, 2, 3, 4}
    out = []
    for k, part in enumerate((pm, pm_num)):
        d = tmp_path / str(k)
        d.mkdir()
        s = capi.Solver(write_dg_case(d, mg.write_rkdg_task_xml(t), mg.write_proc(part)))
        s.set_dg_coeffs(U0)
        s.step(4)
        out.append(s.dg_coeffs())
    o = oracle.OracleDG(t, pm_num)
    o.set_coeffs(U0)
    o.step(4)
    assert np.array_equal(bits(out[0]), bits(out[1]))
    assert np.array_equal(bits(out[1]), bits(o.state()["U"]))
