"""FVM_TVD_IMPLICIT on the GPU against the oracle and the reference's own runs.

The block system (diagonal and face blocks, right-hand side, cTau) equals the oracle's
bit for bit (the Godunov right-hand side within 1e-12: CUDA's exp/log); states after
the reference's run loop match the reference's fixtures within 1e-10 relative (the
GMRES reductions run in a different order on the GPU) with the same flags, CFL number
and iteration counts.
"""
import os

import numpy as np
import pytest

from conftest import implicit_golden_names, load_golden, write_case
from test_oracle_implicit import implicit_mesh, implicit_task, oracle_of, run_to
from cfd2d import meshgen as mg

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def gpu_of(capi, tmp_path, g, inject=True):
    s = capi.Solver(write_case(tmp_path, g))
    if inject and g["U0"].size:
        s.set_state(g["U0"])
    return s


def gpu_run_to(s, steps, cap=1000):
    for _ in range(cap):
        if s.get_info().step >= steps:
            return
        s.step(1)
    raise AssertionError("step counter did not reach STEP_MAX")


def close(a, b):
    """max |a - b| relative to |b|, with entries near zero measured against 1e-3 of their row's largest"""
    scale = np.maximum(np.abs(b), np.abs(b).max(axis=-1, keepdims=True) * 1e-3)
    scale = np.where(scale > 0, scale, 1.0)
    return float(np.max(np.abs(a - b) / scale))


@pytest.mark.parametrize("name", implicit_golden_names())
def test_implicit_system_equals_oracle(capi, oracle, tmp_path, name):
    g = load_golden(name)
    s = gpu_of(capi, tmp_path, g)
    o = oracle_of(oracle, g)
    D, O, b, ct = s.implicit_system()
    D2, O2, b2, ct2 = o.system()
    assert np.array_equal(D, D2)  # (== on values: the sign of a zero block entry is free)
    assert np.array_equal(O, O2)
    assert np.array_equal(ct, ct2)
    if implicit_task(g).flux == "GODUNOV":
        assert close(b, b2) < 1e-12
    else:
        assert np.array_equal(b.view(np.int64), b2.view(np.int64))
    # the state is not advanced by the query
    assert np.array_equal(s.state(), g["U0"] if g["U0"].size else g["ref_U_init"])


@pytest.mark.parametrize("name", implicit_golden_names())
def test_implicit_run_matches_reference(capi, tmp_path, name):
    g = load_golden(name)
    s = gpu_of(capi, tmp_path, g)
    gpu_run_to(s, int(g["steps"]))
    st = s.implicit_stats()
    U = s.state()
    assert close(U, g["ref_U"]) < RTOL
    assert np.array_equal(s.flags(), g["ref_flags"])
    assert close(s.time_step(), g["ref_cTau"]) < RTOL
    assert st["iters"] == int(g["ref_iters"])
    assert st["rel"] == pytest.approx(float(g["ref_rel"]), rel=1e-4)
    if implicit_task(g).steady:
        assert st["cfl"] == float(g["ref_cfl"])


@pytest.mark.parametrize("name", implicit_golden_names())
def test_implicit_vtk_at_start_equals_reference(capi, tmp_path, monkeypatch, name):
    g = load_golden(name)
    s = gpu_of(capi, tmp_path, g, inject=False)
    monkeypatch.chdir(tmp_path)
    s.save_vtk(0)
    assert (tmp_path / "res_0000000000.vtk").read_text() == str(g["ref_vtk0"])


def make_case(tmp_path, n=24, seed=31, **kw):
    kinds = kw.pop("kinds", ("BOUND_INLET",))
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, 0.1, seed)
    m.bseg_bnd = (m.bseg_side % len(kinds)).astype(np.int32)
    bnds = [mg.ImplicitBoundary(edge_type=k + 1, kind=kd, T=1.0, p=1.0, u=1.0, v=0.0) for k, kd in enumerate(kinds)]
    t = mg.ImplicitTask(regions=[mg.ImplicitRegion(cell_type=0, u=1.0, v=0.0, T=1.0, p=1.0)], boundaries=bnds, **kw)
    (tmp_path / "task.xml").write_text(mg.write_implicit_task_xml(t))
    for ext, txt in mg.write_triangle(m, [b.edge_type for b in bnds]).items():
        (tmp_path / ("mesh" + ext)).write_text(txt)
    U0 = mg.isentropic_vortex(m.centroids(), 5.0, 5.0, 5.0)
    return m, t, U0, str(tmp_path / "task.xml")


@pytest.mark.parametrize("kw", [
    dict(flux="LAX", tau=0.1, step_max=3),
    dict(flux="GODUNOV", tau=0.1, step_max=3, kinds=("BOUND_WALL", "BOUND_OUTLET")),
    dict(flux="LAX", tau=0.05, step_max=3, smoothing=(1, 0.3)),
    dict(flux="LAX", steady=1, step_max=5, cfl=(3.0, 1.5, 20.0, 1, 1.0e9), kinds=("BOUND_INLET", "BOUND_OUTLET")),
], ids=["lax", "godunov_wall", "smoothing", "steady_cfl"])
def test_implicit_matches_oracle(capi, oracle, tmp_path, kw):
    """Larger meshes than the fixtures (1152 cells), smoothing (the oracle follows the
    evident intent of smoothingDelta), the CFL rules."""
    m, t, U0, path = make_case(tmp_path, **kw)
    s = capi.Solver(path)
    s.set_state(U0)
    o = oracle.implicit_from_task(t, m, U0=U0)
    for _ in range(t.step_max):
        s.step(1)
        o.step(1)
        st, oi = s.implicit_stats(), o.info()
        assert (st["iters"], st["status"], st["n_lim"]) == (oi["iters"], oi["status"], oi["n_lim"])
        if t.steady:
            assert st["cfl"] == oi["cfl"]
    U, ct, fl = o.state()
    assert close(s.state(), U) < RTOL
    assert np.array_equal(s.flags(), fl)
    assert s.get_info().step == oi["step"]


def test_implicit_mesh_arrays_equal_mesh_files(capi, tmp_path):
    """cfd2d_create_with_mesh builds the same Triangle topology from arrays."""
    m, t, U0, path = make_case(tmp_path, n=12, flux="LAX", tau=0.1, step_max=2)
    a = capi.Solver(path)
    b = capi.Solver(path, mesh=m)
    for s in (a, b):
        s.set_state(U0)
        s.step(2)
    assert np.array_equal(a.state(), b.state())


def test_implicit_handle_rejects_explicit_entry_points(capi, tmp_path):
    m, t, U0, path = make_case(tmp_path, n=6, flux="LAX", tau=0.1, step_max=2)
    s = capi.Solver(path)
    with pytest.raises(capi.CfdError) as e:
        s.residual()
    assert e.value.code == 6
    info = s.get_info()
    assert info.n_cells == 72 and info.step == 0


def test_implicit_run_writes_reference_log(capi, tmp_path, monkeypatch):
    """run(): the loop while t < TMAX and step < STEP_MAX with the reference's output cadence."""
    m, t, U0, path = make_case(tmp_path, n=8, flux="LAX", tau=0.1, step_max=4, file_output_step=2,
                               log_output_step=1)
    monkeypatch.chdir(tmp_path)
    s = capi.Solver(path)
    s.run()
    assert s.get_info().step == 4
    names = sorted(p for p in os.listdir(tmp_path) if p.endswith(".vtk"))
    assert names == ["res_0000000000.vtk", "res_0000000002.vtk", "res_0000000004.vtk"]


@pytest.mark.parametrize("name", implicit_golden_names())
def test_implicit_run_loop_equals_reference(capi, tmp_path, monkeypatch, name):
    """cfd2d_run: FVM_TVD_IMPLICIT::run's loop (t < TMAX, step < STEP_MAX, failed steady solves
    not counted) reaches the reference's final state."""
    g = load_golden(name)
    s = gpu_of(capi, tmp_path, g)
    monkeypatch.chdir(tmp_path)
    s.run()
    assert s.get_info().step == int(g["steps"])
    assert close(s.state(), g["ref_U"]) < RTOL
    assert np.array_equal(s.flags(), g["ref_flags"])


def test_implicit_restart_is_bit_exact(capi, tmp_path):
    """cfd2d_save_state / cfd2d_load_state on an implicit handle (steady: the CFL number and the
    solve status travel with the state): the resumed run equals the uninterrupted one bit for bit."""
    m, t, U0, path = make_case(tmp_path, n=16, flux="LAX", steady=1, step_max=8,
                               cfl=(3.0, 1.5, 20.0, 1, 1.0e9), kinds=("BOUND_INLET", "BOUND_OUTLET"))
    a = capi.Solver(path)
    a.set_state(U0)
    a.step(3)
    a.save_state(str(tmp_path / "r.bin"))
    a.step(3)
    b = capi.Solver(path)
    b.load_state(str(tmp_path / "r.bin"))
    b.step(3)
    assert np.array_equal(a.state(), b.state())
    assert np.array_equal(a.time_step(), b.time_step())
    assert a.get_info().step == b.get_info().step
    assert a.implicit_stats()["cfl"] == b.implicit_stats()["cfl"]


@pytest.mark.parametrize("gm", [(3, 40, 1e-7), (4, 40, 1e-7), (2, 60, 1e-8), (5, 12, 1e-9)],
                         ids=["k3", "k4", "k2", "k5_iteration_limit"])
def test_implicit_restarted_gmres_matches_oracle(capi, oracle, tmp_path, gm):
    """<GMRES krylov max_iter tolerance> (an extension; the reference fixes 30, 20, 1e-7): a small
    Krylov dimension makes the solver restart from the true residual, on the device (the
    restart graph) and in the oracle alike."""
    m, t, U0, path = make_case(tmp_path, n=16, flux="LAX", tau=0.1, step_max=3, gmres=gm)
    s = capi.Solver(path)
    s.set_state(U0)
    o = oracle.implicit_from_task(t, m, U0=U0)
    for _ in range(t.step_max):
        s.step(1)
        o.step(1)
        st, oi = s.implicit_stats(), o.info()
        assert (st["iters"], st["status"]) == (oi["iters"], oi["status"])
        assert st["rel"] == pytest.approx(oi["rel"], rel=1e-3, abs=1e-14)
    assert st["iters"] > gm[0]  # at least one restart happened
    U, ct, fl = o.state()
    assert close(s.state(), U) < RTOL


@pytest.mark.parametrize("bad", ["nan", "negative_density"])
def test_implicit_nonphysical_state_is_reported(capi, tmp_path, bad):
    """A NaN or negative density in the state makes the step return CFD2D_ERR_NONPHYSICAL; the
    handle stays usable and a good state then steps cleanly."""
    m, t, U0, path = make_case(tmp_path, n=8, flux="LAX", tau=0.05, step_max=2)
    s = capi.Solver(path)
    U = U0.copy()
    U[0, 5] = np.nan if bad == "nan" else -1.0
    s.set_state(U)
    assert s.step(1, allow_warnings=True) == capi.ERR_NONPHYSICAL
    s.set_state(U0)
    assert s.step(1) == capi.OK
    assert np.all(np.isfinite(s.state()))


def test_implicit_full_size_step_matches_oracle(capi, oracle, tmp_path):
    """The bench workload itself (2,097,152 triangles, LAX, TAU 0.002): the assembled system equals
    the oracle's bit for bit and one step agrees within 1e-10 with the same GMRES iteration count."""
    from cfd2d import cases
    t, m, U0 = cases.vortex_implicit(1024, flux="LAX", tau=0.002)
    s = capi.Solver(cases.write_implicit_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0)
    o = oracle.implicit_from_task(t, m, U0=U0)
    D, O, b, ct = s.implicit_system()
    D2, O2, b2, ct2 = o.system()
    assert np.array_equal(D, D2) and np.array_equal(O, O2)
    assert np.array_equal(b.view(np.int64), b2.view(np.int64))
    del D, O, D2, O2
    s.step(1)
    o.step(1)
    assert s.implicit_stats()["iters"] == o.info()["iters"]
    assert close(s.state(), o.state()[0]) < RTOL


def test_implicit_steady_run_stops_when_solves_keep_failing(capi, tmp_path, monkeypatch):
    """A steady run whose every solve fails would loop forever in the reference (the step
    counter only advances on success); the library stops with CFD2D_ERR_SOLVER."""
    m, t, U0, path = make_case(tmp_path, n=6, flux="LAX", steady=1, step_max=3, cfl=(2.0, 1.5, 10.0, 1, 1.0e9),
                               gmres=(30, 1, 1e-14))
    monkeypatch.chdir(tmp_path)
    s = capi.Solver(path)
    with pytest.raises(capi.CfdError) as e:
        s.run()
    assert e.value.code == 506
    st = s.implicit_stats()
    assert st["status"] != 0 and st["cfl"] == pytest.approx(0.1)
