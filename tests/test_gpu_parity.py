"""GPU parity: the CUDA path (through the C ABI) against the reference and the oracle.

Bar: FP64 results equal the reference's bit for bit wherever only +,-,*,/ and
sqrt are involved (every flux but the exact Godunov solver, whose exp/log come
from a different math library on each side: there the tolerance is 1e-12
relative, the target the method states). The mixed form is held to 1e-6
relative L1 density/energy error against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, write_case
from cfd2d import cases
from test_oracle_golden import bits_equal, mesh_of, task_of

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def l1_rel(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


@pytest.mark.parametrize("name", golden_names())
def test_reference_fixture_drop_in(capi, tmp_path, name):
    """task.xml + UNV through cfd2d_create: the reference's own outputs."""
    g = load_golden(name)
    s = capi.Solver(write_case(tmp_path, g))
    if g["U0"].size:
        s.set_state(g["U0"], reset_time_step=True)
    assert s.tau == g["ref_tau"]
    assert bits_equal(s.state(), g["ref_U_init"])
    s.step(int(g["steps"]))
    U = s.state()
    assert rel_err(U, g["ref_U"]) <= FP64_TOL
    assert rel_err(s.time_step(), g["ref_cTau"]) <= FP64_TOL
    assert np.array_equal(s.flags(), g["ref_flags"])


def test_reference_fixture_berkeley_triangle(capi, tmp_path):
    g = load_golden("berkeley_triangle")
    s = capi.Solver(write_case(tmp_path, g))
    assert s.tau == g["ref_tau"]
    s.step(int(g["steps"]))
    assert bits_equal(s.state(), g["ref_U"])  # one point per edge: no flux, as in the reference


FLUXES = ["LAX", "ROE", "HLLC", "GODUNOV"]
RECONS = ["NONE", "LINEAR", "MINMOD"]
SCHEMES = ["EULER", "HEUN", "SSPRK3"]
KINDS = ("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP")


def _oracle_for(oracle, t, m, U0):
    return oracle.solver_from_task(t, m, U0=U0, flux=t.flux, recon=t.reconstruction, scheme=t.time_scheme)


@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("scheme", SCHEMES)
def test_methods_vs_oracle_fp64(capi, oracle, tmp_path, flux, recon, scheme):
    t, m, U0 = cases.vortex(12, flux=flux, recon=recon, scheme=scheme, steps=8, bnd_kinds=KINDS, seed=7)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0, reset_time_step=True)
    o = _oracle_for(oracle, t, m, U0)
    assert s.tau == o.tau
    s.step(t.step_max)
    o.step(t.step_max)
    Uo, cto, flo = o.state()
    U = s.state()
    if flux == "GODUNOV":
        assert rel_err(U, Uo) <= FP64_TOL
    else:
        assert bits_equal(U, Uo)
    assert np.array_equal(s.flags(), flo)


@pytest.mark.parametrize("flux", ["LAX", "ROE", "HLLC"])
def test_local_time_step_vs_oracle(capi, oracle, tmp_path, flux):
    t, m, U0 = cases.vortex(12, flux=flux, recon="MINMOD", scheme="SSPRK3", steps=6, steady=1, seed=8)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0, reset_time_step=True)
    o = _oracle_for(oracle, t, m, U0)
    s.step(t.step_max); o.step(t.step_max)
    Uo, cto, _ = o.state()
    assert bits_equal(s.state(), Uo)
    assert bits_equal(s.time_step(), cto)


@pytest.mark.parametrize("flux", ["LAX", "HLLC", "ROE"])
def test_residual_vs_oracle(capi, oracle, tmp_path, flux):
    t, m, U0 = cases.vortex(10, flux=flux, recon="MINMOD", scheme="SSPRK3", bnd_kinds=KINDS, seed=9)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0)
    o = _oracle_for(oracle, t, m, U0)
    assert bits_equal(s.residual(), o.residual())


def test_plain_vortex_lf_euler_full_length(capi, oracle, tmp_path):
    """20,000-triangle vortex, LF first order, explicit Euler, CFL 0.5, 200 steps, FP64."""
    t, m, U0 = cases.vortex(100, flux="LAX", recon="NONE", scheme="EULER", cfl=0.5, steps=200, seed=1)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0, reset_time_step=True)
    o = _oracle_for(oracle, t, m, U0)
    s.step(200); o.step(200)
    Uo, _, _ = o.state()
    U = s.state()
    assert bits_equal(U[0], Uo[0]) and bits_equal(U[3], Uo[3])
    assert bits_equal(U, Uo)


def test_mixed_precision_vs_fp64_oracle(capi, oracle, tmp_path):
    t, m, U0 = cases.vortex(24, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=40, seed=10,
                            precision="MIXED")
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0, reset_time_step=True)
    o = _oracle_for(oracle, t, m, U0)
    s.step(t.step_max); o.step(t.step_max)
    Uo, _, _ = o.state()
    U = s.state()
    assert l1_rel(U[0], Uo[0]) <= MIXED_TOL
    assert l1_rel(U[3], Uo[3]) <= MIXED_TOL
    assert not bits_equal(U, Uo)  # the faces really ran in FP32


def test_four_quadrant_mixed_vs_fp64(capi, tmp_path):
    t, m, _ = cases.four_quadrant(128, steps=50)
    a = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    t.precision = "MIXED"
    b = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    a.step(50); b.step(50)
    Ua, Ub = a.state(), b.state()
    assert l1_rel(Ub[0], Ua[0]) <= MIXED_TOL and l1_rel(Ub[3], Ua[3]) <= MIXED_TOL


def test_deterministic_run_to_run(capi, tmp_path):
    t, m, _ = cases.four_quadrant(64, steps=20)
    p = cases.write_task(t, m, str(tmp_path))
    a = capi.Solver(p, mesh=m); a.step(20)
    b = capi.Solver(p, mesh=m); b.step(20)
    assert bits_equal(a.state(), b.state())


def test_cell_order_does_not_change_results(capi, tmp_path):
    """RCM storage order and the file order give the same bits (fixed gather order)."""
    g = load_golden("shuffled_mesh")
    t, m = task_of(g), mesh_of(g)
    t.flux, t.reconstruction, t.time_scheme = "HLLC", "MINMOD", "SSPRK3"
    xml = cases.write_task(t, m, str(tmp_path))
    a = capi.Solver(xml, mesh=m)
    txt = open(xml).read().replace("<control>", '<control>\n    <REORDER value="NONE" />')
    (tmp_path / "task2.xml").write_text(txt)
    b = capi.Solver(str(tmp_path / "task2.xml"), mesh=m)
    a.step(10); b.step(10)
    assert bits_equal(a.state(), b.state())


def test_state_round_trip_through_permutation(capi, tmp_path):
    g = load_golden("shuffled_mesh")
    s = capi.Solver(write_case(tmp_path, g))
    U = np.random.default_rng(0).uniform(0.5, 2.0, (4, s.n))
    s.set_state(U)
    assert bits_equal(s.state(), U)


def test_mass_conserved_with_walls(capi, tmp_path):
    t, m, U0 = cases.vortex(32, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=50,
                            bnd_kinds=("BOUND_WALL_SLIP",) * 4, seed=11)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_state(U0, reset_time_step=True)
    c0 = s.conservation()
    s.step(50)
    c1 = s.conservation()
    assert abs(c1[0] - c0[0]) <= 1e-13 * abs(c0[0])


def test_newton_cap_reports_instead_of_spinning(capi, tmp_path):
    """p ratio 52 with the unlimited Godunov method hangs the reference
    (negative face pressure in rim_orig's Newton loop); here the loop is capped
    and the call returns a status."""
    t, m, _ = cases.four_quadrant(32, flux="GODUNOV", recon="LINEAR", scheme="HEUN", steps=30)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    rc = s.step(30, allow_warnings=True)
    assert rc in (capi.OK, capi.ERR_NEWTON_CAP, capi.ERR_NONPHYSICAL)


def test_full_size_four_quadrant_step_vs_oracle(capi, oracle, tmp_path):
    """2,097,152 triangles (1024 x 1024 x 2), HLLC + minmod + SSP-RK3: one full step, bit for bit."""
    t, m, _ = cases.four_quadrant(1024, steps=1)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    o = _oracle_for(oracle, t, m, None)
    assert s.tau == o.tau
    s.step(1); o.step(1)
    Uo, _, _ = o.state()
    U = s.state()
    assert bits_equal(U, Uo)
    # checksum of checksums, the mixed form at full size
    t.precision = "MIXED"
    b = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    b.step(1)
    Ub = b.state()
    assert l1_rel(Ub[0], U[0]) <= MIXED_TOL and l1_rel(Ub[3], U[3]) <= MIXED_TOL


@pytest.mark.parametrize("which,name", [(0, "division by reciprocal"), (1, "widening"), (2, "narrowing"),
                                        (3, "minmod sign test")])
def test_device_arithmetic_helpers(capi, which, name):
    """The FP64 division through a precomputed reciprocal must equal '/' bit for
    bit on the device; the integer-pipe conversions must match the hardware's;
    the integer-pipe minmod must equal the reference's expression bit for bit."""
    assert capi.selftest(which, 200_000_000 if which == 0 else 50_000_000, seed=12345) == 0, name
