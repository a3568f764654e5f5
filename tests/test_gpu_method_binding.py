"""The reference-side binding on the GPU: the FVM_TVD_GPU Method subclass
(oracle/dropin/fvm_tvd_gpu.h), created by a main that follows the reference's
src/main.cpp and Solver::initMethod, driven through Method::init/run/done on reference
tasks, writes the files the reference wrote for them.

Built on this machine from the subclass and the stand-in Method interface
(oracle/dropin/iface: the reference's method.h is not shipped here), plus, where the
reference's source tree is present (CFD2D_REFERENCE_SRC), against the reference's own
headers and objects; tests/test_method_binding.py builds both on any machine.
"""
import os
import subprocess

import pytest

from conftest import ROOT, load_golden, write_case

pytestmark = pytest.mark.gpu

ORACLE = os.path.join(ROOT, "oracle")
REF = os.environ.get("CFD2D_REFERENCE_SRC", "")


def _executables():
    r = subprocess.run(["make", "-C", ORACLE, "dropin-standin"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    exes = [os.path.join(ORACLE, "build", "cfd2d_dropin_standin")]
    if REF and os.path.isdir(os.path.join(REF, "src", "methods")):
        r = subprocess.run(["make", "-C", ORACLE, "dropin"], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        exes.append(os.path.join(ORACLE, "_ref", "cfd2d_dropin"))
    return exes


def _same_vtk(got: str, ref: str, rel=1e-12):
    """Same lines and words; numbers within the FP64 bar (the exact Godunov solver's
    exp/log last bits differ between CUDA and the host libm)."""
    gl, rl = got.split("\n"), ref.split("\n")
    assert len(gl) == len(rl)
    for a, b in zip(gl, rl):
        ta, tb = a.split(" "), b.split(" ")
        assert len(ta) == len(tb)
        for x, y in zip(ta, tb):
            if x != y:
                assert abs(float(x) - float(y)) <= rel * max(abs(float(y)), 1.0), (x, y)


def test_fvm_tvd_task_through_the_method_subclass(capi, tmp_path):
    """FVM_TVD task (two regions, all four boundary kinds, Godunov + Heun, 20 steps): the
    initial file byte for byte, the last one (the final state) to the FP64 bar, the log
    lines of FVM_TVD::run."""
    g = load_golden("shock_tube_4bc")
    for k, exe in enumerate(_executables()):
        d = tmp_path / str(k)
        d.mkdir()
        write_case(d, g)
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        for name, text in zip(g["ref_vtk_names"], g["ref_vtk"]):
            got = (d / str(name)).read_text()
            if str(name) == "res_0000000000.vtk":
                assert got == str(text)
            else:
                _same_vtk(got, str(text))
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith(("time step:", "step:", "File '"))]
        assert lines == str(g["ref_log"]).splitlines()


def test_fem_rkdg_task_through_the_method_subclass(capi, tmp_path):
    """FEM_RKDG task on a DECOMP mesh part: the initial PVTU/VTU pair byte for byte and the
    reference's time-step line."""
    g = load_golden("rkdg_quadrants_lax_3pt")
    for k, exe in enumerate(_executables()):
        d = tmp_path / str(k)
        (d / "mesh").mkdir(parents=True)
        (d / "task.xml").write_text(str(g["task_xml"]))
        (d / "mesh" / "mesh.0000.proc").write_text(str(g["proc"]))
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert (d / "res_0000000000.pvtu").read_text() == str(g["ref_pvtu0"])
        assert (d / "vtk_data" / "res_0000000000.0000.vtu").read_text() == str(g["ref_vtu0"])
        assert "UNSTEADY. Proc =    0. Time step TAU = 1.000000e-03." in r.stdout


def test_library_error_through_the_method_subclass(capi, tmp_path):
    """A task the library rejects (a boundary condition of unknown type, the reference's
    error 102) ends the program the reference's way: the message by log(), EXIT(1)."""
    g = load_golden("shock_tube_4bc")
    for k, exe in enumerate(_executables()):
        d = tmp_path / str(k)
        d.mkdir()
        write_case(d, g)
        xml = (d / "task.xml").read_text()
        assert "BOUND_OUTLET" in xml
        (d / "task.xml").write_text(xml.replace("BOUND_OUTLET", "BOUND_NOWHERE", 1))
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=120)
        assert r.returncode == 1 and r.stdout.startswith("ERROR: "), r.stdout + r.stderr
        assert (d / "task.log").read_text().startswith("ERROR: ")
