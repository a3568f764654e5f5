"""The drop-in end to end: cfd-2d_gb300/lib/cfd2d_gpu (the reference's main on the
GPU path) on a reference task, against the reference's own outputs.

FVM_TVD::run writes res_%010d.vtk every FILE_OUTPUT_STEP and a log line every
LOG_OUTPUT_STEP (src/methods/fvm_tvd.cpp:452-459, 501-600); the fixture holds
the files and lines the reference wrote for the same task and mesh.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, load_golden, write_case

pytestmark = pytest.mark.gpu

EXE = os.path.join(PKG, "lib", "cfd2d_gpu")


def _same_vtk(got: str, ref: str, rel=1e-12):
    """Same layout and words; numbers equal to the FP64 bar (this task uses the exact
    Godunov solver, whose exp/log last bits differ between CUDA and the host libm)."""
    gl, rl = got.split("\n"), ref.split("\n")
    assert len(gl) == len(rl)
    scale = 0.0
    for a, b in zip(gl, rl):
        ta, tb = a.split(" "), b.split(" ")
        assert len(ta) == len(tb)          # same separators and padding
        for x, y in zip(ta, tb):
            if x == y:
                continue
            fx, fy = float(x), float(y)    # only numbers may differ
            scale = max(scale, abs(fy))
            assert abs(fx - fy) <= rel * max(abs(fy), 1.0), (x, y)


def test_executable_reproduces_reference_files_and_log(capi, tmp_path):
    g = load_golden("shock_tube_4bc")
    write_case(tmp_path, g)
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    for name, text in zip(g["ref_vtk_names"], g["ref_vtk"]):
        got = (tmp_path / str(name)).read_text()
        if str(name) == "res_0000000000.vtk":
            assert got == str(text)        # the initial state: byte for byte
        else:
            _same_vtk(got, str(text))
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith(("time step:", "step:", "File '"))]
    assert lines == str(g["ref_log"]).splitlines()
    log = (tmp_path / "task.log").read_text()
    assert "step: 20" in log


def test_run_loop_honours_step_max(capi, tmp_path):
    g = load_golden("shock_tube_4bc")
    s = capi.Solver(write_case(tmp_path, g))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        s.run()
    finally:
        os.chdir(cwd)
    inf = s.get_info()
    assert inf.step == int(g["steps"])
    assert abs(inf.time - int(g["steps"]) * float(g["ref_tau"])) <= 1e-15
    assert np.max(np.abs(s.state() - g["ref_U"])) <= 1e-12 * np.max(np.abs(g["ref_U"]))


def test_run_reports_a_vtk_write_failure(capi, tmp_path):
    """run() writes its files from a host thread; a file that cannot be written
    (here a directory stands where res_0000000020.vtk goes) is run()'s error status,
    after every other file has been written."""
    g = load_golden("shock_tube_4bc")
    s = capi.Solver(write_case(tmp_path, g))
    (tmp_path / "res_0000000020.vtk").mkdir()
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        with pytest.raises(capi.CfdError) as e:
            s.run()
        assert e.value.code == 301
    finally:
        os.chdir(cwd)
    assert (tmp_path / "res_0000000000.vtk").is_file()
    assert s.get_info().step == int(g["steps"])
