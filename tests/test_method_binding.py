"""The reference-side binding (CPU part): the FVM_TVD_GPU Method subclass that a
maintainer adds to cfd-2d (oracle/dropin/fvm_tvd_gpu.h), with a main that follows the
reference's src/main.cpp and Solver::initMethod, builds and links against
libcfd2d_gpu.so, and without a GPU reports the library's error the reference's way
(log() into task.log, EXIT(1)).

Two builds: against the reference's own method.h / global.h, grid and global objects
(needs the reference's source tree, named by CFD2D_REFERENCE_SRC; skipped elsewhere),
and against the stand-in interface oracle/dropin/iface (anywhere). The GPU run that
compares the files with the reference's is tests/test_gpu_method_binding.py.
"""
import os
import subprocess

import pytest

from conftest import ROOT, load_golden, write_case

ORACLE = os.path.join(ROOT, "oracle")
REF = os.environ.get("CFD2D_REFERENCE_SRC", "")


def _no_gpu():
    import torch
    return not torch.cuda.is_available()


def _build(target):
    env = dict(os.environ)
    r = subprocess.run(["make", "-C", ORACLE, target], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


def _run_without_gpu(exe, tmp_path):
    write_case(tmp_path, load_golden("shock_tube_4bc"))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1, r.stdout + r.stderr                  # EXIT(1)
    assert "ERROR: no CUDA device" in r.stdout                     # log() to stdout
    assert "ERROR: no CUDA device" in (tmp_path / "task.log").read_text()  # and to hLog


@pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "src", "methods"))),
                    reason="the reference's source tree (CFD2D_REFERENCE_SRC) is not on this machine")
def test_subclass_builds_against_the_reference_headers(capi, tmp_path):
    _build("dropin")
    exe = os.path.join(ORACLE, "_ref", "cfd2d_dropin")
    assert os.path.isfile(exe)
    if _no_gpu():
        _run_without_gpu(exe, tmp_path)


def test_subclass_builds_against_the_standin_interface(capi, tmp_path):
    _build("dropin-standin")
    exe = os.path.join(ORACLE, "build", "cfd2d_dropin_standin")
    assert os.path.isfile(exe)
    if _no_gpu():
        _run_without_gpu(exe, tmp_path)


def test_unknown_method_is_the_reference_error(capi, tmp_path):
    _build("dropin-standin")
    (tmp_path / "task.xml").write_text('<?xml version="1.0"?>\n<task method="FEM_DG_IMPLICIT">\n</task>\n')
    r = subprocess.run([os.path.join(ORACLE, "build", "cfd2d_dropin_standin")], cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 255 and "ERROR: unknown method." in r.stdout   # exit(-1)
