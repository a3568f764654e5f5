"""Shared fixtures. GPU tests are marked ``gpu``; everything else runs on CPU."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cfd-2d_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    """Fixtures of the explicit method (reference FVM_TVD runs on UNV meshes)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not p.endswith("berkeley_triangle.npz")
                  and not os.path.basename(p).startswith(("implicit_", "rkdg_")))


def implicit_golden_names():
    """Fixtures of the implicit method (reference FVM_TVD_IMPLICIT runs, make_golden_implicit.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "implicit_*.npz")))


def rkdg_golden_names():
    """Fixtures of the discontinuous Galerkin method (reference FEM_RKDG runs, make_golden_rkdg.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "rkdg_*.npz")))


def rkdg_task(g):
    """The RkdgTask of a FEM_RKDG fixture."""
    import json
    from cfd2d import meshgen as mg
    d = json.loads(str(g["task_json"]))
    d["regions"] = [mg.Region(**r) for r in d["regions"]]
    d["boundaries"] = [mg.Boundary(**b) for b in d["boundaries"]]
    d["materials"] = [tuple(m) for m in d["materials"]]
    return mg.RkdgTask(**d)


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def capi():
    import importlib.util
    sys.path.insert(0, PKG)
    spec = importlib.util.spec_from_file_location("build_cfd2d", os.path.join(PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    from cfd2d import capi as c
    c.set_verbosity(0)
    return c


def write_case(tmp_path, g, key_unv="mesh_unv"):
    """Write a golden case's task.xml and mesh file(s) into tmp_path; returns the task path."""
    (tmp_path / "task.xml").write_text(str(g["task_xml"]))
    if key_unv in g:
        (tmp_path / "mesh.unv").write_text(str(g[key_unv]))
    for ext in ("node", "ele", "neigh", "poly"):
        k = "mesh_" + ext
        if k in g:
            (tmp_path / ("mesh." + ext)).write_text(str(g[k]))
    return str(tmp_path / "task.xml")
