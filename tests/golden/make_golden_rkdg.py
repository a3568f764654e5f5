"""Generate the FEM_RKDG golden fixtures by running the reference's own FEM_RKDG.

oracle/_ref/ref_fem_rkdg is the reference's src/methods/fem_rkdg.cpp (with src/global.cpp,
src/bnd_cond.cpp, src/mesh/grid.cpp, src/tinyxml/*) compiled by `make -C oracle reference`;
its getF, which returns a dangling reference, is replaced by the same body returning a
valid one (oracle/ref/ref_rkdg.cpp). Each fixture stores the inputs (task.xml, the
mesh/mesh.0000.proc text, the task parameters, optional initial P1 coefficients and an
imposed time step) and the reference's outputs: the coefficients after init and after the
steps, cTau, TAU, the residuals, the step-0 VTU and PVTU files and the log.

Run where the reference source tree is present (it is needed to build the reference):
    python tests/golden/make_golden_rkdg.py
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cfd-2d_gb300"))
sys.path.insert(0, ROOT)

from cfd2d import cases  # noqa: E402
from cfd2d import meshgen as mg  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

CASES = {
    # four gentle quadrant states from the task's regions, one boundary kind per side
    "rkdg_quadrants_godunov": dict(kind="quadrants", n=8, flux="GODUNOV", gp_cell=4, gp_edge=3, steps=6),
    "rkdg_quadrants_lax_3pt": dict(kind="quadrants", n=8, flux="LAX", gp_cell=3, gp_edge=3, steps=6),
    "rkdg_quadrants_steady": dict(kind="quadrants", n=8, flux="GODUNOV", gp_cell=4, gp_edge=3, steps=5, steady=1),
    "rkdg_two_materials_lax": dict(kind="quadrants", n=8, flux="LAX", gp_cell=4, gp_edge=3, steps=5,
                                   materials=[("gas", 8.314472, 3.5, 0.0, 0.0), ("heavy", 8.314472, 4.0, 0.0, 0.0)]),
    # the isentropic vortex as P1 coefficients (every basis function active)
    "rkdg_vortex_godunov": dict(kind="vortex", n=8, flux="GODUNOV", gp_cell=4, gp_edge=3, steps=6, tau=0.01),
    "rkdg_vortex_lax_2pt": dict(kind="vortex", n=8, flux="LAX", gp_cell=3, gp_edge=2, steps=6, tau=0.01,
                                impose_tau=0.01),
    "rkdg_vortex_steady_walls": dict(kind="vortex", n=8, flux="LAX", gp_cell=4, gp_edge=3, steps=4, steady=1,
                                     cfl=0.1, kinds=("BOUND_OUTLET", "BOUND_WALL_SLIP")),
}


def build(spec):
    spec = dict(spec)
    kind = spec.pop("kind")
    impose = spec.pop("impose_tau", None)
    if kind == "quadrants":
        t, m, pm, U0 = cases.rkdg_quadrants(**spec)
    else:
        t, m, pm, U0 = cases.rkdg_vortex(**spec)
    return t, m, pm, U0, impose


def main():
    for name, spec in CASES.items():
        t, m, pm, U0, impose = build(spec)
        xml = mg.write_rkdg_task_xml(t)
        proc = mg.write_proc(pm)
        ref = po.run_reference_rkdg(xml, proc, spec["steps"], U0=U0, tau=impose)
        fi, ff = ref["init"], ref["state"]
        vtu = ref["vtu"]
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), task_xml=np.array(xml), proc=np.array(proc),
            task_json=np.array(json.dumps(dataclasses.asdict(t))),
            U0=np.zeros((0,)) if U0 is None else U0, impose_tau=np.float64(np.nan if impose is None else impose),
            steps=np.int32(spec["steps"]),
            ref_U_init=fi["U"], ref_cTau_init=fi["cTau"], ref_tau=np.float64(ff["tau"]),
            ref_U=ff["U"], ref_cTau=ff["cTau"], ref_res=ff["res"], ref_invA=ref["geom"]["invA"],
            ref_vtu0=np.array(vtu["vtk_data/res_0000000000.0000.vtu"]), ref_pvtu0=np.array(vtu["res_0000000000.pvtu"]),
            ref_stdout=np.array(ref["stdout"]))
        moved = float(np.abs(ff["U"] - fi["U"]).max())
        assert np.isfinite(ff["U"]).all(), name
        print(f"{name}: cells={len(pm.tris)} steps={spec['steps']} TAU={ff['tau']:.6g} moved={moved:.3e} "
              f"res={ff['res']}")


if __name__ == "__main__":
    main()
