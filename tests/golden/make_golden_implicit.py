"""Generate the implicit-method golden fixtures by running the reference's own FVM_TVD_IMPLICIT.

oracle/_ref/ref_fvm_tvd_implicit is the reference's src/methods/fvm_tvd_implicit.cpp
(with src/global.cpp, src/mesh/*, src/methods/solvers/CSR.cpp, src/tinyxml/*) compiled
unmodified by `make -C oracle reference`; HYPRE, which the reference calls for its
linear solve and which is not part of its tree, is replaced by the oracle's GMRES
(oracle/ref/ref_implicit.cpp). Each fixture stores the inputs (task.xml, the Triangle
mesh files and arrays, the task parameters, an optional per-cell initial state) and
the reference's outputs after STEP_MAX steps (state, cTau, flags, CFL, the last
solve's iterations and residual) and its step-0 VTK file.

Run where the reference source tree is present (it is needed to build the reference):
    python tests/golden/make_golden_implicit.py
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

from cfd2d import meshgen as mg  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def case(n, *, seed, kinds=("BOUND_INLET",), vortex=True, two_regions=False, two_materials=False, **task_kw):
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, 0.1, seed)
    m.bseg_bnd = (m.bseg_side % len(kinds)).astype(np.int32)
    bnds = [mg.ImplicitBoundary(edge_type=k + 1, kind=kd, T=1.0, p=1.0, u=1.0, v=0.0) for k, kd in enumerate(kinds)]
    if two_materials:  # the right half is a second gas (Cp 4.0: gamma 1.2625)
        task_kw["materials"] = [("gas", 8.314472, 3.5, 0.0, 0.0), ("heavy", 8.314472, 4.0, 0.0, 0.0)]
    if two_regions:
        m.cell_region = (m.centroids()[:, 0] > 5.0).astype(np.int32)
        regs = [mg.ImplicitRegion(cell_type=3, u=0.0, v=0.0, T=1.0, p=1.0),
                mg.ImplicitRegion(cell_type=7, u=0.0, v=0.0, T=1.0, p=0.6, mat=1 if two_materials else 0)]
    else:
        regs = [mg.ImplicitRegion(cell_type=0, u=1.0, v=0.0, T=1.0, p=1.0)]
    t = mg.ImplicitTask(regions=regs, boundaries=bnds, **task_kw)
    U0 = mg.isentropic_vortex(m.centroids(), 5.0, 5.0, 5.0) if vortex else None
    return m, t, U0


CASES = {
    "implicit_vortex_lax": dict(n=8, seed=21, tau=0.05, step_max=4, flux="LAX"),
    "implicit_vortex_godunov": dict(n=8, seed=22, tau=0.05, step_max=4, flux="GODUNOV"),
    "implicit_bc_steady": dict(n=8, seed=23, steady=1, step_max=6, flux="LAX",
                               kinds=("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL", "BOUND_OUTLET"),
                               cfl=(2.0, 1.5, 10.0, 2, 1.0e9)),
    "implicit_limits": dict(n=8, seed=24, tau=0.05, step_max=5, flux="LAX",
                            limits=(0.85, 1.0e8, 1.0e-8, 1.0e8, 1.0e8)),
    "implicit_steady_limits_godunov": dict(n=8, seed=25, steady=1, step_max=6, flux="GODUNOV",
                                           cfl=(2.0, 1.5, 10.0, 2, 3.0), limits=(0.85, 1.0e8, 1.0e-8, 1.0e8, 1.3)),
    "implicit_two_materials": dict(n=10, seed=27, tau=0.05, step_max=4, flux="LAX", vortex=False, two_regions=True,
                                   two_materials=True, kinds=("BOUND_WALL", "BOUND_OUTLET")),
    "implicit_two_region_wall": dict(n=10, seed=26, steady=1, step_max=5, flux="GODUNOV", vortex=False,
                                     two_regions=True, kinds=("BOUND_WALL",), cfl=(1.0, 1.2, 4.0, 1, 1.0e9)),
}


def main():
    for name, kw in CASES.items():
        kw = dict(kw)
        m, t, U0 = case(kw.pop("n"), seed=kw.pop("seed"), kinds=kw.pop("kinds", ("BOUND_INLET",)),
                        vortex=kw.pop("vortex", True), two_regions=kw.pop("two_regions", False),
                        two_materials=kw.pop("two_materials", False), **kw)
        xml = mg.write_implicit_task_xml(t)
        files = mg.write_triangle(m, [b.edge_type for b in t.boundaries], [r.cell_type for r in t.regions])
        ref = po.run_reference_implicit(xml, files, U0=U0)
        fi, ff = ref["init"], ref["state"]
        vtk0 = ref["vtk"]["res_0000000000.vtk"]
        task_json = json.dumps(dataclasses.asdict(t))
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), task_xml=np.array(xml), task_json=np.array(task_json),
            **{"mesh" + ext.replace(".", "_"): np.array(txt) for ext, txt in files.items()},
            nodes=m.nodes, tris=m.tris, cell_region=m.cell_region, bsegs=m.bsegs, bseg_bnd=m.bseg_bnd,
            U0=np.zeros((0,)) if U0 is None else U0, steps=np.int32(t.step_max),
            ref_U_init=fi["U"], ref_U=ff["U"], ref_cTau=ff["cTau"], ref_flags=ff["flags"],
            ref_cfl=np.float64(ff["cfl"]), ref_iters=np.int32(ff["iters"]), ref_rel=np.float64(ff["rel"]),
            ref_vtk0=np.array(vtk0))
        print(f"{name}: cells={len(m.tris)} steps={t.step_max} iters={ff['iters']} rel={ff['rel']:.3e} "
              f"cfl={ff['cfl']} flagged={int(((ff['flags'] & 2) > 0).sum())} moved={not np.array_equal(fi['U'], ff['U'])}")


if __name__ == "__main__":
    main()
