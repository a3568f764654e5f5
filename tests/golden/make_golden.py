"""Generate the golden fixtures by running the reference's own FVM_TVD.

The reference ships no tests or golden vectors for its solver, so these
fixtures pin parity by executing the reference itself: oracle/_ref/ref_fvm_tvd
is the reference's src/methods/fvm_tvd.cpp, src/bnd_cond.cpp, src/global.cpp,
src/mesh/* and src/tinyxml/* compiled unmodified (make -C oracle reference),
driven by oracle/ref/ref_driver.cpp. Each fixture stores the inputs (task.xml,
the mesh files and arrays, an optional per-cell initial state) and the
reference's outputs (its Grid, its TAU, and the state after STEP_MAX steps).

Run where the reference source tree is present (it is needed to build the reference):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cfd-2d_gb300"))
sys.path.insert(0, ROOT)

from cfd2d import meshgen as mg  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

BK4 = ("BOUND_WALL_NO_SLIP", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_INLET")


def two_region_case(n, steps, seed, pr=0.5, bkinds=BK4, steady=0, shuffle=False):
    m = mg.jittered_square(n, 0.0, 1.0, 0.0, 1.0, 0.1, seed)
    if shuffle:  # arbitrary element order, node order and vertex rotation
        rng = np.random.Generator(np.random.PCG64(seed + 100))
        perm_n = rng.permutation(len(m.nodes))
        inv = np.empty_like(perm_n); inv[perm_n] = np.arange(len(perm_n))
        m.nodes = m.nodes[perm_n]
        m.tris = inv[m.tris].astype(np.int32)
        m.bsegs = inv[m.bsegs].astype(np.int32)
        pc = rng.permutation(len(m.tris))
        m.tris = m.tris[pc]
        rot = rng.integers(0, 3, len(m.tris))
        m.tris = np.stack([np.roll(t, r) for t, r in zip(m.tris, rot)]).astype(np.int32)
        pb = rng.permutation(len(m.bsegs))
        m.bsegs = m.bsegs[pb]; m.bseg_side = m.bseg_side[pb]
    m.cell_region = (m.centroids()[:, 0] > 0.5).astype(np.int32)
    m.bseg_bnd = m.bseg_side.copy()
    t = mg.Task(regions=[mg.Region("left", 0.0, 0.0, 1.0, 1.0), mg.Region("right", 0.0, 0.0, 1.0, pr)],
                boundaries=[mg.Boundary(f"bnd{k}", bk, k + 1, 0.1, 0.0, 1.0, 1.0) for k, bk in enumerate(bkinds)],
                step_max=steps, steady=steady, file_output_step=steps, log_output_step=max(1, steps // 2))
    return m, t, None


def vortex_case(n, steps, seed, steady=0, limits=None, beta=5.0):
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, 0.1, seed)
    m.bseg_bnd = np.zeros(len(m.bsegs), np.int32)
    t = mg.Task(regions=[mg.Region("fluid", 1.0, 0.0, 1.0, 1.0)],
                boundaries=[mg.Boundary("farfield", "BOUND_INLET", 1, 1.0, 0.0, 1.0, 1.0)],
                step_max=steps, steady=steady)
    if limits is not None:
        t.limits = limits
    U0 = mg.isentropic_vortex(m.centroids(), beta, 5.0, 5.0)
    return m, t, U0


CASES = {
    # reference mode (Godunov, unlimited linear, Heun) through the XML-only path
    "shock_tube_4bc": lambda: two_region_case(16, 20, seed=11),
    # arbitrary element / node ordering: exercises neighbour search and edge numbering
    "shuffled_mesh": lambda: two_region_case(12, 10, seed=12, pr=0.6, shuffle=True),
    # per-cell initial vortex, far-field inlet everywhere, global time step
    "vortex_global_dt": lambda: vortex_case(16, 20, seed=13),
    # local time step (STEADY=1): cTau recomputed per cell every step
    "vortex_local_dt": lambda: vortex_case(16, 20, seed=14, steady=1),
    # |u| limit below the vortex peak: LIM flags, neighbour remediation and flag release after 0x20 steps
    "vortex_limits": lambda: vortex_case(12, 40, seed=15, limits=(1e-8, 1e8, 1e-8, 1e8, 1.55)),
}


def main():
    os.makedirs(HERE, exist_ok=True)
    for name, make in CASES.items():
        m, t, U0 = make()
        region_names = [r.name for r in t.regions]
        bnd_names = [b.name for b in t.boundaries]
        xml = mg.write_task_xml(t)
        unv = mg.write_unv(m, region_names, bnd_names)
        ref = po.run_reference(xml, unv, U0)
        g, fi, ff = ref["grid"], ref["init"], ref["final"]
        solver_lines = [ln for ln in ref["stdout"].splitlines() if ln.startswith(("time step:", "step:", "File '"))]
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            task_xml=np.array(xml), mesh_unv=np.array(unv),
            ref_vtk_names=np.array(list(ref["vtk"].keys())), ref_vtk=np.array(list(ref["vtk"].values())),
            ref_log=np.array("\n".join(solver_lines)),
            nodes=m.nodes, tris=m.tris, cell_region=m.cell_region, bsegs=m.bsegs, bseg_bnd=m.bseg_bnd,
            region_names=np.array(region_names), bnd_names=np.array(bnd_names),
            U0=np.zeros((0,)) if U0 is None else U0, steps=np.int32(t.step_max),
            ref_tau=np.float64(fi["tau"]), ref_U_init=fi["U"], ref_U=ff["U"], ref_cTau=ff["cTau"],
            ref_flags=ff["flags"], **{"grid_" + k: v for k, v in g.items()})
        print(f"{name}: cells={len(m.tris)} steps={t.step_max} tau={fi['tau']:.6e} "
              f"flagged={int(((ff['flags'] & 2) > 0).sum())} ref_seconds={ff['seconds']:.4f}")
    # Berkeley-Triangle reader: 1 point per edge in the reference, so no flux at all
    m, t, U0 = two_region_case(8, 5, seed=16)
    t.mesh_type = "berkeley_triangle"; t.mesh_name = "mesh"
    t.regions[0].name, t.regions[1].name = "0", "1"
    files = mg.write_triangle(m, [b.edge_type for b in t.boundaries])
    xml = mg.write_task_xml(t)
    import subprocess, tempfile
    with tempfile.TemporaryDirectory() as d:
        open(os.path.join(d, "task.xml"), "w").write(xml)
        for ext, txt in files.items():
            open(os.path.join(d, "mesh" + ext), "w").write(txt)
        r = subprocess.run([po.REF_BIN, "task.xml", "out"], cwd=d, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stdout + r.stderr
        g = po.read_ref_grid(os.path.join(d, "out.grid.bin"))
        fi = po.read_ref_state(os.path.join(d, "out.init.bin"))
        ff = po.read_ref_state(os.path.join(d, "out.state.bin"))
    np.savez_compressed(
        os.path.join(HERE, "berkeley_triangle.npz"), task_xml=np.array(xml),
        **{"mesh" + ext.replace(".", "_"): np.array(txt) for ext, txt in files.items()},
        nodes=m.nodes, tris=m.tris, cell_region=m.cell_region, bsegs=m.bsegs, bseg_bnd=m.bseg_bnd,
        steps=np.int32(t.step_max), ref_tau=np.float64(fi["tau"]), ref_U_init=fi["U"], ref_U=ff["U"],
        ref_cTau=ff["cTau"], ref_flags=ff["flags"], **{"grid_" + k: v for k, v in g.items()})
    print("berkeley_triangle: unchanged state =", bool(np.array_equal(fi["U"], ff["U"])))


if __name__ == "__main__":
    main()
