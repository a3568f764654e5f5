"""Seeded synthetic workloads (the configurations the solver is measured on).

Each builder returns (task, mesh, U0): a task description, the mesh arrays
and the per-cell initial conserved state (None = the task's regions).
"""
from __future__ import annotations

import math
import os
import tempfile

import numpy as np

from . import meshgen as mg

GAMMA = 1.4
FREE = (1.0, 1.0, 0.0, 1.0)  # rho, u, v, p of the vortex free stream


def vortex(n: int, *, beta=5.0, mach=None, seed=1, jitter=0.1, flux="LAX", recon="NONE", scheme="EULER",
           cfl=0.5, steps=200, steady=0, precision=None, bnd_kinds=None):
    """Isentropic vortex on [0,10]^2 (n x n x 2 triangles), free stream rho=p=1.

    mach=None gives u=1 (the 20,000-triangle plain case); otherwise u = mach*sqrt(gamma).
    Far field: BOUND_INLET with the free stream on all sides (or the kinds given per side).
    """
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, jitter, seed)
    u_inf = 1.0 if mach is None else mach * math.sqrt(GAMMA)
    kinds = bnd_kinds or ("BOUND_INLET",) * 4
    bnds = [mg.Boundary(f"side{k}", kind, k + 1, u_inf, 0.0, 1.0, 1.0) for k, kind in enumerate(kinds)]
    m.bseg_bnd = m.bseg_side.copy()
    t = mg.Task(regions=[mg.Region("fluid", u_inf, 0.0, 1.0, 1.0)], boundaries=bnds, steady=steady, cfl=cfl,
                step_max=steps, flux=flux, reconstruction=recon, time_scheme=scheme, precision=precision)
    U0 = mg.isentropic_vortex(m.centroids(), beta, 5.0, 5.0, u_inf=u_inf)
    return t, m, U0


def four_quadrant(n: int, *, seed=2, jitter=0.05, flux="HLLC", recon="MINMOD", scheme="SSPRK3", cfl=0.4,
                  steps=1000, precision=None, steady=0):
    """Four-quadrant Riemann problem on [0,1]^2 (n x n x 2 triangles), outlets all round.

    Quadrant states (rho, u, v, p): NE (1.5, 0, 0, 1.5), NW (0.5323, 1.206, 0, 0.3),
    SW (0.138, 1.206, 1.206, 0.029), SE (0.5323, 0, 1.206, 0.3); a cell's quadrant
    is the one holding its centroid. Four XML regions, so the reference's own
    region initialisation sets the state.
    """
    m = mg.jittered_square(n, 0.0, 1.0, 0.0, 1.0, jitter, seed)
    m.cell_region = mg.quadrant_regions(m.centroids())
    regs = []
    for q in mg.QUADRANT_ORDER:
        r, u, v, p = mg.FOUR_QUADRANT[q]
        regs.append(mg.Region(q, u, v, p / r, p))  # T = p / rho with gR/M = 1
    t = mg.Task(regions=regs, boundaries=[mg.Boundary("outlet", "BOUND_OUTLET", 1)], steady=steady, cfl=cfl,
                step_max=steps, flux=flux, reconstruction=recon, time_scheme=scheme, precision=precision)
    m.bseg_bnd = np.zeros(len(m.bsegs), np.int32)
    return t, m, None


def write_task(task, mesh, directory=None, with_unv=False) -> str:
    """task.xml (and optionally mesh.unv) in a directory; returns the task path."""
    d = directory or tempfile.mkdtemp(prefix="cfd2d_")
    if with_unv:
        with open(os.path.join(d, "mesh.unv"), "w") as f:
            f.write(mg.write_unv(mesh, [r.name for r in task.regions], [b.name for b in task.boundaries]))
    path = os.path.join(d, "task.xml")
    with open(path, "w") as f:
        f.write(mg.write_task_xml(task))
    return path


def vortex_adjoint(n: int, *, steps=200, mach=None, beta=5.0, seed=4, jitter=0.1, flux="HLLC", recon="MINMOD",
                   scheme="SSPRK3", cfl=0.5, bnd_kinds=None, box=((6.0, 8.0), (4.0, 6.0))):
    """Differentiation workload: the isentropic vortex with the objective
    J = sum over cells whose centroid lies in box of S * (p - 1)^2.

    The global time step is pinned by TAU in the task (0.99 of the CFL value of
    the unperturbed state), so it does not move with the state being
    differentiated. Returns (task, mesh, U0, weights, u0_of_mach) where
    u0_of_mach(M) gives the initial state for another free-stream Mach number.
    """
    t, m, U0 = vortex(n, beta=beta, mach=mach, seed=seed, jitter=jitter, flux=flux, recon=recon, scheme=scheme,
                      cfl=cfl, steps=steps, bnd_kinds=bnd_kinds)
    xy = m.centroids()
    p = m.nodes[m.tris]
    S = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                     (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    (x0, x1), (y0, y1) = box
    inside = (xy[:, 0] >= x0) & (xy[:, 0] <= x1) & (xy[:, 1] >= y0) & (xy[:, 1] <= y1)
    w = np.where(inside, S, 0.0)
    # CFL time step of the unperturbed state (the reference's area-based formula)
    r, ru, rv, rE = U0
    u, v = ru / r, rv / r
    pr = (GAMMA - 1.0) * (rE - 0.5 * r * (u * u + v * v))
    c = np.sqrt(GAMMA * pr / r)
    t.tau = 0.99 * float(np.min(cfl * S / np.maximum(np.abs(u) + c, np.abs(v) + c)))

    def u0_of_mach(M):
        return mg.isentropic_vortex(xy, beta, 5.0, 5.0, u_inf=M * math.sqrt(GAMMA))
    return t, m, U0, w, u0_of_mach


def batched_vortices(count: int = 256, *, seed=3, min_cells=10_000, max_cells=400_000, flux="ROE", recon="MINMOD",
                     scheme="SSPRK3", cfl=0.5, steps=500, precision=None):
    """Batch of isentropic vortices on [0,10]^2 with uneven sizes.

    Triangle counts N_k are drawn log-uniform in [min_cells, max_cells]
    (n_k = round(sqrt(N_k / 2)) squares per side), free-stream Mach uniform in
    [0.1, 0.8] (u = M sqrt(gamma), rho = p = 1), vortex strength uniform in
    [1, 5]; instance k's mesh jitter seed is seed * 1000 + k. Returns a list of
    (task, mesh, U0).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    N = np.exp(rng.uniform(np.log(min_cells), np.log(max_cells), count))
    mach = rng.uniform(0.1, 0.8, count)
    beta = rng.uniform(1.0, 5.0, count)
    out = []
    for k in range(count):
        n = max(2, int(round(math.sqrt(N[k] / 2.0))))
        t, m, U0 = vortex(n, beta=float(beta[k]), mach=float(mach[k]), seed=seed * 1000 + k, flux=flux, recon=recon,
                          scheme=scheme, cfl=cfl, steps=steps, precision=precision)
        out.append((t, m, U0))
    return out


def vortex_implicit(n: int, *, flux="LAX", tau=0.002, steps=100, beta=5.0, seed=4, jitter=0.1, steady=0,
                    cfl=(1.0, 1.0, 1.0, 1000000, 1.0e9)):
    """The isentropic vortex (strength beta at (5, 5), free stream rho=u=p=1) on [0,10]^2 for the
    implicit method FVM_TVD_IMPLICIT: n x n x 2 triangles, all boundaries BOUND_INLET with the
    free stream, time step tau (unsteady) or the CFL rules (steady)."""
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, jitter, seed)
    m.bseg_bnd = np.zeros(len(m.bsegs), np.int32)
    bnds = [mg.ImplicitBoundary(edge_type=1, kind="BOUND_INLET", T=1.0, p=1.0, u=1.0, v=0.0)]
    t = mg.ImplicitTask(regions=[mg.ImplicitRegion(cell_type=0, u=1.0, v=0.0, T=1.0, p=1.0)], boundaries=bnds,
                        steady=steady, tau=tau, step_max=steps, flux=flux, cfl=cfl)
    U0 = mg.isentropic_vortex(m.centroids(), beta, 5.0, 5.0)
    return t, m, U0


def write_implicit_task(task, mesh, directory=None, with_mesh_files=False) -> str:
    """task.xml of an implicit task (and optionally its Triangle mesh files); returns the task path."""
    d = directory or tempfile.mkdtemp(prefix="cfd2d_imp_")
    path = os.path.join(d, "task.xml")
    with open(path, "w") as f:
        f.write(mg.write_implicit_task_xml(task))
    if with_mesh_files:
        files = mg.write_triangle(mesh, [b.edge_type for b in task.boundaries], [r.cell_type for r in task.regions])
        for ext, txt in files.items():
            with open(os.path.join(d, task.mesh_name + ext), "w") as f:
                f.write(txt)
    return path


# ---------------------------------------------------------------- FEM_RKDG (P1 discontinuous Galerkin)

MILD_QUADRANTS = {  # (rho, u, v, p): a gentle four-state problem the unlimited P1 method survives
    "NE": (1.0, 0.1, 0.0, 1.0),
    "NW": (1.1, 0.0, 0.1, 1.05),
    "SW": (0.95, 0.1, 0.1, 0.98),
    "SE": (1.05, -0.1, 0.0, 1.1),
}


def dg_cell_frame(pm):
    """Cell centres and the basis scales HX, HY of a .proc part the way Grid::readMeshFiles
    forms them (src/mesh/grid.cpp:306-317)."""
    p = pm.nodes[pm.tris]
    cx = (p[:, 0, 0] + p[:, 1, 0] + p[:, 2, 0]) / 3.0
    cy = (p[:, 0, 1] + p[:, 1, 1] + p[:, 2, 1]) / 3.0

    def h(k):
        a = np.abs(p[:, 0, k] - p[:, 1, k]); b = np.abs(p[:, 1, k] - p[:, 2, k]); c = np.abs(p[:, 0, k] - p[:, 2, k])
        return np.maximum(a, np.maximum(b, c))
    return cx, cy, h(0), h(1)


def dg_p1_coeffs(pm, field):
    """P1 coefficients (nc, 12: ro[3] ru[3] rv[3] re[3]) of a smooth conserved field
    field(x, y) -> (4, n): the centre value and the centred-difference slopes times HX, HY."""
    cx, cy, HX, HY = dg_cell_frame(pm)
    d = 1.0e-6
    U = field(cx, cy)
    Ux = (field(cx + d, cy) - field(cx - d, cy)) / (2.0 * d)
    Uy = (field(cx, cy + d) - field(cx, cy - d)) / (2.0 * d)
    out = np.empty((len(cx), 12))
    for v in range(4):
        out[:, 3 * v] = U[v]
        out[:, 3 * v + 1] = Ux[v] * HX
        out[:, 3 * v + 2] = Uy[v] * HY
    return out


def rkdg_vortex(n: int, *, flux="GODUNOV", gp_cell=4, gp_edge=3, tau=2.0e-3, beta=2.0, seed=5, jitter=0.1,
                steps=10, steady=0, cfl=0.3, rk=None, kinds=("BOUND_INLET",)):
    """Isentropic vortex (strength beta at (5, 5), free stream rho=u=p=1) on [0,10]^2 for FEM_RKDG:
    n x n x 2 triangles, P1 coefficients of the exact field at t = 0, free-stream boundaries
    (or the kinds given, cycled over the four sides). Returns (task, mesh, part, U0)."""
    m = mg.jittered_square(n, 0.0, 10.0, 0.0, 10.0, jitter, seed)
    m.bseg_bnd = (m.bseg_side % len(kinds)).astype(np.int32)
    bnds = [mg.Boundary(f"side{k}", kd, k + 1, 1.0, 0.0, 1.0, 1.0) for k, kd in enumerate(kinds)]
    t = mg.RkdgTask(regions=[mg.Region("fluid", 1.0, 0.0, 1.0, 1.0)], boundaries=bnds, steady=steady, tau=tau,
                    tmax=tau * steps, cfl=cfl, gp_cell=gp_cell, gp_edge=gp_edge, flux=flux, rk=rk)
    pm = mg.proc_mesh(m, [r.name for r in t.regions], [b.name for b in bnds])

    def field(x, y):
        return mg.isentropic_vortex(np.stack([x, y], axis=1), beta, 5.0, 5.0)
    return t, m, pm, dg_p1_coeffs(pm, field)


def rkdg_quadrants(n: int, *, flux="GODUNOV", gp_cell=4, gp_edge=3, tau=1.0e-3, seed=6, jitter=0.1, steps=10,
                   steady=0, cfl=0.3, rk=None,
                   kinds=("BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_INLET", "BOUND_WALL_NO_SLIP"), materials=None):
    """Four gentle quadrant states (MILD_QUADRANTS) on [0,1]^2 set by the task's regions (the
    reference's own initialisation), one boundary kind per side. Returns (task, mesh, part, None)."""
    m = mg.jittered_square(n, 0.0, 1.0, 0.0, 1.0, jitter, seed)
    m.cell_region = mg.quadrant_regions(m.centroids())
    m.bseg_bnd = (m.bseg_side % len(kinds)).astype(np.int32)
    regs = []
    for k, q in enumerate(mg.QUADRANT_ORDER):
        r, u, v, p = MILD_QUADRANTS[q]
        regs.append(mg.Region(q, u, v, p / r, p, mat=(k % 2) if materials else 0))
    bnds = [mg.Boundary(f"b{k}", kd, k + 1, 0.1, 0.05, 1.0, 1.02) for k, kd in enumerate(kinds)]
    kw = dict(materials=materials) if materials else {}
    t = mg.RkdgTask(regions=regs, boundaries=bnds, steady=steady, tau=tau, tmax=tau * steps, cfl=cfl,
                    gp_cell=gp_cell, gp_edge=gp_edge, flux=flux, rk=rk, **kw)
    pm = mg.proc_mesh(m, [r.name for r in regs], [b.name for b in bnds])
    return t, m, pm, None


def write_rkdg_task(task, pm, directory=None) -> str:
    """task.xml and mesh/mesh.0000.proc in a directory; returns the task path (the method
    reads the mesh part relative to the working directory)."""
    d = directory or tempfile.mkdtemp(prefix="cfd2d_dg_")
    os.makedirs(os.path.join(d, "mesh"), exist_ok=True)
    with open(os.path.join(d, "mesh", "mesh.0000.proc"), "w") as f:
        f.write(mg.write_proc(pm))
    path = os.path.join(d, "task.xml")
    with open(path, "w") as f:
        f.write(mg.write_rkdg_task_xml(task))
    return path
