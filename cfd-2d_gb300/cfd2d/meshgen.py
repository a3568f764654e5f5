"""Seeded synthetic triangle meshes and the reference's input formats.

A mesh here is the input half of the solver's drop-in interface: node
coordinates, triangles, a region index per triangle and a list of boundary
segments with a boundary index each. The same arrays can be written as a
Salome UNV file plus an FVM_TVD ``task.xml`` (the formats the reference reads,
src/mesh/MeshReaderSalomeUnv.cpp:267-447 and src/methods/fvm_tvd.cpp:26-128) or
handed to the library directly.

Generator: an n x n grid of squares on a rectangle, each square split into two
counter-clockwise triangles by the same diagonal; interior nodes jittered by
i.i.d. U(-a*h, +a*h) per coordinate from numpy's PCG64 with a stated seed;
boundary nodes are not moved.
"""
from __future__ import annotations

import io
import math
from dataclasses import dataclass, field

import numpy as np

SIDE_BOTTOM, SIDE_RIGHT, SIDE_TOP, SIDE_LEFT = 0, 1, 2, 3


@dataclass
class Mesh:
    nodes: np.ndarray            # (nn, 2) float64
    tris: np.ndarray             # (nc, 3) int32, counter-clockwise, 0-based
    cell_region: np.ndarray      # (nc,) int32, index into the task's region list
    bsegs: np.ndarray            # (nb, 2) int32 node pairs on the boundary
    bseg_bnd: np.ndarray         # (nb,) int32, index into the task's boundary list
    bseg_side: np.ndarray = field(default=None)  # (nb,) int32 side tag of the square

    @property
    def n_cells(self) -> int:
        return int(self.tris.shape[0])

    def centroids(self) -> np.ndarray:
        """Cell centres the way the reference forms them: (x0+x1+x2)/3."""
        p = self.nodes[self.tris]
        return np.stack([(p[:, 0, 0] + p[:, 1, 0] + p[:, 2, 0]) / 3.0,
                         (p[:, 0, 1] + p[:, 1, 1] + p[:, 2, 1]) / 3.0], axis=1)


def jittered_square(n: int, x0: float, x1: float, y0: float, y1: float,
                    jitter: float, seed: int) -> Mesh:
    """n x n squares x 2 triangles on [x0,x1]x[y0,y1], interior jitter a=jitter."""
    hx = (x1 - x0) / n
    hy = (y1 - y0) / n
    i = np.arange(n + 1)
    X, Y = np.meshgrid(x0 + i * hx, y0 + i * hy)        # row j = y index
    nodes = np.stack([X.ravel(), Y.ravel()], axis=1).astype(np.float64)
    nodes[n * (n + 1):, 1] = y1                         # exact top edge
    nodes[n::n + 1, 0] = x1                             # exact right edge
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        d = rng.uniform(-jitter, jitter, size=(n + 1, n + 1, 2))
        inner = np.zeros((n + 1, n + 1), dtype=bool)
        inner[1:n, 1:n] = True
        inner = inner.ravel()
        dd = d.reshape(-1, 2)
        nodes[inner, 0] += dd[inner, 0] * hx
        nodes[inner, 1] += dd[inner, 1] * hy
    k = (np.arange(n)[None, :] + (n + 1) * np.arange(n)[:, None]).ravel()   # lower-left node
    k00, k10, k01, k11 = k, k + 1, k + n + 1, k + n + 2
    tris = np.empty((2 * n * n, 3), dtype=np.int32)
    tris[0::2] = np.stack([k00, k10, k11], axis=1)
    tris[1::2] = np.stack([k00, k11, k01], axis=1)
    # boundary segments, side by side
    s = np.arange(n)
    bottom = np.stack([s, s + 1], axis=1)
    right = np.stack([n + (n + 1) * s, n + (n + 1) * (s + 1)], axis=1)
    top = np.stack([n * (n + 1) + s + 1, n * (n + 1) + s], axis=1)
    left = np.stack([(n + 1) * (s + 1), (n + 1) * s], axis=1)
    bsegs = np.concatenate([bottom, right, top, left]).astype(np.int32)
    side = np.repeat(np.arange(4, dtype=np.int32), n)
    return Mesh(nodes=nodes, tris=tris, cell_region=np.zeros(2 * n * n, np.int32),
                bsegs=bsegs, bseg_bnd=np.zeros(4 * n, np.int32), bseg_side=side)


# ---------------------------------------------------------------- initial data

GAMMA = 1.4


def cons_from_prim(r, u, v, p, gam=GAMMA):
    """(rho, u, v, p) -> (rho, rho u, rho v, rho E) for a calorically perfect gas."""
    r = np.asarray(r, np.float64)
    e = p / (r * (gam - 1.0))
    return np.stack([r, r * u, r * v, r * (e + 0.5 * (u * u + v * v))])


def isentropic_vortex(xy: np.ndarray, beta: float, xc: float, yc: float,
                      u_inf: float = 1.0, v_inf: float = 0.0, gam: float = GAMMA):
    """Isentropic vortex of strength beta on a free stream rho=p=1 (R=1), at centroids.

    du = -beta/(2 pi) (y-yc) exp((1-r^2)/2), dv = beta/(2 pi) (x-xc) exp((1-r^2)/2),
    T = 1 - (gam-1) beta^2 / (8 gam pi^2) exp(1-r^2), rho = T^(1/(gam-1)), p = rho T.
    """
    dx = xy[:, 0] - xc
    dy = xy[:, 1] - yc
    r2 = dx * dx + dy * dy
    ex = np.exp(0.5 * (1.0 - r2))
    u = u_inf - beta / (2.0 * math.pi) * dy * ex
    v = v_inf + beta / (2.0 * math.pi) * dx * ex
    T = 1.0 - (gam - 1.0) * beta * beta / (8.0 * gam * math.pi * math.pi) * ex * ex
    r = T ** (1.0 / (gam - 1.0))
    p = r * T
    return cons_from_prim(r, u, v, p, gam)


FOUR_QUADRANT = {  # (rho, u, v, p) by quadrant of the unit square split at (1/2, 1/2)
    "NE": (1.5, 0.0, 0.0, 1.5),
    "NW": (0.5323, 1.206, 0.0, 0.3),
    "SW": (0.138, 1.206, 1.206, 0.029),
    "SE": (0.5323, 0.0, 1.206, 0.3),
}
QUADRANT_ORDER = ("NE", "NW", "SW", "SE")


def quadrant_regions(xy: np.ndarray, xs: float = 0.5, ys: float = 0.5) -> np.ndarray:
    """Region index per cell by centroid: 0 NE, 1 NW, 2 SW, 3 SE."""
    east = xy[:, 0] > xs
    north = xy[:, 1] > ys
    reg = np.where(north, np.where(east, 0, 1), np.where(east, 3, 2))
    return reg.astype(np.int32)


# ---------------------------------------------------------------- UNV writer

def write_unv(mesh: Mesh, region_names, bnd_names) -> str:
    """Salome UNV text with blocks 2411 (nodes), 2412 (edges + triangles), 2467 (groups).

    Coordinates use Python's shortest round-trip form, so the reader gets the
    very same doubles back. Every cell goes into the group of its region and
    every boundary segment into the group of its boundary, which is how the
    reference binds regions and boundary conditions by name
    (src/mesh/MeshReaderSalomeUnv.cpp:219-248).
    """
    out = io.StringIO()
    w = out.write
    w("    -1\n  2411\n")
    for i, (x, y) in enumerate(mesh.nodes):
        w(f"{i + 1:10d}{1:10d}{1:10d}{11:10d}\n")
        w(f"  {repr(float(x))}  {repr(float(y))}  0.0\n")
    w("    -1\n    -1\n  2412\n")
    label = 0
    edge_labels = []
    for (a, b) in mesh.bsegs:
        label += 1
        edge_labels.append(label)
        w(f"{label:10d}{11:10d}{2:10d}{1:10d}{7:10d}{2:10d}\n")
        w(f"{0:10d}{1:10d}{1:10d}\n")
        w(f"{a + 1:10d}{b + 1:10d}\n")
    cell_labels = []
    for (a, b, c) in mesh.tris:
        label += 1
        cell_labels.append(label)
        w(f"{label:10d}{41:10d}{2:10d}{1:10d}{7:10d}{3:10d}\n")
        w(f"{a + 1:10d}{b + 1:10d}{c + 1:10d}\n")
    w("    -1\n    -1\n  2467\n")
    groups = []
    edge_labels = np.asarray(edge_labels)
    cell_labels = np.asarray(cell_labels)
    for k, name in enumerate(bnd_names):
        groups.append((name, edge_labels[mesh.bseg_bnd == k]))
    for k, name in enumerate(region_names):
        groups.append((name, cell_labels[mesh.cell_region == k]))
    for g, (name, labels) in enumerate(groups):
        n = len(labels)
        w(f"{g + 1:10d}{0:10d}{0:10d}{0:10d}{0:10d}{0:10d}{0:10d}{n:10d}\n")
        w(f"{name}\n")
        for j in range(0, n - 1, 2):
            w(f"{8:10d}{labels[j]:10d}{0:10d}{0:10d}{8:10d}{labels[j + 1]:10d}{0:10d}{0:10d}\n")
        if n % 2 == 1:
            w(f"{8:10d}{labels[-1]:10d}{0:10d}{0:10d}\n")
    w("    -1\n")
    return out.getvalue()


def triangle_neighbours(tris: np.ndarray) -> np.ndarray:
    """Berkeley-Triangle .neigh convention: neighbour j is across the edge opposite node j; -1 if none."""
    nc = len(tris)
    a = np.concatenate([tris[:, 1], tris[:, 2], tris[:, 0]])
    b = np.concatenate([tris[:, 2], tris[:, 0], tris[:, 1]])
    cell = np.tile(np.arange(nc), 3)
    slot = np.repeat(np.arange(3), nc)
    key = np.minimum(a, b).astype(np.int64) * (1 << 32) + np.maximum(a, b)
    order = np.argsort(key, kind="stable")
    ks = key[order]
    nb = -np.ones((nc, 3), np.int64)
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    i0, i1 = order[same], order[same + 1]
    nb[cell[i0], slot[i0]] = cell[i1]
    nb[cell[i1], slot[i1]] = cell[i0]
    return nb.astype(np.int32)


def write_triangle(mesh: Mesh, bnd_markers, region_attr=None) -> dict:
    """Berkeley-Triangle files (.node .ele .neigh .poly), 1-based, as the reference reads them
    (src/mesh/MeshReaderBerkleyTriangle.cpp:3-170). The .ele attribute is the region index
    (or ``region_attr[cell_region]``, e.g. the implicit method's cell types), which becomes the
    cell's region name ("0", "1", ...); the .poly marker of a boundary segment is
    ``bnd_markers[bseg_bnd]`` and binds to a boundCond by its edgeType."""
    nn, nc = len(mesh.nodes), len(mesh.tris)
    attr = mesh.cell_region if region_attr is None else np.asarray(region_attr)[mesh.cell_region]
    node = [f"{nn} 2 0 1"] + [f"{i + 1} {repr(float(x))} {repr(float(y))} 0" for i, (x, y) in enumerate(mesh.nodes)]
    ele = [f"{nc} 3 1"] + [f"{i + 1} {a + 1} {b + 1} {c + 1} {int(r)}"
                           for i, ((a, b, c), r) in enumerate(zip(mesh.tris, attr))]
    nb = triangle_neighbours(mesh.tris)
    neigh = [f"{nc} 3"] + [f"{i + 1} {x + 1 if x >= 0 else -1} {y + 1 if y >= 0 else -1} {z + 1 if z >= 0 else -1}"
                           for i, (x, y, z) in enumerate(nb)]
    poly = ["0 2 0 1", f"{len(mesh.bsegs)} 1"] + [f"{k + 1} {a + 1} {b + 1} {int(bnd_markers[int(s)])}"
                                                for k, ((a, b), s) in enumerate(zip(mesh.bsegs, mesh.bseg_bnd))]
    return {ext: "\n".join(lines) + "\n" for ext, lines in
            ((".node", node), (".ele", ele), (".neigh", neigh), (".poly", poly))}


# ---------------------------------------------------------------- task.xml

@dataclass
class Region:
    name: str
    u: float
    v: float
    T: float
    p: float
    mat: int = 0


@dataclass
class Boundary:
    name: str
    kind: str                    # BOUND_INLET / BOUND_OUTLET / BOUND_WALL_SLIP / BOUND_WALL_NO_SLIP
    edge_type: int = 1
    u: float = 0.0
    v: float = 0.0
    T: float = 1.0
    p: float = 1.0


@dataclass
class Task:
    regions: list
    boundaries: list
    steady: int = 0
    tau: float = 1.0e8
    tmax: float = 1.0e8
    cfl: float = 0.5
    step_max: int = 10
    file_output_step: int = 1000000
    log_output_step: int = 1000000
    limits: tuple = (1.0e-8, 1.0e8, 1.0e-8, 1.0e8, 1.0e8)   # ro min/max, p min/max, u max
    # (name, M, Cp, K, ML); M = gR and Cp = 3.5 give gR/M = 1, Cv = 2.5, gamma = 1.4, T = p/rho
    materials: list = field(default_factory=lambda: [("gas", 8.314472, 3.5, 0.0, 0.0)])
    mesh_name: str = "mesh.unv"
    mesh_type: str = "salome_unv"
    # optional GPU method selections (absent -> reference behaviour)
    flux: str | None = None
    reconstruction: str | None = None
    time_scheme: str | None = None
    precision: str | None = None
    reorder: str | None = None        # NONE / RCM / HILBERT
    fused_stage: str | None = None    # "1" runs the mixed form's stages as one tiled kernel
    adjoint_store: str | None = None  # NONE / PRIMITIVES / ALL: what the adjoint keeps per recorded stage
    adjoint_memory: float | None = None  # device-memory budget of the handle for the adjoint, bytes
    flux_pipeline: str | None = None  # mixed form: ON (default) / OFF, the software-pipelined flux kernel
    method: str = "FVM_TVD"


def _v(x) -> str:
    return repr(float(x))


def write_task_xml(t: Task) -> str:
    rmin, rmax, pmin, pmax, umax = t.limits
    L = ['<?xml version="1.0" encoding="UTF-8"?>', f'<task method="{t.method}">', "  <control>",
         f'    <STEADY value="{int(t.steady)}" />', f'    <TAU value="{_v(t.tau)}" />',
         f'    <TMAX value="{_v(t.tmax)}" />', f'    <CFL value="{_v(t.cfl)}" />',
         f'    <STEP_MAX value="{int(t.step_max)}" />',
         f'    <FILE_OUTPUT_STEP value="{int(t.file_output_step)}" />',
         f'    <LOG_OUTPUT_STEP value="{int(t.log_output_step)}" />']
    for tag, val in (("FLUX", t.flux), ("RECONSTRUCTION", t.reconstruction),
                     ("TIME_SCHEME", t.time_scheme), ("PRECISION", t.precision), ("REORDER", t.reorder),
                     ("FUSED_STAGE", t.fused_stage), ("ADJOINT_STORE", t.adjoint_store),
                     ("ADJOINT_MEMORY", None if t.adjoint_memory is None else _v(t.adjoint_memory)),
                     ("FLUX_PIPELINE", t.flux_pipeline)):
        if val is not None:
            L.append(f'    <{tag} value="{val}" />')
    L += ["  </control>", "  <limits>", f'    <ro min="{_v(rmin)}" max="{_v(rmax)}" />',
          f'    <p min="{_v(pmin)}" max="{_v(pmax)}" />', f'    <u max="{_v(umax)}" />', "  </limits>",
          f'  <materials count="{len(t.materials)}">']
    for k, (name, M, Cp, K, ML) in enumerate(t.materials):
        L += [f'    <material id="{k}">', f"      <name>{name}</name>", "      <parameters>",
              f'        <M value="{_v(M)}" />', f'        <Cp value="{_v(Cp)}" />',
              f'        <K value="{_v(K)}" />', f'        <ML value="{_v(ML)}" />',
              "      </parameters>", "    </material>"]
    L += ["  </materials>", f'  <regions count="{len(t.regions)}">']
    for k, r in enumerate(t.regions):
        L += [f'    <region id="{k}">', f'      <material id="{r.mat}" />', '      <cell type="3" />',
              f"      <name>{r.name}</name>", "      <parameters>", f'        <Vx value="{_v(r.u)}" />',
              f'        <Vy value="{_v(r.v)}" />', f'        <T value="{_v(r.T)}" />',
              f'        <P value="{_v(r.p)}" />', "      </parameters>", "    </region>"]
    L += ["  </regions>", "  <boundaries>"]
    for b in t.boundaries:
        L += [f'    <boundCond edgeType="{b.edge_type}">', f"      <type>{b.kind}</type>",
              f"      <name>{b.name}</name>"]
        if b.kind == "BOUND_INLET":
            L += ["      <parameters>", f'        <Vx value="{_v(b.u)}" />', f'        <Vy value="{_v(b.v)}" />',
                  f'        <T value="{_v(b.T)}" />', f'        <P value="{_v(b.p)}" />', "      </parameters>"]
        L.append("    </boundCond>")
    L += ["  </boundaries>", "  <mesh>", f'    <name value="{t.mesh_name}" />',
          f'    <filesType value="{t.mesh_type}" />', "  </mesh>", "</task>", ""]
    return "\n".join(L)


# ------------------------------------------------- task.xml of FVM_TVD_IMPLICIT

@dataclass
class ImplicitRegion:
    cell_type: int          # the .ele attribute of its cells
    u: float
    v: float
    T: float
    p: float
    mat: int = 0


@dataclass
class ImplicitBoundary:
    edge_type: int          # the .poly marker of its segments
    kind: str               # BOUND_INLET / BOUND_OUTLET / BOUND_WALL
    T: float = 1.0
    p: float = 1.0
    u: float = 0.0
    v: float = 0.0


@dataclass
class ImplicitTask:
    """task.xml of the reference's FVM_TVD_IMPLICIT (src/methods/fvm_tvd_implicit.cpp:13-184):
    Triangle files read by Grid::initFromFiles, regions bound by cell type, boundaries by
    edge type; the CFL block is read for steady runs only."""
    regions: list
    boundaries: list
    steady: int = 0
    tau: float = 1.0e-3
    tmax: float = 1.0e8
    step_max: int = 10
    file_output_step: int = 1000000
    log_output_step: int = 1000000
    flux: str = "LAX"                  # GODUNOV / LAX
    cfl: tuple = (1.0, 1.0, 1.0, 1000000, 1.0e9)  # start, scale, max, step, max_limited_cells
    smoothing: tuple = (0, 0.0)        # using, coefficient
    limits: tuple = (1.0e-8, 1.0e8, 1.0e-8, 1.0e8, 1.0e8)
    materials: list = field(default_factory=lambda: [("gas", 8.314472, 3.5, 0.0, 0.0)])
    mesh_name: str = "mesh"
    precision: str | None = None       # GPU option: FP64 (default)
    reorder: str | None = None
    gmres: tuple | None = None         # (krylov, max_iter, tolerance); None: the reference's (30, 20, 1e-7)


def write_implicit_task_xml(t: ImplicitTask) -> str:
    rmin, rmax, pmin, pmax, umax = t.limits
    start, scale, cmax, cstep, maxlim = t.cfl
    L = ['<?xml version="1.0" encoding="UTF-8"?>', '<task method="FVM_TVD_IMPLICIT">', "  <control>",
         f'    <STEADY value="{int(t.steady)}" />', f'    <TAU value="{_v(t.tau)}" />',
         f'    <TMAX value="{_v(t.tmax)}" />', f'    <STEP_MAX value="{int(t.step_max)}" />',
         f'    <FILE_OUTPUT_STEP value="{int(t.file_output_step)}" />',
         f'    <LOG_OUTPUT_STEP value="{int(t.log_output_step)}" />', f'    <FLUX value="{t.flux}" />',
         "    <CFL>", f'      <start value="{_v(start)}" />', f'      <scale value="{_v(scale)}" />',
         f'      <max value="{_v(cmax)}" />', f'      <step value="{int(cstep)}" />',
         f'      <max_limited_cells value="{_v(maxlim)}" />', "    </CFL>"]
    for tag, val in (("PRECISION", t.precision), ("REORDER", t.reorder)):
        if val is not None:
            L.append(f'    <{tag} value="{val}" />')
    if t.gmres is not None:
        k, it, tol = t.gmres
        L.append(f'    <GMRES krylov="{int(k)}" max_iter="{int(it)}" tolerance="{_v(tol)}" />')
    L += ["  </control>", "  <smoothing>", f'    <using value="{int(t.smoothing[0])}" />',
          f'    <coefficient value="{_v(t.smoothing[1])}" />', "  </smoothing>",
          "  <limits>", f'    <ro min="{_v(rmin)}" max="{_v(rmax)}" />',
          f'    <p min="{_v(pmin)}" max="{_v(pmax)}" />', f'    <u max="{_v(umax)}" />', "  </limits>",
          f'  <materials count="{len(t.materials)}">']
    for k, (name, M, Cp, K, ML) in enumerate(t.materials):
        L += [f'    <material id="{k}">', f"      <name>{name}</name>", "      <parameters>",
              f'        <M value="{_v(M)}" />', f'        <Cp value="{_v(Cp)}" />',
              f'        <K value="{_v(K)}" />', f'        <ML value="{_v(ML)}" />',
              "      </parameters>", "    </material>"]
    L += ["  </materials>", f'  <regions count="{len(t.regions)}">']
    for k, r in enumerate(t.regions):
        L += [f'    <region id="{k}">', f'      <material id="{r.mat}" />', f'      <cell type="{int(r.cell_type)}" />',
              "      <parameters>", f'        <Vx value="{_v(r.u)}" />', f'        <Vy value="{_v(r.v)}" />',
              f'        <T value="{_v(r.T)}" />', f'        <P value="{_v(r.p)}" />', "      </parameters>",
              "    </region>"]
    L += ["  </regions>", f'  <boundaries count="{len(t.boundaries)}">']
    for b in t.boundaries:
        L += [f'    <boundCond edgeType="{int(b.edge_type)}">', f"      <type>{b.kind}</type>"]
        if b.kind == "BOUND_INLET":
            L += ["      <parameters>", f'        <T value="{_v(b.T)}" />', f'        <P value="{_v(b.p)}" />',
                  f'        <Vx value="{_v(b.u)}" />', f'        <Vy value="{_v(b.v)}" />', "      </parameters>"]
        L.append("    </boundCond>")
    L += ["  </boundaries>", "  <mesh>", f'    <name value="{t.mesh_name}" />', "  </mesh>", "</task>", ""]
    return "\n".join(L)


# ------------------------------------------------------- FEM_RKDG: .proc mesh parts and task.xml

EDGE_TYPE_NAMED = 0x100  # Edge::TYPE_NAMED, src/mesh/grid.h:70


@dataclass
class ProcMesh:
    """One mesh part the way the DECOMP method writes it for a single process
    (src/methods/decomp.cpp:296-331) and Grid::readMeshFiles reads it
    (src/mesh/grid.cpp:275-420): nodes, triangles with a region name each, and edges
    as node pairs with a type (0 inside; EDGE_TYPE_NAMED with a boundary name, or a
    numeric edgeType). Coordinates are what the file holds (printed with %25.15e)."""
    nodes: np.ndarray          # (nn, 2) float64
    tris: np.ndarray           # (nc, 3) int32
    cell_names: list           # (nc,) region name per cell
    edges: np.ndarray          # (ne, 2) int32
    edge_type: np.ndarray      # (ne,) int32
    edge_names: list           # (ne,) boundary name ("" inside)


def proc_mesh(mesh: Mesh, region_names, bnd_names=None, bnd_types=None) -> ProcMesh:
    """The single-process part of a mesh. Edges are numbered in order of first appearance
    over the cells (cell i, its sides (t0,t1), (t1,t2), (t2,t0)), oriented as first seen.
    Boundary edges carry the boundary of their segment: by name (bnd_names, the UNV
    groups' way) or by number (bnd_types, the Triangle markers' way)."""
    nodes = np.array([[float(f"{x:25.15e}"), float(f"{y:25.15e}")] for x, y in mesh.nodes])
    tris = mesh.tris.astype(np.int32)
    a = tris.reshape(-1)
    b = tris[:, [1, 2, 0]].reshape(-1)
    key = np.minimum(a, b).astype(np.int64) * (1 << 32) + np.maximum(a, b)
    uniq, first = np.unique(key, return_index=True)
    order = np.sort(first)
    edges = np.stack([a[order], b[order]], axis=1).astype(np.int32)
    ekey = key[order]
    bkey = np.minimum(mesh.bsegs[:, 0], mesh.bsegs[:, 1]).astype(np.int64) * (1 << 32) + \
        np.maximum(mesh.bsegs[:, 0], mesh.bsegs[:, 1])
    pos = {int(k): i for i, k in enumerate(ekey)}
    etype = np.zeros(len(edges), np.int32)
    enames = [""] * len(edges)
    for s, k in enumerate(bkey):
        e = pos[int(k)]
        bi = int(mesh.bseg_bnd[s])
        if bnd_types is None:
            etype[e] = EDGE_TYPE_NAMED
            enames[e] = bnd_names[bi]
        else:
            etype[e] = int(bnd_types[bi])
            enames[e] = str(int(bnd_types[bi]))
    return ProcMesh(nodes=nodes, tris=tris, cell_names=[region_names[int(r)] for r in mesh.cell_region],
                    edges=edges, edge_type=etype, edge_names=enames)


def write_proc(pm: ProcMesh) -> str:
    """mesh.0000.proc text of a single-process part (the DECOMP writer's layout)."""
    out = io.StringIO()
    w = out.write
    nn, nc, ne = len(pm.nodes), len(pm.tris), len(pm.edges)
    w(f"{nn} {nn}\n")
    for i, (x, y) in enumerate(pm.nodes):
        w(f"{i:6d} {x:25.15e} {y:25.15e}\n")
    w(f"\n{nc} {nc}\n")
    for i, (t, nm) in enumerate(zip(pm.tris, pm.cell_names)):
        w(f"{i:6d} {t[0]:6d} {t[1]:6d} {t[2]:6d} {nm}\n")
    w(f"\n{ne} {ne}\n")
    for i, ((p, q), ty, nm) in enumerate(zip(pm.edges, pm.edge_type, pm.edge_names)):
        w(f"{i:6d} {p:6d} {q:6d} {int(ty):6d} {nm if ty != 0 else ''}\n")
    w("\n0\n\n0 0\n")
    return out.getvalue()


def read_proc(text: str) -> ProcMesh:
    """Parse a single-process .proc part (whitespace-separated, as fscanf reads it)."""
    tok = text.split()
    k = 0

    def nxt():
        nonlocal k
        k += 1
        return tok[k - 1]
    nn, nnx = int(nxt()), int(nxt())
    nodes = np.empty((nnx, 2))
    for i in range(nnx):
        nxt()
        nodes[i] = float(nxt()), float(nxt())
    nc, ncx = int(nxt()), int(nxt())
    tris = np.empty((ncx, 3), np.int32)
    names = []
    for i in range(ncx):
        nxt()
        tris[i] = int(nxt()), int(nxt()), int(nxt())
        names.append(nxt())
    ne, nex = int(nxt()), int(nxt())
    edges = np.empty((nex, 2), np.int32)
    et = np.zeros(nex, np.int32)
    en = [""] * nex
    for i in range(nex):
        nxt()
        edges[i] = int(nxt()), int(nxt())
        et[i] = int(nxt())
        if et[i] != 0:
            en[i] = nxt()
    return ProcMesh(nodes=nodes, tris=tris, cell_names=names, edges=edges, edge_type=et, edge_names=en)


@dataclass
class RkdgTask:
    """task.xml of the reference's FEM_RKDG (src/methods/fem_rkdg.cpp:23-380): the mesh is
    read from mesh/mesh.0000.proc in the working directory; regions are bound by name,
    boundaries by name (named edges) or edgeType."""
    regions: list              # Region (name, u, v, T, p, mat)
    boundaries: list           # Boundary (name, kind, edge_type, u, v, T, p)
    steady: int = 0
    tau: float = 1.0e-3
    tmax: float = 1.0e8
    cfl: float = 0.5
    file_output_step: int = 1000000
    log_output_step: int = 1000000
    func_count: int = 3
    gp_cell: int = 4
    gp_edge: int = 3
    flux: str = "GODUNOV"      # GODUNOV / LAX (anything else: GODUNOV)
    materials: list = field(default_factory=lambda: [("gas", 8.314472, 3.5, 0.0, 0.0)])
    rk: str | None = None      # GPU option RK_MODE: REFERENCE (default) / HEUN


def write_rkdg_task_xml(t: RkdgTask) -> str:
    L = ['<?xml version="1.0" encoding="UTF-8"?>', '<task method="FEM_RKDG">', "  <control>",
         f'    <STEADY value="{int(t.steady)}" />', f'    <TAU value="{_v(t.tau)}" />',
         f'    <TMAX value="{_v(t.tmax)}" />', f'    <CFL value="{_v(t.cfl)}" />',
         f'    <FILE_OUTPUT_STEP value="{int(t.file_output_step)}" />',
         f'    <LOG_OUTPUT_STEP value="{int(t.log_output_step)}" />',
         f'    <BASE_FUNC_COUNT value="{int(t.func_count)}" />', f'    <GP_CELL_COUNT value="{int(t.gp_cell)}" />',
         f'    <GP_EDGE_COUNT value="{int(t.gp_edge)}" />', f'    <FLUX value="{t.flux}" />']
    if t.rk is not None:
        L.append(f'    <RK_MODE value="{t.rk}" />')
    L += ["  </control>", f'  <materials count="{len(t.materials)}">']
    for k, (name, M, Cp, K, ML) in enumerate(t.materials):
        L += [f'    <material id="{k}">', f"      <name>{name}</name>", "      <parameters>",
              f'        <M value="{_v(M)}" />', f'        <Cp value="{_v(Cp)}" />',
              f'        <K value="{_v(K)}" />', f'        <ML value="{_v(ML)}" />',
              "      </parameters>", "    </material>"]
    L += ["  </materials>", f'  <regions count="{len(t.regions)}">']
    for k, r in enumerate(t.regions):
        L += [f'    <region id="{k}">', f'      <material id="{r.mat}" />', '      <cell type="3" />',
              f"      <name>{r.name}</name>", "      <parameters>", f'        <Vx value="{_v(r.u)}" />',
              f'        <Vy value="{_v(r.v)}" />', f'        <T value="{_v(r.T)}" />',
              f'        <P value="{_v(r.p)}" />', "      </parameters>", "    </region>"]
    L += ["  </regions>", "  <boundaries>"]
    for b in t.boundaries:
        L += [f'    <boundCond edgeType="{b.edge_type}">', f"      <type>{b.kind}</type>",
              f"      <name>{b.name}</name>"]
        if b.kind == "BOUND_INLET":
            L += ["      <parameters>", f'        <Vx value="{_v(b.u)}" />', f'        <Vy value="{_v(b.v)}" />',
                  f'        <T value="{_v(b.T)}" />', f'        <P value="{_v(b.p)}" />', "      </parameters>"]
        L.append("    </boundCond>")
    L += ["  </boundaries>", "</task>", ""]
    return "\n".join(L)
