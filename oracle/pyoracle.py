"""ctypes binding of the C oracle and a runner for the reference's own FVM_TVD.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, to check the GPU results against. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libcfd2d_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_fvm_tvd")
REF_IMP_BIN = os.path.join(HERE, "_ref", "ref_fvm_tvd_implicit")

FLUX = {"GODUNOV": 0, "LAX": 1, "ROE": 2, "HLLC": 3}
RECON = {"NONE": 0, "LINEAR": 1, "MINMOD": 2}
TIME = {"EULER": 0, "HEUN": 1, "SSPRK3": 2}
BND = {"BOUND_INLET": 1, "BOUND_OUTLET": 2, "BOUND_WALL_SLIP": 3, "BOUND_WALL_NO_SLIP": 4}
IBND = {"BOUND_INLET": 1, "BOUND_OUTLET": 2, "BOUND_WALL": 3}


class Params(C.Structure):
    _fields_ = [("flux", C.c_int), ("recon", C.c_int), ("scheme", C.c_int), ("steady", C.c_int),
                ("newton_cap", C.c_int), ("pad", C.c_int),
                ("tau_xml", C.c_double), ("cfl", C.c_double),
                ("lim_rmin", C.c_double), ("lim_rmax", C.c_double), ("lim_pmin", C.c_double),
                ("lim_pmax", C.c_double), ("lim_umax", C.c_double), ("gam_flux", C.c_double)]


class ImpParams(C.Structure):
    _fields_ = [("flux", C.c_int), ("steady", C.c_int), ("smoothing", C.c_int), ("cfl_step", C.c_int),
                ("gmres_maxit", C.c_int), ("gmres_kdim", C.c_int), ("newton_cap", C.c_int), ("pad", C.c_int),
                ("tau_xml", C.c_double), ("cfl", C.c_double), ("cfl_scale", C.c_double), ("cfl_max", C.c_double),
                ("max_lim_cells", C.c_double), ("smoothing_par", C.c_double),
                ("lim_rmin", C.c_double), ("lim_rmax", C.c_double), ("lim_pmin", C.c_double),
                ("lim_pmax", C.c_double), ("lim_umax", C.c_double), ("gmres_eps", C.c_double)]


def build(quiet: bool = True) -> str:
    """Compile the restatement (make -C oracle restatement)."""
    r = subprocess.run(["make", "-C", HERE, "restatement"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, I, D, U = C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint)
        IP = C.POINTER(C.c_int)
        L.orc_mesh_build.argtypes = [I, D, I, IP, IP, I, IP, IP, I, C.POINTER(P)]
        L.orc_mesh_sizes.argtypes = [P, IP, IP]
        L.orc_mesh_export.argtypes = [P, IP, D, D, IP, IP, IP, IP, D, D, D]
        L.orc_mesh_free.argtypes = [P]
        L.orc_region_state.argtypes = [C.c_double] * 6 + [D]
        L.orc_solver_create.argtypes = [P, C.POINTER(Params), I, D, IP, I, IP, D, D, C.POINTER(P)]
        L.orc_tau.argtypes = [P]; L.orc_tau.restype = C.c_double
        L.orc_step.argtypes = [P, I]
        L.orc_get_state.argtypes = [P, D, D, U]
        L.orc_set_state.argtypes = [P, D]
        L.orc_residual.argtypes = [P, D]
        L.orc_solver_free.argtypes = [P]
        L.orc_imp_create.argtypes = [P, C.POINTER(ImpParams), I, D, IP, I, IP, D, D, C.POINTER(P)]
        L.orc_imp_step.argtypes = [P, I]
        L.orc_imp_get_state.argtypes = [P, D, D, U]
        L.orc_imp_set_state.argtypes = [P, D]
        L.orc_imp_system.argtypes = [P, D, D, D, D]
        L.orc_imp_lim_count.argtypes = [P]
        L.orc_imp_info.argtypes = [P, D, D, IP, IP, D, IP]
        L.orc_imp_free.argtypes = [P]
        L.orc_gmres_block.argtypes = [I, IP, D, D, D, D, C.c_double, I, I, IP, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class OracleMesh:
    """Edge structure built by the reference's reader rules (see cfd2d_oracle.h)."""

    def __init__(self, nodes, tris, bsegs, bseg_bnd, berkeley_neigh=None, legacy=False):
        L = lib()
        self.nodes = np.ascontiguousarray(nodes, np.float64)
        self.tris = np.ascontiguousarray(tris, np.int32)
        bs = np.ascontiguousarray(bsegs, np.int32)
        bb = np.ascontiguousarray(bseg_bnd, np.int32)
        nb = np.ascontiguousarray(berkeley_neigh, np.int32) if berkeley_neigh is not None else None
        h = C.c_void_p()
        rc = L.orc_mesh_build(len(self.nodes), _d(self.nodes), len(self.tris), _i(self.tris),
                              _i(nb) if nb is not None else None, len(bs), _i(bs), _i(bb),
                              (2 if legacy else 1) if nb is not None else 0, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle mesh build failed ({rc})")
        self.h = h
        nc, ne = C.c_int(), C.c_int()
        L.orc_mesh_sizes(h, C.byref(nc), C.byref(ne))
        self.nc, self.ne = nc.value, ne.value

    @classmethod
    def from_mesh(cls, mesh):
        return cls(mesh.nodes, mesh.tris, mesh.bsegs, mesh.bseg_bnd)

    def export(self) -> dict:
        nc, ne = self.nc, self.ne
        out = dict(cell_edges=np.zeros((nc, 3), np.int32), cell_S=np.zeros(nc), cell_c=np.zeros((nc, 2)),
                   edge_n12=np.zeros((ne, 2), np.int32), edge_c12=np.zeros((ne, 2), np.int32),
                   edge_bnd=np.zeros(ne, np.int32), edge_npts=np.zeros(ne, np.int32),
                   edge_n=np.zeros((ne, 2)), edge_l=np.zeros(ne), edge_pts=np.zeros((ne, 3, 2)))
        lib().orc_mesh_export(self.h, _i(out["cell_edges"]), _d(out["cell_S"]), _d(out["cell_c"]),
                              _i(out["edge_n12"]), _i(out["edge_c12"]), _i(out["edge_bnd"]),
                              _i(out["edge_npts"]), _d(out["edge_n"]), _d(out["edge_l"]), _d(out["edge_pts"]))
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_free(self.h)
            self.h = None


def region_state(M, Cp, u, v, T, p) -> np.ndarray:
    out = np.zeros(4)
    lib().orc_region_state(M, Cp, u, v, T, p, _d(out))
    return out


class OracleSolver:
    def __init__(self, mesh: OracleMesh, *, flux="GODUNOV", recon="LINEAR", scheme="HEUN", steady=0,
                 tau=1e8, cfl=0.5, limits=(1e-8, 1e8, 1e-8, 1e8, 1e8), gam_flux=1.4, newton_cap=1000,
                 materials=((8.314472, 3.5),), cell_mat=None, bnd_kind=(), bnd_par=None, U0=None):
        L = lib()
        self.mesh = mesh
        p = Params(FLUX[flux], RECON[recon], TIME[scheme], int(steady), int(newton_cap), 0,
                   float(tau), float(cfl), *[float(x) for x in limits], float(gam_flux))
        mat = np.ascontiguousarray(np.asarray(materials, np.float64).reshape(-1, 2))
        cm = np.ascontiguousarray(np.zeros(mesh.nc, np.int32) if cell_mat is None else cell_mat, np.int32)
        bk = np.ascontiguousarray([BND[k] if isinstance(k, str) else int(k) for k in bnd_kind], np.int32)
        bp = np.ascontiguousarray(np.zeros((len(bk), 4)) if bnd_par is None else bnd_par, np.float64)
        U = np.ascontiguousarray(U0, np.float64).reshape(4, mesh.nc)
        h = C.c_void_p()
        rc = L.orc_solver_create(mesh.h, C.byref(p), len(mat), _d(mat), _i(cm), len(bk),
                                 _i(bk) if len(bk) else None, _d(bp), _d(U), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle solver create failed ({rc})")
        self.h = h

    @property
    def tau(self) -> float:
        return lib().orc_tau(self.h)

    def step(self, n: int) -> int:
        return lib().orc_step(self.h, int(n))

    def state(self):
        nc = self.mesh.nc
        U = np.zeros((4, nc)); ct = np.zeros(nc); fl = np.zeros(nc, np.uint32)
        lib().orc_get_state(self.h, _d(U), _d(ct), fl.ctypes.data_as(C.POINTER(C.c_uint)))
        return U, ct, fl

    def set_state(self, U):
        U = np.ascontiguousarray(U, np.float64)
        lib().orc_set_state(self.h, _d(U))

    def residual(self) -> np.ndarray:
        R = np.zeros((4, self.mesh.nc))
        lib().orc_residual(self.h, _d(R))
        return R

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_solver_free(self.h)
            self.h = None


class OracleImplicit:
    """The oracle's FVM_TVD_IMPLICIT (orc_imp_* in cfd2d_oracle.c)."""

    def __init__(self, mesh: OracleMesh, *, flux="LAX", steady=0, tau=1e-3, cfl=(1.0, 1.0, 1.0, 1000000, 1e9),
                 smoothing=(0, 0.0), limits=(1e-8, 1e8, 1e-8, 1e8, 1e8), gmres=(1e-7, 20, 30), newton_cap=1000,
                 materials=((8.314472, 3.5),), cell_mat=None, bnd_kind=(), bnd_par=None, U0=None):
        L = lib()
        self.mesh = mesh
        start, scale, cmax, cstep, maxlim = cfl
        p = ImpParams(FLUX[flux], int(steady), int(smoothing[0]), int(cstep), int(gmres[1]), int(gmres[2]),
                      int(newton_cap), 0, float(tau), float(start), float(scale), float(cmax), float(maxlim),
                      float(smoothing[1]), *[float(x) for x in limits], float(gmres[0]))
        mat = np.ascontiguousarray(np.asarray(materials, np.float64).reshape(-1, 2))
        cm = np.ascontiguousarray(np.zeros(mesh.nc, np.int32) if cell_mat is None else cell_mat, np.int32)
        bk = np.ascontiguousarray([IBND[k] if isinstance(k, str) else int(k) for k in bnd_kind], np.int32)
        bp = np.ascontiguousarray(np.zeros((len(bk), 4)) if bnd_par is None else bnd_par, np.float64)
        U = np.ascontiguousarray(U0, np.float64).reshape(4, mesh.nc)
        h = C.c_void_p()
        rc = L.orc_imp_create(mesh.h, C.byref(p), len(mat), _d(mat), _i(cm), len(bk),
                              _i(bk) if len(bk) else None, _d(bp), _d(U), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle implicit create failed ({rc})")
        self.h = h

    def step(self, n: int) -> int:
        return lib().orc_imp_step(self.h, int(n))

    def state(self):
        nc = self.mesh.nc
        U = np.zeros((4, nc)); ct = np.zeros(nc); fl = np.zeros(nc, np.uint32)
        lib().orc_imp_get_state(self.h, _d(U), _d(ct), fl.ctypes.data_as(C.POINTER(C.c_uint)))
        return U, ct, fl

    def set_state(self, U):
        lib().orc_imp_set_state(self.h, _d(np.ascontiguousarray(U, np.float64)))

    def system(self):
        nc = self.mesh.nc
        diag = np.zeros((nc, 4, 4)); off = np.zeros((nc, 3, 4, 4)); rhs = np.zeros((nc, 4)); ct = np.zeros(nc)
        lib().orc_imp_system(self.h, _d(diag), _d(off), _d(rhs), _d(ct))
        return diag, off, rhs, ct

    def info(self) -> dict:
        t, cfl, rel = C.c_double(), C.c_double(), C.c_double()
        step, it, st = C.c_int(), C.c_int(), C.c_int()
        lib().orc_imp_info(self.h, C.byref(t), C.byref(cfl), C.byref(step), C.byref(it), C.byref(rel), C.byref(st))
        return dict(t=t.value, cfl=cfl.value, step=step.value, iters=it.value, rel=rel.value, status=st.value,
                    n_lim=lib().orc_imp_lim_count(self.h))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_imp_free(self.h)
            self.h = None


def implicit_from_task(task, mesh, omesh: OracleMesh | None = None, U0=None, **over) -> OracleImplicit:
    """Oracle implicit solver configured like FVM_TVD_IMPLICIT::init from ``task`` (an ImplicitTask);
    ``mesh.cell_region`` indexes task.regions, ``mesh.bseg_bnd`` task.boundaries."""
    from cfd2d import meshgen
    if omesh is None:  # .neigh as the loader holds it: 0-based, -2 for none
        nb = meshgen.triangle_neighbours(mesh.tris)
        omesh = OracleMesh(mesh.nodes, mesh.tris, mesh.bsegs, mesh.bseg_bnd,
                           berkeley_neigh=np.where(nb >= 0, nb, -2), legacy=True)
    mats = [(m[1], m[2]) for m in task.materials]
    cell_mat = np.asarray([r.mat for r in task.regions], np.int32)[mesh.cell_region]
    if U0 is None:
        reg_U = np.stack([region_state(*mats[r.mat], r.u, r.v, r.T, r.p) for r in task.regions])
        U0 = reg_U[mesh.cell_region].T.copy()
    bk = [b.kind for b in task.boundaries]
    bp = np.asarray([[b.T, b.p, b.u, b.v] for b in task.boundaries], np.float64).reshape(-1, 4)
    kw = dict(flux=task.flux, steady=task.steady, tau=task.tau, cfl=task.cfl, smoothing=task.smoothing,
              limits=task.limits, materials=mats, cell_mat=cell_mat, bnd_kind=bk, bnd_par=bp, U0=U0)
    if getattr(task, "gmres", None) is not None:
        k, it, tol = task.gmres
        kw["gmres"] = (float(tol), int(it), int(k))
    kw.update(over)
    return OracleImplicit(omesh, **kw)


def run_reference_implicit(task_xml: str, tri_files: dict, U0=None, timeout=300, workdir=None) -> dict:
    """Run the reference's own FVM_TVD_IMPLICIT (oracle/_ref/ref_fvm_tvd_implicit) on one case;
    tri_files: extension -> text of mesh.node/.ele/.neigh/.poly."""
    if not os.path.exists(REF_IMP_BIN):
        raise FileNotFoundError(REF_IMP_BIN + " (build with: make -C oracle reference REF=<reference checkout>)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        open(os.path.join(d, "task.xml"), "w").write(task_xml)
        for ext, text in tri_files.items():
            open(os.path.join(d, "mesh" + ext), "w").write(text)
        args = [REF_IMP_BIN, "task.xml", "out"]
        if U0 is not None:
            np.ascontiguousarray(U0, np.float64).tofile(os.path.join(d, "init.bin"))
            args.append("init.bin")
        r = subprocess.run(args, cwd=d, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
        out = {}
        for tag in ("init", "state"):
            raw = open(os.path.join(d, f"out.{tag}.bin"), "rb").read()
            nc, iters = (int(x) for x in np.frombuffer(raw[:8], np.int32))
            tau, secs, cfl, rel = np.frombuffer(raw, np.float64, 4, 16)
            off = 48
            U = np.frombuffer(raw, np.float64, 4 * nc, off).reshape(4, nc).copy(); off += 32 * nc
            ct = np.frombuffer(raw, np.float64, nc, off).copy(); off += 8 * nc
            fl = np.frombuffer(raw, np.uint32, nc, off).copy()
            out[tag] = dict(U=U, cTau=ct, flags=fl, tau=float(tau), seconds=float(secs), cfl=float(cfl),
                            iters=iters, rel=float(rel))
        out["stdout"] = r.stdout
        out["vtk"] = {f: open(os.path.join(d, f)).read() for f in sorted(os.listdir(d)) if f.endswith(".vtk")}
        return out


# ------------------------------------------------------------- task helpers

def solver_from_task(task, mesh, omesh: OracleMesh | None = None, U0=None, **over) -> OracleSolver:
    """Oracle solver configured like FVM_TVD::init configures itself from ``task``."""
    omesh = omesh or OracleMesh.from_mesh(mesh)
    mats = [(m[1], m[2]) for m in task.materials]
    cell_mat = np.asarray([task.regions[r].mat for r in range(len(task.regions))], np.int32)[mesh.cell_region]
    if U0 is None:
        reg_U = np.stack([region_state(*mats[r.mat], r.u, r.v, r.T, r.p) for r in task.regions])
        U0 = reg_U[mesh.cell_region].T.copy()
    bk = [b.kind for b in task.boundaries]
    bp = np.asarray([[b.u, b.v, b.T, b.p] for b in task.boundaries], np.float64)
    kw = dict(flux=task.flux or "GODUNOV", recon=task.reconstruction or "LINEAR",
              scheme=task.time_scheme or "HEUN", steady=task.steady, tau=task.tau, cfl=task.cfl,
              limits=task.limits, materials=mats, cell_mat=cell_mat, bnd_kind=bk, bnd_par=bp, U0=U0)
    kw.update(over)
    return OracleSolver(omesh, **kw)


# ------------------------------------------------------------- reference runs

def read_ref_grid(path) -> dict:
    raw = open(path, "rb").read()
    nc, ne, nn, _ = np.frombuffer(raw[:16], np.int32)
    off = 16
    out = {}

    def take(name, dtype, count, shape):
        nonlocal off
        a = np.frombuffer(raw, dtype, count, off).reshape(shape).copy()
        off += a.nbytes
        out[name] = a
    take("nodes", np.float64, nn * 2, (nn, 2))
    take("cell_nodes", np.int32, nc * 3, (nc, 3))
    take("cell_edges", np.int32, nc * 3, (nc, 3))
    take("cell_S", np.float64, nc, (nc,))
    take("cell_c", np.float64, nc * 2, (nc, 2))
    take("edge_n12", np.int32, ne * 2, (ne, 2))
    take("edge_c12", np.int32, ne * 2, (ne, 2))
    take("edge_type", np.int32, ne, (ne,))
    take("edge_bnd", np.int32, ne, (ne,))
    take("edge_npts", np.int32, ne, (ne,))
    take("edge_n", np.float64, ne * 2, (ne, 2))
    take("edge_l", np.float64, ne, (ne,))
    take("edge_pts", np.float64, ne * 6, (ne, 3, 2))
    assert off == len(raw)
    return out


def read_ref_state(path) -> dict:
    raw = open(path, "rb").read()
    nc = int(np.frombuffer(raw[:4], np.int32)[0])
    tau, secs = np.frombuffer(raw, np.float64, 2, 16)
    off = 32
    U = np.frombuffer(raw, np.float64, 4 * nc, off).reshape(4, nc).copy(); off += 32 * nc
    ct = np.frombuffer(raw, np.float64, nc, off).copy(); off += 8 * nc
    fl = np.frombuffer(raw, np.uint32, nc, off).copy()
    return dict(U=U, tau=float(tau), seconds=float(secs), cTau=ct, flags=fl)


def run_reference(task_xml: str, unv_text: str, U0=None, timeout=120, workdir=None) -> dict:
    """Run the reference's own FVM_TVD (oracle/_ref/ref_fvm_tvd) on one case."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN + " (build with: make -C oracle reference REF=<reference checkout>)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        open(os.path.join(d, "task.xml"), "w").write(task_xml)
        open(os.path.join(d, "mesh.unv"), "w").write(unv_text)
        args = [REF_BIN, "task.xml", "out"]
        if U0 is not None:
            np.ascontiguousarray(U0, np.float64).tofile(os.path.join(d, "init.bin"))
            args.append("init.bin")
        r = subprocess.run(args, cwd=d, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
        vtk = {f: open(os.path.join(d, f)).read() for f in sorted(os.listdir(d)) if f.endswith(".vtk")}
        return dict(grid=read_ref_grid(os.path.join(d, "out.grid.bin")),
                    init=read_ref_state(os.path.join(d, "out.init.bin")),
                    final=read_ref_state(os.path.join(d, "out.state.bin")),
                    stdout=r.stdout, vtk=vtk)


# ------------------------------------------------------------- FEM_RKDG

REF_DG_BIN = os.path.join(HERE, "_ref", "ref_fem_rkdg")
DG_RK = {"REFERENCE": 0, "HEUN": 1}


class DgParams(C.Structure):
    _fields_ = [("steady", C.c_int), ("flux", C.c_int), ("gp_cell", C.c_int), ("gp_edge", C.c_int),
                ("rk_mode", C.c_int), ("newton_cap", C.c_int),
                ("tau", C.c_double), ("tmax", C.c_double), ("cfl", C.c_double)]


def _dg_lib():
    L = lib()
    if not getattr(L, "_dg_ready", False):
        P, I, D = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        IP = C.POINTER(C.c_int)
        L.orc_dg_create.argtypes = [C.POINTER(DgParams), I, D, I, IP, IP, I, IP, IP, I, D, I, IP, D]
        L.orc_dg_create.restype = P
        L.orc_dg_set.argtypes = [P, D]
        L.orc_dg_set_tau.argtypes = [P, C.c_double]
        L.orc_dg_step.argtypes = [P, I]; L.orc_dg_step.restype = C.c_uint
        L.orc_dg_get.argtypes = [P, D, D, D]
        L.orc_dg_geom.argtypes = [P, IP, IP, D, D, D]
        L.orc_dg_centre.argtypes = [P, D]
        L.orc_dg_free.argtypes = [P]
        L._dg_ready = True
    return L


def dg_binding(task, pm):
    """Region index per cell (by name, getRegion(typeName)) and boundary index per edge
    (by name for named edges, else by edgeType; -1 inside), as FEM_RKDG::init binds them
    (src/methods/fem_rkdg.cpp:196-248, 1382-1401)."""
    names = {r.name: k for k, r in enumerate(task.regions)}
    creg = np.array([names[n] for n in pm.cell_names], np.int32)
    ebnd = np.full(len(pm.edges), -1, np.int32)
    for e, (ty, nm) in enumerate(zip(pm.edge_type, pm.edge_names)):
        if ty == 0:
            continue
        for k, b in enumerate(task.boundaries):
            if (ty == 0x100 and b.name == nm) or (ty != 0x100 and ty == b.edge_type):
                ebnd[e] = k
                break
        else:
            raise ValueError(f"unknown edge type of edge {e}")
    return creg, ebnd


class OracleDG:
    """The C restatement of FEM_RKDG on one .proc mesh part (see cfd2d_oracle.h)."""

    def __init__(self, task, pm, *, rk=None, newton_cap=100):
        L = _dg_lib()
        rk = rk or task.rk or "REFERENCE"
        p = DgParams(int(task.steady), FLUX.get(task.flux, 0) if task.flux in ("GODUNOV", "LAX") else 0,
                     int(task.gp_cell), int(task.gp_edge), DG_RK[rk], int(newton_cap),
                     float(task.tau), float(task.tmax), float(task.cfl))
        creg, ebnd = dg_binding(task, pm)
        mats = task.materials
        reg = np.array([[mats[r.mat][1], mats[r.mat][2], r.u, r.v, r.T, r.p] for r in task.regions], np.float64)
        bkind = np.array([BND[b.kind] for b in task.boundaries], np.int32)
        bpar = np.array([[b.u, b.v, b.T, b.p] for b in task.boundaries], np.float64).reshape(-1, 4)
        self.nodes = np.ascontiguousarray(pm.nodes, np.float64)
        self.tris = np.ascontiguousarray(pm.tris, np.int32)
        self.edges = np.ascontiguousarray(pm.edges, np.int32)
        self._keep = (creg, ebnd, reg, bkind, bpar)
        self.h = L.orc_dg_create(C.byref(p), len(self.nodes), _d(self.nodes), len(self.tris), _i(self.tris),
                                 _i(creg), len(self.edges), _i(self.edges), _i(ebnd), len(reg), _d(reg),
                                 len(bkind), _i(bkind), _d(bpar))
        if not self.h:
            raise RuntimeError("orc_dg_create failed")
        self.nc, self.ne = len(self.tris), len(self.edges)

    def set_coeffs(self, U):
        U = np.ascontiguousarray(U, np.float64).reshape(self.nc, 12)
        _dg_lib().orc_dg_set(self.h, _d(U))

    def set_tau(self, tau):
        _dg_lib().orc_dg_set_tau(self.h, float(tau))

    def step(self, n: int) -> int:
        return int(_dg_lib().orc_dg_step(self.h, int(n)))

    def state(self) -> dict:
        U = np.empty((self.nc, 12)); ct = np.empty(self.nc); sc = np.empty(7)
        _dg_lib().orc_dg_get(self.h, _d(U), _d(ct), _d(sc))
        return dict(U=U, cTau=ct, tau=float(sc[0]), t=float(sc[1]), res=sc[2:6].copy(), step=int(sc[6]))

    def geom(self) -> dict:
        ce = np.empty((self.nc, 3), np.int32); cc = np.empty((self.ne, 2), np.int32)
        c6 = np.empty((self.nc, 6)); ia = np.empty((self.nc, 9)); e4 = np.empty((self.ne, 4))
        _dg_lib().orc_dg_geom(self.h, _i(ce), _i(cc), _d(c6), _d(ia), _d(e4))
        return dict(cedge=ce, c1c2=cc, cell6=c6, invA=ia, edge4=e4)

    def centre(self) -> np.ndarray:
        out = np.empty((self.nc, 4))
        _dg_lib().orc_dg_centre(self.h, _d(out))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            _dg_lib().orc_dg_free(self.h)
            self.h = None


def run_reference_rkdg(task_xml: str, proc_text: str, steps: int, U0=None, tau=None, timeout=300,
                       workdir=None) -> dict:
    """Run the reference's own FEM_RKDG (oracle/_ref/ref_fem_rkdg, see oracle/ref/ref_rkdg.cpp)
    on one case: mesh/mesh.0000.proc = proc_text; U0: (nc, 12) coefficients or None; tau: a
    time step to impose after init. Returns the dumps, stdout and the VTU/PVTU files."""
    if not os.path.exists(REF_DG_BIN):
        raise FileNotFoundError(REF_DG_BIN + " (build with: make -C oracle reference REF=<reference checkout>)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        os.makedirs(os.path.join(d, "mesh"))
        open(os.path.join(d, "task.xml"), "w").write(task_xml)
        open(os.path.join(d, "mesh", "mesh.0000.proc"), "w").write(proc_text)
        args = [REF_DG_BIN, "task.xml", "out", str(int(steps))]
        if U0 is not None or tau is not None:
            if U0 is not None:
                np.ascontiguousarray(U0, np.float64).tofile(os.path.join(d, "init.bin"))
            args.append("init.bin" if U0 is not None else "-")
        if tau is not None:
            args.append(repr(float(tau)))
        r = subprocess.run(args, cwd=d, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
        out = {}
        for tag in ("init", "state"):
            raw = open(os.path.join(d, f"out.{tag}.bin"), "rb").read()
            nc = int(np.frombuffer(raw[:4], np.int32)[0])
            sc = np.frombuffer(raw, np.float64, 6, 16)
            off = 64
            U = np.frombuffer(raw, np.float64, 12 * nc, off).reshape(nc, 12).copy(); off += 96 * nc
            ct = np.frombuffer(raw, np.float64, nc, off).copy()
            out[tag] = dict(U=U, cTau=ct, tau=float(sc[0]), tmax=float(sc[1]), res=sc[2:6].copy())
        raw = open(os.path.join(d, "out.geom.bin"), "rb").read()
        nc, ne, nn, gc, ge, fc = (int(x) for x in np.frombuffer(raw[:24], np.int32))
        off = 32
        g = {}
        g["cedge"] = np.frombuffer(raw, np.int32, 3 * nc, off).reshape(nc, 3).copy(); off += 12 * nc
        g["c1c2"] = np.frombuffer(raw, np.int32, 2 * ne, off).reshape(ne, 2).copy(); off += 8 * ne
        g["cell6"] = np.frombuffer(raw, np.float64, 6 * nc, off).reshape(nc, 6).copy(); off += 48 * nc
        g["cgp"] = np.frombuffer(raw, np.float64, 3 * gc * nc, off).reshape(nc, gc, 3).copy(); off += 24 * gc * nc
        g["invA"] = np.frombuffer(raw, np.float64, 9 * nc, off).reshape(nc, 9).copy(); off += 72 * nc
        g["edge4"] = np.frombuffer(raw, np.float64, 4 * ne, off).reshape(ne, 4).copy(); off += 32 * ne
        g["egp"] = np.frombuffer(raw, np.float64, 3 * ge * ne, off).reshape(ne, ge, 3).copy()
        out["geom"] = g
        out["stdout"] = r.stdout
        files = {}
        for root, _, fs in os.walk(d):
            for f in fs:
                if f.endswith(".vtu") or f.endswith(".pvtu"):
                    full = os.path.join(root, f)
                    files[os.path.relpath(full, d)] = open(full).read()
        out["vtu"] = files
        return out
