"""ctypes binding of libcfd2d_gpu.so (include/cfd2d.h).

Mirrors the reference's Method interface for FVM_TVD (src/methods/method.h:6-11):
``Solver(task_xml)`` is init, ``run()`` is run, ``close()`` is done. There is no
fallback: if the shared library is missing or cannot be loaded, importing the
solver raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libcfd2d_gpu.so")

OK = 0
ERR_NEWTON_CAP = 503
ERR_NONPHYSICAL = 504


class CfdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cfd2d error {code}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("xy", C.POINTER(C.c_double)), ("n_cells", C.c_int),
                ("tri", C.POINTER(C.c_int)), ("cell_region", C.POINTER(C.c_int)), ("n_bsegs", C.c_int),
                ("bseg", C.POINTER(C.c_int)), ("bseg_bnd", C.POINTER(C.c_int))]


class Info(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_edges", C.c_int), ("n_boundary_edges", C.c_int), ("n_nodes", C.c_int),
                ("step", C.c_int), ("flux", C.c_int), ("recon", C.c_int), ("scheme", C.c_int),
                ("precision", C.c_int), ("steady", C.c_int), ("time", C.c_double), ("tau", C.c_double),
                ("device_bytes", C.c_size_t), ("n_instances", C.c_int)]


class ImplicitStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("n_limited", C.c_int), ("pad", C.c_int),
                ("rel_residual", C.c_double), ("cfl", C.c_double)]


# every symbol include/cfd2d.h declares, with its ctypes signature
_P, _I, _D = C.c_void_p, C.c_int, C.POINTER(C.c_double)
_IP, _UP = C.POINTER(C.c_int), C.POINTER(C.c_uint)
SIGNATURES = {
    "cfd2d_create": [C.c_char_p, C.POINTER(_P)],
    "cfd2d_create_with_mesh": [C.c_char_p, C.POINTER(MeshDesc), C.POINTER(_P)],
    "cfd2d_step": [_P, _I],
    "cfd2d_run": [_P],
    "cfd2d_destroy": [_P],
    "cfd2d_get_info": [_P, C.POINTER(Info)],
    "cfd2d_get_state": [_P, _D, _D, _D, _D],
    "cfd2d_set_state": [_P, _D, _D, _D, _D, _I],
    "cfd2d_get_time_step": [_P, _D],
    "cfd2d_get_flags": [_P, _UP],
    "cfd2d_residual": [_P, _D],
    "cfd2d_conservation": [_P, _D],
    "cfd2d_save_vtk": [_P, _I],
    "cfd2d_batch_create": [_I, C.POINTER(C.c_char_p), C.POINTER(MeshDesc), C.POINTER(_P)],
    "cfd2d_batch_instance": [_P, _I, _IP, _IP, _D, _D],
    "cfd2d_autotune": [_P, C.c_char_p],
    "cfd2d_load_tuning": [_P, C.c_char_p],
    "cfd2d_set_objective": [_P, _I, _D, C.c_double],
    "cfd2d_forward": [_P, _I, _I, _D],
    "cfd2d_backward": [_P, _D, _D],
    "cfd2d_set_boundary": [_P, _I, _D],
    "cfd2d_timed_steps": [_P, _I, _D],
    "cfd2d_profile_steps": [_P, _I, _D, _IP],
    "cfd2d_save_state": [_P, C.c_char_p],
    "cfd2d_load_state": [_P, C.c_char_p],
    "cfd2d_residual_first_order_static": [_I, _I, _P, _P, _P, _P, _P, _I, _IP, _D, C.c_double, C.c_double, _I,
                                          _P, _P, _P],
    "cfd2d_static_reset": [],
    "cfd2d_implicit_system": [_P, _D, _D, _D, _D],
    "cfd2d_implicit_stats": [_P, C.POINTER(ImplicitStats)],
    "cfd2d_dg_get_coeffs": [_P, _D],
    "cfd2d_dg_set_coeffs": [_P, _D],
    "cfd2d_dg_set_time_step": [_P, C.c_double],
    "cfd2d_dg_residuals": [_P, _D],
    "cfd2d_selftest": [_I, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)],
    "cfd2d_set_device": [_I],
    "cfd2d_last_error": [C.c_char_p, C.c_size_t],
    "cfd2d_set_verbosity": [_I],
    "cfd2d_set_log_file": [C.c_char_p],
    "cfd2d_mesh_load": [C.c_char_p, C.POINTER(_P)],
    "cfd2d_mesh_build": [C.POINTER(MeshDesc), _IP, C.POINTER(_P)],
    "cfd2d_mesh_sizes": [_P, _IP, _IP],
    "cfd2d_mesh_export": [_P, _IP, _D, _D, _IP, _IP, _IP, _IP, _D, _D, _D],
    "cfd2d_mesh_order": [_P, _I, _IP],
    "cfd2d_mesh_free": [_P],
}

_lib = None


def lib():
    """Load the library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().cfd2d_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int, allow=(OK,)) -> int:
    if rc not in allow:
        raise CfdError(rc, last_error())
    return rc


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def mesh_desc(nodes, tris, cell_region, bsegs, bseg_bnd):
    """MeshDesc over contiguous copies (returned alongside to keep them alive)."""
    keep = [np.ascontiguousarray(nodes, np.float64), np.ascontiguousarray(tris, np.int32),
            np.ascontiguousarray(cell_region, np.int32), np.ascontiguousarray(bsegs, np.int32),
            np.ascontiguousarray(bseg_bnd, np.int32)]
    d = MeshDesc(len(keep[0]), _d(keep[0]), len(keep[1]), _i(keep[1]), _i(keep[2]), len(keep[3]), _i(keep[3]),
                 _i(keep[4]))
    return d, keep


def selftest(which: int, n: int, seed: int = 1) -> int:
    """Mismatch count of a device arithmetic helper against the hardware operation."""
    out = C.c_longlong(-1)
    check(lib().cfd2d_selftest(int(which), int(n), int(seed), C.byref(out)))
    return out.value


def set_device(device: int):
    check(lib().cfd2d_set_device(int(device)))


def set_verbosity(level: int):
    lib().cfd2d_set_verbosity(int(level))


def _count_boundaries(task_xml: str) -> int:
    import xml.etree.ElementTree as ET
    try:
        return len(ET.parse(task_xml).getroot().find("boundaries").findall("boundCond"))
    except Exception:
        return 0


class Solver:
    """One FVM_TVD instance on the GPU."""

    def __init__(self, task_xml: str, mesh=None):
        L = lib()
        h = C.c_void_p()
        if mesh is None:
            check(L.cfd2d_create(task_xml.encode(), C.byref(h)))
        else:
            d, self._keep = mesh_desc(mesh.nodes, mesh.tris, mesh.cell_region, mesh.bsegs, mesh.bseg_bnd)
            check(L.cfd2d_create_with_mesh(task_xml.encode(), C.byref(d), C.byref(h)))
        self.h = h
        self.info = self.get_info()
        self.n = self.info.n_cells
        self._nbnd = _count_boundaries(task_xml)

    def get_info(self) -> Info:
        inf = Info()
        check(lib().cfd2d_get_info(self.h, C.byref(inf)))
        return inf

    def step(self, n: int = 1, allow_warnings: bool = False) -> int:
        allow = (OK, ERR_NEWTON_CAP, ERR_NONPHYSICAL) if allow_warnings else (OK,)
        return check(lib().cfd2d_step(self.h, int(n)), allow)

    def run(self) -> int:
        return check(lib().cfd2d_run(self.h), (OK, ERR_NEWTON_CAP, ERR_NONPHYSICAL))

    def state(self, out=None) -> np.ndarray:
        U = np.empty((4, self.n)) if out is None else out
        check(lib().cfd2d_get_state(self.h, _d(U[0]), _d(U[1]), _d(U[2]), _d(U[3])))
        return U

    def set_state(self, U, reset_time_step: bool = False):
        U = np.ascontiguousarray(U, np.float64).reshape(4, self.n)
        check(lib().cfd2d_set_state(self.h, _d(U[0]), _d(U[1]), _d(U[2]), _d(U[3]), int(reset_time_step)))

    def time_step(self) -> np.ndarray:
        t = np.empty(self.n)
        check(lib().cfd2d_get_time_step(self.h, _d(t)))
        return t

    def flags(self) -> np.ndarray:
        f = np.empty(self.n, np.uint32)
        check(lib().cfd2d_get_flags(self.h, f.ctypes.data_as(C.POINTER(C.c_uint))))
        return f

    def residual(self) -> np.ndarray:
        R = np.empty((4, self.n))
        check(lib().cfd2d_residual(self.h, _d(R)))
        return R

    def conservation(self) -> np.ndarray:
        s = np.empty(4)
        check(lib().cfd2d_conservation(self.h, _d(s)))
        return s

    def save_state(self, path: str):
        check(lib().cfd2d_save_state(self.h, path.encode()))

    def load_state(self, path: str):
        check(lib().cfd2d_load_state(self.h, path.encode()))

    def save_vtk(self, step: int):
        check(lib().cfd2d_save_vtk(self.h, int(step)))

    # ---- discrete adjoint
    def set_objective(self, kind: int, weights, p_ref: float = 0.0):
        w = np.ascontiguousarray(weights, np.float64)
        check(lib().cfd2d_set_objective(self.h, int(kind), _d(w), float(p_ref)))

    def forward(self, nsteps: int, checkpoint_every: int) -> float:
        J = np.zeros(1)
        check(lib().cfd2d_forward(self.h, int(nsteps), int(checkpoint_every), _d(J)))
        return float(J[0])

    def backward(self):
        """(dJ/dU0 as 4 x n_cells, dJ/d(Vx, Vy, T, P) per boundary as n_bnd x 4)."""
        g = np.empty((4, self.n))
        nb = max(self._nbnd, 1)
        gb = np.zeros((nb, 4))
        check(lib().cfd2d_backward(self.h, _d(g), _d(gb)))
        return g, gb[:self._nbnd]

    def set_boundary(self, b: int, par):
        p = np.ascontiguousarray(par, np.float64)
        check(lib().cfd2d_set_boundary(self.h, int(b), _d(p)))

    def autotune(self, json_path: str | None = None):
        check(lib().cfd2d_autotune(self.h, json_path.encode() if json_path else None))

    def load_tuning(self, json_path: str):
        check(lib().cfd2d_load_tuning(self.h, json_path.encode()))

    def timed_steps(self, n: int) -> float:
        """Device milliseconds for n steps (CUDA events on the solver's stream)."""
        ms = np.zeros(1)
        check(lib().cfd2d_timed_steps(self.h, int(n), _d(ms)))
        return float(ms[0])

    def profile_steps(self, n: int):
        """Per kernel kind (grad, flux, update, remediate): device ms and launch counts over n steps."""
        ms = np.zeros(4); cnt = np.zeros(4, np.int32)
        check(lib().cfd2d_profile_steps(self.h, int(n), _d(ms), _i(cnt)))
        return ms, cnt

    def implicit_system(self):
        """FVM_TVD_IMPLICIT: (diag (nc,4,4), off (nc,3,4,4), rhs (nc,4), cTau (nc)) of the current state."""
        nc = self.get_info().n_cells
        diag = np.zeros((nc, 4, 4)); off = np.zeros((nc, 3, 4, 4)); rhs = np.zeros((nc, 4)); ct = np.zeros(nc)
        check(lib().cfd2d_implicit_system(self.h, _d(diag), _d(off), _d(rhs), _d(ct)))
        return diag, off, rhs, ct

    def implicit_stats(self) -> dict:
        st = ImplicitStats()
        check(lib().cfd2d_implicit_stats(self.h, C.byref(st)))
        return dict(iters=st.iterations, status=st.status, n_lim=st.n_limited, rel=st.rel_residual, cfl=st.cfl)

    # FEM_RKDG handles: P1 coefficients, 12 per cell (ro[3] ru[3] rv[3] re[3])
    def dg_coeffs(self, out=None) -> np.ndarray:
        U = np.empty((self.n, 12)) if out is None else out
        check(lib().cfd2d_dg_get_coeffs(self.h, _d(U)))
        return U

    def set_dg_coeffs(self, U):
        U = np.ascontiguousarray(U, np.float64).reshape(self.n, 12)
        check(lib().cfd2d_dg_set_coeffs(self.h, _d(U)))

    def dg_coeffs_into(self, ptr):
        """cfd2d_dg_get_coeffs into a raw pointer (host, pinned or device)."""
        check(lib().cfd2d_dg_get_coeffs(self.h, C.cast(ptr, C.POINTER(C.c_double))))

    def set_dg_coeffs_from(self, ptr):
        check(lib().cfd2d_dg_set_coeffs(self.h, C.cast(ptr, C.POINTER(C.c_double))))

    def dg_set_time_step(self, tau: float):
        check(lib().cfd2d_dg_set_time_step(self.h, float(tau)))

    def dg_residuals(self) -> np.ndarray:
        r = np.zeros(4)
        check(lib().cfd2d_dg_residuals(self.h, _d(r)))
        return r

    def state_into(self, ptrs):
        """get_state into four raw host pointers (e.g. pinned buffers)."""
        P = C.POINTER(C.c_double)
        check(lib().cfd2d_get_state(self.h, *[C.cast(p, P) for p in ptrs]))

    def set_state_from(self, ptrs, reset_time_step: bool = False):
        P = C.POINTER(C.c_double)
        check(lib().cfd2d_set_state(self.h, *[C.cast(p, P) for p in ptrs], int(reset_time_step)))

    @property
    def tau(self) -> float:
        return self.get_info().tau

    def close(self):
        if getattr(self, "h", None):
            lib().cfd2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch(Solver):
    """Many independent instances solved together (cfd2d_batch_create)."""

    def __init__(self, task_xmls, meshes=None):
        L = lib()
        n = len(task_xmls)
        paths = (C.c_char_p * n)(*[p.encode() for p in task_xmls])
        h = C.c_void_p()
        if meshes is None:
            check(L.cfd2d_batch_create(n, paths, None, C.byref(h)))
        else:
            descs = (MeshDesc * n)()
            self._keep = []
            for k, m in enumerate(meshes):
                d, keep = mesh_desc(m.nodes, m.tris, m.cell_region, m.bsegs, m.bseg_bnd)
                descs[k] = d
                self._keep.append(keep)
            check(L.cfd2d_batch_create(n, paths, descs, C.byref(h)))
        self.h = h
        self.info = self.get_info()
        self.n = self.info.n_cells
        self._nbnd = sum(_count_boundaries(p) for p in task_xmls)
        self.count = n

    def instance(self, k: int):
        """(cell_offset, n_cells, tau, time) of instance k."""
        off, nc = C.c_int(), C.c_int()
        tau, t = np.zeros(1), np.zeros(1)
        check(lib().cfd2d_batch_instance(self.h, int(k), C.byref(off), C.byref(nc), _d(tau), _d(t)))
        return off.value, nc.value, float(tau[0]), float(t[0])


class Mesh:
    """Host-only edge structure as the reference's readers build it (no GPU needed)."""

    def __init__(self, task_xml: str | None = None, nodes=None, tris=None, bsegs=None, bseg_bnd=None,
                 berkeley_neigh=None):
        L = lib()
        h = C.c_void_p()
        if task_xml is not None:
            check(L.cfd2d_mesh_load(task_xml.encode(), C.byref(h)))
        else:
            d, self._keep = mesh_desc(nodes, tris, np.zeros(len(tris), np.int32), bsegs, bseg_bnd)
            nb = np.ascontiguousarray(berkeley_neigh, np.int32) if berkeley_neigh is not None else None
            self._keep.append(nb)
            check(L.cfd2d_mesh_build(C.byref(d), _i(nb) if nb is not None else None, C.byref(h)))
        self.h = h
        nc, ne = C.c_int(), C.c_int()
        check(L.cfd2d_mesh_sizes(h, C.byref(nc), C.byref(ne)))
        self.nc, self.ne = nc.value, ne.value

    def export(self) -> dict:
        nc, ne = self.nc, self.ne
        o = dict(cell_edges=np.zeros((nc, 3), np.int32), cell_S=np.zeros(nc), cell_c=np.zeros((nc, 2)),
                 edge_n12=np.zeros((ne, 2), np.int32), edge_c12=np.zeros((ne, 2), np.int32),
                 edge_bnd=np.zeros(ne, np.int32), edge_npts=np.zeros(ne, np.int32), edge_n=np.zeros((ne, 2)),
                 edge_l=np.zeros(ne), edge_pts=np.zeros((ne, 3, 2)))
        check(lib().cfd2d_mesh_export(self.h, _i(o["cell_edges"]), _d(o["cell_S"]), _d(o["cell_c"]),
                                      _i(o["edge_n12"]), _i(o["edge_c12"]), _i(o["edge_bnd"]), _i(o["edge_npts"]),
                                      _d(o["edge_n"]), _d(o["edge_l"]), _d(o["edge_pts"])))
        return o

    def order(self, rcm: bool = True) -> np.ndarray:
        p = np.zeros(self.nc, np.int32)
        check(lib().cfd2d_mesh_order(self.h, int(rcm), _i(p)))
        return p

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.cfd2d_mesh_free(self.h)
            self.h = None
