"""cfd2d_residual_first_order_static: the entry point that allocates nothing.

Callers recording a CUDA graph, or living inside a framework that owns the
device's memory pool, cannot let the library call cudaMalloc when they call in.
This entry point keeps its only scratch (one FP64 flux per edge) in a fixed
device array inside the library and writes the residual into the caller's
buffer. Its result must equal the handle-based cfd2d_residual of a solver
created with RECONSTRUCTION NONE, bit for bit (the FP64 bar of these tests), on
two calls in a row: the second call must not see anything the first call left
in the shared array. Collected last so a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

from cfd2d import cases

pytestmark = pytest.mark.gpu

KINDS = ("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP")
KIND_CODE = {"BOUND_INLET": 1, "BOUND_OUTLET": 2, "BOUND_WALL_SLIP": 3, "BOUND_WALL_NO_SLIP": 4}


def _static_residual(capi, dev, U_dev, R_dev, t, flux_code):
    import torch
    kinds = np.array([KIND_CODE[b.kind] for b in t.boundaries], np.int32)
    par = np.array([[b.u, b.v, b.T, b.p] for b in t.boundaries], np.float64)
    M, Cp = t.materials[0][1], t.materials[0][2]
    rc = capi.lib().cfd2d_residual_first_order_static(
        dev["nc"], dev["ne"], C.c_void_p(dev["cell_edges"].data_ptr()), C.c_void_p(dev["c12"].data_ptr()),
        C.c_void_p(dev["n"].data_ptr()), C.c_void_p(dev["l"].data_ptr()), C.c_void_p(dev["bnd"].data_ptr()),
        len(kinds), kinds.ctypes.data_as(C.POINTER(C.c_int)), par.ctypes.data_as(C.POINTER(C.c_double)),
        M, Cp, flux_code, C.c_void_p(U_dev.data_ptr()), C.c_void_p(R_dev.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("flux", ["HLLC", "LAX", "ROE", "GODUNOV"])
def test_static_residual_matches_handle_residual_twice(capi, tmp_path, flux):
    import torch
    t, m, U0 = cases.vortex(20, flux=flux, recon="NONE", scheme="EULER", bnd_kinds=KINDS, seed=21)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    mesh = capi.Mesh(nodes=m.nodes, tris=m.tris, bsegs=m.bsegs, bseg_bnd=m.bseg_bnd).export()
    cuda = torch.device("cuda:0")
    dev = {"nc": m.n_cells, "ne": len(mesh["edge_l"]),
           "cell_edges": torch.from_numpy(mesh["cell_edges"].ravel()).to(cuda),
           "c12": torch.from_numpy(mesh["edge_c12"].ravel()).to(cuda),
           "n": torch.from_numpy(mesh["edge_n"].ravel()).to(cuda),
           "l": torch.from_numpy(mesh["edge_l"]).to(cuda),
           "bnd": torch.from_numpy(mesh["edge_bnd"]).to(cuda)}
    flux_code = {"GODUNOV": 0, "LAX": 1, "ROE": 2, "HLLC": 3}[flux]
    U1 = U0
    U2 = U0 * np.array([[1.02], [0.97], [1.05], [1.01]])  # a second, different state
    R_dev = torch.full((4, m.n_cells), float("nan"), dtype=torch.float64, device=cuda)
    for U in (U1, U2):
        s.set_state(U)
        R_ref = s.residual()
        U_dev = torch.from_numpy(np.ascontiguousarray(U)).to(cuda)
        assert _static_residual(capi, dev, U_dev, R_dev, t, flux_code) == capi.OK
        R = R_dev.cpu().numpy()
        if flux == "GODUNOV":   # exp/log inside the exact solver: the FP64 tolerance
            assert np.max(np.abs(R - R_ref)) <= 1e-12 * np.max(np.abs(R_ref))
        else:
            assert np.array_equal(R.view(np.int64), R_ref.view(np.int64))


def test_static_residual_without_boundary_conditions(capi, tmp_path):
    """n_bnd == 0 is a valid call: every cell whose three edges are interior gets the
    handle's residual bit for bit; cells on a boundary edge (which would need a
    boundary condition) get NaN, and nothing reads outside the arrays."""
    import torch
    t, m, U0 = cases.vortex(20, flux="HLLC", recon="NONE", scheme="EULER", bnd_kinds=KINDS, seed=22)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    mesh = capi.Mesh(nodes=m.nodes, tris=m.tris, bsegs=m.bsegs, bseg_bnd=m.bseg_bnd).export()
    cuda = torch.device("cuda:0")
    ce = mesh["cell_edges"].reshape(-1, 3)
    c12 = mesh["edge_c12"].reshape(-1, 2)
    interior = np.all(c12[ce][:, :, 1] >= 0, axis=1)
    assert interior.sum() > 0 and (~interior).sum() > 0
    dev = {k: torch.from_numpy(np.ascontiguousarray(mesh[v]).ravel()).to(cuda)
           for k, v in (("cell_edges", "cell_edges"), ("c12", "edge_c12"), ("n", "edge_n"), ("l", "edge_l"),
                        ("bnd", "edge_bnd"))}
    s.set_state(U0)
    R_ref = s.residual()
    U_dev = torch.from_numpy(np.ascontiguousarray(U0)).to(cuda)
    R_dev = torch.zeros((4, m.n_cells), dtype=torch.float64, device=cuda)
    p = lambda x: C.c_void_p(x.data_ptr())
    rc = capi.lib().cfd2d_residual_first_order_static(
        m.n_cells, len(mesh["edge_l"]), p(dev["cell_edges"]), p(dev["c12"]), p(dev["n"]), p(dev["l"]),
        p(dev["bnd"]), 0, None, None, t.materials[0][1], t.materials[0][2], 3, p(U_dev), p(R_dev),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rc == capi.OK
    R = R_dev.cpu().numpy()
    assert np.array_equal(R[:, interior].view(np.int64), R_ref[:, interior].view(np.int64))
    assert np.all(np.isnan(R[:, ~interior]))


def test_static_residual_rejects_unknown_boundary_kind(capi):
    import torch
    cuda = torch.device("cuda:0")
    buf = torch.zeros(16, dtype=torch.float64, device=cuda)
    ibuf = torch.zeros(16, dtype=torch.int32, device=cuda)
    p = lambda x: C.c_void_p(x.data_ptr())
    par = np.zeros(8)
    for bad in (0, 5, -1):
        kinds = np.array([2, bad], np.int32)
        rc = capi.lib().cfd2d_residual_first_order_static(
            4, 4, p(ibuf), p(ibuf), p(buf), p(buf), p(ibuf), 2,
            kinds.ctypes.data_as(C.POINTER(C.c_int)), par.ctypes.data_as(C.POINTER(C.c_double)),
            8.314472, 3.5, 3, p(buf), p(buf), None)
        assert rc == 6  # CFD2D_ERR_INVALID_ARG, before anything is launched


def test_static_residual_rejects_oversized_mesh(capi):
    import torch
    cuda = torch.device("cuda:0")
    buf = torch.zeros(16, dtype=torch.float64, device=cuda)
    ibuf = torch.zeros(16, dtype=torch.int32, device=cuda)
    p = lambda x: C.c_void_p(x.data_ptr())
    kinds = np.array([2], np.int32)
    par = np.zeros(4)
    rc = capi.lib().cfd2d_residual_first_order_static(
        4, 262144 + 1, p(ibuf), p(ibuf), p(buf), p(buf), p(ibuf), 1,
        kinds.ctypes.data_as(C.POINTER(C.c_int)), par.ctypes.data_as(C.POINTER(C.c_double)),
        8.314472, 3.5, 3, p(buf), p(buf), None)
    assert rc == 505  # CFD2D_ERR_CAPACITY, before anything is launched
