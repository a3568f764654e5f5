"""Restart files (cfd2d_save_state / cfd2d_load_state) and host-side fault injection.

A run stopped, saved and resumed in a new handle continues bit for bit as if it
had not stopped; a non-physical state injected into the host buffers before
upload is reported as a status (CFD2D_ERR_NONPHYSICAL), never as a GPU fault."""
import numpy as np
import pytest

from cfd2d import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,steady", [(None, 0), (None, 1), ("MIXED", 0), ("MIXED", 1)])
def test_restart_continues_bit_for_bit(capi, tmp_path, precision, steady):
    t, m, U0 = cases.vortex(48, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=30, steady=steady,
                            precision=precision)
    t.limits = (1e-8, 1e8, 1e-8, 1e8, 1.55)  # limiter flags, their ageing and release travel in the file
    path = cases.write_task(t, m, str(tmp_path))
    a = capi.Solver(path, mesh=m)
    a.set_state(U0, reset_time_step=True)
    a.step(12)
    f = str(tmp_path / "state.bin")
    a.save_state(f)
    a.step(18)
    b = capi.Solver(path, mesh=m)
    b.load_state(f)
    assert b.get_info().step == 12
    b.step(18)
    assert np.array_equal(a.state(), b.state())
    assert np.array_equal(a.flags(), b.flags())
    assert np.array_equal(a.time_step(), b.time_step())
    assert a.get_info().time == b.get_info().time


def test_restart_rejects_another_mesh(capi, tmp_path):
    t, m, U0 = cases.vortex(16, steps=2)
    a = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    f = str(tmp_path / "state.bin")
    a.save_state(f)
    t2, m2, _ = cases.vortex(20, steps=2)
    d = tmp_path / "other"
    d.mkdir()
    b = capi.Solver(cases.write_task(t2, m2, str(d)), mesh=m2)
    with pytest.raises(capi.CfdError):
        b.load_state(f)


@pytest.mark.parametrize("precision", [None, "MIXED"])
@pytest.mark.parametrize("bad", ["negative_density", "nan_energy"])
def test_injected_nonphysical_state_is_a_status(capi, tmp_path, precision, bad):
    t, m, U0 = cases.vortex(32, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=3, precision=precision)
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    U = U0.copy()
    k = m.n_cells // 2
    if bad == "negative_density":
        U[0, k] = -U[0, k]
    else:
        U[3, k] = np.nan
    s.set_state(U)
    rc = s.step(3, allow_warnings=True)
    assert rc == capi.ERR_NONPHYSICAL
    s.set_state(U0)  # the handle stays usable
    assert s.step(1, allow_warnings=True) == capi.OK


def test_state_exchange_with_device_and_pinned_buffers(capi, tmp_path):
    """cfd2d_set_state / cfd2d_get_state accept device buffers of the handle's GPU and pinned host
    buffers as well as pageable ones, with identical results."""
    torch = pytest.importorskip("torch")
    from cfd2d import cases
    t, m, U0 = cases.vortex(12, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=5)
    path = cases.write_task(t, m, str(tmp_path))
    ref = capi.Solver(path, mesh=m)
    ref.set_state(U0)
    ref.step(2)
    want = ref.state()
    for kind in ("cuda", "pinned"):
        s = capi.Solver(path, mesh=m)
        src = torch.from_numpy(U0.copy())
        src = src.cuda() if kind == "cuda" else src.pin_memory()
        dst = torch.zeros_like(src)
        torch.cuda.synchronize()  # device data handed to the library must be ready
        s.set_state_from([src[k].data_ptr() for k in range(4)])
        s.step(2)
        s.state_into([dst[k].data_ptr() for k in range(4)])
        got = dst.cpu().numpy()
        assert np.array_equal(got.view(np.int64), want.view(np.int64)), kind
