"""The mixed form's tiled stage kernels against the same form on its per-kernel path:
FUSED_STAGE 1 (gradients, fluxes and update of a tile of cells in one launch, from
shared memory), FUSED_STAGE 2 (the per-kernel gradients, then the fluxes of a tile's
edges in shared memory and its cells' update in one launch) and FUSED_STAGE 3 (the flux
kernel forms its two cells' gradients; no gradient kernel). Identical inputs and
identical arithmetic, so identical bits."""
import numpy as np
import pytest

from cfd2d import cases

pytestmark = pytest.mark.gpu


MODES = ("1", "2", "3")


def _pair(capi, tmp_path, t, m, U0=None, mode="1", **kw):
    out = []
    kw.setdefault("reorder", "HILBERT")
    for fused in ("0", mode):
        t.precision = "MIXED"
        t.fused_stage = fused
        for k, v in kw.items():
            setattr(t, k, v)
        d = tmp_path / ("a" if fused == "0" else "b")
        d.mkdir(exist_ok=True)
        s = capi.Solver(cases.write_task(t, m, str(d)), mesh=m)
        if U0 is not None:
            s.set_state(U0, reset_time_step=True)
        out.append(s)
    return out


def _is_fused(s, mode="1"):
    """Profile one step (it is taken): the tiled paths launch no separate update kernel, FUSED_STAGE 1
    no separate gradient kernel either; FUSED_STAGE 3 no gradient kernel but its update kernel."""
    ms, cnt = s.profile_steps(1)
    if mode == "3":
        return cnt[0] == 0 and cnt[1] > 0 and cnt[2] > 0
    return (cnt[0] == 0 or mode == "2") and cnt[2] == 0 and cnt[1] > 0


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("flux,recon,scheme", [("HLLC", "MINMOD", "SSPRK3"), ("ROE", "MINMOD", "HEUN"),
                                               ("LAX", "LINEAR", "SSPRK3"), ("HLLC", "NONE", "HEUN"),
                                               ("GODUNOV", "LINEAR", "SSPRK3")])
def test_fused_equals_per_kernel_vortex(capi, tmp_path, flux, recon, scheme, mode):
    kinds = ("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP")
    t, m, U0 = cases.vortex(96, flux=flux, recon=recon, scheme=scheme, steps=12, bnd_kinds=kinds)
    a, b = _pair(capi, tmp_path, t, m, U0, mode=mode)
    fa, fb = _is_fused(a, mode), _is_fused(b, mode)  # each check takes one step on its solver
    if not (mode == "3" and recon == "NONE"):  # no gradients to form: FUSED_STAGE 3 is the per-kernel path
        assert not fa and fb
    a.step(12)
    b.step(12)
    assert np.array_equal(a.state(), b.state())
    assert np.array_equal(a.time_step(), b.time_step())


@pytest.mark.parametrize("mode", MODES)
def test_fused_equals_per_kernel_local_time_step(capi, tmp_path, mode):
    t, m, U0 = cases.vortex(80, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=10, steady=1)
    a, b = _pair(capi, tmp_path, t, m, U0, mode=mode)
    a.step(10)
    b.step(10)
    assert np.array_equal(a.state(), b.state())
    assert np.array_equal(a.time_step(), b.time_step())


@pytest.mark.parametrize("mode", MODES)
def test_fused_equals_per_kernel_limits_and_remediation(capi, tmp_path, mode):
    """A |u| limit below the vortex peak flags cells (frozen, then remediated)."""
    t, m, U0 = cases.vortex(64, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=30)
    t.limits = (1e-8, 1e8, 1e-8, 1e8, 1.55)
    a, b = _pair(capi, tmp_path, t, m, U0, mode=mode)
    a.step(30)
    b.step(30)
    assert np.array_equal(a.flags(), b.flags())
    assert (a.flags() & 2).any() or (a.flags() > 0).any()
    assert np.array_equal(a.state(), b.state())


@pytest.mark.parametrize("mode", MODES)
def test_fused_four_quadrant_full_size(capi, tmp_path, mode):
    """2,097,152 triangles, HLLC + minmod + SSP-RK3, 5 steps: the bench workload."""
    t, m, _ = cases.four_quadrant(1024, steps=5)
    a, b = _pair(capi, tmp_path, t, m, mode=mode)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.state(), b.state())


@pytest.mark.parametrize("mode", MODES)
def test_fused_with_rcm_order(capi, tmp_path, mode):
    """Long thin tiles (RCM order) still fit and still give the per-kernel bits."""
    t, m, U0 = cases.vortex(64, flux="HLLC", recon="MINMOD", scheme="SSPRK3", steps=8)
    a, b = _pair(capi, tmp_path, t, m, U0, mode=mode, reorder="RCM")
    assert not _is_fused(a, mode) and _is_fused(b, mode)
    a.step(8)
    b.step(8)
    assert np.array_equal(a.state(), b.state())


@pytest.mark.parametrize("flux,recon", [("HLLC", "MINMOD"), ("ROE", "MINMOD"), ("GODUNOV", "LINEAR"),
                                        ("LAX", "NONE")])
def test_pipelined_flux_equals_one_thread_per_edge(capi, tmp_path, flux, recon):
    """The mixed form's default flux kernel (persistent, cp.async-pipelined gathers) against
    the one-thread-per-edge kernel (FLUX_PIPELINE OFF): the same fluxes, the same bits."""
    kinds = ("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP")
    t, m, U0 = cases.vortex(150, flux=flux, recon=recon, scheme="SSPRK3", steps=10, bnd_kinds=kinds)
    out = []
    for pipe in ("OFF", "ON"):
        t.precision = "MIXED"
        t.fused_stage = "0"  # the per-kernel path, whose flux kernel the option selects
        t.flux_pipeline = pipe
        d = tmp_path / pipe
        d.mkdir(exist_ok=True)
        s = capi.Solver(cases.write_task(t, m, str(d)), mesh=m)
        s.set_state(U0, reset_time_step=True)
        s.step(10)
        out.append(s.state())
    assert np.array_equal(out[0].view(np.int64), out[1].view(np.int64))
