"""Discrete adjoint (cfd2d_forward / cfd2d_backward) against central finite differences.

J = sum over cells in a box of S (p - 1)^2 after the run; gradients with
respect to the initial conserved state, the inlet parameters and the
free-stream Mach number. Bar: 1e-5 relative agreement with central FD at
eps = 1e-6 (directions are seeded unit vectors in the 4 N-dimensional state).
"""
import math

import numpy as np
import pytest

from cfd2d import cases

pytestmark = pytest.mark.gpu

TOL = 1e-5
KINDS = ("BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP")


def _solver(capi, tmp_path, t, m, w):
    s = capi.Solver(cases.write_task(t, m, str(tmp_path)), mesh=m)
    s.set_objective(0, w, 1.0)
    return s


def _J(s, U, steps, k):
    s.set_state(U)
    return s.forward(steps, k)


def _fd_check(s, U0, g, steps, k, ndir, seed, eps=1e-6):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for _ in range(ndir):
        d = rng.standard_normal(U0.shape)
        d /= np.linalg.norm(d)
        fd = (_J(s, U0 + eps * d, steps, k) - _J(s, U0 - eps * d, steps, k)) / (2 * eps)
        ad = float(np.sum(g * d))
        worst = max(worst, abs(ad - fd) / max(abs(fd), 1e-3 * np.linalg.norm(g)))
    return worst


@pytest.mark.parametrize("flux,recon,scheme,kinds", [
    ("HLLC", "MINMOD", "SSPRK3", None),
    ("HLLC", "LINEAR", "HEUN", KINDS),
    ("LAX", "NONE", "EULER", KINDS),
    ("LAX", "MINMOD", "SSPRK3", KINDS),
])
def test_adjoint_state_gradient_vs_fd(capi, tmp_path, flux, recon, scheme, kinds):
    t, m, U0, w, _ = cases.vortex_adjoint(24, steps=12, flux=flux, recon=recon, scheme=scheme, bnd_kinds=kinds)
    s = _solver(capi, tmp_path, t, m, w)
    s.set_state(U0)
    J0 = s.forward(12, 5)          # segments of 5, 5, 2 steps
    g, gb = s.backward()
    assert J0 > 0 and np.all(np.isfinite(g))
    assert _fd_check(s, U0, g, 12, 5, ndir=6, seed=1) <= TOL


def test_adjoint_boundary_and_mach_gradients_vs_fd(capi, tmp_path):
    t, m, U0, w, u0_of = cases.vortex_adjoint(24, steps=10, mach=0.5)
    s = _solver(capi, tmp_path, t, m, w)
    s.set_state(U0)
    s.forward(10, 4)
    g, gb = s.backward()
    eps = 1e-6
    # inlet Vx of side 0 only
    b0 = [t.boundaries[0].u, t.boundaries[0].v, t.boundaries[0].T, t.boundaries[0].p]

    def J_vx(vx):
        s.set_boundary(0, [vx] + b0[1:])
        return _J(s, U0, 10, 4)
    fd = (J_vx(b0[0] + eps) - J_vx(b0[0] - eps)) / (2 * eps)
    s.set_boundary(0, b0)
    assert abs(gb[0, 0] - fd) <= TOL * max(abs(fd), 1e-8)
    # free-stream Mach: initial state and every inlet's Vx = M sqrt(gamma)
    M = 0.5
    sg = math.sqrt(cases.GAMMA)
    dU = (u0_of(M + 1e-7) - u0_of(M - 1e-7)) / 2e-7  # the initial state's Mach derivative
    ad = float(np.sum(g * dU)) + sg * float(np.sum(gb[:, 0]))

    def J_mach(Mv):
        for b in range(len(t.boundaries)):
            bb = t.boundaries[b]
            s.set_boundary(b, [Mv * sg, bb.v, bb.T, bb.p])
        return _J(s, u0_of(Mv), 10, 4)
    fd = (J_mach(M + eps) - J_mach(M - eps)) / (2 * eps)
    assert abs(ad - fd) <= 1e-4 * abs(fd)


def test_adjoint_matches_cpu_reference_fd(capi, oracle, tmp_path):
    """The CPU solver's finite differences are the reference gradient: its
    forward equals the GPU's bit for bit, so its FD equals the GPU FD."""
    t, m, U0, w, _ = cases.vortex_adjoint(16, steps=6, flux="HLLC", recon="MINMOD", scheme="SSPRK3")
    s = _solver(capi, tmp_path, t, m, w)
    s.set_state(U0)
    s.forward(6, 3)
    g, _ = s.backward()
    rng = np.random.default_rng(9)

    def J_cpu(U):
        o = oracle.solver_from_task(t, m, U0=U, flux="HLLC", recon="MINMOD", scheme="SSPRK3")
        o.step(6)
        Uf, _, _ = o.state()
        r, ru, rv, rE = Uf
        p = (rE / r - 0.5 * ((ru / r) ** 2 + (rv / r) ** 2)) * r * 0.4
        return float(np.sum(w * (p - 1.0) ** 2))
    for _ in range(2):
        d = rng.standard_normal(U0.shape); d /= np.linalg.norm(d)
        fd_cpu = (J_cpu(U0 + 1e-6 * d) - J_cpu(U0 - 1e-6 * d)) / 2e-6
        assert abs(float(np.sum(g * d)) - fd_cpu) <= TOL * max(abs(fd_cpu), 1e-3 * np.linalg.norm(g))


def test_adjoint_of_mixed_forward_tracks_fp64(capi, tmp_path):
    t, m, U0, w, _ = cases.vortex_adjoint(24, steps=10)
    a = _solver(capi, tmp_path, t, m, w)
    t.precision = "MIXED"
    b = _solver(capi, tmp_path, t, m, w)
    for s in (a, b):
        s.set_state(U0)
        s.forward(10, 4)
    ga, _ = a.backward()
    gb, _ = b.backward()
    assert np.linalg.norm(gb - ga) <= 1e-5 * np.linalg.norm(ga)


def test_full_size_adjoint_64_directions(capi, tmp_path):
    """131,072 triangles (256 x 256 x 2), HLLC + minmod + SSP-RK3, 200 steps,
    checkpoint every 20: every one of 64 seeded directions within 1e-5 of central FD at
    eps = 1e-6. A direction's error is |g.d - fd| / max(|fd|, 1e-3 |g|); |g| / sqrt(4 N)
    is the typical directional derivative, so the floor only keeps near-zero directions
    from dividing by FD round-off. The errors of all directions are printed."""
    t, m, U0, w, _ = cases.vortex_adjoint(256, steps=200)
    s = _solver(capi, tmp_path, t, m, w)
    s.set_state(U0)
    s.forward(200, 20)
    g, _ = s.backward()
    errs = []
    rng = np.random.default_rng(4)
    for _ in range(64):
        d = rng.standard_normal(U0.shape); d /= np.linalg.norm(d)
        fd = (_J(s, U0 + 1e-6 * d, 200, 20) - _J(s, U0 - 1e-6 * d, 200, 20)) / 2e-6
        errs.append(abs(float(np.sum(g * d)) - fd) / max(abs(fd), 1e-3 * np.linalg.norm(g)))
    errs = np.array(errs)
    print("per-direction relative FD error:", " ".join("%.2e" % e for e in errs))
    print("max %.3e median %.3e" % (errs.max(), np.median(errs)))
    assert errs.max() <= TOL, errs


def test_combined_mixed_adjoint_within_memory_budget(capi, tmp_path):
    """The combined configuration's path at reduced size: four-quadrant Riemann problem,
    FP32 faces / FP64 accumulation, HLLC + minmod + SSP-RK3, J = sum over the central
    quarter of S rho^2, checkpointed forward and mixed adjoint with an ADJOINT_MEMORY
    budget that the full store (primitives and gradients) would exceed. The handle stays
    within the budget, its gradient equals the unconstrained run's bit for bit (the store
    modes re-derive what they do not keep), and it stays close to the FP64 gradient."""
    t, m, _ = cases.four_quadrant(48, seed=5, steps=12)
    U0 = None  # the task's own initial state (four regions), read from the first handle
    xy = m.centroids()
    p = m.nodes[m.tris]
    S = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                     (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    w = np.where((xy[:, 0] >= 0.25) & (xy[:, 0] <= 0.75) & (xy[:, 1] >= 0.25) & (xy[:, 1] <= 0.75), S, 0.0)
    t.precision = "MIXED"
    runs = {}
    for name, budget in (("free", None), ("budget", "probe")):
        d = tmp_path / name
        d.mkdir()
        if budget == "probe":  # the unconstrained handle's bytes less half of its full store
            nst, k, nc = 3, 4, m.n_cells
            full_store = k * nst * 12 * nc * 4
            t.adjoint_memory = float(runs["free"][2] - full_store // 2)
        s = capi.Solver(cases.write_task(t, m, str(d)), mesh=m)
        s.set_objective(1, w, 0.0)
        if U0 is None:
            U0 = s.state()
        s.set_state(U0)
        J = s.forward(12, 4)
        g, _ = s.backward()
        runs[name] = (J, g, s.get_info().device_bytes)
        s.close()
    assert runs["budget"][2] <= t.adjoint_memory < runs["free"][2]
    assert runs["budget"][0] == runs["free"][0] and np.array_equal(runs["budget"][1], runs["free"][1])
    t.precision = None
    t.adjoint_memory = None
    d = tmp_path / "fp64"
    d.mkdir()
    s = capi.Solver(cases.write_task(t, m, str(d)), mesh=m)
    s.set_objective(1, w, 0.0)
    s.set_state(U0)
    s.forward(12, 4)
    g64, _ = s.backward()
    gmx = runs["free"][1]
    assert np.all(np.isfinite(gmx)) and np.all(np.isfinite(g64))
    # at the four-quadrant discontinuities minmod's branch (a b > 0, |a| < |b|) follows FP32
    # rounding in the mixed forward and FP64 rounding in the other, and its derivative jumps
    # between branches, so the two gradients differ by a few 1e-3 (the smooth vortex: 1e-5).
    # The same kinks make central differences unreliable here; the FD checks run on the
    # smooth vortex above.
    assert np.linalg.norm(gmx - g64) <= 1e-2 * np.linalg.norm(g64)


@pytest.mark.parametrize("precision", [None, "MIXED"])
def test_adjoint_store_modes_give_the_same_gradient(capi, tmp_path, precision):
    """Recorded stages keep their states only, their primitives too, primitives and
    gradients, or these and the HLLC flux evaluations' records (face states, sound speeds,
    minmod's branches): whatever is not kept is re-derived by the forward's own kernels,
    and the recorded values are the ones they re-derive, so the gradient is the same bit
    for bit."""
    t, m, U0, w, _ = cases.vortex_adjoint(32, steps=9)
    t.precision = precision
    grads = []
    modes = ("NONE", "PRIMITIVES", "ALL") + (("FLUXES",) if precision is None else ())  # records: FP64 faces
    for mode in modes:
        t.adjoint_store = mode
        d = tmp_path / mode
        d.mkdir()
        s = capi.Solver(cases.write_task(t, m, str(d)), mesh=m)
        s.set_objective(0, w, 1.0)
        s.set_state(U0)
        s.forward(9, 4)
        g, gb = s.backward()
        grads.append((g, gb))
    for g, gb in grads[1:]:
        assert np.array_equal(g, grads[0][0]) and np.array_equal(gb, grads[0][1])
