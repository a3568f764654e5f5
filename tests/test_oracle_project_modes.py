"""The oracle's own arithmetic for the modes the reference does not have (HLLC, Roe, minmod),
checked on the CPU against a plain IEEE restatement in numpy.

HLLC's and Roe's divisions and square roots in the oracle (and, bit for bit, on the GPU) are
Newton-refined sequences from binary32 seeds, Roe's averages come from reciprocal square
roots, HLLC's star flux is formed in one division and minmod's Green-Gauss gradients use
host-formed weights: rounding differs from the textbook expressions. Here the textbook
expressions (Toro's HLLC star state, Roe's averages with the Harten-Hyman fix, the reference's
Green-Gauss formula) are evaluated with numpy's IEEE operations and the oracle's residual
must agree to 1e-12 of the largest face flux. Four-quadrant mesh, outlets all round, the
state perturbed so that minmod takes all three branches.
"""
import numpy as np
import pytest

from cfd2d import cases

GAM = 1.4  # FVM_TVD::run's flux gamma, src/methods/fvm_tvd.cpp:345,398


def _prims(U):
    r = U[0]
    u, v, E = U[1] / r, U[2] / r, U[3] / r
    p = r * (E - 0.5 * (u * u + v * v)) * (GAM - 1.0)  # the task's gas: Cp 3.5, Cv 2.5
    return np.stack([r, u, v, p])


def _phys(q, E, un, nx, ny):
    r, u, v, p = q
    m = r * un
    return np.stack([m, m * u + p * nx, m * v + p * ny, (E + p) * un])


def _energy(q):
    r, u, v, p = q
    return p / (GAM - 1.0) + 0.5 * r * (u * u + v * v)


def _hllc(qL, qR, nx, ny):
    """Toro (Riemann Solvers and Numerical Methods for Fluid Dynamics, sec. 10.4-10.6), Davis
    wave speeds, the star states U*_K = rho_K (S_K - un_K)/(S_K - S*) [1, u*, v*, E*]."""
    unL, unR = qL[1] * nx + qL[2] * ny, qR[1] * nx + qR[2] * ny
    cL, cR = np.sqrt(GAM * qL[3] / qL[0]), np.sqrt(GAM * qR[3] / qR[0])
    EL, ER = _energy(qL), _energy(qR)
    SL, SR = np.minimum(unL - cL, unR - cR), np.maximum(unL + cL, unR + cR)
    mL, mR = qL[0] * (SL - unL), qR[0] * (SR - unR)
    Ss = (qR[3] - qL[3] + mL * unL - mR * unR) / (mL - mR)
    FL, FR = _phys(qL, EL, unL, nx, ny), _phys(qR, ER, unR, nx, ny)

    def star(q, E, un, S, F):
        k = q[0] * (S - un) / (S - Ss)
        Us = k * np.stack([np.ones_like(k), q[1] + (Ss - un) * nx, q[2] + (Ss - un) * ny,
                           E / q[0] + (Ss - un) * (Ss + q[3] / (q[0] * (S - un)))])
        U = np.stack([q[0], q[0] * q[1], q[0] * q[2], E])
        return F + S * (Us - U)

    FsL, FsR = star(qL, EL, unL, SL, FL), star(qR, ER, unR, SR, FR)
    return np.where(SL >= 0, FL, np.where(SR <= 0, FR, np.where(Ss >= 0, FsL, FsR)))


def _roe(qL, qR, nx, ny):
    """Roe (1981) with the Harten-Hyman entropy fix on the acoustic waves (as in the
    reference's roe_orig averages, src/global.cpp:407-441)."""
    G1 = GAM - 1.0
    unL, unR = qL[1] * nx + qL[2] * ny, qR[1] * nx + qR[2] * ny
    EL, ER = _energy(qL), _energy(qR)
    HL, HR = (EL + qL[3]) / qL[0], (ER + qR[3]) / qR[0]
    sL, sR = np.sqrt(qL[0]), np.sqrt(qR[0])
    ut = (sL * qL[1] + sR * qR[1]) / (sL + sR)
    vt = (sL * qL[2] + sR * qR[2]) / (sL + sR)
    Ht = (sL * HL + sR * HR) / (sL + sR)
    q2 = ut * ut + vt * vt
    c = np.sqrt(G1 * (Ht - 0.5 * q2))
    unt = ut * nx + vt * ny
    rt = sL * sR
    dr, dp, dun = qR[0] - qL[0], qR[3] - qL[3], unR - unL
    dtx, dty = (qR[1] - qL[1]) - dun * nx, (qR[2] - qL[2]) - dun * ny
    a1 = (dp - rt * c * dun) / (2 * c * c)
    a2 = dr - dp / (c * c)
    a4 = (dp + rt * c * dun) / (2 * c * c)
    l1, l4 = unt - c, unt + c
    cL, cR = np.sqrt(GAM * qL[3] / qL[0]), np.sqrt(GAM * qR[3] / qR[0])
    d1 = np.maximum(0, np.maximum(l1 - (unL - cL), (unR - cR) - l1))
    d4 = np.maximum(0, np.maximum(l4 - (unL + cL), (unR + cR) - l4))
    al1, al4, al2 = np.maximum(np.abs(l1), d1), np.maximum(np.abs(l4), d4), np.abs(unt)
    w1, w2, w4, ws = al1 * a1, al2 * a2, al4 * a4, al2 * rt
    D = np.stack([w1 + w2 + w4,
                  w1 * (ut - c * nx) + w2 * ut + ws * dtx + w4 * (ut + c * nx),
                  w1 * (vt - c * ny) + w2 * vt + ws * dty + w4 * (vt + c * ny),
                  w1 * (Ht - unt * c) + w2 * 0.5 * q2 + ws * (ut * dtx + vt * dty) + w4 * (Ht + unt * c)])
    return 0.5 * (_phys(qL, EL, unL, nx, ny) + _phys(qR, ER, unR, nx, ny) - D)


def _minmod(a, b):
    return np.where(a * b > 0, np.where(np.abs(a) < np.abs(b), a, b), 0.0)


def _residual(ex, U, flux, recon):
    """stage_residual of FVM_TVD (src/methods/fvm_tvd.cpp:324-365) with outlets (ghost = the
    state itself) in plain IEEE arithmetic, per edge vectorised."""
    q = _prims(U)
    c1, c2 = ex["edge_c12"][:, 0], ex["edge_c12"][:, 1]
    inner = c2 >= 0
    c2s = np.where(inner, c2, c1)
    nx, ny, l = ex["edge_n"][:, 0], ex["edge_n"][:, 1], ex["edge_l"]
    qL, qRc = q[:, c1], q[:, c2s]  # on the boundary the outlet ghost of the centre state
    nc = U.shape[1]
    g = np.zeros((4, 2, nc))
    if recon == "MINMOD":  # Green-Gauss: (1/S) sum over faces of (phi_1 + phi_2)/2 n l
        h = 0.5 * (qL + qRc)
        for d, n in enumerate((nx, ny)):
            for k in range(4):
                np.add.at(g[k, d], c1, h[k] * n * l)
                np.add.at(g[k, d], c2[inner], -(h[k] * n * l)[inner])
        g /= ex["cell_S"]
    flux_fn = _hllc if flux == "HLLC" else _roe
    F = np.zeros((4, len(l)))
    branches = np.zeros(3, int)  # minmod: zero, the projection, the difference
    for gp in (1, 2):
        P = ex["edge_pts"][:, gp]
        pL, pR = qL, qRc
        if recon == "MINMOD":
            def rec(cc, own, other):
                d = P - ex["cell_c"][cc]
                a, b = g[:, 0, cc] * d[:, 0] + g[:, 1, cc] * d[:, 1], other - own
                branches[:] += [np.sum(a * b <= 0), np.sum((a * b > 0) & (np.abs(a) < np.abs(b))),
                                np.sum((a * b > 0) & (np.abs(a) >= np.abs(b)))]
                return own + _minmod(a, b)
            pL, pR = rec(c1, qL, qRc), rec(c2s, qRc, qL)
        pR = np.where(inner, pR, pL)  # outlet: the ghost of the reconstructed state
        F += flux_fn(pL, pR, nx, ny)
    F *= 0.5 * l
    R = np.zeros((4, nc))
    for k in range(4):
        np.add.at(R[k], c1, -F[k])
        np.add.at(R[k], c2[inner], F[k][inner])
    return R, np.abs(F).max(axis=1), branches


@pytest.mark.parametrize("flux", ["HLLC", "ROE"])
@pytest.mark.parametrize("recon", ["NONE", "MINMOD"])
def test_oracle_project_fluxes_match_ieee_restatement(oracle, flux, recon):
    t, m, _ = cases.four_quadrant(12, flux=flux, recon=recon, scheme="SSPRK3")
    om = oracle.OracleMesh.from_mesh(m)
    ex = om.export()
    s0 = oracle.solver_from_task(t, m, om)
    U, _, _ = s0.state()
    rng = np.random.default_rng(7)
    U = U * (1.0 + 0.05 * rng.standard_normal(U.shape))  # minmod sees all three branches
    U[0] = np.abs(U[0]); U[3] = np.abs(U[3]) + 0.2 * U[0]
    s = oracle.solver_from_task(t, m, om, U0=U)
    R_orc = s.residual()
    R_ref, scale, branches = _residual(ex, U, flux, recon)
    err = np.abs(R_orc - R_ref).max(axis=1) / scale
    assert np.all(err <= 1e-12), (flux, recon, err)
    if recon == "MINMOD":
        assert np.all(branches > 0), branches
