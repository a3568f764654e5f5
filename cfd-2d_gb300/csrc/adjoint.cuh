// Reverse-mode (vector-Jacobian) pieces of the FP64 step, written by hand: for
// each forward function f(x) below, vjp_f accumulates x_bar += (df/dx)^T y_bar.
// Each follows the forward expression in kernels.cuh line by line, so the
// adjoint is the exact derivative of the discrete scheme the solver runs
// (branches of min/max, minmod and the HLLC wave pattern are taken as the
// forward pass took them).
#pragma once
#include "kernels.cuh"

namespace cfd2d {

// convertConsToPar: (rho, rho u, rho v, rho E) -> (r, u, v, p)
__device__ __forceinline__ void vjp_cons2prim(const double* U, double gm1, const Prim<double>& pb, double* Ub) {
    const double ro = U[0], iro = 1.0 / ro;  // the reverse sweep needs no bit parity: one reciprocal
    const double u = U[1] * iro, v = U[2] * iro, E = U[3] * iro;
    const double e = E - 0.5 * (u * u + v * v);
    // p = r e gm1
    double rb = pb.r + pb.p * e * gm1;
    const double eb = pb.p * ro * gm1;
    // e = E - (u^2 + v^2)/2
    const double Eb = eb;
    const double ub = pb.u - eb * u, vb = pb.v - eb * v;
    Ub[1] += ub * iro;
    Ub[2] += vb * iro;
    Ub[3] += Eb * iro;
    rb -= (ub * u + vb * v + Eb * E) * iro;
    Ub[0] += rb;
}

// Tc = (p / (r gm1)) / Cv
__device__ __forceinline__ void vjp_temperature(const Prim<double>& q, double gm1, double Cv, double Tb,
                                                Prim<double>& qb) {
    const double k = 1.0 / (q.r * gm1 * Cv);
    qb.p += Tb * k;
    qb.r -= Tb * (q.p * k) / q.r;
}

// ghost_state(b, q, Tc, n, M): the reference's CFDBnd*::run + URS(2) for the density.
// bp_bar receives d/d(Vx, Vy, T, P) of an inlet's parameters.
__device__ __forceinline__ void vjp_ghost(const DevBnd& b, const Prim<double>& q, double Tc, double nx, double ny,
                                          double M, const Prim<double>& gb, Prim<double>& qb, double& Tcb,
                                          double* bp_bar) {
    if (b.kind == BND_INLET) {
        const double k = M / (b.T * GAS_R);
        bp_bar[0] += gb.u;
        bp_bar[1] += gb.v;
        bp_bar[3] += gb.p + gb.r * k;
        bp_bar[2] -= gb.r * (b.p * k) / b.T;
        return;
    }
    const double k = M / (Tc * GAS_R);
    qb.p += gb.p + gb.r * k;
    Tcb -= gb.r * (q.p * k) / Tc;
    if (b.kind == BND_OUTLET) {
        qb.u += gb.u;
        qb.v += gb.v;
    } else {  // wall: u_g = u - 2 nx Un, v_g = v - 2 ny Un, Un = u nx + v ny
        const double Unb = -2.0 * (nx * gb.u + ny * gb.v);
        qb.u += gb.u + Unb * nx;
        qb.v += gb.v + Unb * ny;
    }
}

// phys_flux(f, r, u, v, p, E, un, n)
__device__ __forceinline__ void vjp_phys(double r, double u, double v, double p, double E, double un, double nx,
                                         double ny, const double* fb, double& rb, double& ub, double& vb, double& pb,
                                         double& Eb, double& unb) {
    const double m = r * un;
    const double mb = fb[0] + fb[1] * u + fb[2] * v;
    ub += fb[1] * m;
    vb += fb[2] * m;
    pb += fb[1] * nx + fb[2] * ny + fb[3] * un;
    Eb += fb[3] * un;
    unb += fb[3] * (E + p) + mb * r;
    rb += mb * un;
}

// Lax-Friedrichs (flux_lax in kernels.cuh)
__device__ __forceinline__ void vjp_lax(const Prim<double>& L, const Prim<double>& R, double nx, double ny,
                                        double GAM, const double* fb, Prim<double>& Lb, Prim<double>& Rb) {
    const double unl = L.u * nx + L.v * ny, unr = R.u * nx + R.v * ny;
    const double aL = GAM * L.p / L.r, aR = GAM * R.p / R.r;
    const double cL = sqrt(aL), cR = sqrt(aR);
    const double s1 = fabs(unl) + cL, s2 = fabs(unr) + cR;
    const bool first = s1 > s2;  // t_max(a, b) = a > b ? a : b
    const double alpha = first ? s1 : s2;
    const double rol = L.r, rul = L.r * L.u, rvl = L.r * L.v;
    const double G1 = GAM - 1.0;
    const double rel = L.p / G1 + 0.5 * L.r * (L.u * L.u + L.v * L.v);
    const double ror = R.r, rur = R.r * R.u, rvr = R.r * R.v;
    const double rer = R.p / G1 + 0.5 * R.r * (R.u * R.u + R.v * R.v);
    const double frl = rol * unl, frr = ror * unr;
    const double h0 = 0.5 * fb[0], h1 = 0.5 * fb[1], h2 = 0.5 * fb[2], h3 = 0.5 * fb[3];
    // f0 = .5(frr + frl - alpha (ror - rol)), f1 = .5(frr uR + frl uL + (pR + pL) nx - alpha (rur - rul))
    // f2 = .5(frr vR + frl vL + (pR + pL) ny - alpha (rvr - rvl)), f3 = .5((rer + pR) unr + (rel + pL) unl - alpha (rer - rel))
    double frrb = h0 + h1 * R.u + h2 * R.v, frlb = h0 + h1 * L.u + h2 * L.v;
    double alphab = -(h0 * (ror - rol) + h1 * (rur - rul) + h2 * (rvr - rvl) + h3 * (rer - rel));
    double rorb = -h0 * alpha, rolb = h0 * alpha, rurb = -h1 * alpha, rulb = h1 * alpha;
    double rvrb = -h2 * alpha, rvlb = h2 * alpha, rerb = h3 * unr - h3 * alpha, relb = h3 * unl + h3 * alpha;
    Rb.u += h1 * frr; Lb.u += h1 * frl; Rb.v += h2 * frr; Lb.v += h2 * frl;
    Rb.p += h1 * nx + h2 * ny + h3 * unr; Lb.p += h1 * nx + h2 * ny + h3 * unl;
    double unrb = h3 * (rer + R.p), unlb = h3 * (rel + L.p);
    // fr = ro un
    rorb += frrb * unr; unrb += frrb * ror; rolb += frlb * unl; unlb += frlb * rol;
    // re = p/G1 + .5 r (u^2 + v^2)
    Rb.p += rerb / G1; rorb += rerb * 0.5 * (R.u * R.u + R.v * R.v);
    Rb.u += rerb * R.r * R.u; Rb.v += rerb * R.r * R.v;
    Lb.p += relb / G1; rolb += relb * 0.5 * (L.u * L.u + L.v * L.v);
    Lb.u += relb * L.r * L.u; Lb.v += relb * L.r * L.v;
    // ru, rv
    rorb += rurb * R.u + rvrb * R.v; Rb.u += rurb * R.r; Rb.v += rvrb * R.r;
    rolb += rulb * L.u + rvlb * L.v; Lb.u += rulb * L.r; Lb.v += rvlb * L.r;
    Rb.r += rorb; Lb.r += rolb;
    // alpha = max(|unl| + cL, |unr| + cR)
    if (first) { unlb += alphab * (unl >= 0 ? 1.0 : -1.0); const double ab = 0.5 * alphab / (cL * L.r); Lb.p += ab * GAM; Lb.r -= ab * aL; }
    else { unrb += alphab * (unr >= 0 ? 1.0 : -1.0); const double ab = 0.5 * alphab / (cR * R.r); Rb.p += ab * GAM; Rb.r -= ab * aR; }
    Lb.u += unlb * nx; Lb.v += unlb * ny; Rb.u += unrb * nx; Rb.v += unrb * ny;
}

// HLLC in the single-division star-flux form (flux_hllc in kernels.cuh)
__device__ __forceinline__ void vjp_hllc(const Prim<double>& L, const Prim<double>& R, double nx, double ny,
                                         double GAM, const double* fb, Prim<double>& Lb, Prim<double>& Rb) {
    const double IG1 = 1.0 / (GAM - 1.0);
    const double aL = GAM * L.p / L.r, aR = GAM * R.p / R.r;
    const double cL = sqrt(aL), cR = sqrt(aR);
    const double unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    const double EL = energy(L.r, L.u, L.v, L.p, IG1);
    const double ER = energy(R.r, R.u, R.v, R.p, IG1);
    const double sl1 = unL - cL, sl2 = unR - cR, sr1 = unL + cL, sr2 = unR + cR;
    const bool l1 = sl1 < sl2, r1 = sr1 > sr2;
    const double SL = l1 ? sl1 : sl2, SR = r1 ? sr1 : sr2;
    double unLb = 0, unRb = 0, ELb = 0, ERb = 0, SLb = 0, SRb = 0, cLb = 0, cRb = 0;
    if (SL >= 0.0 || SR <= 0.0) {  // supersonic: the upwind side's physical flux
        if (SL >= 0.0) vjp_phys(L.r, L.u, L.v, L.p, EL, unL, nx, ny, fb, Lb.r, Lb.u, Lb.v, Lb.p, ELb, unLb);
        else vjp_phys(R.r, R.u, R.v, R.p, ER, unR, nx, ny, fb, Rb.r, Rb.u, Rb.v, Rb.p, ERb, unRb);
    } else {
        const double mL = L.r * (SL - unL), mR = R.r * (SR - unR);
        const double num = fma(-mR, unR, fma(mL, unL, R.p - L.p)), den = mL - mR;
        const double Ss = num / den;
        const bool left = Ss >= 0.0;
        const Prim<double>& K = left ? L : R;
        const double SK = left ? SL : SR, unK = left ? unL : unR, EK = left ? EL : ER, mK = left ? mL : mR;
        const double m = K.r * unK;
        const double FK0 = m, FK1 = m * K.u + K.p * nx, FK2 = m * K.v + K.p * ny, FK3 = (EK + K.p) * unK;
        const double ps = fma(mK, Ss - unK, K.p);
        const double inv = 1.0 / (SK - Ss);
        const double sp = SK * ps;
        const double A0 = SK * K.r - FK0, A1 = SK * (K.r * K.u) - FK1, A2 = SK * (K.r * K.v) - FK2,
                     A3 = SK * EK - FK3;
        const double h0 = Ss * A0, h1 = Ss * A1 + sp * nx, h2 = Ss * A2 + sp * ny, h3 = Ss * A3 + sp * Ss;
        // f_k = h_k inv
        const double hb0 = fb[0] * inv, hb1 = fb[1] * inv, hb2 = fb[2] * inv, hb3 = fb[3] * inv;
        const double invb = fb[0] * h0 + fb[1] * h1 + fb[2] * h2 + fb[3] * h3;
        double Ssb = hb0 * A0 + hb1 * A1 + hb2 * A2 + hb3 * (A3 + sp);
        const double A0b = hb0 * Ss, A1b = hb1 * Ss, A2b = hb2 * Ss, A3b = hb3 * Ss;
        const double spb = hb1 * nx + hb2 * ny + hb3 * Ss;
        // inv = 1/(SK - Ss)
        double SKb = -invb * inv * inv;
        Ssb += invb * inv * inv;
        // sp = SK ps
        SKb += spb * ps;
        const double psb = spb * SK;
        // ps = pK + mK (Ss - unK)
        double Krb = 0, Kub = 0, Kvb = 0, Kpb = psb, EKb = 0, unKb = -psb * mK, mKb = psb * (Ss - unK);
        Ssb += psb * mK;
        // A_k
        SKb += A0b * K.r + A1b * (K.r * K.u) + A2b * (K.r * K.v) + A3b * EK;
        Krb += A0b * SK + A1b * SK * K.u + A2b * SK * K.v;
        Kub += A1b * SK * K.r;
        Kvb += A2b * SK * K.r;
        EKb += A3b * SK;
        const double FKb[4] = {-A0b, -A1b, -A2b, -A3b};
        vjp_phys(K.r, K.u, K.v, K.p, EK, unK, nx, ny, FKb, Krb, Kub, Kvb, Kpb, EKb, unKb);
        // route the K-side adjoints
        double mLb = 0, mRb = 0;
        if (left) {
            Lb.r += Krb; Lb.u += Kub; Lb.v += Kvb; Lb.p += Kpb; ELb += EKb; unLb += unKb; SLb += SKb; mLb += mKb;
        } else {
            Rb.r += Krb; Rb.u += Kub; Rb.v += Kvb; Rb.p += Kpb; ERb += EKb; unRb += unKb; SRb += SKb; mRb += mKb;
        }
        // Ss = num / den
        const double iden = 1.0 / den;
        const double numb = Ssb * iden, denb = -Ssb * Ss * iden;
        Rb.p += numb; Lb.p -= numb;
        mLb += numb * unL + denb; unLb += numb * mL;
        mRb += -numb * unR - denb; unRb -= numb * mR;
        // mL = rL (SL - unL), mR = rR (SR - unR)
        Lb.r += mLb * (SL - unL); SLb += mLb * L.r; unLb -= mLb * L.r;
        Rb.r += mRb * (SR - unR); SRb += mRb * R.r; unRb -= mRb * R.r;
        // SL = min(sl1, sl2), SR = max(sr1, sr2)
        if (l1) { unLb += SLb; cLb -= SLb; } else { unRb += SLb; cRb -= SLb; }
        if (r1) { unLb += SRb; cLb += SRb; } else { unRb += SRb; cRb += SRb; }
    }
    // E = p IG1 + .5 r (u^2 + v^2)
    Lb.p += ELb * IG1; Lb.r += ELb * 0.5 * (L.u * L.u + L.v * L.v); Lb.u += ELb * L.r * L.u; Lb.v += ELb * L.r * L.v;
    Rb.p += ERb * IG1; Rb.r += ERb * 0.5 * (R.u * R.u + R.v * R.v); Rb.u += ERb * R.r * R.u; Rb.v += ERb * R.r * R.v;
    // un = u nx + v ny
    Lb.u += unLb * nx; Lb.v += unLb * ny; Rb.u += unRb * nx; Rb.v += unRb * ny;
    // c = sqrt(GAM p / r): dc = (GAM dp - a dr) / (2 c r)
    if (cLb != 0.0) { const double ab = 0.5 * cLb / (cL * L.r); Lb.p += ab * GAM; Lb.r -= ab * aL; }
    if (cRb != 0.0) { const double ab = 0.5 * cRb / (cR * R.r); Rb.p += ab * GAM; Rb.r -= ab * aR; }
}

// One side's reconstruction p = q + delta(a, nb - q) with the projections
// a = g . dl already formed (in the forward's operation order): pb -> qb, gb
// (8: r, p, u, v gradients, through a) and nbb (the minmod neighbour values).
template <int RECON>
__device__ __forceinline__ void vjp_reconstruct_a(const Prim<double>& q, const double* a, double dx, double dy,
                                                  const Prim<double>& nb, const Prim<double>& pb, Prim<double>& qb,
                                                  double* gb, Prim<double>& nbb) {
    const double qv[4] = {q.r, q.p, q.u, q.v}, nv[4] = {nb.r, nb.p, nb.u, nb.v};
    const double pv[4] = {pb.r, pb.p, pb.u, pb.v};
    double qbv[4] = {0, 0, 0, 0}, nbv[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double db = pv[k];
        qbv[k] += db;
        if (RECON == RECON_LINEAR) {
            gb[2 * k] += db * dx;
            gb[2 * k + 1] += db * dy;
            continue;
        }
        const double b = nv[k] - qv[k];  // minmod(a, b): a*b > 0 ? (|a| < |b| ? a : b) : 0
        if (a[k] * b > 0.0) {
            if (fabs(a[k]) < fabs(b)) { gb[2 * k] += db * dx; gb[2 * k + 1] += db * dy; }
            else { nbv[k] += db; qbv[k] -= db; }
        }
    }
    qb.r += qbv[0]; qb.p += qbv[1]; qb.u += qbv[2]; qb.v += qbv[3];
    nbb.r += nbv[0]; nbb.p += nbv[1]; nbb.u += nbv[2]; nbb.v += nbv[3];
}

// Projections a = g . dl of one side's four gradients, as reconstruct() forms them.
template <int RECON>
__device__ __forceinline__ void project(const double* g, double dx, double dy, double* a) {
    a[0] = proj<double, RECON>(g[0], g[1], dx, dy);
    a[1] = proj<double, RECON>(g[2], g[3], dx, dy);
    a[2] = proj<double, RECON>(g[4], g[5], dx, dy);
    a[3] = proj<double, RECON>(g[6], g[7], dx, dy);
}

// The forward reconstruction from the projections (kernels.cuh reconstruct).
template <int RECON>
__device__ __forceinline__ Prim<double> recon_a(const Prim<double>& q, const double* a, const Prim<double>& nb) {
    Prim<double> p = q;
    double d0 = a[0], d1 = a[1], d2 = a[2], d3 = a[3];
    if (RECON == RECON_MINMOD) {
        d0 = minmod(d0, nb.r - q.r);
        d1 = minmod(d1, nb.p - q.p);
        d2 = minmod(d2, nb.u - q.u);
        d3 = minmod(d3, nb.v - q.v);
    }
    p.r += d0; p.p += d1; p.u += d2; p.v += d3;
    return p;
}

// One side's reconstruction p = q + delta(g . dl, nb - q) (kernels.cuh reconstruct):
// pb -> qb, gb (8: r, p, u, v gradients) and nbb (the minmod neighbour values).
template <int RECON>
__device__ __forceinline__ void vjp_reconstruct(const Prim<double>& q, const double* g, double dx, double dy,
                                                const Prim<double>& nb, const Prim<double>& pb, Prim<double>& qb,
                                                double* gb, Prim<double>& nbb) {
    const double qv[4] = {q.r, q.p, q.u, q.v}, nv[4] = {nb.r, nb.p, nb.u, nb.v};
    const double pv[4] = {pb.r, pb.p, pb.u, pb.v};
    double qbv[4] = {0, 0, 0, 0}, nbv[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double db = pv[k];
        qbv[k] += db;
        if (RECON == RECON_LINEAR) {
            gb[2 * k] += db * dx;
            gb[2 * k + 1] += db * dy;
        } else {
            const double a = g[2 * k] * dx + g[2 * k + 1] * dy, b = nv[k] - qv[k];
            if (a * b > 0.0) {
                if (fabs(a) < fabs(b)) { gb[2 * k] += db * dx; gb[2 * k + 1] += db * dy; }
                else { nbv[k] += db; qbv[k] -= db; }
            }
        }
    }
    qb.r += qbv[0]; qb.p += qbv[1]; qb.u += qbv[2]; qb.v += qbv[3];
    nbb.r += nbv[0]; nbb.p += nbv[1]; nbb.u += nbv[2]; nbb.v += nbv[3];
}

}  // namespace cfd2d
