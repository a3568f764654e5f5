// Reverse-mode (vector-Jacobian) pieces of the step, written by hand: for each
// forward function f(x) below, vjp_f accumulates x_bar += (df/dx)^T y_bar. T is
// the face precision, as in the forward kernels (double: the FP64 drop-in;
// float: the mixed form's FP32 faces). Each follows the forward expression in
// kernels.cuh line by line and recomputes the forward values with the forward's
// own expressions, so the adjoint is the exact derivative of the discrete scheme
// the solver runs (branches of min/max, minmod and the HLLC wave pattern are
// taken as the forward pass took them). The reverse arithmetic itself needs no
// bit parity.
#pragma once
#include "kernels.cuh"

namespace cfd2d {

// x + a b with one rounding. The reverse sweep's sums of products need no bit parity,
// so they are fused explicitly (the FP64 translation unit is built without automatic
// contraction, which the recomputed forward values need).
template <typename T> __device__ __forceinline__ T madd(T x, T a, T b) { return t_fma(a, b, x); }

// Accumulators start at -0: x + (-0) == x for every x, so the first addition folds away.
template <typename T> __device__ __forceinline__ T acc0() { return T(-0.0); }
template <typename T> __device__ __forceinline__ Prim<T> zero_prim() {
    Prim<T> z;
    z.r = acc0<T>(); z.u = acc0<T>(); z.v = acc0<T>(); z.p = acc0<T>();
    return z;
}

// Conversions between the FP64 per-cell quantities and the face precision
// (integer-pipe narrowing / widening for FP32, identity for FP64).
template <typename T> __device__ __forceinline__ T to_face(double x);
template <> __device__ __forceinline__ double to_face<double>(double x) { return x; }
template <> __device__ __forceinline__ float to_face<float>(double x) { return narrow(x); }
__device__ __forceinline__ double to_wide(double x) { return x; }
__device__ __forceinline__ double to_wide(float x) { return widen(x); }

// A running sum in the face precision kept exact for FP32 (Knuth's TwoSum into a
// value and an error term, so cancelling face contributions lose nothing to the
// summation) and plain for FP64; value() rounds it once into FP64.
template <typename T> struct SumAcc;
template <> struct SumAcc<double> {
    double s = -0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ double face() const { return s; }
};
template <> struct SumAcc<float> {
    float hi = -0.0f, lo = -0.0f;
    __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum(hi, x, t, e);
        hi = t;
        lo += e;
    }
    __device__ __forceinline__ double value() const { return widen(hi) + widen(lo); }
    __device__ __forceinline__ float face() const { return hi + lo; }
};

template <typename T> __device__ __forceinline__ const T* invS_of(const DevCase& c);
template <> __device__ __forceinline__ const double* invS_of<double>(const DevCase& c) { return c.invS; }
template <> __device__ __forceinline__ const float* invS_of<float>(const DevCase& c) { return c.invS32; }

// convertConsToPar: (rho, rho u, rho v, rho E) -> (r, u, v, p), U in the face precision
template <typename T>
__device__ __forceinline__ void vjp_cons2prim(const T* U, T gm1, const Prim<T>& pb, T* Ub) {
    const T ro = U[0], iro = T(1.0) / ro;
    const T u = U[1] * iro, v = U[2] * iro, E = U[3] * iro;
    const T e = E - T(0.5) * (u * u + v * v);
    // p = r e gm1
    T rb = pb.r + pb.p * e * gm1;
    const T eb = pb.p * ro * gm1;
    // e = E - (u^2 + v^2)/2
    const T Eb = eb;
    const T ub = pb.u - eb * u, vb = pb.v - eb * v;
    Ub[1] += ub * iro;
    Ub[2] += vb * iro;
    Ub[3] += Eb * iro;
    rb -= (ub * u + vb * v + Eb * E) * iro;
    Ub[0] += rb;
}

// The same VJP with the conserved state expressed through the stage's primitives
// (E = p/(r gm1) + (u^2 + v^2)/2): no read of the FP64 state.
template <typename T>
__device__ __forceinline__ void vjp_cons2prim_q(const Prim<T>& q, T gm1, const Prim<T>& pb, T* Ub) {
    // derivative factors only: Newton-refined reciprocal and quotient (FP64; FP32 divides)
    const T ro = q.r, iro = hllc_recip(ro), u = q.u, v = q.v;
    const T e = hllc_quot(q.p, ro * gm1);
    const T E = madd(e, T(0.5), t_fma(u, u, v * v));
    T rb = madd(pb.r, pb.p * e, gm1);
    const T eb = pb.p * ro * gm1;
    const T Eb = eb;
    const T ub = madd(pb.u, -eb, u), vb = madd(pb.v, -eb, v);
    Ub[1] = madd(Ub[1], ub, iro);
    Ub[2] = madd(Ub[2], vb, iro);
    Ub[3] = madd(Ub[3], Eb, iro);
    rb = madd(rb, -madd(madd(ub * u, vb, v), Eb, E), iro);
    Ub[0] += rb;
}

// Tc = (p / (r gm1)) / Cv
template <typename T>
__device__ __forceinline__ void vjp_temperature(const Prim<T>& q, T gm1, T Cv, T Tb, Prim<T>& qb) {
    const T k = T(1.0) / (q.r * gm1 * Cv);
    qb.p += Tb * k;
    qb.r -= Tb * (q.p * k) / q.r;
}

// ghost_state(b, q, Tc, n, M): the reference's CFDBnd*::run + URS(2) for the density.
// bp_bar receives d/d(Vx, Vy, T, P) of an inlet's parameters.
template <typename T>
__device__ __forceinline__ void vjp_ghost(const DevBnd& b, const Prim<T>& q, T Tc, T nx, T ny, T M,
                                          const Prim<T>& gb, Prim<T>& qb, T& Tcb, T* bp_bar) {
    if (b.kind == BND_INLET) {
        const T bT = T(b.T), bP = T(b.p);
        const T k = M / (bT * T(GAS_R));
        bp_bar[0] += gb.u;
        bp_bar[1] += gb.v;
        bp_bar[3] += gb.p + gb.r * k;
        bp_bar[2] -= gb.r * (bP * k) / bT;
        return;
    }
    const T k = M / (Tc * T(GAS_R));
    qb.p += gb.p + gb.r * k;
    Tcb -= gb.r * (q.p * k) / Tc;
    if (b.kind == BND_OUTLET) {
        qb.u += gb.u;
        qb.v += gb.v;
    } else {  // wall: u_g = u - 2 nx Un, v_g = v - 2 ny Un, Un = u nx + v ny
        const T Unb = T(-2.0) * (nx * gb.u + ny * gb.v);
        qb.u += gb.u + Unb * nx;
        qb.v += gb.v + Unb * ny;
    }
}

// phys_flux(f, r, u, v, p, E, un, n)
template <typename T>
__device__ __forceinline__ void vjp_phys(T r, T u, T v, T p, T E, T un, T nx, T ny, const T* fb, T& rb, T& ub,
                                         T& vb, T& pb, T& Eb, T& unb) {
    const T m = r * un;
    const T mb = madd(madd(fb[0], fb[1], u), fb[2], v);
    ub = madd(ub, fb[1], m);
    vb = madd(vb, fb[2], m);
    pb = madd(madd(madd(pb, fb[1], nx), fb[2], ny), fb[3], un);
    Eb = madd(Eb, fb[3], un);
    unb = madd(madd(unb, fb[3], E + p), mb, r);
    rb = madd(rb, mb, un);
}

// Lax-Friedrichs (flux_lax in kernels.cuh)
template <typename T>
__device__ __forceinline__ void vjp_lax(const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1, const T* fb,
                                        Prim<T>& Lb, Prim<T>& Rb) {
    const T unl = L.u * nx + L.v * ny, unr = R.u * nx + R.v * ny;
    const T aL = GAM * L.p / L.r, aR = GAM * R.p / R.r;
    const T cL = t_sqrt(aL), cR = t_sqrt(aR);
    const T s1 = t_abs(unl) + cL, s2 = t_abs(unr) + cR;
    const bool first = s1 > s2;  // t_max(a, b) = a > b ? a : b
    const T alpha = first ? s1 : s2;
    const T rol = L.r, rul = L.r * L.u, rvl = L.r * L.v;
    const T rel = div_by(L.p, GAM - T(1.0), IG1) + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    const T ror = R.r, rur = R.r * R.u, rvr = R.r * R.v;
    const T rer = div_by(R.p, GAM - T(1.0), IG1) + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    const T frl = rol * unl, frr = ror * unr;
    const T h0 = T(0.5) * fb[0], h1 = T(0.5) * fb[1], h2 = T(0.5) * fb[2], h3 = T(0.5) * fb[3];
    // f0 = .5(frr + frl - alpha (ror - rol)), f1 = .5(frr uR + frl uL + (pR + pL) nx - alpha (rur - rul))
    // f2 = .5(frr vR + frl vL + (pR + pL) ny - alpha (rvr - rvl)), f3 = .5((rer + pR) unr + (rel + pL) unl - alpha (rer - rel))
    const T frrb = h0 + h1 * R.u + h2 * R.v, frlb = h0 + h1 * L.u + h2 * L.v;
    const T alphab = -(h0 * (ror - rol) + h1 * (rur - rul) + h2 * (rvr - rvl) + h3 * (rer - rel));
    T rorb = -h0 * alpha, rolb = h0 * alpha, rurb = -h1 * alpha, rulb = h1 * alpha;
    T rvrb = -h2 * alpha, rvlb = h2 * alpha, rerb = h3 * unr - h3 * alpha, relb = h3 * unl + h3 * alpha;
    Rb.u += h1 * frr; Lb.u += h1 * frl; Rb.v += h2 * frr; Lb.v += h2 * frl;
    Rb.p += h1 * nx + h2 * ny + h3 * unr; Lb.p += h1 * nx + h2 * ny + h3 * unl;
    T unrb = h3 * (rer + R.p), unlb = h3 * (rel + L.p);
    // fr = ro un
    rorb += frrb * unr; unrb += frrb * ror; rolb += frlb * unl; unlb += frlb * rol;
    // re = p/G1 + .5 r (u^2 + v^2)
    Rb.p += rerb * IG1; rorb += rerb * T(0.5) * (R.u * R.u + R.v * R.v);
    Rb.u += rerb * R.r * R.u; Rb.v += rerb * R.r * R.v;
    Lb.p += relb * IG1; rolb += relb * T(0.5) * (L.u * L.u + L.v * L.v);
    Lb.u += relb * L.r * L.u; Lb.v += relb * L.r * L.v;
    // ru, rv
    rorb += rurb * R.u + rvrb * R.v; Rb.u += rurb * R.r; Rb.v += rvrb * R.r;
    rolb += rulb * L.u + rvlb * L.v; Lb.u += rulb * L.r; Lb.v += rvlb * L.r;
    Rb.r += rorb; Lb.r += rolb;
    // alpha = max(|unl| + cL, |unr| + cR)
    if (first) {
        unlb += alphab * (unl >= T(0) ? T(1.0) : T(-1.0));
        const T ab = T(0.5) * alphab / (cL * L.r);
        Lb.p += ab * GAM; Lb.r -= ab * aL;
    } else {
        unrb += alphab * (unr >= T(0) ? T(1.0) : T(-1.0));
        const T ab = T(0.5) * alphab / (cR * R.r);
        Rb.p += ab * GAM; Rb.r -= ab * aR;
    }
    Lb.u += unlb * nx; Lb.v += unlb * ny; Rb.u += unrb * nx; Rb.v += unrb * ny;
}

// Ss = num / den as the forward forms it (hllc_quot: the forward's quotient bit for bit),
// with an approximation of 1/den for the derivatives (the Newton reciprocal hllc_quot
// starts from; FP32: a division)
__device__ __forceinline__ double star_speed(double num, double den, double& iden) {
    iden = hllc_in_range(den) ? hllc_rcp1(den) : 1.0 / den;
    return hllc_quot(num, den);
}
__device__ __forceinline__ float star_speed(float num, float den, float& iden) {
    iden = 1.0f / den;
    return num / den;
}

// HLLC in the single-division star-flux form (flux_hllc in kernels.cuh), with the forward's
// sound speeds cL, cR given
template <typename T>
__device__ __forceinline__ void vjp_hllc_c(const Prim<T>& L, const Prim<T>& R, T cL, T cR, T nx, T ny, T GAM, T IG1,
                                           const T* fb, Prim<T>& Lb, Prim<T>& Rb) {
    const T unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    const T EL = energy(L.r, L.u, L.v, L.p, IG1);
    const T ER = energy(R.r, R.u, R.v, R.p, IG1);
    const T sl1 = unL - cL, sl2 = unR - cR, sr1 = unL + cL, sr2 = unR + cR;
    const bool l1 = sl1 < sl2, r1 = sr1 > sr2;
    const T SL = l1 ? sl1 : sl2, SR = r1 ? sr1 : sr2;
    T unLb = acc0<T>(), unRb = acc0<T>(), ELb = acc0<T>(), ERb = acc0<T>();
    T SLb = acc0<T>(), SRb = acc0<T>(), cLb = acc0<T>(), cRb = acc0<T>();
    if (SL >= T(0.0) || SR <= T(0.0)) {  // supersonic: the upwind side's physical flux
        if (SL >= T(0.0)) vjp_phys(L.r, L.u, L.v, L.p, EL, unL, nx, ny, fb, Lb.r, Lb.u, Lb.v, Lb.p, ELb, unLb);
        else vjp_phys(R.r, R.u, R.v, R.p, ER, unR, nx, ny, fb, Rb.r, Rb.u, Rb.v, Rb.p, ERb, unRb);
    } else {
        const T mL = L.r * (SL - unL), mR = R.r * (SR - unR);
        const T num = t_fma(-mR, unR, t_fma(mL, unL, R.p - L.p)), den = mL - mR;
        T iden;
        const T Ss = star_speed(num, den, iden);
        const bool left = Ss >= T(0.0);
        const Prim<T>& K = left ? L : R;
        const T SK = left ? SL : SR, unK = left ? unL : unR, EK = left ? EL : ER, mK = left ? mL : mR;
        T FK[4];
        phys_flux(FK, K.r, K.u, K.v, K.p, EK, unK, nx, ny);
        const T ps = t_fma(mK, Ss - unK, K.p);
        const T inv = hllc_recip(SK - Ss);
        const T sp = SK * ps;
        // A_k and h_k only feed the derivatives: fused freely
        const T A0 = madd(-FK[0], SK, K.r), A1 = madd(-FK[1], SK, K.r * K.u), A2 = madd(-FK[2], SK, K.r * K.v),
                A3 = madd(-FK[3], SK, EK);
        const T h0 = Ss * A0, h1 = madd(Ss * A1, sp, nx), h2 = madd(Ss * A2, sp, ny), h3 = madd(Ss * A3, sp, Ss);
        // f_k = h_k inv
        const T hb0 = fb[0] * inv, hb1 = fb[1] * inv, hb2 = fb[2] * inv, hb3 = fb[3] * inv;
        const T invb = madd(madd(madd(fb[0] * h0, fb[1], h1), fb[2], h2), fb[3], h3);
        T Ssb = madd(madd(madd(hb0 * A0, hb1, A1), hb2, A2), hb3, A3 + sp);
        const T A0b = hb0 * Ss, A1b = hb1 * Ss, A2b = hb2 * Ss, A3b = hb3 * Ss;
        const T spb = madd(madd(hb1 * nx, hb2, ny), hb3, Ss);
        // inv = 1/(SK - Ss)
        const T ii = invb * inv * inv;
        T SKb = -ii;
        Ssb += ii;
        // sp = SK ps
        SKb = madd(SKb, spb, ps);
        const T psb = spb * SK;
        // ps = pK + mK (Ss - unK)
        T Krb = acc0<T>(), Kub = acc0<T>(), Kvb = acc0<T>(), Kpb = psb, EKb = acc0<T>();
        T unKb = -psb * mK;
        const T mKb = psb * (Ss - unK);
        Ssb = madd(Ssb, psb, mK);
        // A_k
        SKb = madd(madd(madd(madd(SKb, A0b, K.r), A1b, K.r * K.u), A2b, K.r * K.v), A3b, EK);
        const T A1S = A1b * SK, A2S = A2b * SK;
        Krb = madd(madd(madd(Krb, A0b, SK), A1S, K.u), A2S, K.v);
        Kub = madd(Kub, A1S, K.r);
        Kvb = madd(Kvb, A2S, K.r);
        EKb = madd(EKb, A3b, SK);
        const T FKb[4] = {-A0b, -A1b, -A2b, -A3b};
        vjp_phys(K.r, K.u, K.v, K.p, EK, unK, nx, ny, FKb, Krb, Kub, Kvb, Kpb, EKb, unKb);
        // route the K-side adjoints
        T mLb = acc0<T>(), mRb = acc0<T>();
        if (left) {
            Lb.r += Krb; Lb.u += Kub; Lb.v += Kvb; Lb.p += Kpb; ELb += EKb; unLb += unKb; SLb += SKb; mLb += mKb;
        } else {
            Rb.r += Krb; Rb.u += Kub; Rb.v += Kvb; Rb.p += Kpb; ERb += EKb; unRb += unKb; SRb += SKb; mRb += mKb;
        }
        // Ss = num / den
        const T numb = Ssb * iden, denb = -Ssb * Ss * iden;
        Rb.p += numb; Lb.p -= numb;
        mLb = madd(mLb + denb, numb, unL); unLb = madd(unLb, numb, mL);
        mRb = madd(mRb - denb, -numb, unR); unRb = madd(unRb, -numb, mR);
        // mL = rL (SL - unL), mR = rR (SR - unR)
        Lb.r = madd(Lb.r, mLb, SL - unL); SLb = madd(SLb, mLb, L.r); unLb = madd(unLb, -mLb, L.r);
        Rb.r = madd(Rb.r, mRb, SR - unR); SRb = madd(SRb, mRb, R.r); unRb = madd(unRb, -mRb, R.r);
        // SL = min(sl1, sl2), SR = max(sr1, sr2)
        if (l1) { unLb += SLb; cLb -= SLb; } else { unRb += SLb; cRb -= SLb; }
        if (r1) { unLb += SRb; cLb += SRb; } else { unRb += SRb; cRb += SRb; }
    }
    // E = p IG1 + .5 r (u^2 + v^2)
    {
        const T eL = ELb * L.r, eR = ERb * R.r;
        Lb.p = madd(Lb.p, ELb, IG1); Lb.r = madd(Lb.r, ELb * T(0.5), t_fma(L.u, L.u, L.v * L.v));
        Lb.u = madd(Lb.u, eL, L.u); Lb.v = madd(Lb.v, eL, L.v);
        Rb.p = madd(Rb.p, ERb, IG1); Rb.r = madd(Rb.r, ERb * T(0.5), t_fma(R.u, R.u, R.v * R.v));
        Rb.u = madd(Rb.u, eR, R.u); Rb.v = madd(Rb.v, eR, R.v);
    }
    // un = u nx + v ny
    Lb.u = madd(Lb.u, unLb, nx); Lb.v = madd(Lb.v, unLb, ny);
    Rb.u = madd(Rb.u, unRb, nx); Rb.v = madd(Rb.v, unRb, ny);
    // c = sqrt(GAM p / r) = sqrt(a): dc = (GAM dp - a dr) / (2 c r), a = c^2
    if (cLb != T(0.0)) {
        const T ab = hllc_quot(T(0.5) * cLb, cL * L.r);
        Lb.p = madd(Lb.p, ab, GAM); Lb.r = madd(Lb.r, -ab, cL * cL);
    }
    if (cRb != T(0.0)) {
        const T ab = hllc_quot(T(0.5) * cRb, cR * R.r);
        Rb.p = madd(Rb.p, ab, GAM); Rb.r = madd(Rb.r, -ab, cR * cR);
    }
}

// FP64 faces: the VJP of the FP64 forward's arrangement (flux_hllc_c<double> in kernels.cuh:
// S_K U_K - F_K from m_K = rho_K d_K, d_K = S_K - un_K, and only the used side's energy),
// recomputing the forward's values and branches with its own expressions.
__device__ __forceinline__ void vjp_hllc_c(const Prim<double>& L, const Prim<double>& R, double cL, double cR,
                                           double nx, double ny, double GAM, double IG1, const double* fb,
                                           Prim<double>& Lb, Prim<double>& Rb) {
    typedef double T;
    const T unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    const T sl1 = unL - cL, sl2 = unR - cR, sr1 = unL + cL, sr2 = unR + cR;
    const bool l1 = sl1 < sl2, r1 = sr1 > sr2;
    const T SL = l1 ? sl1 : sl2, SR = r1 ? sr1 : sr2;
    T unLb = acc0<T>(), unRb = acc0<T>(), SLb = acc0<T>(), SRb = acc0<T>(), cLb = acc0<T>(), cRb = acc0<T>();
    // E = p IG1 + .5 r (u^2 + v^2): the adjoint Eb of one side's energy into its state
    auto energy_bar = [&](const Prim<T>& q, T Eb, Prim<T>& qb) {
        const T e = Eb * q.r;
        qb.p = madd(qb.p, Eb, IG1); qb.r = madd(qb.r, Eb * T(0.5), t_fma(q.u, q.u, q.v * q.v));
        qb.u = madd(qb.u, e, q.u); qb.v = madd(qb.v, e, q.v);
    };
    if (SL >= T(0.0) || SR <= T(0.0)) {  // supersonic: the upwind side's physical flux
        T Eb = acc0<T>();
        if (SL >= T(0.0)) {
            vjp_phys(L.r, L.u, L.v, L.p, energy(L.r, L.u, L.v, L.p, IG1), unL, nx, ny, fb, Lb.r, Lb.u, Lb.v, Lb.p,
                     Eb, unLb);
            energy_bar(L, Eb, Lb);
        } else {
            vjp_phys(R.r, R.u, R.v, R.p, energy(R.r, R.u, R.v, R.p, IG1), unR, nx, ny, fb, Rb.r, Rb.u, Rb.v, Rb.p,
                     Eb, unRb);
            energy_bar(R, Eb, Rb);
        }
    } else {
        const T dL = SL - unL, dR = SR - unR;
        const T mL = L.r * dL, mR = R.r * dR;
        const T num = t_fma(-mR, unR, t_fma(mL, unL, R.p - L.p)), den = mL - mR;
        T iden;
        const T Ss = star_speed(num, den, iden);
        const bool left = Ss >= T(0.0);
        const Prim<T>& K = left ? L : R;
        const T SK = left ? SL : SR, unK = left ? unL : unR, dK = left ? dL : dR, mK = left ? mL : mR;
        const T EK = energy(K.r, K.u, K.v, K.p, IG1);
        const T A1 = t_fma(mK, K.u, -(K.p * nx)), A2 = t_fma(mK, K.v, -(K.p * ny)), A3 = t_fma(EK, dK, -(K.p * unK));
        const T ps = t_fma(mK, Ss - unK, K.p);
        const T inv = hllc_recip(SK - Ss);
        const T sp = SK * ps;
        // h0 = Ss mK, h1 = Ss A1 + sp nx, h2 = Ss A2 + sp ny, h3 = Ss A3 + sp Ss; f_k = h_k inv
        const T h0 = Ss * mK, h1 = madd(Ss * A1, sp, nx), h2 = madd(Ss * A2, sp, ny), h3 = madd(Ss * A3, sp, Ss);
        const T hb0 = fb[0] * inv, hb1 = fb[1] * inv, hb2 = fb[2] * inv, hb3 = fb[3] * inv;
        const T invb = madd(madd(madd(fb[0] * h0, fb[1], h1), fb[2], h2), fb[3], h3);
        T Ssb = madd(madd(madd(hb0 * mK, hb1, A1), hb2, A2), hb3, A3 + sp);
        T mKb = hb0 * Ss;
        const T A1b = hb1 * Ss, A2b = hb2 * Ss, A3b = hb3 * Ss;
        const T spb = madd(madd(hb1 * nx, hb2, ny), hb3, Ss);
        // inv = 1/(SK - Ss)
        const T ii = invb * inv * inv;
        T SKb = -ii;
        Ssb += ii;
        // sp = SK ps
        SKb = madd(SKb, spb, ps);
        const T psb = spb * SK;
        // ps = pK + mK (Ss - unK)
        T Krb = acc0<T>(), Kub = acc0<T>(), Kvb = acc0<T>(), Kpb = psb;
        T unKb = -psb * mK;
        mKb = madd(mKb, psb, Ss - unK);
        Ssb = madd(Ssb, psb, mK);
        // A1 = mK u - p nx, A2 = mK v - p ny, A3 = EK dK - p unK
        mKb = madd(madd(mKb, A1b, K.u), A2b, K.v);
        Kub = madd(Kub, A1b, mK);
        Kvb = madd(Kvb, A2b, mK);
        Kpb = madd(madd(madd(Kpb, -A1b, nx), -A2b, ny), -A3b, unK);
        const T EKb = A3b * dK;
        T dKb = A3b * EK;
        unKb = madd(unKb, -A3b, K.p);
        // Ss = num / den
        const T numb = Ssb * iden, denb = -Ssb * Ss * iden;
        Rb.p += numb; Lb.p -= numb;
        T mLb = madd(denb, numb, unL), mRb = madd(-denb, -numb, unR);
        unLb = madd(unLb, numb, mL); unRb = madd(unRb, -numb, mR);
        T dLb = acc0<T>(), dRb = acc0<T>();
        // route the K side (its m, d, state, energy and speeds) to L or R
        if (left) {
            mLb += mKb; dLb += dKb; unLb += unKb; SLb += SKb;
            Lb.r += Krb; Lb.u += Kub; Lb.v += Kvb; Lb.p += Kpb;
            energy_bar(L, EKb, Lb);
        } else {
            mRb += mKb; dRb += dKb; unRb += unKb; SRb += SKb;
            Rb.r += Krb; Rb.u += Kub; Rb.v += Kvb; Rb.p += Kpb;
            energy_bar(R, EKb, Rb);
        }
        // mL = rL dL, dL = SL - unL (and R)
        Lb.r = madd(Lb.r, mLb, dL); dLb = madd(dLb, mLb, L.r);
        Rb.r = madd(Rb.r, mRb, dR); dRb = madd(dRb, mRb, R.r);
        SLb += dLb; unLb -= dLb;
        SRb += dRb; unRb -= dRb;
        // SL = min(sl1, sl2), SR = max(sr1, sr2)
        if (l1) { unLb += SLb; cLb -= SLb; } else { unRb += SLb; cRb -= SLb; }
        if (r1) { unLb += SRb; cLb += SRb; } else { unRb += SRb; cRb += SRb; }
    }
    // un = u nx + v ny
    Lb.u = madd(Lb.u, unLb, nx); Lb.v = madd(Lb.v, unLb, ny);
    Rb.u = madd(Rb.u, unRb, nx); Rb.v = madd(Rb.v, unRb, ny);
    // c = sqrt(GAM p / r) = sqrt(a): dc = (GAM dp - a dr) / (2 c r), a = c^2
    if (cLb != T(0.0)) {
        const T ab = hllc_quot(T(0.5) * cLb, cL * L.r);
        Lb.p = madd(Lb.p, ab, GAM); Lb.r = madd(Lb.r, -ab, cL * cL);
    }
    if (cRb != T(0.0)) {
        const T ab = hllc_quot(T(0.5) * cRb, cR * R.r);
        Rb.p = madd(Rb.p, ab, GAM); Rb.r = madd(Rb.r, -ab, cR * cR);
    }
}

template <typename T>
__device__ __forceinline__ void vjp_hllc(const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1, const T* fb,
                                         Prim<T>& Lb, Prim<T>& Rb) {
    const T cL = hllc_sound(GAM * L.p, L.r), cR = hllc_sound(GAM * R.p, R.r);  // the forward's values
    vjp_hllc_c(L, R, cL, cR, nx, ny, GAM, IG1, fb, Lb, Rb);
}

template <int FLUX, typename T>
__device__ __forceinline__ void vjp_flux(const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1, const T* fb,
                                         Prim<T>& Lb, Prim<T>& Rb) {
    if (FLUX == FLUX_HLLC) vjp_hllc(L, R, nx, ny, GAM, IG1, fb, Lb, Rb);
    else vjp_lax(L, R, nx, ny, GAM, IG1, fb, Lb, Rb);
}

// One side's reconstruction p = q + delta(a, nb - q) with the projections
// a = g . dl already formed (in the forward's operation order): pb -> qb, gb
// (8: r, p, u, v gradients, through a) and nbb (the minmod neighbour values).
// The minmod branch is the forward's own decision (mm_pos, mm_first).
template <int RECON, typename T>
__device__ __forceinline__ void vjp_reconstruct_a(const Prim<T>& q, const T* a, T dx, T dy, const Prim<T>& nb,
                                                  const Prim<T>& pb, Prim<T>& qb, T* gb, Prim<T>& nbb) {
    const T qv[4] = {q.r, q.p, q.u, q.v}, nv[4] = {nb.r, nb.p, nb.u, nb.v};
    const T pv[4] = {pb.r, pb.p, pb.u, pb.v};
    T qbv[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()}, nbv[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const T db = pv[k];
        qbv[k] += db;
        if (RECON == RECON_LINEAR) {
            gb[2 * k] = madd(gb[2 * k], db, dx);
            gb[2 * k + 1] = madd(gb[2 * k + 1], db, dy);
            continue;
        }
        const T b = nv[k] - qv[k];
        if (mm_pos(a[k], b)) {
            if (mm_first(a[k], b)) { gb[2 * k] = madd(gb[2 * k], db, dx); gb[2 * k + 1] = madd(gb[2 * k + 1], db, dy); }
            else { nbv[k] += db; qbv[k] -= db; }
        }
    }
    qb.r += qbv[0]; qb.p += qbv[1]; qb.u += qbv[2]; qb.v += qbv[3];
    nbb.r += nbv[0]; nbb.p += nbv[1]; nbb.u += nbv[2]; nbb.v += nbv[3];
}

// The same VJP with minmod's branches read from the forward's record (code: 2 bits per
// variable r, p, u, v; 1 the projection, 2 the neighbour difference, 0 neither) instead
// of being recomputed: the same operations on the same values.
template <int RECON, typename T>
__device__ __forceinline__ void vjp_reconstruct_code(unsigned code, T dx, T dy, const Prim<T>& pb, Prim<T>& qb,
                                                     T* gb, Prim<T>& nbb) {
    const T pv[4] = {pb.r, pb.p, pb.u, pb.v};
    T qbv[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()}, nbv[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const T db = pv[k];
        qbv[k] += db;
        const unsigned br = RECON == RECON_LINEAR ? 1u : (code >> (2 * k)) & 3u;
        if (br == 1u) { gb[2 * k] = madd(gb[2 * k], db, dx); gb[2 * k + 1] = madd(gb[2 * k + 1], db, dy); }
        else if (br == 2u) { nbv[k] += db; qbv[k] -= db; }
    }
    qb.r += qbv[0]; qb.p += qbv[1]; qb.u += qbv[2]; qb.v += qbv[3];
    nbb.r += nbv[0]; nbb.p += nbv[1]; nbb.u += nbv[2]; nbb.v += nbv[3];
}

// Projections a = g . dl of one side's four gradients, as reconstruct() forms them.
template <int RECON, typename T>
__device__ __forceinline__ void project(const T* g, T dx, T dy, T* a) {
    a[0] = proj<T, RECON>(g[0], g[1], dx, dy);
    a[1] = proj<T, RECON>(g[2], g[3], dx, dy);
    a[2] = proj<T, RECON>(g[4], g[5], dx, dy);
    a[3] = proj<T, RECON>(g[6], g[7], dx, dy);
}

// The forward reconstruction from the projections (kernels.cuh reconstruct).
template <int RECON, typename T>
__device__ __forceinline__ Prim<T> recon_a(const Prim<T>& q, const T* a, const Prim<T>& nb) {
    Prim<T> p = q;
    T d0 = a[0], d1 = a[1], d2 = a[2], d3 = a[3];
    if (RECON == RECON_MINMOD) {
        d0 = minmod(d0, nb.r - q.r);
        d1 = minmod(d1, nb.p - q.p);
        d2 = minmod(d2, nb.u - q.u);
        d3 = minmod(d3, nb.v - q.v);
    }
    p.r += d0; p.p += d1; p.u += d2; p.v += d3;
    return p;
}

}  // namespace cfd2d
