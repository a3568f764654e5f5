// Device code of the GB300 FVM_TVD path, templated on the face precision T
// (double for the FP64 drop-in, float for the mixed form). Included by
// kern_fp64.cu (built with -fmad=false so every product and sum rounds on its
// own, as in the reference's x86/ARM build) and by kern_mixed.cu.
//
// Bit-reproducibility without atomics: every interior edge flux is computed
// once (k_flux, one thread per edge) and each cell gathers its three edge
// fluxes in ascending original edge number with the reference's signs
// (c1: -=, c2: +=, src/methods/fvm_tvd.cpp:353-363). That is the order in which
// the reference's edge loop accumulates into each cell, so the FP64 sums are
// the reference's sums.
#pragma once
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace cfd2d {

template <typename T>
struct Prim { T r, u, v, p; };

__device__ __forceinline__ double t_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float t_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double t_exp(double x) { return exp(x); }
__device__ __forceinline__ float t_exp(float x) { return expf(x); }
__device__ __forceinline__ double t_log(double x) { return log(x); }
__device__ __forceinline__ float t_log(float x) { return logf(x); }
__device__ __forceinline__ double t_abs(double x) { return fabs(x); }
__device__ __forceinline__ float t_abs(float x) { return fabsf(x); }
template <typename T> __device__ __forceinline__ T t_max(T a, T b) { return a > b ? a : b; }  // _max_, src/mesh/grid.h:102
template <typename T> __device__ __forceinline__ T t_min(T a, T b) { return a < b ? a : b; }

template <typename T> __device__ __forceinline__ const T* W_of(const DevCase& c);
template <> __device__ __forceinline__ const double* W_of<double>(const DevCase& c) { return c.W64; }
template <> __device__ __forceinline__ const float* W_of<float>(const DevCase& c) { return c.W32; }
template <typename T> __device__ __forceinline__ T* Wm_of(const DevCase& c);
template <> __device__ __forceinline__ double* Wm_of<double>(const DevCase& c) { return c.W64; }
template <> __device__ __forceinline__ float* Wm_of<float>(const DevCase& c) { return c.W32; }
template <typename T> __device__ __forceinline__ T* G_of(const DevCase& c);
template <> __device__ __forceinline__ double* G_of<double>(const DevCase& c) { return c.G64; }
template <> __device__ __forceinline__ float* G_of<float>(const DevCase& c) { return c.G32; }
template <typename T> __device__ __forceinline__ T* F_of(const DevCase& c);
template <> __device__ __forceinline__ double* F_of<double>(const DevCase& c) { return c.F64; }
template <> __device__ __forceinline__ float* F_of<float>(const DevCase& c) { return c.F32; }
template <typename T> __device__ __forceinline__ const T* NX_of(const DevCase& c);
template <> __device__ __forceinline__ const double* NX_of<double>(const DevCase& c) { return c.nx; }
template <> __device__ __forceinline__ const float* NX_of<float>(const DevCase& c) { return c.nx32; }
template <typename T> __device__ __forceinline__ const T* NY_of(const DevCase& c);
template <> __device__ __forceinline__ const double* NY_of<double>(const DevCase& c) { return c.ny; }
template <> __device__ __forceinline__ const float* NY_of<float>(const DevCase& c) { return c.ny32; }
template <typename T> __device__ __forceinline__ const T* L_of(const DevCase& c);
template <> __device__ __forceinline__ const double* L_of<double>(const DevCase& c) { return c.l; }
template <> __device__ __forceinline__ const float* L_of<float>(const DevCase& c) { return c.l32; }
template <typename T> __device__ __forceinline__ const T* DL_of(const DevCase& c);
template <> __device__ __forceinline__ const double* DL_of<double>(const DevCase& c) { return c.dl; }
template <> __device__ __forceinline__ const float* DL_of<float>(const DevCase& c) { return c.dl32; }

__device__ __forceinline__ DevMat mat_of(const DevCase& c, int cell) {
    return c.cmat ? c.mats[c.cmat[cell]] : c.mat0;
}

template <typename T>
__device__ __forceinline__ Prim<T> load_prim(const T* __restrict__ W, int n, int i) {
    Prim<T> q;
    q.r = W[i]; q.u = W[n + i]; q.v = W[2 * n + i]; q.p = W[3 * n + i];
    return q;
}

template <typename T>
__device__ __forceinline__ void store_prim(T* __restrict__ W, int n, int i, const Prim<T>& q) {
    W[i] = q.r; W[n + i] = q.u; W[2 * n + i] = q.v; W[3 * n + i] = q.p;
}

// convertConsToPar + Material::URS(0), src/methods/fvm_tvd.cpp:803-813, src/global.cpp:15-18
template <typename T>
__device__ __forceinline__ Prim<T> cons2prim(T ro, T ru, T rv, T re, T gm1) {
    Prim<T> q;
    q.r = ro;
    q.u = ru / ro;
    q.v = rv / ro;
    T E = re / ro;
    T e = E - T(0.5) * (q.u * q.u + q.v * q.v);
    q.p = q.r * e * gm1;
    return q;
}

// Material::URS(1) temperature of a state: e = p/(r (gam-1)), T = e/Cv
template <typename T>
__device__ __forceinline__ T temperature(const Prim<T>& q, T gm1, T Cv) {
    T e = q.p / (q.r * gm1);
    return e / Cv;
}

// Ghost state: CFDBnd*::run then URS(2) for the density, src/bnd_cond.cpp:75-110,
// src/methods/fvm_tvd.cpp:694-705. Tc is the (stale) cell-centre temperature the
// reference carries in pL.T. Only r, u, v, p are consumed downstream.
template <typename T>
__device__ __forceinline__ Prim<T> ghost_state(const DevBnd& b, const Prim<T>& q, T Tc, T nx, T ny, T M) {
    Prim<T> g;
    T Tg;
    if (b.kind == BND_INLET) {
        g.u = T(b.u); g.v = T(b.v); g.p = T(b.p); Tg = T(b.T);
    } else if (b.kind == BND_OUTLET) {
        g = q; Tg = Tc;
    } else {  // BOUND_WALL_SLIP; BOUND_WALL_NO_SLIP is the slip class in the reference (src/bnd_cond.cpp:50-55)
        T Un = q.u * nx + q.v * ny;
        T Vx = nx * Un * T(2.0), Vy = ny * Un * T(2.0);
        g.u = q.u - Vx; g.v = q.v - Vy; g.p = q.p; Tg = Tc;
    }
    g.r = g.p * M / (Tg * T(GAS_R));
    return g;
}

// MINMOD, src/methods/LimiterDGCockburn.cpp:110-123
template <typename T>
__device__ __forceinline__ T minmod(T a, T b) {
    if (a * b > T(0)) return t_abs(a) < t_abs(b) ? a : b;
    return T(0);
}

// ------------------------------------------------------------------ fluxes

// Exact Riemann solver rim_orig (src/global.cpp:232-405), structured, with a cap
// on its Newton loop (the reference has none and can spin forever).
template <typename T>
__device__ __forceinline__ bool riemann_exact(T& RI, T& EI, T& PI, T& UI, T& VI, T RB, T PB, T UB, T VB, T RE,
                                              T PE, T UE, T VE, T GAM, int cap) {
    const T AGAM = (GAM - T(1.0));
    const T DGAM = (T(2.0) / AGAM);
    const T GGAM = (t_sqrt(GAM * AGAM));
    const T HGAM = (AGAM / T(2.0));
    const T FGAM = (T(3.0) * GAM - T(1.0));
    const T OGAM = (AGAM / (T(2.0) * GAM));
    const T QGAM = (GAM + T(1.0));
    const T PGAM = (QGAM / (T(2.0) * GAM));
    const T RGAM = (T(4.0) * GAM);
    const T SGAM = (GAM * AGAM);
    const T TGAM = (QGAM / T(2.0));
    T US = T(0.0), UF = T(0.0);
    T RF, RS, EF, ES, SBL, SFL, SSL, SEL, D, P;
    const T eps = T(1.0e-5);
    T CB = t_sqrt(GAM * PB / RB);
    T CE = t_sqrt(GAM * PE / RE);
    T EB = CB * CB / SGAM;
    T EE = CE * CE / SGAM;
    T RCB = RB * CB;
    T RCE = RE * CE;
    T DU = UB - UE;
    bool hit = false;
    if (DU < T(-2.0) * (CB + CE) / AGAM) {  // vacuum
        RF = T(0.0); RS = T(0.0); EF = T(0.0); ES = T(0.0);
        SBL = UB - CB;
        SFL = UB + T(2.0) * CB / AGAM;
        SSL = UE - T(2.0) * CE / AGAM;
        SEL = UE + CE;
    } else {
        P = (PB * RCE + PE * RCB + DU * RCB * RCE) / (RCB + RCE);
        int it = 0;
        for (;;) {
            T F1, FS1, F2, FS2;
            if (P < eps) P = eps;
            T PPB = P / PB;
            if (PB > P) {
                T ZFB = CB * t_exp(t_log(PPB) * OGAM);
                F1 = DGAM * (ZFB - CB);
                FS1 = ZFB / (GAM * P);
            } else {
                T PKB = PGAM * PPB + OGAM;
                T ZNB = RCB * t_sqrt(PKB);
                F1 = (P - PB) / ZNB;
                FS1 = (QGAM * PPB + FGAM) / (RGAM * ZNB * PKB);
            }
            T PPE = P / PE;
            if (PE > P) {
                T ZFE = CE * t_exp(t_log(PPE) * OGAM);
                F2 = DGAM * (ZFE - CE);
                FS2 = ZFE / (GAM * P);
            } else {
                T PKE = PGAM * PPE + OGAM;
                T ZNE = RCE * t_sqrt(PKE);
                F2 = (P - PE) / ZNE;
                FS2 = (QGAM * PPE + FGAM) / (RGAM * ZNE * PKE);
            }
            T DP = (DU - F1 - F2) / (FS1 + FS2);
            P = P + DP;
            if (!(t_abs(DU - F1 - F2) > eps)) break;
            if (++it >= cap) { hit = true; break; }
        }
        T PPB = P / PB, PPE = P / PE;
        T ZFB = CB * t_exp(t_log(PPB) * OGAM);
        T ZFE = CE * t_exp(t_log(PPE) * OGAM);
        if (!(PB > P)) {
            D = UB - t_sqrt((TGAM * P + HGAM * PB) / RB);
            T UBD = UB - D, RUBD = RB * UBD;
            RF = RUBD * RUBD / (PB - P + RUBD * UBD);
            UF = D + RUBD / RF;
            EF = P / (AGAM * RF);
            SBL = D; SFL = D;
        } else {
            EF = ZFB * ZFB / SGAM;
            UF = UB + DGAM * (CB - ZFB);
            RF = P / (AGAM * EF);
            SBL = UB - CB;
            SFL = UF - ZFB;
        }
        if (!(PE > P)) {
            D = UE + t_sqrt((TGAM * P + HGAM * PE) / RE);
            T UED = UE - D, RUED = RE * UED;
            RS = RUED * RUED / (PE - P + RUED * UED);
            US = D + RUED / RS;
            ES = P / (AGAM * RS);
            SEL = D; SSL = D;
        } else {
            ES = ZFE * ZFE / SGAM;
            US = UE - DGAM * (CE - ZFE);
            RS = P / (AGAM * ES);
            SSL = US + ZFE;
            SEL = UE + CE;
        }
    }
    if (SEL <= T(0.0)) { RI = RE; EI = EE; UI = UE; VI = VE; }
    else if (SBL >= T(0.0)) { RI = RB; EI = EB; UI = UB; VI = VB; }
    else if ((SSL >= T(0.0)) && (SFL <= T(0.0))) {
        if (US >= T(0.0)) { RI = RF; EI = EF; UI = UF; VI = VB; }
        else { RI = RS; EI = ES; UI = US; VI = VE; }
    } else if (SFL > T(0.0)) {
        UI = (UB + DGAM * GGAM * t_sqrt(EB)) / (T(1) + DGAM);
        VI = VB;
        EI = (UI * UI) / SGAM;
        RI = RB * t_exp(t_log(EI / EB) * (T(1) / AGAM));
    } else {
        UI = (UE - DGAM * GGAM * t_sqrt(EE)) / (T(1) + DGAM);
        VI = VE;
        EI = (UI * UI) / SGAM;
        RI = RE * t_exp(t_log(EI / EE) * (T(1) / AGAM));
    }
    PI = AGAM * EI * RI;
    return hit;
}

// Godunov flux, FVM_TVD::calcFlux, src/methods/fvm_tvd.cpp:602-622
template <typename T>
__device__ __forceinline__ bool flux_godunov(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, int cap) {
    T RI, EI, PI, UN, UT;
    T unl = L.u * nx + L.v * ny;
    T unr = R.u * nx + R.v * ny;
    T utl = L.u * ny - L.v * nx;
    T utr = R.u * ny - R.v * nx;
    bool hit = riemann_exact(RI, EI, PI, UN, UT, L.r, L.p, unl, utl, R.r, R.p, unr, utr, GAM, cap);
    T UI = UN * nx + UT * ny;
    T VI = UN * ny - UT * nx;
    f[0] = RI * UN;
    f[1] = f[0] * UI + PI * nx;
    f[2] = f[0] * VI + PI * ny;
    f[3] = (RI * (EI + T(0.5) * (UI * UI + VI * VI)) + PI) * UN;
    return hit;
}

// Lax-Friedrichs (Rusanov), the reference's template src/methods/fvm_tvd_implicit.cpp:939-960
template <typename T>
__device__ __forceinline__ void flux_lax(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM) {
    T unl = L.u * nx + L.v * ny;
    T unr = R.u * nx + R.v * ny;
    T alpha = t_max(t_abs(unl) + t_sqrt(GAM * L.p / L.r), t_abs(unr) + t_sqrt(GAM * R.p / R.r));
    T rol = L.r, rul = L.r * L.u, rvl = L.r * L.v;
    T rel = L.p / (GAM - T(1.0)) + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    T ror = R.r, rur = R.r * R.u, rvr = R.r * R.v;
    T rer = R.p / (GAM - T(1.0)) + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    T frl = rol * unl, frr = ror * unr;
    f[0] = T(0.5) * (frr + frl - alpha * (ror - rol));
    f[1] = T(0.5) * (frr * R.u + frl * L.u + (R.p + L.p) * nx - alpha * (rur - rul));
    f[2] = T(0.5) * (frr * R.v + frl * L.v + (R.p + L.p) * ny - alpha * (rvr - rvl));
    f[3] = T(0.5) * ((rer + R.p) * unr + (rel + L.p) * unl - alpha * (rer - rel));
}

template <typename T>
__device__ __forceinline__ void phys_flux(T* f, T r, T u, T v, T p, T E, T un, T nx, T ny) {
    T m = r * un;
    f[0] = m;
    f[1] = m * u + p * nx;
    f[2] = m * v + p * ny;
    f[3] = (E + p) * un;
}

// HLLC (Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, sec. 10.4-10.5),
// Davis wave speeds S_L = min(unL-cL, unR-cR), S_R = max(unL+cL, unR+cR).
template <typename T>
__device__ __forceinline__ void flux_hllc(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM) {
    T cL = t_sqrt(GAM * L.p / L.r), cR = t_sqrt(GAM * R.p / R.r);
    T unL = L.u * nx + L.v * ny, unR = R.u * nx + R.v * ny;
    T EL = L.p / (GAM - T(1.0)) + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    T ER = R.p / (GAM - T(1.0)) + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    T SL = t_min(unL - cL, unR - cR), SR = t_max(unL + cL, unR + cR);
    if (SL >= T(0.0)) { phys_flux(f, L.r, L.u, L.v, L.p, EL, unL, nx, ny); return; }
    if (SR <= T(0.0)) { phys_flux(f, R.r, R.u, R.v, R.p, ER, unR, nx, ny); return; }
    T mL = L.r * (SL - unL), mR = R.r * (SR - unR);
    T Ss = (R.p - L.p + mL * unL - mR * unR) / (mL - mR);
    const bool left = Ss >= T(0.0);
    const Prim<T>& K = left ? L : R;
    T SK = left ? SL : SR, unK = left ? unL : unR, EK = left ? EL : ER, mK = left ? mL : mR;
    T FK[4];
    phys_flux(FK, K.r, K.u, K.v, K.p, EK, unK, nx, ny);
    T fac = mK / (SK - Ss);
    T ds = Ss - unK;
    T U0 = fac;
    T U1 = fac * (K.u + ds * nx);
    T U2 = fac * (K.v + ds * ny);
    T U3 = fac * (EK / K.r + ds * (Ss + K.p / mK));
    f[0] = FK[0] + SK * (U0 - K.r);
    f[1] = FK[1] + SK * (U1 - K.r * K.u);
    f[2] = FK[2] + SK * (U2 - K.r * K.v);
    f[3] = FK[3] + SK * (U3 - EK);
}

// Roe flux (Roe 1981) in the face-normal frame with the Harten-Hyman entropy fix
// on the acoustic waves: delta = max(0, lam~ - lam_L, lam_R - lam~), |lam~| -> delta
// where |lam~| < delta. Roe averages as in roe_orig (src/global.cpp:407-441).
template <typename T>
__device__ __forceinline__ void flux_roe(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM) {
    T G1 = GAM - T(1.0);
    T unL = L.u * nx + L.v * ny, unR = R.u * nx + R.v * ny;
    T EL = L.p / G1 + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    T ER = R.p / G1 + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    T HL = (EL + L.p) / L.r, HR = (ER + R.p) / R.r;
    T sL = t_sqrt(L.r), sR = t_sqrt(R.r);
    T w = T(1.0) / (sL + sR);
    T ut = (sL * L.u + sR * R.u) * w;
    T vt = (sL * L.v + sR * R.v) * w;
    T Ht = (sL * HL + sR * HR) * w;
    T q2 = ut * ut + vt * vt;
    T c2 = G1 * (Ht - T(0.5) * q2);
    T c = t_sqrt(c2);
    T unt = ut * nx + vt * ny;
    T rt = sL * sR;
    T dr = R.r - L.r, dp = R.p - L.p, dun = unR - unL;
    T dtx = (R.u - L.u) - dun * nx, dty = (R.v - L.v) - dun * ny;
    T a1 = (dp - rt * c * dun) / (T(2.0) * c2);
    T a2 = dr - dp / c2;
    T a4 = (dp + rt * c * dun) / (T(2.0) * c2);
    T l1 = unt - c, l4 = unt + c;
    T cL = t_sqrt(GAM * L.p / L.r), cR = t_sqrt(GAM * R.p / R.r);
    T d1 = t_max(T(0.0), t_max(l1 - (unL - cL), (unR - cR) - l1));
    T d4 = t_max(T(0.0), t_max(l4 - (unL + cL), (unR + cR) - l4));
    T al1 = t_abs(l1); if (al1 < d1) al1 = d1;
    T al4 = t_abs(l4); if (al4 < d4) al4 = d4;
    T al2 = t_abs(unt);
    T w1 = al1 * a1, w2 = al2 * a2, w4 = al4 * a4, ws = al2 * rt;
    T D0 = w1 + w2 + w4;
    T D1 = w1 * (ut - c * nx) + (w2 * ut + ws * dtx) + w4 * (ut + c * nx);
    T D2 = w1 * (vt - c * ny) + (w2 * vt + ws * dty) + w4 * (vt + c * ny);
    T D3 = w1 * (Ht - unt * c) + (w2 * (T(0.5) * q2) + ws * (ut * dtx + vt * dty)) + w4 * (Ht + unt * c);
    T FL[4], FR[4];
    phys_flux(FL, L.r, L.u, L.v, L.p, EL, unL, nx, ny);
    phys_flux(FR, R.r, R.u, R.v, R.p, ER, unR, nx, ny);
    f[0] = T(0.5) * (FL[0] + FR[0] - D0);
    f[1] = T(0.5) * (FL[1] + FR[1] - D1);
    f[2] = T(0.5) * (FL[2] + FR[2] - D2);
    f[3] = T(0.5) * (FL[3] + FR[3] - D3);
}

template <typename T, int FLUX>
__device__ __forceinline__ bool num_flux(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, int cap) {
    if (FLUX == FLUX_LAX) { flux_lax(f, L, R, nx, ny, GAM); return false; }
    if (FLUX == FLUX_ROE) { flux_roe(f, L, R, nx, ny, GAM); return false; }
    if (FLUX == FLUX_HLLC) { flux_hllc(f, L, R, nx, ny, GAM); return false; }
    return flux_godunov(f, L, R, nx, ny, GAM, cap);
}

// ------------------------------------------------------------------ kernels

// Green-Gauss gradients of r, p, u, v (calcGrad, src/methods/fvm_tvd.cpp:242-301),
// gathered per cell over its faces in ascending original edge order.
template <typename T>
__global__ void __launch_bounds__(256) k_grad(const DevCase c) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const T* __restrict__ W = W_of<T>(c);
    const Prim<T> q = load_prim(W, nc, i);
    T g0 = T(0.0), g1 = T(0.0), g2 = T(0.0), g3 = T(0.0), g4 = T(0.0), g5 = T(0.0), g6 = T(0.0), g7 = T(0.0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const int e = f >> 1;
        const bool side2 = f & 1;
        const T nx = NX_of<T>(c)[e], ny = NY_of<T>(c)[e], l = L_of<T>(c)[e];
        Prim<T> o;
        const int j = side2 ? c.ec1[e] : c.ec2[e];
        if (j >= 0) {
            o = load_prim(W, nc, j);
        } else {
            const DevMat mt = mat_of(c, i);
            const T Tc = temperature(q, T(mt.gm1), T(mt.Cv));
            o = ghost_state(c.bnds[c.ebnd[e]], q, Tc, nx, ny, T(mt.M));
        }
        const T hr = (q.r + o.r) / T(2), hp = (q.p + o.p) / T(2);
        const T hu = (q.u + o.u) / T(2), hv = (q.v + o.v) / T(2);
        const T ax = hr * nx * l, ay = hr * ny * l, bx = hp * nx * l, by = hp * ny * l;
        const T cx = hu * nx * l, cy = hu * ny * l, dx = hv * nx * l, dy = hv * ny * l;
        if (side2) {
            g0 = g0 - ax; g1 = g1 - ay; g2 = g2 - bx; g3 = g3 - by;
            g4 = g4 - cx; g5 = g5 - cy; g6 = g6 - dx; g7 = g7 - dy;
        } else {
            g0 = g0 + ax; g1 = g1 + ay; g2 = g2 + bx; g3 = g3 + by;
            g4 = g4 + cx; g5 = g5 + cy; g6 = g6 + dx; g7 = g7 + dy;
        }
    }
    const T s = T(c.S[i]);
    T* __restrict__ G = G_of<T>(c);
    G[i] = g0 / s; G[nc + i] = g1 / s; G[2 * nc + i] = g2 / s; G[3 * nc + i] = g3 / s;
    G[4 * nc + i] = g4 / s; G[5 * nc + i] = g5 / s; G[6 * nc + i] = g6 / s; G[7 * nc + i] = g7 / s;
}

template <typename T, int RECON>
__device__ __forceinline__ void reconstruct(Prim<T>& q, const T* g, T dx, T dy, const Prim<T>& nb) {
    T dr = g[0] * dx + g[1] * dy;
    T dp = g[2] * dx + g[3] * dy;
    T du = g[4] * dx + g[5] * dy;
    T dv = g[6] * dx + g[7] * dy;
    if (RECON == RECON_MINMOD) {
        dr = minmod(dr, nb.r - q.r);
        dp = minmod(dp, nb.p - q.p);
        du = minmod(du, nb.u - q.u);
        dv = minmod(dv, nb.v - q.v);
    }
    q.r += dr; q.p += dp; q.u += du; q.v += dv;
}

// Edge flux over the edge's two Gauss points, times l/2 (src/methods/fvm_tvd.cpp:329-352).
template <typename T, int FLUX, int RECON>
__global__ void __launch_bounds__(256) k_flux(const DevCase c) {
    const int ne = c.ne, nc = c.nc;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const T* __restrict__ W = W_of<T>(c);
    const T* __restrict__ G = G_of<T>(c);
    const T* __restrict__ DL = DL_of<T>(c);
    const T nx = NX_of<T>(c)[e], ny = NY_of<T>(c)[e], l = L_of<T>(c)[e];
    const T GAM = T(c.gam_flux);
    const int c1 = c.ec1[e];
    const bool inner = e < c.n_int;
    const Prim<T> qL = load_prim(W, nc, c1);
    T gL[8], gR[8];
    if (RECON != RECON_NONE)
#pragma unroll
        for (int k = 0; k < 8; k++) gL[k] = G[k * nc + c1];
    Prim<T> qR = qL, gc = qL;
    DevBnd b{};
    T Tc = T(0), M = T(0);
    if (inner) {
        const int c2 = c.ec2[e];
        qR = load_prim(W, nc, c2);
        if (RECON != RECON_NONE)
#pragma unroll
            for (int k = 0; k < 8; k++) gR[k] = G[k * nc + c2];
    } else {
        b = c.bnds[c.ebnd[e]];
        const DevMat mt = mat_of(c, c1);
        Tc = temperature(qL, T(mt.gm1), T(mt.Cv));
        M = T(mt.M);
        if (RECON == RECON_MINMOD) gc = ghost_state(b, qL, Tc, nx, ny, M);
    }
    T fs[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
    bool hit = false;
#pragma unroll
    for (int gp = 0; gp < 2; gp++) {
        Prim<T> pL = qL, pR;
        if (RECON != RECON_NONE)
            reconstruct<T, RECON>(pL, gL, DL[(4 * gp) * ne + e], DL[(4 * gp + 1) * ne + e], inner ? qR : gc);
        if (inner) {
            pR = qR;
            if (RECON != RECON_NONE)
                reconstruct<T, RECON>(pR, gR, DL[(4 * gp + 2) * ne + e], DL[(4 * gp + 3) * ne + e], qL);
        } else {
            pR = ghost_state(b, pL, Tc, nx, ny, M);
        }
        T f[4];
        hit |= num_flux<T, FLUX>(f, pL, pR, nx, ny, GAM, c.newton_cap);
        fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
        if (RECON == RECON_NONE) {  // both Gauss points see the cell-centre states
            fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
            break;
        }
    }
    if (hit) atomicOr(c.err, ERRBIT_NEWTON_CAP);
    const T lh = l * T(0.5);
    T* __restrict__ F = F_of<T>(c);
    F[e] = fs[0] * lh; F[ne + e] = fs[1] * lh; F[2 * ne + e] = fs[2] * lh; F[3 * ne + e] = fs[3] * lh;
}

template <typename T>
__device__ __forceinline__ Prim<T> prim_face_of(double ro, double ru, double rv, double re, double gm1);
template <>
__device__ __forceinline__ Prim<double> prim_face_of<double>(double ro, double ru, double rv, double re, double gm1) {
    return cons2prim<double>(ro, ru, rv, re, gm1);
}
template <>
__device__ __forceinline__ Prim<float> prim_face_of<float>(double ro, double ru, double rv, double re, double gm1) {
    return cons2prim<float>(float(ro), float(ru), float(rv), float(re), float(gm1));
}

// local time step of one cell (calcTimeStep STEADY branch, src/methods/fvm_tvd.cpp:218-224)
__device__ __forceinline__ void local_dt(const DevCase& c, int i, const Prim<double>& q, const DevMat& mt) {
    double cz = sqrt(mt.gam * q.p / q.r);
    double t = c.cfl_number * c.S[i] / t_max(fabs(q.u) + cz, fabs(q.v) + cz);
    c.ctau_next[i] = t;
    c.cfl[i] = t / c.S[i];
}

__device__ __forceinline__ bool outside_limits(const DevCase& c, const Prim<double>& q) {  // :439-446
    return q.r < c.lim_rmin || q.r > c.lim_rmax || q.p < c.lim_pmin || q.p > c.lim_pmax ||
           fabs(q.u) > c.lim_umax || fabs(q.v) > c.lim_umax;
}

// One Runge-Kutta stage update with the residual gathered from the edge fluxes.
// SCHEME/STAGE: Euler (0), Heun (0,1; src/methods/fvm_tvd.cpp:366-447), SSP-RK3 Shu-Osher (0,1,2).
template <typename T, int SCHEME, int STAGE>
__global__ void __launch_bounds__(256) k_update(const DevCase c) {
    constexpr bool FINAL = (SCHEME == TIME_EULER && STAGE == 0) || (SCHEME == TIME_HEUN && STAGE == 1) ||
                           (SCHEME == TIME_SSPRK3 && STAGE == 2);
    const int nc = c.nc, ne = c.ne;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    if (STAGE == 0 && c.steady) c.ctau[i] = c.ctau_next[i];  // the step now running uses ctau_next
    if (c.flags[i] & 0x2u) {  // cellIsLim: no update; later stages read B
        if (STAGE == 0 && !FINAL)
#pragma unroll
            for (int k = 0; k < 4; k++) c.B[k * nc + i] = c.A[k * nc + i];
        if (FINAL) atomicAdd(c.n_lim, 1);
        return;
    }
    const T* __restrict__ F = F_of<T>(c);
    double R0 = 0.0, R1 = 0.0, R2 = 0.0, R3 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const int e = f >> 1;
        const double f0 = double(F[e]), f1 = double(F[ne + e]), f2 = double(F[2 * ne + e]), f3 = double(F[3 * ne + e]);
        if (f & 1) { R0 = R0 + f0; R1 = R1 + f1; R2 = R2 + f2; R3 = R3 + f3; }
        else { R0 = R0 - f0; R1 = R1 - f1; R2 = R2 - f2; R3 = R3 - f3; }
    }
    const double cf = c.cfl[i];
    const double* __restrict__ src = STAGE == 0 ? c.A : c.B;
    double u0 = src[i] + cf * R0, u1 = src[nc + i] + cf * R1, u2 = src[2 * nc + i] + cf * R2,
           u3 = src[3 * nc + i] + cf * R3;
    double* dst = FINAL ? c.A : c.B;
    if (SCHEME == TIME_HEUN && STAGE == 1) {
        u0 = 0.5 * (c.A[i] + u0); u1 = 0.5 * (c.A[nc + i] + u1);
        u2 = 0.5 * (c.A[2 * nc + i] + u2); u3 = 0.5 * (c.A[3 * nc + i] + u3);
    } else if (SCHEME == TIME_SSPRK3 && STAGE == 1) {
        u0 = 0.75 * c.A[i] + 0.25 * u0; u1 = 0.75 * c.A[nc + i] + 0.25 * u1;
        u2 = 0.75 * c.A[2 * nc + i] + 0.25 * u2; u3 = 0.75 * c.A[3 * nc + i] + 0.25 * u3;
    } else if (SCHEME == TIME_SSPRK3 && STAGE == 2) {
        const double c13 = 1.0 / 3.0, c23 = 2.0 / 3.0;
        u0 = c13 * c.A[i] + c23 * u0; u1 = c13 * c.A[nc + i] + c23 * u1;
        u2 = c13 * c.A[2 * nc + i] + c23 * u2; u3 = c13 * c.A[3 * nc + i] + c23 * u3;
    }
    dst[i] = u0; dst[nc + i] = u1; dst[2 * nc + i] = u2; dst[3 * nc + i] = u3;
    const DevMat mt = mat_of(c, i);
    if (FINAL) {
        const Prim<double> q = cons2prim<double>(u0, u1, u2, u3, mt.gm1);
        if (outside_limits(c, q)) {
            c.flags[i] |= 0x2u;
            atomicAdd(c.n_lim, 1);
        }
        if (!(q.r > 0.0) || !(q.p > 0.0)) atomicOr(c.err, ERRBIT_NONPHYSICAL);
        if (c.steady) local_dt(c, i, q, mt);
        Prim<T> w;
        w.r = T(q.r); w.u = T(q.u); w.v = T(q.v); w.p = T(q.p);
        store_prim(Wm_of<T>(c), nc, i, w);
    } else {
        store_prim(Wm_of<T>(c), nc, i, prim_face_of<T>(u0, u1, u2, u3, mt.gm1));
    }
}

// remediateLimCells, src/methods/fvm_tvd.cpp:464-499: flagged cells, in original
// cell order and one after another (each may read a neighbour remediated just
// before it), take the area-weighted mean of the c2 cells of their edges.
template <typename T>
__global__ void __launch_bounds__(1024) k_remediate(const DevCase c) {
    __shared__ int list[1024];
    __shared__ int cnt;
    const int nc = c.nc;
    if (*c.n_lim == 0) return;
    for (int base = 0; base < nc; base += blockDim.x) {
        const int o = base + threadIdx.x;
        const int i = o < nc ? c.iperm[o] : -1;
        const bool fl = o < nc && (c.flags[i] & 0x2u);
        const unsigned ball = __ballot_sync(0xffffffffu, fl);
        __shared__ int wsum[32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) wsum[warp] = __popc(ball);
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) { int t = wsum[w]; wsum[w] = s; s += t; }
            cnt = s;
        }
        __syncthreads();
        if (fl) list[wsum[warp] + __popc(ball & ((1u << lane) - 1u))] = i;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 0; k < cnt; k++) {
                const int ci = list[k];
                double S = 0.0, a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
                for (int q = 0; q < 3; q++) {
                    const int j = c.rem_nb[q * nc + ci];
                    if (j >= 0) {
                        const double s = c.S[j];
                        S += s;
                        a0 += c.A[j] * s; a1 += c.A[nc + j] * s; a2 += c.A[2 * nc + j] * s; a3 += c.A[3 * nc + j] * s;
                    }
                }
                const double u0 = a0 / S, u1 = a1 / S, u2 = a2 / S, u3 = a3 / S;
                c.A[ci] = u0; c.A[nc + ci] = u1; c.A[2 * nc + ci] = u2; c.A[3 * nc + ci] = u3;
                unsigned f = c.flags[ci] + 0x010000u;
                if (f & 0x200000u) f &= 0x001110u;
                c.flags[ci] = f;
                const DevMat mt = mat_of(c, ci);
                const Prim<double> q = cons2prim<double>(u0, u1, u2, u3, mt.gm1);
                if (c.steady) local_dt(c, ci, q, mt);
                Prim<T> w;
                w.r = T(q.r); w.u = T(q.u); w.v = T(q.v); w.p = T(q.p);
                store_prim(Wm_of<T>(c), nc, ci, w);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *c.n_lim = 0;
}

// Primitives of A for every cell (+ local time step when steady).
template <typename T>
__global__ void __launch_bounds__(256) k_prims(const DevCase c) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const DevMat mt = mat_of(c, i);
    const Prim<double> q = cons2prim<double>(c.A[i], c.A[nc + i], c.A[2 * nc + i], c.A[3 * nc + i], mt.gm1);
    if (c.steady) {
        local_dt(c, i, q, mt);
        c.ctau[i] = c.ctau_next[i];
    }
    Prim<T> w;
    w.r = T(q.r); w.u = T(q.u); w.v = T(q.v); w.p = T(q.p);
    store_prim(Wm_of<T>(c), nc, i, w);
}

// Residual of the current edge fluxes (the reference's *_int arrays) for every cell.
template <typename T>
__global__ void __launch_bounds__(256) k_residual(const DevCase c, double* __restrict__ R) {
    const int nc = c.nc, ne = c.ne;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const T* __restrict__ F = F_of<T>(c);
    double r[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const int e = f >> 1;
        for (int q = 0; q < 4; q++) {
            const double v = double(F[q * ne + e]);
            r[q] = (f & 1) ? r[q] + v : r[q] - v;
        }
    }
    for (int q = 0; q < 4; q++) R[q * nc + i] = r[q];
}

}  // namespace cfd2d
