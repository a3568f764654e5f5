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

#include <cmath>

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
__device__ __forceinline__ double t_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float t_fma(float a, float b, float c) { return fmaf(a, b, c); }
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
template <typename T> struct CellFaces { const T *nx, *ny, *l; };
template <typename T> __device__ __forceinline__ CellFaces<T> cf_of(const DevCase& c);
template <> __device__ __forceinline__ CellFaces<double> cf_of<double>(const DevCase& c) {
    return CellFaces<double>{c.cf_nx, c.cf_ny, c.cf_l};
}
template <typename T> __device__ __forceinline__ const T* DL_of(const DevCase& c);
template <> __device__ __forceinline__ const double* DL_of<double>(const DevCase& c) { return c.dl; }
template <> __device__ __forceinline__ const float* DL_of<float>(const DevCase& c) { return c.dl32; }

__device__ __forceinline__ DevMat mat_of(const DevCase& c, int cell) {
    return c.cmat ? c.mats[c.cmat[cell]] : c.mat0;
}

// Records gathered by index are stored as array-of-structures so a neighbour's
// data arrives in 16-byte vector loads: W (r, u, v, p) and F (4 fluxes) are one
// 4-vector per cell / edge, G (8 gradient components) two.
__device__ __forceinline__ void ld4(const float* __restrict__ p, int i, float* v) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p) + i);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double* __restrict__ p, int i, double* v) {
    const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
    const double2 a = __ldg(q), b = __ldg(q + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float* __restrict__ p, int i, float a0, float a1, float a2, float a3) {
    reinterpret_cast<float4*>(p)[i] = make_float4(a0, a1, a2, a3);
}
__device__ __forceinline__ void st4(double* __restrict__ p, int i, double a0, double a1, double a2, double a3) {
    double2* q = reinterpret_cast<double2*>(p) + 2 * (size_t)i;
    q[0] = make_double2(a0, a1);
    q[1] = make_double2(a2, a3);
}
template <typename T>
__device__ __forceinline__ void ld8(const T* __restrict__ p, int i, T* v) {
    ld4(p, 2 * i, v);
    ld4(p, 2 * i + 1, v + 4);
}
template <typename T>
__device__ __forceinline__ void st8(T* __restrict__ p, int i, const T* v) {
    st4(p, 2 * i, v[0], v[1], v[2], v[3]);
    st4(p, 2 * i + 1, v[4], v[5], v[6], v[7]);
}

// Per-item data a kernel reads once and no later kernel of the stage reads again (edge
// geometry, face lists) is loaded with the evict-first hint, so the L2 keeps the cell
// records the neighbour gathers hit.
template <typename T> __device__ __forceinline__ T ldcs(const T* p) { return __ldcs(p); }

template <typename T>
__device__ __forceinline__ Prim<T> load_prim(const T* __restrict__ W, int i) {
    T v[4];
    ld4(W, i, v);
    Prim<T> q;
    q.r = v[0]; q.u = v[1]; q.v = v[2]; q.p = v[3];
    return q;
}

template <typename T>
__device__ __forceinline__ void store_prim(T* __restrict__ W, int i, const Prim<T>& q) {
    st4(W, i, q.r, q.u, q.v, q.p);
}

// Material constants in the face precision (the mixed form keeps FP32 copies so
// its face kernels issue no FP64 instruction).
template <typename T> struct MatT { T M, Cv, gm1; };
template <typename T> __device__ __forceinline__ MatT<T> matT_of(const DevCase& c, int cell);
template <> __device__ __forceinline__ MatT<double> matT_of<double>(const DevCase& c, int cell) {
    const DevMat m = c.cmat ? c.mats[c.cmat[cell]] : c.mat0;
    return MatT<double>{m.M, m.Cv, m.gm1};
}
template <> __device__ __forceinline__ MatT<float> matT_of<float>(const DevCase& c, int cell) {
    if (!c.cmat) return MatT<float>{c.mat0_f[0], c.mat0_f[1], c.mat0_f[2]};
    const DevMat m = c.mats[c.cmat[cell]];
    return MatT<float>{float(m.M), float(m.Cv), float(m.gm1)};
}
template <typename T> __device__ __forceinline__ T gam_of(const DevCase& c);
template <> __device__ __forceinline__ double gam_of<double>(const DevCase& c) { return c.gam_flux; }
template <> __device__ __forceinline__ float gam_of<float>(const DevCase& c) { return c.gam_flux_f; }
template <typename T> __device__ __forceinline__ T ig1_of(const DevCase& c);
template <> __device__ __forceinline__ double ig1_of<double>(const DevCase& c) { return c.ig1_flux; }
template <> __device__ __forceinline__ float ig1_of<float>(const DevCase& c) { return c.ig1_flux_f; }

// a / b correctly rounded from y = RN(1/b): q = RN(a y), r = a - b q exactly
// (one FMA), result RN(q + r y) (Markstein, "IA-64 and Elementary Functions",
// 2000, the division theorem). Three FP64 instructions instead of a full
// division; the exponent guard keeps a, y and the quotient far from underflow
// and overflow, where the theorem needs no extra conditions. A zero dividend
// over a finite y (b nonzero, not NaN) gives the zero with the sign of a XOR b,
// built on the integer pipe (zero gradients and velocities are common). Other
// operands (subnormal, huge, inf, NaN, b zero) divide outright.
// The outright division sits in a function of its own so that the compiler
// branches to it instead of evaluating it beside the common path.
static __device__ __noinline__ double div_outright(double a, double b) { return a / b; }
__device__ __forceinline__ double div_rn(double a, double b, double y) {
    const long long ia = __double_as_longlong(a), iy = __double_as_longlong(y);
    const int ea = (int)((ia >> 52) & 0x7ff);
    const int ey = (int)((iy >> 52) & 0x7ff);
    const int eq = ea + ey - 1023;
    if (__builtin_expect(ea > 0x100 && ea < 0x700 && ey > 0x100 && ey < 0x700 && eq > 0x100 && eq < 0x700, 1)) {
        const double q = a * y;
        const double r = fma(-q, b, a);
        return fma(r, y, q);
    }
    if ((ia & 0x7fffffffffffffffll) == 0 && ey < 0x7ff)
        return __longlong_as_double((ia ^ iy) & (long long)0x8000000000000000ull);
    return div_outright(a, b);
}
// -x when s, else x: a sign-bit flip on the integer pipe (x - y is x + (-y) in IEEE).
__device__ __forceinline__ double neg_if(double x, bool s) {
    return __hiloint2double(__double2hiint(x) ^ (s ? (int)0x80000000 : 0), __double2loint(x));
}
__device__ __forceinline__ float neg_if(float x, bool s) { return __int_as_float(__float_as_int(x) ^ (s ? (int)0x80000000 : 0)); }
// a / b given y = RN(1/b): the correctly rounded quotient in FP64, a * y in the FP32 faces.
__device__ __forceinline__ double div_by(double a, double b, double y) { return div_rn(a, b, y); }
__device__ __forceinline__ float div_by(float a, float, float y) { return a * y; }

// FP32 <-> FP64 conversions on the integer pipe. GB300's FP64 unit issues ~2
// instructions per clock and SM, and the hardware conversions run there; these
// bit-level versions keep the mixed form's update kernel off that unit.
// Widening is exact for zero, normal, infinite and NaN floats (the mixed kernels
// run with FTZ, so no subnormal float reaches it; one would read as zero).
__device__ __forceinline__ double widen(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned ex = (b >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(b & 0x80000000u) << 32;
    if (ex == 0) return __longlong_as_double((long long)sgn);
    const unsigned long long e64 = ex == 0xffu ? 0x7ffull : (unsigned long long)(ex + (1023 - 127));
    return __longlong_as_double((long long)(sgn | (e64 << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// Narrowing rounds to nearest (ties away from zero), flushes below FLT_MIN to
// zero, saturates to infinity and keeps NaN a NaN.
__device__ __forceinline__ float narrow(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffull);
    if (e == 0x7ff) return __uint_as_float(sgn | ((b & 0xfffffffffffffull) ? 0x7fc00000u : 0x7f800000u));
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sgn);
    if (ef >= 0xff) return __uint_as_float(sgn | 0x7f800000u);
    const unsigned m = (unsigned)(b >> 29) & 0x7fffffu;
    const unsigned rnd = (unsigned)(b >> 28) & 1u;
    return __uint_as_float((sgn | ((unsigned)ef << 23) | m) + rnd);  // a carry moves into the exponent
}

// convertConsToPar + Material::URS(0), src/methods/fvm_tvd.cpp:803-813, src/global.cpp:15-18
template <typename T>
__device__ __forceinline__ Prim<T> cons2prim(T ro, T ru, T rv, T re, T gm1) {
    Prim<T> q;
    q.r = ro;
    T E;
    if constexpr (sizeof(T) == 8) {  // the three quotients by ro share one reciprocal
        const double y = 1.0 / ro;
        q.u = div_rn(ru, ro, y);
        q.v = div_rn(rv, ro, y);
        E = div_rn(re, ro, y);
    } else {
        q.u = ru / ro;
        q.v = rv / ro;
        E = re / ro;
    }
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

// MINMOD, src/methods/LimiterDGCockburn.cpp:110-123: a*b > 0 ? (|a| < |b| ? a : b) : 0,
// split into its two decisions so that the adjoint takes exactly the forward's branch.
// mm_pos is the test a*b > 0. On the integer pipe: a zero operand gives a product of
// +-0 or NaN (0 * inf), never > 0; for normal or infinite operands of one sign whose
// exponent fields sum to at least 972, |a b| >= 2^(ea+eb-2046) >= 2^-1074, so the
// rounded product is > 0 (or +inf); NaN or opposite signs fail the test. Subnormal
// operands and products near the underflow threshold take the FP64 multiply and read
// the sign of its bits (positive, non-NaN doubles are exactly the patterns in
// (0, 0x7ff0...0]). mm_first is |a| < |b| on magnitude bits, which orders non-NaN
// values like fabs does. Bit for bit the reference's result.
static __device__ __noinline__ double mul_outright(double a, double b) { return a * b; }
__device__ __forceinline__ bool mm_pos(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7fffffffffffffffll, mb = ib & 0x7fffffffffffffffll;
    if (ma == 0 || mb == 0) return false;
    const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
    if (__builtin_expect(ea >= 1 && eb >= 1 && ea + eb >= 972, 1))
        return (ia ^ ib) >= 0 && ma <= 0x7ff0000000000000ll && mb <= 0x7ff0000000000000ll;
    const long long pb = __double_as_longlong(mul_outright(a, b));  // a branch, not a predicated multiply
    return pb > 0 && pb <= 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool mm_first(double a, double b) {
    return (__double_as_longlong(a) & 0x7fffffffffffffffll) < (__double_as_longlong(b) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ bool mm_pos(float a, float b) {
    const int pb = __float_as_int(a * b);
    return pb > 0 && pb <= 0x7f800000;
}
__device__ __forceinline__ bool mm_first(float a, float b) {
    return (__float_as_int(a) & 0x7fffffff) < (__float_as_int(b) & 0x7fffffff);
}
template <typename T>
__device__ __forceinline__ T minmod(T a, T b) {
    return mm_pos(a, b) ? (mm_first(a, b) ? a : b) : T(0.0);
}

// ------------------------------------------------------------------ fluxes

// a / b: from y = RN(1/b) when RECIP (correctly rounded, the same bits as '/', div_rn),
// else '/' itself; the FP32 faces always divide outright
template <bool RECIP>
__device__ __forceinline__ double div_x(double a, double b, double y) { return RECIP ? div_rn(a, b, y) : a / b; }
template <bool RECIP>
__device__ __forceinline__ float div_x(float a, float b, float) { return a / b; }

// Exact Riemann solver rim_orig (src/global.cpp:232-405), structured, with a cap
// on its Newton loop (the reference has none and can spin forever). With RECIP the
// quotients by the side densities (yRB, yRE = their reciprocals), by the side pressures
// and by the gas constants go through div_rn: the same bits, a third of the FP64 work of
// a division each.
template <typename T, bool RECIP = false>
__device__ __forceinline__ bool riemann_exact(T& RI, T& EI, T& PI, T& UI, T& VI, T RB, T PB, T UB, T VB, T RE,
                                              T PE, T UE, T VE, const RimGas<T>& g, int cap, T yRB = T(0),
                                              T yRE = T(0)) {
    const T GAM = g.GAM, AGAM = g.AGAM, DGAM = g.DGAM, GGAM = g.GGAM, HGAM = g.HGAM, FGAM = g.FGAM;
    const T OGAM = g.OGAM, QGAM = g.QGAM, PGAM = g.PGAM, RGAM = g.RGAM, SGAM = g.SGAM, TGAM = g.TGAM;
    T US = T(0.0), UF = T(0.0);
    T RF, RS, EF, ES, SBL, SFL, SSL, SEL, D, P;
    const T eps = T(1.0e-5);
    T CB = t_sqrt(div_x<RECIP>(GAM * PB, RB, yRB));
    T CE = t_sqrt(div_x<RECIP>(GAM * PE, RE, yRE));
    T EB = div_x<RECIP>(CB * CB, SGAM, g.iSGAM);
    T EE = div_x<RECIP>(CE * CE, SGAM, g.iSGAM);
    T RCB = RB * CB;
    T RCE = RE * CE;
    T DU = UB - UE;
    bool hit = false;
    if (DU < div_x<RECIP>(T(-2.0) * (CB + CE), AGAM, g.iAGAM)) {  // vacuum
        RF = T(0.0); RS = T(0.0); EF = T(0.0); ES = T(0.0);
        SBL = UB - CB;
        SFL = UB + div_x<RECIP>(T(2.0) * CB, AGAM, g.iAGAM);
        SSL = UE - div_x<RECIP>(T(2.0) * CE, AGAM, g.iAGAM);
        SEL = UE + CE;
    } else {
        P = (PB * RCE + PE * RCB + DU * RCB * RCE) / (RCB + RCE);
        const T yPB = RECIP ? T(1) / PB : T(0), yPE = RECIP ? T(1) / PE : T(0);
        int it = 0;
        for (;;) {
            T F1, FS1, F2, FS2;
            if (P < eps) P = eps;
            T PPB = div_x<RECIP>(P, PB, yPB);
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
            T PPE = div_x<RECIP>(P, PE, yPE);
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
        // the reference forms ZFB and ZFE here for both sides; each is read only on its
        // rarefaction branch, so it is formed there (same value, no exp/log for a shock)
        if (!(PB > P)) {
            D = UB - t_sqrt(div_x<RECIP>(TGAM * P + HGAM * PB, RB, yRB));
            T UBD = UB - D, RUBD = RB * UBD;
            RF = RUBD * RUBD / (PB - P + RUBD * UBD);
            UF = D + RUBD / RF;
            EF = P / (AGAM * RF);
            SBL = D; SFL = D;
        } else {
            const T ZFB = CB * t_exp(t_log(div_x<RECIP>(P, PB, yPB)) * OGAM);
            EF = div_x<RECIP>(ZFB * ZFB, SGAM, g.iSGAM);
            UF = UB + DGAM * (CB - ZFB);
            RF = P / (AGAM * EF);
            SBL = UB - CB;
            SFL = UF - ZFB;
        }
        if (!(PE > P)) {
            D = UE + t_sqrt(div_x<RECIP>(TGAM * P + HGAM * PE, RE, yRE));
            T UED = UE - D, RUED = RE * UED;
            RS = RUED * RUED / (PE - P + RUED * UED);
            US = D + RUED / RS;
            ES = P / (AGAM * RS);
            SEL = D; SSL = D;
        } else {
            const T ZFE = CE * t_exp(t_log(div_x<RECIP>(P, PE, yPE)) * OGAM);
            ES = div_x<RECIP>(ZFE * ZFE, SGAM, g.iSGAM);
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
        UI = div_x<RECIP>(UB + DGAM * GGAM * t_sqrt(EB), T(1) + DGAM, g.i1DGAM);
        VI = VB;
        EI = div_x<RECIP>(UI * UI, SGAM, g.iSGAM);
        RI = RB * t_exp(t_log(EI / EB) * g.eAGAM);
    } else {
        UI = div_x<RECIP>(UE - DGAM * GGAM * t_sqrt(EE), T(1) + DGAM, g.i1DGAM);
        VI = VE;
        EI = div_x<RECIP>(UI * UI, SGAM, g.iSGAM);
        RI = RE * t_exp(t_log(EI / EE) * g.eAGAM);
    }
    PI = AGAM * EI * RI;
    return hit;
}

// Godunov flux, FVM_TVD::calcFlux, src/methods/fvm_tvd.cpp:602-622 (FEM_RKDG's, :918-937, is
// the same). With RECIP: a fixed gas and the side densities' reciprocals yL, yR.
template <typename T, bool RECIP = false>
__device__ __forceinline__ bool flux_godunov(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny,
                                             const RimGas<T>& g, int cap, T yL = T(0), T yR = T(0)) {
    T RI, EI, PI, UN, UT;
    T unl = L.u * nx + L.v * ny;
    T unr = R.u * nx + R.v * ny;
    T utl = L.u * ny - L.v * nx;
    T utr = R.u * ny - R.v * nx;
    bool hit = riemann_exact<T, RECIP>(RI, EI, PI, UN, UT, L.r, L.p, unl, utl, R.r, R.p, unr, utr, g, cap, yL, yR);
    T UI = UN * nx + UT * ny;
    T VI = UN * ny - UT * nx;
    f[0] = RI * UN;
    f[1] = f[0] * UI + PI * nx;
    f[2] = f[0] * VI + PI * ny;
    f[3] = (RI * (EI + T(0.5) * (UI * UI + VI * VI)) + PI) * UN;
    return hit;
}

template <typename T>
__device__ __forceinline__ bool flux_godunov(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, int cap) {
    return flux_godunov<T, false>(f, L, R, nx, ny, rim_gas<T>(GAM), cap);
}

// Lax-Friedrichs (Rusanov), the reference's template src/methods/fvm_tvd_implicit.cpp:939-960
// (FEM_RKDG's, :938-958, is the same). With RECIP the quotients by the densities use their
// reciprocals yL, yR (div_rn: the same bits).
template <typename T, bool RECIP = false>
__device__ __forceinline__ void flux_lax(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1,
                                         T yL = T(0), T yR = T(0)) {
    T unl = L.u * nx + L.v * ny;
    T unr = R.u * nx + R.v * ny;
    T alpha = t_max(t_abs(unl) + t_sqrt(div_x<RECIP>(GAM * L.p, L.r, yL)),
                    t_abs(unr) + t_sqrt(div_x<RECIP>(GAM * R.p, R.r, yR)));
    T rol = L.r, rul = L.r * L.u, rvl = L.r * L.v;
    T rel = div_by(L.p, GAM - T(1.0), IG1) + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    T ror = R.r, rur = R.r * R.u, rvr = R.r * R.v;
    T rer = div_by(R.p, GAM - T(1.0), IG1) + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    T frl = rol * unl, frr = ror * unr;
    f[0] = T(0.5) * (frr + frl - alpha * (ror - rol));
    f[1] = T(0.5) * (frr * R.u + frl * L.u + (R.p + L.p) * nx - alpha * (rur - rul));
    f[2] = T(0.5) * (frr * R.v + frl * L.v + (R.p + L.p) * ny - alpha * (rvr - rvl));
    f[3] = T(0.5) * ((rer + R.p) * unr + (rel + L.p) * unl - alpha * (rer - rel));
}

// The fluxes below (HLLC, Roe, the minmod increment) have no counterpart in the
// reference; their multiply-adds are fused, exactly as the oracle defines them.
template <typename T>
__device__ __forceinline__ void phys_flux(T* f, T r, T u, T v, T p, T E, T un, T nx, T ny) {
    T m = r * un;
    f[0] = m;
    f[1] = t_fma(m, u, p * nx);
    f[2] = t_fma(m, v, p * ny);
    f[3] = (E + p) * un;
}
template <typename T> __device__ __forceinline__ T dot2(T a, T x, T b, T y) { return t_fma(a, x, b * y); }
template <typename T> __device__ __forceinline__ T energy(T r, T u, T v, T p, T IG1) {
    return t_fma(p, IG1, (T(0.5) * r) * t_fma(u, u, v * v));
}

// Newton-refined quotient, reciprocal and sound speed of the FP64 HLLC flux. HLLC has no
// counterpart in the reference, so its arithmetic is this project's definition and the
// oracle performs the very same operations (same bits): a binary32 seed, then FP64 Newton
// steps with fused multiply-adds (Newton-Raphson for 1/b and for sqrt(a/r), the final
// quotient corrected as in Markstein, "IA-64 and Elementary Functions", 2000). The seed
// is x truncated to binary32 (sign, rebiased exponent, top 23 fraction bits: integer
// operations) and the binary32 operations are correctly rounded (IEEE), so every step is
// defined bit for bit. Within |x| in [2^-60, 2^60) every binary32 value stays normal and
// every result is within about one ulp of the exact one; other operands take the IEEE
// expression. Each costs 4-6 FP64 instructions where a division or square root costs ~9.
__device__ __forceinline__ bool hllc_in_range(double x) {  // 2^-60 <= |x| < 2^60
    const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
    return e >= 1023 - 60 && e < 1023 + 60;
}
__device__ __forceinline__ float hllc_seed(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned ex = (unsigned)((b >> 52) & 0x7ff) - (1023u - 127u);
    return __uint_as_float(sgn | (ex << 23) | ((unsigned)(b >> 29) & 0x7fffffu));
}
// 1/b to ~2^-46 (one Newton step from the binary32 reciprocal of the seed)
__device__ __forceinline__ double hllc_rcp1(double b) {
    const double y0 = widen(__frcp_rn(hllc_seed(b)));
    return fma(y0, fma(-b, y0, 1.0), y0);
}
// a / b: one Newton step for 1/b, then q = a y corrected once (|a|, |b| in range; a = 0
// gives the IEEE signed zero)
// (the IEEE fallbacks sit in functions of their own so that the compiler branches to them
// instead of issuing them, predicated off, beside the common path)
static __device__ __noinline__ double recip_outright(double b) { return 1.0 / b; }
static __device__ __noinline__ double sound_outright(double a, double r) { return sqrt(a / r); }
__device__ __forceinline__ double hllc_quot(double a, double b) {
    if (hllc_in_range(b)) {
        if (__builtin_expect(hllc_in_range(a), 1)) {
            const double y = hllc_rcp1(b);
            const double q = a * y;
            return fma(fma(-q, b, a), y, q);
        }
        const long long ia = __double_as_longlong(a);
        if ((ia & 0x7fffffffffffffffll) == 0)
            return __longlong_as_double((ia ^ __double_as_longlong(b)) & (long long)0x8000000000000000ull);
    }
    return div_outright(a, b);
}
__device__ __forceinline__ float hllc_quot(float a, float b) { return a / b; }
// 1/b: two Newton steps
__device__ __forceinline__ double hllc_recip(double b) {
    if (__builtin_expect(!hllc_in_range(b), 0)) return recip_outright(b);
    const double y = hllc_rcp1(b);
    return fma(y, fma(-b, y, 1.0), y);
}
__device__ __forceinline__ float hllc_recip(float b) { return 1.0f / b; }
// sqrt(a / r) for a = GAMMA p, r the density (both positive and in range): s0 and
// h = 1/(2 r s0) from binary32, then two steps s <- s + (a - (r s) s) h
__device__ __forceinline__ double hllc_sound(double a, double r) {
    const long long ia = __double_as_longlong(a), ir = __double_as_longlong(r);
    if (__builtin_expect(ia < 0 || ir < 0 || !hllc_in_range(a) || !hllc_in_range(r), 0)) return sound_outright(a, r);
    const float af = hllc_seed(a), rf = hllc_seed(r);
    const float sf = __fsqrt_rn(__fdiv_rn(af, rf));
    const double h = widen(__fdiv_rn(0.5f, __fmul_rn(rf, sf)));
    double s = widen(sf);
    s = fma(fma(-(r * s), s, a), h, s);
    s = fma(fma(-(r * s), s, a), h, s);
    return s;
}
__device__ __forceinline__ float hllc_sound(float a, float r) { return t_sqrt(a / r); }

// HLLC (Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, sec. 10.4-10.6),
// Davis wave speeds S_L = min(unL-cL, unR-cR), S_R = max(unL+cL, unR+cR), star flux
// F*_K = [S*(S_K U_K - F_K) + S_K p* D*] / (S_K - S*), D* = (0, nx, ny, S*),
// p* = p_K + rho_K (S_K - un_K)(S* - un_K): one division instead of Toro's star state;
// S_K U_K - F_K is formed from m_K = rho_K (S_K - un_K) and only the side that is used
// forms its energy. FP64: c = hllc_sound(GAMMA p, rho), S* = hllc_quot,
// 1/(S_K - S*) = hllc_recip.
// FP32 faces (the mixed form): both energies up front and the star flux from the physical
// flux F_K; without branches on the energies this measured faster there (124 against
// 151 us per flux launch at 2.1M triangles).
__device__ __forceinline__ void flux_hllc_c(float* f, const Prim<float>& L, const Prim<float>& R, float cL, float cR,
                                            float nx, float ny, float IG1) {
    float unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    float EL = energy(L.r, L.u, L.v, L.p, IG1);
    float ER = energy(R.r, R.u, R.v, R.p, IG1);
    float SL = t_min(unL - cL, unR - cR), SR = t_max(unL + cL, unR + cR);
    if (SL >= 0.0f) { phys_flux(f, L.r, L.u, L.v, L.p, EL, unL, nx, ny); return; }
    if (SR <= 0.0f) { phys_flux(f, R.r, R.u, R.v, R.p, ER, unR, nx, ny); return; }
    float mL = L.r * (SL - unL), mR = R.r * (SR - unR);
    float Ss = hllc_quot(t_fma(-mR, unR, t_fma(mL, unL, R.p - L.p)), mL - mR);
    const bool left = Ss >= 0.0f;
    const Prim<float>& K = left ? L : R;
    float SK = left ? SL : SR, unK = left ? unL : unR, EK = left ? EL : ER, mK = left ? mL : mR;
    float FK[4];
    phys_flux(FK, K.r, K.u, K.v, K.p, EK, unK, nx, ny);
    float ps = t_fma(mK, Ss - unK, K.p);
    float inv = hllc_recip(SK - Ss);
    float sp = SK * ps;
    f[0] = (Ss * t_fma(SK, K.r, -FK[0])) * inv;
    f[1] = t_fma(Ss, t_fma(SK, K.r * K.u, -FK[1]), sp * nx) * inv;
    f[2] = t_fma(Ss, t_fma(SK, K.r * K.v, -FK[2]), sp * ny) * inv;
    f[3] = t_fma(Ss, t_fma(SK, EK, -FK[3]), sp * Ss) * inv;
}
// FP64 faces: S_K U_K - F_K from m_K, the used side's energy only (fewer FP64 instructions,
// the FP64 unit being the bound there)
template <typename T>
__device__ __forceinline__ void flux_hllc_c(T* f, const Prim<T>& L, const Prim<T>& R, T cL, T cR, T nx, T ny, T IG1) {
    T unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    T SL = t_min(unL - cL, unR - cR), SR = t_max(unL + cL, unR + cR);
    if (SL >= T(0.0)) { phys_flux(f, L.r, L.u, L.v, L.p, energy(L.r, L.u, L.v, L.p, IG1), unL, nx, ny); return; }
    if (SR <= T(0.0)) { phys_flux(f, R.r, R.u, R.v, R.p, energy(R.r, R.u, R.v, R.p, IG1), unR, nx, ny); return; }
    T dL = SL - unL, dR = SR - unR;
    T mL = L.r * dL, mR = R.r * dR;
    T Ss = hllc_quot(t_fma(-mR, unR, t_fma(mL, unL, R.p - L.p)), mL - mR);
    const bool left = Ss >= T(0.0);
    const Prim<T>& K = left ? L : R;
    T SK = left ? SL : SR, unK = left ? unL : unR, dK = left ? dL : dR, mK = left ? mL : mR;
    T EK = energy(K.r, K.u, K.v, K.p, IG1);
    // S_K U_K - F_K = (m_K, m_K u - p nx, m_K v - p ny, E_K (S_K - un_K) - p un_K)
    T A1 = t_fma(mK, K.u, -(K.p * nx)), A2 = t_fma(mK, K.v, -(K.p * ny)), A3 = t_fma(EK, dK, -(K.p * unK));
    T ps = t_fma(mK, Ss - unK, K.p);
    T inv = hllc_recip(SK - Ss);
    T sp = SK * ps;
    f[0] = (Ss * mK) * inv;
    f[1] = t_fma(Ss, A1, sp * nx) * inv;
    f[2] = t_fma(Ss, A2, sp * ny) * inv;
    f[3] = t_fma(Ss, A3, sp * Ss) * inv;
}
template <typename T>
__device__ __forceinline__ void flux_hllc(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1) {
    const T cL = hllc_sound(GAM * L.p, L.r), cR = hllc_sound(GAM * R.p, R.r);
    flux_hllc_c(f, L, R, cL, cR, nx, ny, IG1);
}

// Roe flux (Roe 1981) in the face-normal frame with the Harten-Hyman entropy fix
// on the acoustic waves: delta = max(0, lam~ - lam_L, lam_R - lam~), |lam~| -> delta
// where |lam~| < delta. Roe averages as in roe_orig (src/global.cpp:407-441). FP32 faces
// (the mixed form); the FP64 faces' arithmetic is the overload below.
template <typename T>
__device__ __forceinline__ void flux_roe(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1) {
    T G1 = GAM - T(1.0);
    T unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    T EL = energy(L.r, L.u, L.v, L.p, IG1);
    T ER = energy(R.r, R.u, R.v, R.p, IG1);
    const T yL = T(1.0) / L.r, yR = T(1.0) / R.r;  // each shared by two quotients below
    T HL = div_by(EL + L.p, L.r, yL), HR = div_by(ER + R.p, R.r, yR);
    T sL = t_sqrt(L.r), sR = t_sqrt(R.r);
    T w = T(1.0) / (sL + sR);
    T ut = (sL * L.u + sR * R.u) * w;
    T vt = (sL * L.v + sR * R.v) * w;
    T Ht = (sL * HL + sR * HR) * w;
    T q2 = ut * ut + vt * vt;
    T c2 = G1 * (Ht - T(0.5) * q2);
    T c = t_sqrt(c2);
    T ic2 = T(1.0) / c2;
    T unt = ut * nx + vt * ny;
    T rt = sL * sR;
    T dr = R.r - L.r, dp = R.p - L.p, dun = unR - unL;
    T dtx = (R.u - L.u) - dun * nx, dty = (R.v - L.v) - dun * ny;
    T a1 = (dp - rt * c * dun) * (T(0.5) * ic2);
    T a2 = dr - dp * ic2;
    T a4 = (dp + rt * c * dun) * (T(0.5) * ic2);
    T l1 = unt - c, l4 = unt + c;
    T cL = t_sqrt(div_by(GAM * L.p, L.r, yL)), cR = t_sqrt(div_by(GAM * R.p, R.r, yR));
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

// 1/sqrt(x) for x > 0 in [2^-60, 2^60): t = RN32(1 / RN32(sqrt(x truncated to binary32))),
// then two Newton steps t <- t + (t/2)(1 - x t t); other operands: IEEE
static __device__ __noinline__ double rsqrt_outright(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ double roe_rsqrt(double x) {
    if (__builtin_expect(__double_as_longlong(x) <= 0 || !hllc_in_range(x), 0)) return rsqrt_outright(x);
    double t = widen(__fdiv_rn(1.0f, __fsqrt_rn(hllc_seed(x))));
    t = fma(0.5 * t, fma(-(x * t), t, 1.0), t);
    t = fma(0.5 * t, fma(-(x * t), t, 1.0), t);
    return t;
}
static __device__ __noinline__ double sqrt_outright(double x) { return sqrt(x); }

// The Roe flux with FP64 faces, this project's arithmetic (the oracle's flux_roe does the
// same): the Roe averages from t = 1/sqrt(rho) (sqrt(rho) = rho t, sqrt(rho) H = (E + p) t),
// c~ = c~^2 t~ and 1/c~^2 = t~^2 with t~ = 1/sqrt(c~^2), the side sound speeds as HLLC's,
// 1/(sqrt(rho_L) + sqrt(rho_R)) Newton-refined, and the wave sums fused.
__device__ __forceinline__ void flux_roe(double* f, const Prim<double>& L, const Prim<double>& R, double nx,
                                         double ny, double GAM, double IG1) {
    const double G1 = GAM - 1.0;
    const double unL = dot2(L.u, nx, L.v, ny), unR = dot2(R.u, nx, R.v, ny);
    const double EL = energy(L.r, L.u, L.v, L.p, IG1), ER = energy(R.r, R.u, R.v, R.p, IG1);
    const double tL = roe_rsqrt(L.r), tR = roe_rsqrt(R.r);
    const double sL = L.r * tL, sR = R.r * tR;
    const double w = hllc_recip(sL + sR);
    const double ut = fma(sL, L.u, sR * R.u) * w, vt = fma(sL, L.v, sR * R.v) * w;
    const double Ht = fma(EL + L.p, tL, (ER + R.p) * tR) * w;
    const double q2 = fma(ut, ut, vt * vt);
    const double c2 = G1 * fma(-0.5, q2, Ht);
    double c, ic2;
    if (__builtin_expect(c2 > 0.0 && hllc_in_range(c2), 1)) {
        const double t = roe_rsqrt(c2);
        c = c2 * t;
        ic2 = t * t;
    } else {
        c = sqrt_outright(c2);
        ic2 = recip_outright(c2);
    }
    const double unt = dot2(ut, nx, vt, ny);
    const double rt = sL * sR;
    const double dr = R.r - L.r, dp = R.p - L.p, dun = unR - unL;
    const double dtx = fma(-dun, nx, R.u - L.u), dty = fma(-dun, ny, R.v - L.v);
    const double h = 0.5 * ic2, x = (rt * c) * dun;
    const double a1 = (dp - x) * h, a2 = fma(-dp, ic2, dr), a4 = (dp + x) * h;
    const double l1 = unt - c, l4 = unt + c;
    const double cL = hllc_sound(GAM * L.p, L.r), cR = hllc_sound(GAM * R.p, R.r);
    const double d1 = t_max(0.0, t_max(l1 - (unL - cL), (unR - cR) - l1));
    const double d4 = t_max(0.0, t_max(l4 - (unL + cL), (unR + cR) - l4));
    double al1 = t_abs(l1); if (al1 < d1) al1 = d1;
    double al4 = t_abs(l4); if (al4 < d4) al4 = d4;
    const double al2 = t_abs(unt);
    const double w1 = al1 * a1, w2 = al2 * a2, w4 = al4 * a4, ws = al2 * rt;
    const double cx = c * nx, cy = c * ny, cu = unt * c;
    const double D0 = (w1 + w2) + w4;
    const double D1 = fma(w4, ut + cx, fma(w1, ut - cx, fma(w2, ut, ws * dtx)));
    const double D2 = fma(w4, vt + cy, fma(w1, vt - cy, fma(w2, vt, ws * dty)));
    const double D3 = fma(w4, Ht + cu, fma(w1, Ht - cu, fma(0.5 * w2, q2, ws * dot2(ut, dtx, vt, dty))));
    double FL[4], FR[4];
    phys_flux(FL, L.r, L.u, L.v, L.p, EL, unL, nx, ny);
    phys_flux(FR, R.r, R.u, R.v, R.p, ER, unR, nx, ny);
    f[0] = 0.5 * ((FL[0] + FR[0]) - D0);
    f[1] = 0.5 * ((FL[1] + FR[1]) - D1);
    f[2] = 0.5 * ((FL[2] + FR[2]) - D2);
    f[3] = 0.5 * ((FL[3] + FR[3]) - D3);
}

template <typename T, int FLUX>
__device__ __forceinline__ bool num_flux(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1,
                                         int cap) {
    if (FLUX == FLUX_LAX) { flux_lax(f, L, R, nx, ny, GAM, IG1); return false; }
    if (FLUX == FLUX_ROE) { flux_roe(f, L, R, nx, ny, GAM, IG1); return false; }
    if (FLUX == FLUX_HLLC) { flux_hllc(f, L, R, nx, ny, GAM, IG1); return false; }
    return flux_godunov(f, L, R, nx, ny, GAM, cap);
}
// The same with the FP64 Riemann solver's gas constants formed once (on the host, in the
// same operations): FP64 faces use them, FP32 faces form their own per call as before.
template <typename T, int FLUX>
__device__ __forceinline__ bool num_flux(T* f, const Prim<T>& L, const Prim<T>& R, T nx, T ny, T GAM, T IG1,
                                         int cap, const RimGas<double>& rg) {
    if constexpr (FLUX == FLUX_GODUNOV && sizeof(T) == 8) return flux_godunov<double, false>(f, L, R, nx, ny, rg, cap);
    return num_flux<T, FLUX>(f, L, R, nx, ny, GAM, IG1, cap);
}

// ------------------------------------------------------------------ kernels

// Green-Gauss gradients of r, p, u, v (calcGrad, src/methods/fvm_tvd.cpp:242-301),
// gathered per cell over its faces in ascending original edge order, dividing by S like
// the reference (FP64; the minmod arithmetic is grad_one_mm, the mixed form's grad_one_w).
// One face of the Green-Gauss sum: g +-= (q + o)/2 n l (c2 subtracts, c1 adds).
template <typename T>
__device__ __forceinline__ void grad_face(T* g, const Prim<T>& q, const Prim<T>& o, T nx, T ny, T l, bool side2) {
    // x * 0.5 is the correctly rounded x / 2 (exact halving), without a division
    const T hr = (q.r + o.r) * T(0.5), hp = (q.p + o.p) * T(0.5);
    const T hu = (q.u + o.u) * T(0.5), hv = (q.v + o.v) * T(0.5);
    const T v[8] = {hr * nx * l, hr * ny * l, hp * nx * l, hp * ny * l,
                    hu * nx * l, hu * ny * l, hv * nx * l, hv * ny * l};
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = g[m] + neg_if(v[m], side2);
}
// The ghost of the unreconstructed centre state across boundary edge e (the cell is its c1).
template <typename T>
__device__ __forceinline__ Prim<T> grad_ghost(const DevCase& c, int i, int e, const Prim<T>& q, T nx, T ny) {
    const MatT<T> mt = matT_of<T>(c, i);
    const T Tc = temperature(q, mt.gm1, mt.Cv);
    return ghost_state(c.bnds[c.ebnd[e]], q, Tc, nx, ny, mt.M);
}
// The sum divided by the area through the host-rounded reciprocal (correctly rounded, the
// reference's division); FP64 faces only (the mixed form's gradients are grad_one_w's).
template <typename T>
__device__ __forceinline__ void grad_finish(const DevCase& c, int i, T* g) {
    static_assert(sizeof(T) == 8, "the reference's Green-Gauss rounding is kept in FP64");
    const double s = c.S[i], y = c.invS[i];  // y = RN(1/S), computed on the host
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = div_rn(g[m], s, y);
}

template <typename T>
__device__ __forceinline__ void grad_one(const DevCase& c, int i) {
    const int nc = c.nc;
    const T* __restrict__ W = W_of<T>(c);
    const Prim<T> q = load_prim(W, i);
    T g[8] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
    const CellFaces<T> cf = cf_of<T>(c);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int nb = ldcs(c.cf_nb + k * nc + i);
        const T nx = ldcs(cf.nx + k * nc + i), ny = ldcs(cf.ny + k * nc + i), l = ldcs(cf.l + k * nc + i);
        const bool side2 = nb >= 0 && (nb & 1);
        const Prim<T> o = nb >= 0 ? load_prim(W, nb >> 1) : grad_ghost(c, i, -(nb + 1), q, nx, ny);
        grad_face(g, q, o, nx, ny, l, side2);
    }
    grad_finish(c, i, g);
    st8(G_of<T>(c), i, g);
}

// The FP64 gradients that minmod reconstructs from (this project's arithmetic, the oracle's
// calc_grad_minmod does the same): per face s = q + o and the weights a = RN(RN(n l) / 2)
// formed on the host, g = (sum over the faces, ascending edge order, of +-s a, the first
// term taken as it is) * RN(1/S). 60 FP64 operations per cell where grad_one takes ~128:
// the halving sits in the weights, the division is a product.
__device__ __forceinline__ void grad_one_mm(const DevCase& c, int i) {
    const int nc = c.nc;
    const double* __restrict__ W = c.W64;
    const Prim<double> q = load_prim(W, i);
    double g[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int nb = ldcs(c.cf_nb + k * nc + i);
        const double ax = ldcs(c.cf_ax + k * nc + i), ay = ldcs(c.cf_ay + k * nc + i);
        const bool side2 = nb >= 0 && (nb & 1);
        Prim<double> o;
        if (nb >= 0) {
            o = load_prim(W, nb >> 1);
        } else {
            const double nx = ldcs(c.cf_nx + k * nc + i), ny = ldcs(c.cf_ny + k * nc + i);
            o = grad_ghost(c, i, -(nb + 1), q, nx, ny);
        }
        const double sr = q.r + o.r, sp = q.p + o.p, su = q.u + o.u, sv = q.v + o.v;
        const double v[8] = {sr * ax, sr * ay, sp * ax, sp * ay, su * ax, su * ay, sv * ax, sv * ay};
#pragma unroll
        for (int m = 0; m < 8; m++) g[m] = k == 0 ? neg_if(v[m], side2) : g[m] + neg_if(v[m], side2);
    }
    const double y = c.invS[i];
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = g[m] * y;
    st8(c.G64, i, g);
}

// The mixed form's gradients (FP32 faces, every stage path): per face s = q + o and the
// host-formed weights a = RN32(n l / 2), g = (sum over the faces, ascending edge order, of
// +-s a, the first term taken as it is) * RN32(1/S): 60 FP32 operations per cell where the
// reference's expression takes 104. The sign flips run on the integer pipe, so no product
// is contracted into a sum and every path forms the same bits.
__device__ __forceinline__ void grad_face_w(float* g, const Prim<float>& q, const Prim<float>& o, float ax, float ay,
                                            bool side2, bool first) {
    const float sr = q.r + o.r, sp = q.p + o.p, su = q.u + o.u, sv = q.v + o.v;
    const float v[8] = {sr * ax, sr * ay, sp * ax, sp * ay, su * ax, su * ay, sv * ax, sv * ay};
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = first ? neg_if(v[m], side2) : g[m] + neg_if(v[m], side2);
}
__device__ __forceinline__ void grad_finish_w(const DevCase& c, int i, float* g) {
    const float is = c.invS32[i];
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = g[m] * is;
}
// k_grad's cell for the mixed form: the three faces through the per-cell arrays (the
// boundary ghosts take the edge's normal)
__device__ __forceinline__ void grad_one_w(const DevCase& c, int i) {
    const int nc = c.nc;
    const float* __restrict__ W = c.W32;
    const Prim<float> q = load_prim(W, i);
    float g[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int nb = ldcs(c.cf_nb + k * nc + i);
        const float ax = ldcs(c.cf_ax32 + k * nc + i), ay = ldcs(c.cf_ay32 + k * nc + i);
        const bool side2 = nb >= 0 && (nb & 1);
        Prim<float> o;
        if (nb >= 0) {
            o = load_prim(W, nb >> 1);
        } else {
            const int e = -(nb + 1);
            o = grad_ghost(c, i, e, q, c.nx32[e], c.ny32[e]);
        }
        grad_face_w(g, q, o, ax, ay, side2, k == 0);
    }
    grad_finish_w(c, i, g);
    st8(c.G32, i, g);
}

// 16-byte asynchronous global -> shared copies (cp.async, completion tracked per
// commit group; the waits are hardware waits, no polling).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
// the same, cached in L1 as well (records that neighbouring items read again)
__device__ __forceinline__ void cp_async16_ca(void* smem_dst, const void* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}

// 4-byte asynchronous copy global -> shared, cached in L1 and L2
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src) : "memory");
}

// MM: this project's arithmetic for minmod (FP64 only, grad_one_mm); FP32 faces the mixed
// form's (grad_one_w); else the reference's
template <typename T, bool STRIDE, bool MM = false>
__global__ void __launch_bounds__(256) k_grad(const DevCase c) {
    static_assert(!MM || sizeof(T) == 8, "the minmod gradient arithmetic is FP64's");
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (!STRIDE) {  // one thread per item
        if (i0 < c.nc) {
            if constexpr (MM) grad_one_mm(c, i0);
            else if constexpr (sizeof(T) == 4) grad_one_w(c, i0);
            else grad_one<T>(c, i0);
        }
    } else {
        for (int i = i0; i < c.nc; i += gridDim.x * blockDim.x) {  // persistent grid
            if constexpr (MM) grad_one_mm(c, i);
            else if constexpr (sizeof(T) == 4) grad_one_w(c, i);
            else grad_one<T>(c, i);
        }
    }
}

// Projection g . dl of one gradient: the reference's reconstruction (LINEAR)
// unfused, this project's minmod increment fused.
template <typename T, int RECON>
__device__ __forceinline__ T proj(T gx, T gy, T dx, T dy) {
    if (RECON == RECON_MINMOD) return dot2(gx, dx, gy, dy);
    return gx * dx + gy * dy;
}

// dq = neighbour value minus own centre value per variable (minmod only; formed
// once per edge: the two sides' differences are exact negatives of each other).
// minmod's branch as a 2-bit code: 0 zero (the signs differ), 1 the projection, 2 the difference
template <typename T>
__device__ __forceinline__ unsigned mm_code(T a, T b) {
    return mm_pos(a, b) ? (mm_first(a, b) ? 1u : 2u) : 0u;
}
// Returns minmod's branches for r, p, u, v (2 bits each, in that order; 0 without minmod),
// which the adjoint's recorded path reads instead of recomputing them.
template <typename T, int RECON>
__device__ __forceinline__ unsigned reconstruct(Prim<T>& q, const T* g, T dx, T dy, const Prim<T>& dq) {
    T dr = proj<T, RECON>(g[0], g[1], dx, dy);
    T dp = proj<T, RECON>(g[2], g[3], dx, dy);
    T du = proj<T, RECON>(g[4], g[5], dx, dy);
    T dv = proj<T, RECON>(g[6], g[7], dx, dy);
    unsigned code = 0;
    if (RECON == RECON_MINMOD) {
        code = mm_code(dr, dq.r) | mm_code(dp, dq.p) << 2 | mm_code(du, dq.u) << 4 | mm_code(dv, dq.v) << 6;
        dr = minmod(dr, dq.r);
        dp = minmod(dp, dq.p);
        du = minmod(du, dq.u);
        dv = minmod(dv, dq.v);
    }
    q.r += dr; q.p += dp; q.u += du; q.v += dv;
    return code;
}

// Edge flux over the edge's two Gauss points, times l/2 (src/methods/fvm_tvd.cpp:329-352).
// The edge flux from the two cells' primitives and gradients, both Gauss points,
// times l/2 (src/methods/fvm_tvd.cpp:329-352): out[4] is what F holds for edge e.
// An edge's geometry as the flux reads it: normal, length, the Gauss-point offsets
// (gp0: dxL dyL dxR dyR, gp1: ...; only with reconstruction).
template <typename T> struct EdgeGeo { T nx, ny, l, dl[8]; };
template <typename T, int RECON>
__device__ __forceinline__ EdgeGeo<T> load_geo(const DevCase& c, int e) {
    EdgeGeo<T> g;
    if constexpr (sizeof(T) == 4) {  // FP32 faces: the edge's three 16-byte records
        const float4* __restrict__ r = c.geo32 + 3 * (size_t)e;
        const float4 a = __ldcs(r);
        g.nx = a.x; g.ny = a.y; g.l = a.z;
        if (RECON != RECON_NONE) {
            const float4 b = __ldcs(r + 1), d = __ldcs(r + 2);
            g.dl[0] = b.x; g.dl[1] = b.y; g.dl[2] = b.z; g.dl[3] = b.w;
            g.dl[4] = d.x; g.dl[5] = d.y; g.dl[6] = d.z; g.dl[7] = d.w;
        }
    } else {
        g.nx = ldcs(NX_of<T>(c) + e);
        g.ny = ldcs(NY_of<T>(c) + e);
        g.l = ldcs(L_of<T>(c) + e);
        if (RECON != RECON_NONE) {
            const T* __restrict__ DL = DL_of<T>(c);
#pragma unroll
            for (int k = 0; k < 8; k++) g.dl[k] = ldcs(DL + (size_t)k * c.ne + e);
        }
    }
    return g;
}

// With REC (HLLC only) the evaluation also leaves what the adjoint's recorded path reads
// (FluxRec): per Gauss point the two face states and sound speeds, and minmod's branches.
// SIDE: EDGE_ANY (interior or boundary, decided at run time), EDGE_INNER or EDGE_BOUNDARY
// (known at compile time: the interior instantiation carries no boundary code, which a
// warp would otherwise issue, predicated off, for every interior edge; the adjoint's flux
// kernels use them).
enum { EDGE_ANY = 0, EDGE_INNER = 1, EDGE_BOUNDARY = 2 };
template <int SIDE>
__device__ __forceinline__ bool edge_inner(const DevCase& c, int e) {
    return SIDE == EDGE_INNER ? true : (SIDE == EDGE_BOUNDARY ? false : e < c.n_int);
}
template <typename T, int FLUX, int RECON, bool REC = false, int SIDE = EDGE_ANY>
__device__ __forceinline__ void flux_core(const DevCase& c, int e, int c1, const Prim<T>& qL, const T* gL,
                                          const Prim<T>& qR, const T* gR, T* out, const EdgeGeo<T>& geo,
                                          const FluxRec& rec = FluxRec{}) {
    static_assert(!REC || FLUX == FLUX_HLLC, "flux records are kept for HLLC");
    // qR: the second cell's primitives on interior edges (e < n_int), qL on boundary edges
    const T nx = geo.nx, ny = geo.ny, l = geo.l;
    const T GAM = gam_of<T>(c), IG1 = ig1_of<T>(c);
    const bool inner = edge_inner<SIDE>(c, e);
    Prim<T> gc = qL;
    DevBnd b{};
    T Tc = T(0), M = T(0);
    if (!inner) {
        b = c.bnds[c.ebnd[e]];
        const MatT<T> mt = matT_of<T>(c, c1);
        Tc = temperature(qL, mt.gm1, mt.Cv);
        M = mt.M;
        if (RECON == RECON_MINMOD) gc = ghost_state(b, qL, Tc, nx, ny, M);
    }
    // minmod's neighbour-minus-centre differences of both sides: formed once per edge in
    // FP64 (the FP64 pipe is the bound there); per Gauss point in FP32 (fewer live registers)
    Prim<T> dL = qL, dR = qL;
    if (RECON == RECON_MINMOD && sizeof(T) == 8) {
        const Prim<T>& nb = inner ? qR : gc;
        dL.r = nb.r - qL.r; dL.u = nb.u - qL.u; dL.v = nb.v - qL.v; dL.p = nb.p - qL.p;
        dR.r = neg_if(dL.r, true); dR.u = neg_if(dL.u, true); dR.v = neg_if(dL.v, true); dR.p = neg_if(dL.p, true);
    }
    T fs[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
    bool hit = false;
    unsigned codes = 0;
#pragma unroll
    for (int gp = 0; gp < 2; gp++) {
        Prim<T> pL = qL, pR;
        if (RECON == RECON_MINMOD && sizeof(T) == 4) {
            const Prim<T>& nb = inner ? qR : gc;
            dL.r = nb.r - qL.r; dL.u = nb.u - qL.u; dL.v = nb.v - qL.v; dL.p = nb.p - qL.p;
            dR.r = qL.r - qR.r; dR.u = qL.u - qR.u; dR.v = qL.v - qR.v; dR.p = qL.p - qR.p;
        }
        if (RECON != RECON_NONE)
            codes |= reconstruct<T, RECON>(pL, gL, geo.dl[4 * gp], geo.dl[4 * gp + 1], dL) << (16 * gp);
        if (inner) {
            pR = qR;
            if (RECON != RECON_NONE)
                codes |= reconstruct<T, RECON>(pR, gR, geo.dl[4 * gp + 2], geo.dl[4 * gp + 3], dR) << (16 * gp + 8);
        } else {
            pR = ghost_state(b, pL, Tc, nx, ny, M);
        }
        T f[4];
        if constexpr (REC) {
            const T cL = hllc_sound(GAM * pL.p, pL.r), cR = hllc_sound(GAM * pR.p, pR.r);
            T* v = static_cast<T*>(rec.v) + (size_t)(10 * gp) * c.ne + e;
            const size_t ne = c.ne;
            v[0] = pL.r; v[ne] = pL.u; v[2 * ne] = pL.v; v[3 * ne] = pL.p;
            v[4 * ne] = pR.r; v[5 * ne] = pR.u; v[6 * ne] = pR.v; v[7 * ne] = pR.p;
            v[8 * ne] = cL; v[9 * ne] = cR;
            flux_hllc_c(f, pL, pR, cL, cR, nx, ny, IG1);
        } else {
            hit |= num_flux<T, FLUX>(f, pL, pR, nx, ny, GAM, IG1, c.newton_cap, c.rg_flux);
        }
        // the reference's fluxes sum the Gauss points from +0 (its fSum = 0; fSum += F); this
        // project's own fluxes (HLLC, Roe) start from the first point's flux
        if (gp == 0 && (FLUX == FLUX_HLLC || FLUX == FLUX_ROE)) {
            fs[0] = f[0]; fs[1] = f[1]; fs[2] = f[2]; fs[3] = f[3];
        } else {
            fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
        }
        if (RECON == RECON_NONE) {  // both Gauss points see the cell-centre states
            fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
            break;
        }
    }
    if constexpr (REC) rec.bits[e] = codes;
    if (hit) atomicOr(c.err, ERRBIT_NEWTON_CAP);
    const T lh = l * T(0.5);
    out[0] = fs[0] * lh; out[1] = fs[1] * lh; out[2] = fs[2] * lh; out[3] = fs[3] * lh;
}

// The flux of edge e (what F holds for it) from the stage's W and G (with REC: and its record).
template <typename T, int FLUX, int RECON, bool REC = false, int SIDE = EDGE_ANY>
__device__ __forceinline__ void flux_edge(const DevCase& c, int e, T* out, const FluxRec& rec = FluxRec{}) {
    const T* __restrict__ W = W_of<T>(c);
    const T* __restrict__ G = G_of<T>(c);
    const int c1 = ldcs(c.ec1 + e);
    const bool inner = edge_inner<SIDE>(c, e);
    const Prim<T> qL = load_prim(W, c1);
    T gL[8], gR[8];
    if (RECON != RECON_NONE) ld8(G, c1, gL);
    Prim<T> qR = qL;
    if (inner) {
        const int c2 = ldcs(c.ec2 + e);
        qR = load_prim(W, c2);
        if (RECON != RECON_NONE) ld8(G, c2, gR);
    }
    flux_core<T, FLUX, RECON, REC, SIDE>(c, e, c1, qL, gL, qR, gR, out, load_geo<T, RECON>(c, e), rec);
}

template <typename T, int FLUX, int RECON>
__device__ __forceinline__ void flux_one(const DevCase& c, int e) {
    T out[4];
    flux_edge<T, FLUX, RECON>(c, e, out);
    st4(F_of<T>(c), e, out[0], out[1], out[2], out[3]);
}

// The mixed form's flux kernel as a persistent, software-pipelined loop. A thread works
// through edges e, e + S, e + 2S, ... (S = threads in the grid): while it computes one
// edge, the next edge's inputs -- the two cells' records (W and G, 96 bytes) and the edge's
// geometry (normal, length, Gauss-point offsets) -- are on their way into its own slots of
// shared memory (cp.async), and the cell numbers of the edge after that into registers, so
// no load stalls the arithmetic. Same inputs and arithmetic as k_flux: the same fluxes bit
// for bit. Dynamic shared memory: 2 stages x (6 float4 + 12 float) per thread.
constexpr int kPipeStage = 6 * 16 + 12 * 4;  // bytes per thread and stage
template <int FLUX, int RECON>
__global__ void __launch_bounds__(256, 3) k_flux_pipe(const DevCase c) {
    extern __shared__ float4 stg[];
    const int tid = threadIdx.x, nb = blockDim.x;
    const float4* __restrict__ W4 = reinterpret_cast<const float4*>(c.W32);
    const float4* __restrict__ G4 = reinterpret_cast<const float4*>(c.G32);
    const int stride = gridDim.x * nb;
    const int ne = c.ne, n_int = c.n_int;
    // stage k: 6 float4 columns then 12 float columns, each nb wide
    auto rec = [&](int k) { return reinterpret_cast<float4*>(reinterpret_cast<char*>(stg) + (size_t)k * kPipeStage * nb); };
    auto geo_col = [&](int k, int j) { return reinterpret_cast<float*>(rec(k) + 6 * nb) + (size_t)j * nb + tid; };
    int e = blockIdx.x * nb + tid;
    // cell numbers of the edge whose copies go out next (a, b) and of the one after (a2, b2)
    int a = 0, b = 0, a2 = 0, b2 = 0;
    auto cells = [&](int edge, int& x, int& y) {
        if (edge < ne) {
            x = ldcs(c.ec1 + edge);
            y = edge < n_int ? ldcs(c.ec2 + edge) : x;
        }
    };
    auto issue = [&](int k, int edge, int x, int y) {
        if (edge < ne) {
            float4* sl = rec(k) + tid;
            cp_async16_ca(sl, W4 + x);
            cp_async16_ca(sl + nb, W4 + y);
            if (RECON != RECON_NONE) {
                cp_async16_ca(sl + 2 * nb, G4 + 2 * (size_t)x);
                cp_async16_ca(sl + 3 * nb, G4 + 2 * (size_t)x + 1);
                cp_async16_ca(sl + 4 * nb, G4 + 2 * (size_t)y);
                cp_async16_ca(sl + 5 * nb, G4 + 2 * (size_t)y + 1);
            }
            cp_async4(geo_col(k, 0), c.nx32 + edge);
            cp_async4(geo_col(k, 1), c.ny32 + edge);
            cp_async4(geo_col(k, 2), c.l32 + edge);
            if (RECON != RECON_NONE)
#pragma unroll
                for (int j = 0; j < 8; j++) cp_async4(geo_col(k, 3 + j), c.dl32 + (size_t)j * ne + edge);
        }
        cp_async_commit();
    };
    cells(e, a, b);
    issue(0, e, a, b);
    cells(e + stride, a2, b2);
    for (int k = 0; e < ne; e += stride, k ^= 1) {
        const int c1 = a;
        a = a2; b = b2;
        issue(k ^ 1, e + stride, a, b);     // the next edge's inputs
        cells(e + 2 * stride, a2, b2);      // and the cell numbers of the one after
        cp_async_wait<1>();                 // this edge's inputs (issued one round ago)
        const float4* sl = rec(k) + tid;
        const float4 wl = sl[0];
        const Prim<float> qL{wl.x, wl.y, wl.z, wl.w};
        Prim<float> qR = qL;
        float gL[8], gR[8];
        if (RECON != RECON_NONE) {
            const float4 x0 = sl[2 * nb], x1 = sl[3 * nb];
            gL[0] = x0.x; gL[1] = x0.y; gL[2] = x0.z; gL[3] = x0.w; gL[4] = x1.x; gL[5] = x1.y; gL[6] = x1.z; gL[7] = x1.w;
        }
        if (e < n_int) {
            const float4 wr = sl[nb];
            qR = Prim<float>{wr.x, wr.y, wr.z, wr.w};
            if (RECON != RECON_NONE) {
                const float4 y0 = sl[4 * nb], y1 = sl[5 * nb];
                gR[0] = y0.x; gR[1] = y0.y; gR[2] = y0.z; gR[3] = y0.w; gR[4] = y1.x; gR[5] = y1.y; gR[6] = y1.z; gR[7] = y1.w;
            }
        }
        EdgeGeo<float> geo;
        geo.nx = *geo_col(k, 0);
        geo.ny = *geo_col(k, 1);
        geo.l = *geo_col(k, 2);
        if (RECON != RECON_NONE)
#pragma unroll
            for (int j = 0; j < 8; j++) geo.dl[j] = *geo_col(k, 3 + j);
        float out[4];
        flux_core<float, FLUX, RECON>(c, e, c1, qL, gL, qR, gR, out, geo);
        st4(c.F32, e, out[0], out[1], out[2], out[3]);
    }
    cp_async_wait<0>();
}

template <typename T, int FLUX, int RECON, bool STRIDE>
__global__ void __launch_bounds__(256) k_flux(const DevCase c) {
    const int e0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (!STRIDE) {  // one thread per item
        if (e0 < c.ne) flux_one<T, FLUX, RECON>(c, e0);
    } else {
        for (int e = e0; e < c.ne; e += gridDim.x * blockDim.x) flux_one<T, FLUX, RECON>(c, e);  // persistent grid
    }
}

// Knuth's TwoSum: s + e == a + b exactly (round to nearest, no reassociation).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// The three signed FP32 face fluxes summed as an FP32 pair (TwoSum) and rounded once to
// FP32: at most half an FP32 ulp of the residual, below the FP32 rounding its fluxes
// already carry (cancellation among the three costs nothing), and no FP64 addition on
// the way to the FP64 update.
__device__ __forceinline__ void residual_pair_sum(const float t[3][4], double* R) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float s1, e1, s2, e2;
        two_sum(t[0][q], t[1][q], s1, e1);
        two_sum(s1, t[2][q], s2, e2);
        R[q] = widen(__fadd_rn(s2, __fadd_rn(e1, e2)));
    }
}

// Residual of cell i: the reference's ro_int..re_int (src/methods/fvm_tvd.cpp:353-363).
// FP64 faces: 0 -/+ F in ascending original edge order, the reference's own sums.
// FP32 faces: the three signed fluxes summed exactly as an FP32 pair, then rounded
// once to FP32 (residual_pair_sum).
template <typename T>
__device__ __forceinline__ void gather_residual(const DevCase& c, int i, double* R) {
    const int nc = c.nc;
    const T* __restrict__ F = F_of<T>(c);
    if constexpr (sizeof(T) == 8) {
        R[0] = 0.0; R[1] = 0.0; R[2] = 0.0; R[3] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int f = c.face[k * nc + i];
            double v[4];
            ld4(F, f >> 1, v);
#pragma unroll
            for (int q = 0; q < 4; q++) R[q] = R[q] + neg_if(v[q], !(f & 1));
        }
    } else {
        float t[3][4];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int f = c.face[k * nc + i];
            float v[4];
            ld4(F, f >> 1, v);
#pragma unroll
            for (int q = 0; q < 4; q++) t[k][q] = neg_if(v[q], !(f & 1));
        }
        residual_pair_sum(t, R);
    }
}

template <typename T>
__device__ __forceinline__ Prim<T> prim_face_of(double ro, double ru, double rv, double re, const DevCase& c, int i);
template <>
__device__ __forceinline__ Prim<double> prim_face_of<double>(double ro, double ru, double rv, double re,
                                                             const DevCase& c, int i) {
    return cons2prim<double>(ro, ru, rv, re, mat_of(c, i).gm1);
}
template <>
__device__ __forceinline__ Prim<float> prim_face_of<float>(double ro, double ru, double rv, double re,
                                                           const DevCase& c, int i) {
    return cons2prim<float>(narrow(ro), narrow(ru), narrow(rv), narrow(re), matT_of<float>(c, i).gm1);
}

// local time step of one cell (calcTimeStep STEADY branch, src/methods/fvm_tvd.cpp:218-224)
__device__ __forceinline__ void local_dt(const DevCase& c, int i, const Prim<double>& q, const DevMat& mt) {
    double cz = sqrt(mt.gam * q.p / q.r);
    double t = c.cfl_number * c.S[i] / t_max(fabs(q.u) + cz, fabs(q.v) + cz);
    c.ctau_next[i] = t;
    c.cfl[i] = t / c.S[i];
}

template <typename T>
__device__ __forceinline__ bool outside_limits(const DevCase& c, const Prim<T>& q) {  // :439-446
    if constexpr (sizeof(T) == 8)
        return q.r < c.lim_rmin || q.r > c.lim_rmax || q.p < c.lim_pmin || q.p > c.lim_pmax ||
               fabs(q.u) > c.lim_umax || fabs(q.v) > c.lim_umax;
    else
        return q.r < c.lim_f[0] || q.r > c.lim_f[1] || q.p < c.lim_f[2] || q.p > c.lim_f[3] ||
               fabsf(q.u) > c.lim_f[4] || fabsf(q.v) > c.lim_f[4];
}

// One Runge-Kutta stage update with the residual gathered from the edge fluxes.
// SCHEME/STAGE: Euler (0), Heun (0,1; src/methods/fvm_tvd.cpp:366-447), SSP-RK3 Shu-Osher (0,1,2).
// The last stage checks the limits (in the face precision) and, for a local time
// step, computes the next step's cTau in FP64.
template <int SCHEME, int STAGE>
struct StageKind {
    static constexpr bool FINAL = (SCHEME == TIME_EULER && STAGE == 0) || (SCHEME == TIME_HEUN && STAGE == 1) ||
                                  (SCHEME == TIME_SSPRK3 && STAGE == 2);
};

// Start of a cell's stage update: the step's cTau, and the frozen (LIM-flagged)
// cells, which are not updated (later stages read B). Returns false for those.
template <int SCHEME, int STAGE>
__device__ __forceinline__ bool update_begin(const DevCase& c, int i) {
    constexpr bool FINAL = StageKind<SCHEME, STAGE>::FINAL;
    const int nc = c.nc;
    if (STAGE == 0 && c.steady) c.ctau[i] = c.ctau_next[i];  // the step now running uses ctau_next
    if (c.flags[i] & 0x2u) {  // cellIsLim
        if (STAGE == 0 && !FINAL)
#pragma unroll
            for (int k = 0; k < 4; k++) c.B[k * nc + i] = c.A[k * nc + i];
        if (FINAL) atomicAdd(c.n_lim, 1);
        return false;
    }
    return true;
}

// The stage update of cell i from its residual R: U += cTau/S R, the scheme's
// combination, the next primitives into Wout; the last stage checks the limits
// (in the face precision) and, for a local time step, computes the next step's
// cTau in FP64.
template <typename T, int SCHEME, int STAGE>
__device__ __forceinline__ void update_finish(const DevCase& c, int i, const double* R, T* __restrict__ Wout) {
    constexpr bool FINAL = StageKind<SCHEME, STAGE>::FINAL;
    const int nc = c.nc;
    const double cf = c.cfl[i];
    const double* __restrict__ src = STAGE == 0 ? c.A : c.B;
    double u0 = src[i] + cf * R[0], u1 = src[nc + i] + cf * R[1], u2 = src[2 * nc + i] + cf * R[2],
           u3 = src[3 * nc + i] + cf * R[3];
    double* dst = FINAL ? c.A : c.B;
    if (SCHEME == TIME_SSPRK3) {
        // SSP-RK3 (not in the reference) with fused multiply-adds: X + cf R, then
        // 3/4 U^n + 1/4 X and 1/3 U^n + 2/3 X (the Euler and Heun stages stay unfused: the
        // reference's U += cTau/S R)
        u0 = fma(cf, R[0], src[i]); u1 = fma(cf, R[1], src[nc + i]);
        u2 = fma(cf, R[2], src[2 * nc + i]); u3 = fma(cf, R[3], src[3 * nc + i]);
        if (STAGE == 1) {
            u0 = fma(0.25, u0, 0.75 * c.A[i]); u1 = fma(0.25, u1, 0.75 * c.A[nc + i]);
            u2 = fma(0.25, u2, 0.75 * c.A[2 * nc + i]); u3 = fma(0.25, u3, 0.75 * c.A[3 * nc + i]);
        } else if (STAGE == 2) {
            const double c13 = 1.0 / 3.0, c23 = 2.0 / 3.0;
            u0 = fma(c23, u0, c13 * c.A[i]); u1 = fma(c23, u1, c13 * c.A[nc + i]);
            u2 = fma(c23, u2, c13 * c.A[2 * nc + i]); u3 = fma(c23, u3, c13 * c.A[3 * nc + i]);
        }
    } else if (SCHEME == TIME_HEUN && STAGE == 1) {
        u0 = 0.5 * (c.A[i] + u0); u1 = 0.5 * (c.A[nc + i] + u1);
        u2 = 0.5 * (c.A[2 * nc + i] + u2); u3 = 0.5 * (c.A[3 * nc + i] + u3);
    }
    dst[i] = u0; dst[nc + i] = u1; dst[2 * nc + i] = u2; dst[3 * nc + i] = u3;
    const Prim<T> w = prim_face_of<T>(u0, u1, u2, u3, c, i);
    store_prim(Wout, i, w);
    if (FINAL) {
        if (outside_limits(c, w)) {
            c.flags[i] |= 0x2u;
            atomicAdd(c.n_lim, 1);
        }
        if (!(w.r > T(0)) || !(w.p > T(0))) atomicOr(c.err, ERRBIT_NONPHYSICAL);
        if (c.steady) {
            const DevMat mt = mat_of(c, i);
            local_dt(c, i, cons2prim<double>(u0, u1, u2, u3, mt.gm1), mt);
        }
    }
}

// One Runge-Kutta stage update with the residual gathered from the edge fluxes.
// SCHEME/STAGE: Euler (0), Heun (0,1; src/methods/fvm_tvd.cpp:366-447), SSP-RK3 Shu-Osher (0,1,2).
template <typename T, int SCHEME, int STAGE>
__device__ __forceinline__ void update_one(const DevCase& c, int i) {
    if (!update_begin<SCHEME, STAGE>(c, i)) return;
    double R[4];
    gather_residual<T>(c, i, R);
    update_finish<T, SCHEME, STAGE>(c, i, R, Wm_of<T>(c));
}

// The mixed form's whole Runge-Kutta stage for tiles of cells (persistent CTAs of 256
// threads, each looping over tiles): a tile's and its two-ring halo's primitives are
// staged in shared memory (fetched with cp.async while the CTA works on its previous
// tile), then gradients of the own and first-ring cells, the fluxes of the own
// cells' edges and the own cells' updates run from shared memory. Edges on the tile
// border are evaluated by both tiles, each time with the same inputs and the same
// code as k_grad / k_flux / k_update, so the results are those kernels' bit for
// bit. Primitives are read from w_in and written to w_out (another buffer: the
// neighbouring tiles still read the old values as their halo).
template <int FLUX, int RECON, int SCHEME, int STAGE>
__global__ void __launch_bounds__(256, 5) k_stage_fused(const DevCase c, const DevTiles tl,
                                                     const float* __restrict__ w_in, float* __restrict__ w_out) {
    extern __shared__ float4 smem[];
    float4* Wb[2] = {smem, smem + tl.max_cells};  // primitives of the tile in work / the next tile
    float4* Gs = smem + 2 * tl.max_cells;          // 2 per gradient cell
    float4* Fs = Gs + 2 * tl.max_grad;             // one flux record per edge
    const float4* W4 = reinterpret_cast<const float4*>(w_in);
    float4* Wo = reinterpret_cast<float4*>(w_out);
    auto fetch = [&](int t, float4* dst) {
        const int own0 = t * tl.tile, n_own = min(tl.tile, c.nc - own0);
        const int h0 = tl.halo_off[t], nL = n_own + tl.halo_off[t + 1] - h0;
        for (int k = threadIdx.x; k < nL; k += blockDim.x)
            cp_async16(dst + k, W4 + (k < n_own ? own0 + k : tl.halo[h0 + k - n_own]));
    };
    int b = 0;
    if ((int)blockIdx.x < tl.n_tiles) fetch(blockIdx.x, Wb[0]);
    cp_async_commit();
    for (int t = blockIdx.x; t < tl.n_tiles; t += gridDim.x, b ^= 1) {
        const int tn = t + gridDim.x;
        if (tn < tl.n_tiles) fetch(tn, Wb[b ^ 1]);
        cp_async_commit();
        cp_async_wait<1>();  // this tile's copies have landed (the next tile's may be in flight)
        __syncthreads();
        const float4* Ws = Wb[b];
        const int own0 = t * tl.tile, n_own = min(tl.tile, c.nc - own0);
        const int h0 = tl.halo_off[t], nh1 = tl.n_h1[t];
        const int nG = n_own + nh1;
        const int e0 = tl.edge_off[t], nE = tl.edge_off[t + 1] - e0;
        const int2* __restrict__ gf = tl.gface + 3 * (size_t)tl.gface_off[t];
        auto prim = [&](int k) {
            const float4 a = Ws[k];
            Prim<float> q;
            q.r = a.x; q.u = a.y; q.v = a.z; q.p = a.w;
            return q;
        };
        if (RECON != RECON_NONE) {
            for (int k = threadIdx.x; k < nG; k += blockDim.x) {
                const int i = k < n_own ? own0 + k : tl.halo[h0 + k - n_own];
                const Prim<float> q = prim(k);
                float g[8];
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    const int2 fr = gf[3 * k + f];
                    const int e = fr.x >> 1, nb = fr.y & 0xffff;
                    const Prim<float> o = nb != 0xffff ? prim(nb) : grad_ghost(c, i, e, q, c.nx32[e], c.ny32[e]);
                    grad_face_w(g, q, o, c.ax32[e], c.ay32[e], (fr.x & 1) != 0, f == 0);
                }
                grad_finish_w(c, i, g);
                Gs[2 * k] = make_float4(g[0], g[1], g[2], g[3]);
                Gs[2 * k + 1] = make_float4(g[4], g[5], g[6], g[7]);
            }
            __syncthreads();
        }
        for (int k = threadIdx.x; k < nE; k += blockDim.x) {
            const int2 te = tl.tedge[e0 + k];
            const int e = te.x, l1 = te.y & 0xffff, l2 = (int)((unsigned)te.y >> 16);
            const Prim<float> qL = prim(l1);
            const Prim<float> qR = l2 != 0xffff ? prim(l2) : qL;
            float gL[8], gR[8];
            if (RECON != RECON_NONE) {
                const float4 a = Gs[2 * l1], bb = Gs[2 * l1 + 1];
                gL[0] = a.x; gL[1] = a.y; gL[2] = a.z; gL[3] = a.w; gL[4] = bb.x; gL[5] = bb.y; gL[6] = bb.z; gL[7] = bb.w;
                if (l2 != 0xffff) {
                    const float4 x = Gs[2 * l2], y = Gs[2 * l2 + 1];
                    gR[0] = x.x; gR[1] = x.y; gR[2] = x.z; gR[3] = x.w; gR[4] = y.x; gR[5] = y.y; gR[6] = y.z; gR[7] = y.w;
                }
            }
            float out[4];
            const int c1 = l1 < n_own ? own0 + l1 : tl.halo[h0 + l1 - n_own];
            flux_core<float, FLUX, RECON>(c, e, c1, qL, gL, qR, gR, out, load_geo<float, RECON>(c, e));
            Fs[k] = make_float4(out[0], out[1], out[2], out[3]);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < n_own; k += blockDim.x) {
            const int i = own0 + k;
            if (!update_begin<SCHEME, STAGE>(c, i)) {
                Wo[i] = Ws[k];  // frozen cell: its primitives do not change
                continue;
            }
            float tv[3][4];
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const int2 fr = gf[3 * k + f];
                const float4 v = Fs[(unsigned)fr.y >> 16];
                const bool add = (fr.x & 1) != 0;  // c2 adds the edge flux, c1 subtracts it
                tv[f][0] = neg_if(v.x, !add); tv[f][1] = neg_if(v.y, !add);
                tv[f][2] = neg_if(v.z, !add); tv[f][3] = neg_if(v.w, !add);
            }
            double R[4];
            residual_pair_sum(tv, R);
            update_finish<float, SCHEME, STAGE>(c, i, R, w_out);
        }
        __syncthreads();  // shared buffers are free for the next round
    }
    cp_async_wait<0>();
}

// Gradient of cell i (FP32 faces) from its three 16-byte face records {neighbour, a_x,
// a_y, 0}: the operations of grad_one_w on the same values.
__device__ __forceinline__ void grad_of_cell(const DevCase& c, int i, const Prim<float>& q, float* g) {
    const float4* __restrict__ rec = c.cfrec32 + 3 * (size_t)i;
    const float* __restrict__ W = c.W32;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 r = __ldg(rec + k);
        const int nb = __float_as_int(r.x);
        const bool side2 = nb >= 0 && (nb & 1);
        Prim<float> o;
        if (nb >= 0) {
            o = load_prim(W, nb >> 1);
        } else {
            const int e = -(nb + 1);
            o = grad_ghost(c, i, e, q, c.nx32[e], c.ny32[e]);
        }
        grad_face_w(g, q, o, r.y, r.z, side2, k == 0);
    }
    grad_finish_w(c, i, g);
}

// The mixed form's edge flux with the two cells' Green-Gauss gradients formed in the
// kernel (each cell's once per edge it borders, from the stage's W and the cells' face
// records) instead of read from G: no gradient array written and read back, no gradient
// launch. The same operations on the same values as k_grad + k_flux, so the same fluxes.
template <int FLUX, int RECON>
__global__ void __launch_bounds__(256, 4) k_flux_grad(const DevCase c) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    const float* __restrict__ W = c.W32;
    const int c1 = ldcs(c.ec1 + e);
    const bool inner = e < c.n_int;
    const Prim<float> qL = load_prim(W, c1);
    float gL[8], gR[8];
    grad_of_cell(c, c1, qL, gL);
    Prim<float> qR = qL;
    if (inner) {
        const int c2 = ldcs(c.ec2 + e);
        qR = load_prim(W, c2);
        grad_of_cell(c, c2, qR, gR);
    }
    float out[4];
    flux_core<float, FLUX, RECON>(c, e, c1, qL, gL, qR, gR, out, load_geo<float, RECON>(c, e));
    st4(c.F32, e, out[0], out[1], out[2], out[3]);
}

// The mixed form's flux and update of one stage per tile of cells (one CTA of 256 threads
// per tile): the fluxes of every edge of the tile's own cells (from the stage's W in
// c.W32 and the gradients k_grad left in c.G32, read through the caches) go into shared
// memory, then each own cell gathers its three and updates, writing its new primitives
// to w_out (another buffer: the neighbouring tiles still read the old ones). An edge on
// the tile border is evaluated by both tiles with the same inputs and the same code as
// k_flux, and the cell sums are those of k_update: the per-kernel path's results bit for
// bit, without the edge fluxes' round trip through memory, and with the update's FP64
// work overlapping other tiles' gathers.
template <int FLUX, int RECON, int SCHEME, int STAGE>
__global__ void __launch_bounds__(256) k_flux_update(const DevCase c, const DevTiles tl, float* __restrict__ w_out) {
    extern __shared__ float4 Fs[];
    const int t = blockIdx.x;
    const int own0 = t * tl.tile, n_own = min(tl.tile, c.nc - own0);
    const int e0 = tl.edge_off[t], nE = tl.edge_off[t + 1] - e0;
    for (int k = threadIdx.x; k < nE; k += blockDim.x) {
        float out[4];
        flux_edge<float, FLUX, RECON>(c, tl.tedge[e0 + k].x, out);
        Fs[k] = make_float4(out[0], out[1], out[2], out[3]);
    }
    __syncthreads();
    const int k = threadIdx.x;
    if (k >= n_own) return;
    const int i = own0 + k;
    if (!update_begin<SCHEME, STAGE>(c, i)) {  // frozen cell: its primitives do not change
        reinterpret_cast<float4*>(w_out)[i] = reinterpret_cast<const float4*>(c.W32)[i];
        return;
    }
    const int2* __restrict__ gf = tl.gface + 3 * ((size_t)tl.gface_off[t] + k);
    float tv[3][4];
#pragma unroll
    for (int f = 0; f < 3; f++) {
        const int2 fr = gf[f];
        const float4 v = Fs[(unsigned)fr.y >> 16];
        const bool add = (fr.x & 1) != 0;  // c2 adds the edge flux, c1 subtracts it
        tv[f][0] = neg_if(v.x, !add); tv[f][1] = neg_if(v.y, !add);
        tv[f][2] = neg_if(v.z, !add); tv[f][3] = neg_if(v.w, !add);
    }
    double R[4];
    residual_pair_sum(tv, R);
    update_finish<float, SCHEME, STAGE>(c, i, R, w_out);
}

template <typename T, int SCHEME, int STAGE, bool STRIDE>
__global__ void __launch_bounds__(256) k_update(const DevCase c) {
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (!STRIDE) {  // one thread per item
        if (i0 < c.nc) update_one<T, SCHEME, STAGE>(c, i0);
    } else {
        for (int i = i0; i < c.nc; i += gridDim.x * blockDim.x) update_one<T, SCHEME, STAGE>(c, i);  // persistent grid
    }
}

// remediateLimCells, src/methods/fvm_tvd.cpp:464-499: flagged cells, in original
// cell order and one after another (each may read a neighbour remediated just
// before it), take the area-weighted mean of the c2 cells of their edges.
template <typename T>
__global__ void __launch_bounds__(1024) k_remediate(const DevCase c) {
    __shared__ int list[1024];
    __shared__ int cnt;
    __shared__ int wsum[32];
    const int nc = c.nc;
    if (*c.n_lim == 0) return;
    for (int base = 0; base < nc; base += blockDim.x) {
        const int o = base + threadIdx.x;
        const int i = o < nc ? c.iperm[o] : -1;
        const bool fl = o < nc && (c.flags[i] & 0x2u);
        const unsigned ball = __ballot_sync(0xffffffffu, fl);
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
                if (c.steady) local_dt(c, ci, cons2prim<double>(u0, u1, u2, u3, mt.gm1), mt);
                store_prim(Wm_of<T>(c), ci, prim_face_of<T>(u0, u1, u2, u3, c, ci));
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
    const double u0 = c.A[i], u1 = c.A[nc + i], u2 = c.A[2 * nc + i], u3 = c.A[3 * nc + i];
    if (c.steady) {
        const DevMat mt = mat_of(c, i);
        local_dt(c, i, cons2prim<double>(u0, u1, u2, u3, mt.gm1), mt);
        c.ctau[i] = c.ctau_next[i];
    }
    store_prim(Wm_of<T>(c), i, prim_face_of<T>(u0, u1, u2, u3, c, i));
}

// Residual of the current edge fluxes (the reference's *_int arrays) for every cell.
template <typename T>
__global__ void __launch_bounds__(256) k_residual(const DevCase c, double* __restrict__ R) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double r[4];
    gather_residual<T>(c, i, r);
    for (int q = 0; q < 4; q++) R[q * nc + i] = r[q];
}

}  // namespace cfd2d
