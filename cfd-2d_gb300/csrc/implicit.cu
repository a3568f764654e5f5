// FVM_TVD_IMPLICIT kernels that must equal the reference bit for bit: primitives,
// gradients, Gauss-point fluxes, the block-row assembly and the post-solve update
// (src/methods/fvm_tvd_implicit.cpp). Built with -fmad=false: no product is fused
// into a following sum, every expression is evaluated as the reference writes it.
#include "implicit.hpp"
#include "kernels.cuh"

namespace cfd2d {

namespace {

__device__ __forceinline__ const DevMat& imat(const ImpCase& c, int i) { return c.cmat ? c.mats[c.cmat[i]] : c.mat0; }

// FVM_TVD_IMPLICIT::boundaryCond, :963-1008. INLET: (T, P, Vx, Vy) then URS(2)
// rho = p M / (T gR); OUTLET: the cell state; WALL: the cell state with the normal
// velocity mirrored, u - 2 (u.n) n. Only r, u, v, p are consumed downstream.
__device__ __forceinline__ Prim<double> imp_ghost(const DevBnd& b, const Prim<double>& q, double nx, double ny,
                                                  double M) {
    Prim<double> g = q;
    if (b.kind == IBND_INLET) {
        g.u = b.u; g.v = b.v; g.p = b.p;
        g.r = g.p * M / (b.T * GAS_R);
    } else if (b.kind == IBND_WALL) {
        const double Un = q.u * nx + q.v * ny;
        const double Vx = nx * Un * 2.0, Vy = ny * Un * 2.0;
        g.u = q.u - Vx;
        g.v = q.v - Vy;
    }
    return g;
}

__global__ void __launch_bounds__(256) k_imp_prims(const ImpCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nc) return;
    const int nc = c.nc;
    // convertConsToPar, :1058-1068 (URS(0): p = r e (gam - 1))
    const Prim<double> q = cons2prim<double>(c.A[i], c.A[nc + i], c.A[2 * nc + i], c.A[3 * nc + i], imat(c, i).gm1);
    store_prim(c.W, i, q);
    if (!(q.r > 0.0) || !(q.p > 0.0)) atomicOr(c.err, ERRBIT_NONPHYSICAL);  // non-positive or NaN: reported, not fixed
}

// calcGrad, :186-252: per cell over its faces in ascending edge order, the
// unreconstructed centre states and the implicit method's ghosts.
__global__ void __launch_bounds__(256) k_imp_grad(const ImpCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nc) return;
    const int nc = c.nc;
    const Prim<double> q = load_prim(c.W, i);
    double g[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i], e = f >> 1;
        const bool side2 = f & 1;
        const double nx = c.nx[e], ny = c.ny[e], l = c.l[e];
        Prim<double> o;
        if (e < c.n_int) o = load_prim(c.W, side2 ? c.ec1[e] : c.ec2[e]);
        else o = imp_ghost(c.bnds[c.ebnd[e]], q, nx, ny, imat(c, i).M);
        grad_face(g, q, o, nx, ny, l, side2);
    }
    const double s = c.S[i], y = c.invS[i];
#pragma unroll
    for (int m = 0; m < 8; m++) g[m] = div_rn(g[m], s, y);
    st8(c.G, i, g);
}

// calcRoeAverage (:408-429) over roe_orig (src/global.cpp:407-441) with W = 0:
// the W terms add +0 to sums of squares and change no bit, so they are left out.
struct Roe { double r, u, v, p, E, cz; };
__device__ __forceinline__ Roe roe_average(const Prim<double>& L, const Prim<double>& R, double GAM) {
    const double AGAM = (GAM - 1.0);
    const double fSB = sqrt(L.r), fSE = sqrt(R.r);
    const double fS_ = 1.0 / (fSB + fSE);
    Roe a;
    a.r = fSB * fSE;
    a.u = (fSB * L.u + fSE * R.u) * fS_;
    a.v = (fSB * L.v + fSE * R.v) * fS_;
    const double EB = L.p / (L.r * AGAM), EE = R.p / (R.r * AGAM);
    const double HB = EB + (L.u * L.u + L.v * L.v) * 0.5 + L.p / L.r;
    const double HE = EE + (R.u * R.u + R.v * R.v) * 0.5 + R.p / R.r;
    const double HI = (fSB * HB + fSE * HE) * fS_;
    a.p = (HI - (a.u * a.u + a.v * a.v) * 0.5) * a.r * (GAM - 1.0) / GAM;
    const double e = a.p / (a.r * AGAM);
    a.cz = sqrt(GAM * a.p / a.r);
    a.E = e + 0.5 * (a.u * a.u + a.v * a.v);
    return a;
}

// The two Gauss-point fluxes of an edge times l/2 (run's loop, :612-633): interior
// faces reconstruct linearly from both centres (reconstruct(iFace, pL, pR, p),
// :444-476), boundary faces take the centre state and its ghost.
template <int FLUX>
__global__ void __launch_bounds__(256) k_imp_flux(const ImpCase c) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    const int ne = c.ne;
    const int c1 = c.ec1[e];
    const double nx = c.nx[e], ny = c.ny[e], l = c.l[e];
    const double GAM = c.gam_flux;
    const Prim<double> qL = load_prim(c.W, c1);
    double fs[4] = {0.0, 0.0, 0.0, 0.0};
    bool hit = false;
    if (e < c.n_int) {
        const int c2 = c.ec2[e];
        const Prim<double> qR = load_prim(c.W, c2);
        double gL[8], gR[8];
        ld8(c.G, c1, gL);
        ld8(c.G, c2, gR);
#pragma unroll
        for (int gp = 0; gp < 2; gp++) {
            Prim<double> pL = qL, pR = qR;
            reconstruct<double, RECON_LINEAR>(pL, gL, c.dl[(4 * gp) * ne + e], c.dl[(4 * gp + 1) * ne + e], qL);
            reconstruct<double, RECON_LINEAR>(pR, gR, c.dl[(4 * gp + 2) * ne + e], c.dl[(4 * gp + 3) * ne + e], qR);
            double f[4];
            if constexpr (FLUX == FLUX_LAX) flux_lax(f, pL, pR, nx, ny, GAM, c.ig1_flux);
            else hit |= flux_godunov<double, false>(f, pL, pR, nx, ny, c.rg_flux, c.newton_cap);
            fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
        }
    } else {  // both Gauss points see the same centre state and ghost
        const Prim<double> pR = imp_ghost(c.bnds[c.ebnd[e]], qL, nx, ny, imat(c, c1).M);
        double f[4];
        if constexpr (FLUX == FLUX_LAX) flux_lax(f, qL, pR, nx, ny, GAM, c.ig1_flux);
        else hit |= flux_godunov<double, false>(f, qL, pR, nx, ny, c.rg_flux, c.newton_cap);
        fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
        fs[0] = fs[0] + f[0]; fs[1] = fs[1] + f[1]; fs[2] = fs[2] + f[2]; fs[3] = fs[3] + f[3];
    }
    if (hit) atomicOr(c.err, ERRBIT_NEWTON_CAP);
    const double lh = 0.5 * l;  // right4 -= 0.5*l*fr, :623-633
    st4(c.F, e, fs[0] * lh, fs[1] * lh, fs[2] * lh, fs[3] * lh);
    // calcRoeAverage of the edge's centre states (cellL = c1, cellR = c2 or the ghost,
    // :553-554), for both cells' block rows
    const Prim<double> cR = e < c.n_int ? load_prim(c.W, c.ec2[e]) : imp_ghost(c.bnds[c.ebnd[e]], qL, nx, ny, imat(c, c1).M);
    const Roe a = roe_average(qL, cR, GAM);
    st4(c.R, e, a.u, a.v, a.cz, a.E + a.p / a.r);  // H of eigenValues' callers, :565
}

// (s * 0.5) * l as s * (0.5 l): halving is exact for |s| >= 2^-1021 (exponent field >= 2,
// decided on the integer pipe) and so is 0.5 l, so both round the same real number;
// a zero gives the same signed zero; smaller nonzero s take the two products (out of line,
// so that the common path is not evaluated beside them).
static __device__ __noinline__ double mul_half_l_tiny(double s, double l) { return (s * 0.5) * l; }
__device__ __forceinline__ double mul_half_l(double s, double hl, double l) {
    const long long b = __double_as_longlong(s);
    if (__builtin_expect(((b >> 52) & 0x7ff) >= 2 || (b << 1) == 0, 1)) return s * hl;  // (zeros: +-0 either way)
    return mul_half_l_tiny(s, l);
}
// 0.0 + x: x, with -0 turned into +0 (on the integer pipe)
__device__ __forceinline__ double plus_zero(double x) {
    return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}

// One face's 0.5 l R diag(lam+-) L (eigenValues / rightEigenVector / leftEigenVector /
// calcAP / calcAM, :335-406, scaled by l in run, :572-600) from the Roe state (u, v, c,
// H), with the normal (nx, ny) of the side being assembled. The reference forms
// R diag(lam+) and R diag(lam-) as full 4x4 products and multiplies each by L, summing
// four products from 0 per entry. An entry of R diag(lam+) is R[i][k] lam+_k or zero, and
// a zero term never changes such a sum (started from +0 it cannot become -0), so column k
// contributes to A+ only where lam_k > 0 and to A- only where lam_k < 0, in the
// reference's order of k: the same bits with half the products.
// Adds A+ into dg (the cell's diagonal block; first: dg holds nothing yet, the sums start
// from 0); returns A- in am.
template <bool FIRST>
__device__ __forceinline__ void face_jacobians(double u, double v, double c, double H, double GAM, double nx,
                                               double ny, double l, double* dg, double* am) {
    const double hl = 0.5 * l;
    const double qn = u * nx + v * ny;
    const double q2 = u * u + v * v;
    const double lx = -ny, ly = nx;
    const double ql = u * lx + v * ly;
    const double g1 = GAM - 1.0, c2 = c * c;
    // the quotients of leftEigenVector, each correctly rounded (div_rn equals '/')
    const double yc2 = 1.0 / c2, yc = 1.0 / c;
    const double A0 = div_rn(0.5 * q2 * g1, c2, yc2);
    const double B0 = div_rn(qn, c, yc);
    const double Cu = div_rn(g1 * u, c2, yc2);
    const double Dn = div_rn(nx, c, yc);
    const double Ev = div_rn(g1 * v, c2, yc2);
    const double Fn = div_rn(ny, c, yc);
    const double G0 = div_rn(0.5 * g1, c2, yc2);
    const double Hg = div_rn(g1, c2, yc2);
    const double L[16] = {0.5 * (A0 + B0), -0.5 * (Cu + Dn), -0.5 * (Ev + Fn), G0,
                          1 - A0,          Cu,               Ev,               neg_if(Hg, true),
                          0.5 * (A0 - B0), -0.5 * (Cu - Dn), -0.5 * (Ev - Fn), G0,
                          neg_if(ql, true), lx,              ly,               0.0};
    const double lam[4] = {qn - c, qn, qn + c, qn};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double Rr[4];
        if (i == 0) { Rr[0] = 1.0; Rr[1] = 1.0; Rr[2] = 1.0; Rr[3] = 0.0; }
        if (i == 1) { Rr[0] = u - c * nx; Rr[1] = u; Rr[2] = u + c * nx; Rr[3] = lx; }
        if (i == 2) { Rr[0] = v - c * ny; Rr[1] = v; Rr[2] = v + c * ny; Rr[3] = ly; }
        if (i == 3) { Rr[0] = H - qn * c; Rr[1] = q2 / 2; Rr[2] = H + qn * c; Rr[3] = ql; }
        double sp[4] = {0.0, 0.0, 0.0, 0.0}, sm[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const double t = Rr[k] * lam[k];
            if (lam[k] > 0) {
#pragma unroll
                for (int j = 0; j < 4; j++) sp[j] = sp[j] + t * L[4 * k + j];
            } else if (lam[k] < 0) {
#pragma unroll
                for (int j = 0; j < 4; j++) sm[j] = sm[j] + t * L[4 * k + j];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const double ap = mul_half_l(sp[j], hl, l);
            dg[4 * i + j] = FIRST ? plus_zero(ap) : dg[4 * i + j] + ap;
            am[4 * i + j] = plus_zero(mul_half_l(sm[j], hl, l));
        }
    }
}

// One block row of the system per cell (run's edge loop, :541-634, gathered per
// cell in ascending edge order, and the diagonal S/cTau of :640-664): the Roe
// average of the face's two centre states, the spectral radius (steady), A+ into
// the diagonal block, A- as the face's block, and the right-hand side -sum F l/2.
__global__ void __launch_bounds__(128) k_imp_assemble(const ImpCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nc) return;
    const int nc = c.nc;
    const double GAM = c.gam_flux;
    double dg[16];
#pragma unroll
    for (int m = 0; m < 16; m++) dg[m] = 0.0;
    double rhs[4] = {0.0, 0.0, 0.0, 0.0};
    double lam = 0.0;
#pragma unroll 1
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i], e = f >> 1;
        const bool side2 = f & 1;
        double fe[4];
        ld4(c.F, e, fe);
#pragma unroll
        for (int m = 0; m < 4; m++) rhs[m] = rhs[m] + neg_if(fe[m], !side2);
        const double nx = c.nx[e], ny = c.ny[e], l = c.l[e];
        double a[4];  // the edge's Roe state (u, v, c, H), formed once by k_imp_flux
        ld4(c.R, e, a);
        if (c.steady) lam = lam + (sqrt(a[0] * a[0] + a[1] * a[1]) + a[2]) * l;
        double am[16];
        if (k == 0) face_jacobians<true>(a[0], a[1], a[2], a[3], GAM, neg_if(nx, side2), neg_if(ny, side2), l, dg, am);
        else face_jacobians<false>(a[0], a[1], a[2], a[3], GAM, neg_if(nx, side2), neg_if(ny, side2), l, dg, am);
        const bool inner = e < c.n_int;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            double2* o = reinterpret_cast<double2*>(c.O + oblk(nc, i, k, 0, q));
            o[0] = inner ? make_double2(am[q], am[4 + q]) : make_double2(0.0, 0.0);
            o[1] = inner ? make_double2(am[8 + q], am[12 + q]) : make_double2(0.0, 0.0);
        }
    }
    const double S = c.S[i];
    double tau;
    if (c.steady) {
        tau = 2.0 * (*c.cfl) * S / (lam + 1.0e-100);
        c.ctau[i] = tau;
    } else {
        tau = c.ctau[i];
    }
    const double sd = S / tau;
#pragma unroll
    for (int m = 0; m < 16; m++) dg[m] = (m % 5) == 0 ? dg[m] + sd : plus_zero(dg[m]);  // + 0.0 off the diagonal
#pragma unroll
    for (int q = 0; q < 4; q++) {
        double2* d = reinterpret_cast<double2*>(c.D + dblk(nc, i, 0, q));
        d[0] = make_double2(dg[q], dg[4 + q]);
        d[1] = make_double2(dg[8 + q], dg[12 + q]);
    }
    st4(c.b, i, rhs[0], rhs[1], rhs[2], rhs[3]);
}

__device__ __forceinline__ bool solve_ok(const GmresCtl* g) { return g->final_ && !g->restart && g->status == 0; }

// smoothingDelta, :790-808, for the four components at once (each pass reads and
// writes one component only): x2 = (x + a sum_nb x_nb) / (1 + a n_nb) over the
// unlimited neighbours in ascending edge order. (The reference indexes its
// neighbour sums with 4 i + shift instead of i, past their end; the sums of cell i
// are the evident intent and what is used here.)
__global__ void __launch_bounds__(256) k_imp_smooth(const ImpCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nc || !solve_ok(c.ctl)) return;
    const int nc = c.nc;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    int n = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i], e = f >> 1;
        if (e >= c.n_int) continue;
        const int j = (f & 1) ? c.ec1[e] : c.ec2[e];
        if (c.flags[j] & 0x2u) continue;
        double xj[4];
        ld4(c.x, j, xj);
        for (int m = 0; m < 4; m++) s[m] = s[m] + xj[m];
        n++;
    }
    double xi[4];
    ld4(c.x, i, xi);
    const double a = c.smoothing_par;
    const double den = 1.0 + a * (double)n;
    st4(c.x2, i, (xi[0] + a * s[0]) / den, (xi[1] + a * s[1]) / den, (xi[2] + a * s[2]) / den,
        (xi[3] + a * s[3]) / den);
}

// The update of a solved system with the limits, :675-692.
__global__ void __launch_bounds__(256) k_imp_update(const ImpCase c, const double* __restrict__ dx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = solve_ok(c.ctl);
    bool lim = false;
    if (i < c.nc && ok && !(c.flags[i] & 0x2u)) {
        const int nc = c.nc;
        double d[4];
        ld4(dx, i, d);
        double U0 = c.A[i] + d[0], U1 = c.A[nc + i] + d[1], U2 = c.A[2 * nc + i] + d[2], U3 = c.A[3 * nc + i] + d[3];
        Prim<double> p = cons2prim<double>(U0, U1, U2, U3, imat(c, i).gm1);
        bool f = false;
        if (p.r > c.lim_rmax) { p.r = c.lim_rmax; f = true; }
        if (p.r < c.lim_rmin) { p.r = c.lim_rmin; f = true; }
        if (fabs(p.u) > c.lim_umax) { p.u = c.lim_umax * p.u / fabs(p.u); f = true; }
        if (fabs(p.v) > c.lim_umax) { p.v = c.lim_umax * p.v / fabs(p.v); f = true; }
        if (p.p > c.lim_pmax) { p.p = c.lim_pmax; f = true; }
        if (p.p < c.lim_pmin) { p.p = c.lim_pmin; f = true; }
        if (f) {  // par.e = p/((__GAM-1) r), convertParToCons
            const double e = p.p / ((1.4 - 1) * p.r);
            U0 = p.r;
            U1 = p.r * p.u;
            U2 = p.r * p.v;
            U3 = p.r * (e + 0.5 * (p.u * p.u + p.v * p.v));
            c.flags[i] |= 0x2u;
        }
        c.A[i] = U0; c.A[nc + i] = U1; c.A[2 * nc + i] = U2; c.A[3 * nc + i] = U3;
    }
    if (i < c.nc && ok) lim = (c.flags[i] & 0x2u) != 0;
    if (__syncthreads_or(lim) && threadIdx.x == 0) atomicAdd(c.n_lim, 1);
}

// FVM_TVD_IMPLICIT::remediateLimCells, :740-780: flagged cells in original order,
// one after another; the area-weighted mean of the cells across their faces, taken
// when those areas sum to at least TAU^2; flag aging.
__global__ void __launch_bounds__(1024) k_imp_remediate(const ImpCase c) {
    __shared__ int list[1024];
    __shared__ int cnt;
    __shared__ int wsum[32];
    const int nc = c.nc;
    if (*c.n_lim == 0 || !solve_ok(c.ctl)) return;
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
                    const int f = c.face[q * nc + ci], e = f >> 1;
                    const int j = (f & 1) ? c.ec1[e] : c.ec2[e];
                    if (j >= 0) {
                        const double s = c.S[j];
                        S += s;
                        a0 += c.A[j] * s; a1 += c.A[nc + j] * s; a2 += c.A[2 * nc + j] * s; a3 += c.A[3 * nc + j] * s;
                    }
                }
                if (S >= c.tau_xml * c.tau_xml) {
                    c.A[ci] = a0 / S; c.A[nc + ci] = a1 / S; c.A[2 * nc + ci] = a2 / S; c.A[3 * nc + ci] = a3 / S;
                }
                unsigned f = c.flags[ci] + 0x010000u;
                if (f & 0x200000u) f &= 0x001110u;
                c.flags[ci] = f;
            }
        }
        __syncthreads();
    }
}

// getLimitedCellsCount, :782-788
__global__ void __launch_bounds__(256) k_imp_count(const ImpCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lim = i < c.nc && (c.flags[i] & 0x2u);
    const int n = __syncthreads_count(lim);
    if (threadIdx.x == 0 && n && solve_ok(c.ctl)) atomicAdd(&c.ctl->n_lim, n);
}

__global__ void k_imp_post_begin(const ImpCase c) {
    *c.n_lim = 0;
    c.ctl->n_lim = 0;
}

// storage -> reference cell order of the block system: which 0 = D (16 per cell),
// 1 = O (48 per cell), 2 = b (4 per cell)
__global__ void __launch_bounds__(256) k_imp_permute(const ImpCase c, double* __restrict__ dst, int which) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.nc) return;
    const int i = c.iperm[o], nc = c.nc;
    if (which == 0)
        for (int m = 0; m < 16; m++) dst[16 * (size_t)o + m] = c.D[dblk(nc, i, m >> 2, m & 3)];
    else if (which == 1)
        for (int m = 0; m < 48; m++) dst[48 * (size_t)o + m] = c.O[oblk(nc, i, m >> 4, (m >> 2) & 3, m & 3)];
    else
        for (int m = 0; m < 4; m++) dst[4 * (size_t)o + m] = c.b[4 * (size_t)i + m];
}

inline int blocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void imp_launch_prims(const ImpCase& c, cudaStream_t s) { k_imp_prims<<<blocks(c.nc, 256), 256, 0, s>>>(c); }
void imp_launch_grad(const ImpCase& c, cudaStream_t s) { k_imp_grad<<<blocks(c.nc, 256), 256, 0, s>>>(c); }
void imp_launch_flux(const ImpCase& c, cudaStream_t s) {
    if (c.flux == FLUX_LAX) k_imp_flux<FLUX_LAX><<<blocks(c.ne, 256), 256, 0, s>>>(c);
    else k_imp_flux<FLUX_GODUNOV><<<blocks(c.ne, 256), 256, 0, s>>>(c);
}
void imp_launch_assemble(const ImpCase& c, cudaStream_t s) {
    k_imp_assemble<<<blocks(c.nc, 128), 128, 0, s>>>(c);
}
void imp_launch_post(const ImpCase& c, cudaStream_t s) {
    k_imp_post_begin<<<1, 1, 0, s>>>(c);
    const double* dx = c.x;
    if (c.smoothing) {
        k_imp_smooth<<<blocks(c.nc, 256), 256, 0, s>>>(c);
        dx = c.x2;
    }
    k_imp_update<<<blocks(c.nc, 256), 256, 0, s>>>(c, dx);
    k_imp_remediate<<<1, 1024, 0, s>>>(c);
    k_imp_count<<<blocks(c.nc, 256), 256, 0, s>>>(c);
}
void imp_launch_permute_blocks(const ImpCase& c, double* dst, int which, cudaStream_t s) {
    k_imp_permute<<<blocks(c.nc, 256), 256, 0, s>>>(c, dst, which);
}

}  // namespace cfd2d
