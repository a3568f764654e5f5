// Adjoint kernels for one face precision; included once per precision by
// adjoint.cu (KT = double, with the forward FP64 kernels' -fmad=false) and
// adjoint_mixed.cu (KT = float, with the mixed kernels' flags), so every
// forward value the adjoint recomputes is the forward's own.
//
// Per Runge-Kutta stage s, with stage input X_s and residual R(X_s), the
// forward computes t_s = X_s + cfl * R(X_s). Backward, given the adjoint t_bar
// of t_s and mu = cfl * t_bar (FP64, per cell):
//   k_adj_flux   per edge: F_bar = mu_c2 - mu_c1 (the reference's -=/+=), the
//                VJP of both Gauss-point fluxes, reconstructions and ghost
//                states -> adjoints of the two cells' primitives and gradients
//   k_adj_gather per cell: sum of its faces' contributions (fixed order)
//   k_adj_cell   per cell: VJP of the Green-Gauss gradients (own and the three
//                neighbours' gradient adjoints), of the boundary ghosts and of
//                convertConsToPar; X_bar = t_bar + (dR/dX)^T mu in FP64; the
//                scheme's stage algebra gives the previous stage's t_bar
// Face-level products run in KT; everything accumulated per cell across stages
// and steps (t_bar, lambda, the boundary-parameter sums) is FP64. No atomics:
// every sum is a gather in a fixed order.
#pragma once
#include "adjoint.cuh"

namespace cfd2d {
namespace {

inline int adj_nblk(long n, int b) { return (int)((n + b - 1) / b); }

template <typename T, int FLUX, int RECON, int SIDE>
__device__ __forceinline__ void adj_flux_edge(const DevCase& c, const AdjCase& a, int e);
template <typename T, int FLUX, int RECON>
// FP32 faces: at most 128 registers (two 256-thread blocks' worth per SM), measured
// faster than the compiler's unconstrained choice; FP64 faces: unconstrained. With FP64 faces
// interior and boundary edges (stored last) run their own instantiations.
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 0) k_adj_flux(const DevCase c, const AdjCase a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    if constexpr (sizeof(T) == 8) {  // FP64 faces: no contraction, the same bits in either instantiation
        if (e < c.n_int) adj_flux_edge<T, FLUX, RECON, EDGE_INNER>(c, a, e);
        else adj_flux_edge<T, FLUX, RECON, EDGE_BOUNDARY>(c, a, e);
    } else {
        adj_flux_edge<T, FLUX, RECON, EDGE_ANY>(c, a, e);
    }
}
template <typename T, int FLUX, int RECON, int SIDE>
__device__ __forceinline__ void adj_flux_edge(const DevCase& c, const AdjCase& a, int e) {
    const int ne = c.ne;
    const T* W = W_of<T>(c);
    const T* G = G_of<T>(c);
    const T* DL = DL_of<T>(c);
    const T nx = NX_of<T>(c)[e], ny = NY_of<T>(c)[e], l = L_of<T>(c)[e];
    const T GAM = gam_of<T>(c), IG1 = ig1_of<T>(c);
    const int c1 = c.ec1[e];
    const bool inner = edge_inner<SIDE>(c, e);
    const int c2 = inner ? c.ec2[e] : -1;
    const Prim<T> qL = load_prim(W, c1);
    Prim<T> qR = qL, gc = qL;
    DevBnd b{};
    T Tc = T(0), M = T(0), gm1 = T(0), Cv = T(0);
    T fb[4];
    {
        double m1[4], m2[4] = {0, 0, 0, 0};
        ld4(a.mu, c1, m1);
        if (inner) ld4(a.mu, c2, m2);
        // F = (sum over Gauss points of f) * l/2; R_c1 -= F, R_c2 += F. The difference is
        // formed in FP64 and rounded once into the face precision.
        const double lh = to_wide(l) * (RECON == RECON_NONE ? 1.0 : 0.5);
        for (int k = 0; k < 4; k++) fb[k] = to_face<T>((m2[k] - m1[k]) * lh);
    }
    if (inner) {
        qR = load_prim(W, c2);
    } else {
        b = c.bnds[c.ebnd[e]];
        const MatT<T> mt = matT_of<T>(c, c1);
        gm1 = mt.gm1; Cv = mt.Cv; M = mt.M;
        Tc = temperature(qL, gm1, Cv);
        if (RECON == RECON_MINMOD) gc = ghost_state(b, qL, Tc, nx, ny, M);
    }
    Prim<T> q1b = zero_prim<T>(), q2b = zero_prim<T>(), gcb = zero_prim<T>();
    T g1b[8], g2b[8], bp[4];
#pragma unroll
    for (int k = 0; k < 8; k++) { g1b[k] = acc0<T>(); g2b[k] = acc0<T>(); }
#pragma unroll
    for (int k = 0; k < 4; k++) bp[k] = acc0<T>();
    T Tcb = acc0<T>();
    const int ngp = RECON == RECON_NONE ? 1 : 2;
#pragma unroll 1
    for (int gp = 0; gp < ngp; gp++) {
        Prim<T> pL = qL, pR = qR;
        T aL[4] = {T(0), T(0), T(0), T(0)}, aR[4] = {T(0), T(0), T(0), T(0)};
        T dxL = T(0), dyL = T(0), dxR = T(0), dyR = T(0);
        if (RECON != RECON_NONE) {
            T g[8];
            dxL = DL[(4 * gp) * ne + e]; dyL = DL[(4 * gp + 1) * ne + e];
            ld8(G, c1, g);
            project<RECON>(g, dxL, dyL, aL);
            pL = recon_a<RECON>(qL, aL, inner ? qR : gc);
            if (inner) {
                dxR = DL[(4 * gp + 2) * ne + e]; dyR = DL[(4 * gp + 3) * ne + e];
                ld8(G, c2, g);
                project<RECON>(g, dxR, dyR, aR);
                pR = recon_a<RECON>(qR, aR, qL);
            }
        }
        if (!inner) pR = ghost_state(b, pL, Tc, nx, ny, M);
        Prim<T> pLb = zero_prim<T>(), pRb = zero_prim<T>();
        vjp_flux<FLUX>(pL, pR, nx, ny, GAM, IG1, fb, pLb, pRb);
        if (!inner) vjp_ghost(b, pL, Tc, nx, ny, M, pRb, pLb, Tcb, bp);
        if (RECON == RECON_NONE) {  // both Gauss points see the cell-centre states: one pass, twice the weight
            q1b.r += pLb.r; q1b.u += pLb.u; q1b.v += pLb.v; q1b.p += pLb.p;
            if (inner) { q2b.r += pRb.r; q2b.u += pRb.u; q2b.v += pRb.v; q2b.p += pRb.p; }
        } else if (inner) {
            vjp_reconstruct_a<RECON>(qL, aL, dxL, dyL, qR, pLb, q1b, g1b, q2b);
            vjp_reconstruct_a<RECON>(qR, aR, dxR, dyR, qL, pRb, q2b, g2b, q1b);
        } else {
            vjp_reconstruct_a<RECON>(qL, aL, dxL, dyL, gc, pLb, q1b, g1b, gcb);
        }
    }
    if (!inner) {
        if (RECON == RECON_MINMOD) vjp_ghost(b, qL, Tc, nx, ny, M, gcb, q1b, Tcb, bp);
        vjp_temperature(qL, gm1, Cv, Tcb, q1b);
        double* o = a.eb + 4 * (size_t)(e - c.n_int);  // this edge's own running sum over stages and steps
        o[0] += to_wide(bp[0]); o[1] += to_wide(bp[1]); o[2] += to_wide(bp[2]); o[3] += to_wide(bp[3]);
    }
    T* o = static_cast<T*>(a.eq) + 24 * (size_t)e;
    st4(o, 0, q1b.r, q1b.u, q1b.v, q1b.p);
    st8(o + 4, 0, g1b);
    st4(o + 12, 0, q2b.r, q2b.u, q2b.v, q2b.p);
    st8(o + 16, 0, g2b);
}

// The forward flux kernel of a recomputed stage that also keeps the evaluation's record
// (FluxRec: face states, sound speeds, minmod's branches) for k_adj_flux_rec. Compiled with
// the forward kernels' flags and the same code, so F is the forward's bit for bit.
template <typename T, int RECON>
__global__ void __launch_bounds__(128) k_flux_rec(const DevCase c, const FluxRec r) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    T out[4];
    flux_edge<T, FLUX_HLLC, RECON, true>(c, e, out, r);
    st4(F_of<T>(c), e, out[0], out[1], out[2], out[3]);
}

// k_adj_flux (HLLC) reading the forward's record of each Gauss point instead of
// recomputing the reconstruction, the ghost state, the sound speeds and minmod's
// branches: the same reverse operations on the same values, so the same bits.
template <typename T, int RECON, int SIDE>
__device__ __forceinline__ void adj_flux_rec_edge(const DevCase& c, const AdjCase& a, const FluxRec& r, int e);
template <typename T, int RECON>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 0) k_adj_flux_rec(const DevCase c, const AdjCase a,
                                                                              const FluxRec r) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    if constexpr (sizeof(T) == 8) {
        if (e < c.n_int) adj_flux_rec_edge<T, RECON, EDGE_INNER>(c, a, r, e);
        else adj_flux_rec_edge<T, RECON, EDGE_BOUNDARY>(c, a, r, e);
    } else {
        adj_flux_rec_edge<T, RECON, EDGE_ANY>(c, a, r, e);
    }
}
template <typename T, int RECON, int SIDE>
__device__ __forceinline__ void adj_flux_rec_edge(const DevCase& c, const AdjCase& a, const FluxRec& r, int e) {
    const int ne = c.ne;
    const T* DL = DL_of<T>(c);
    const T nx = NX_of<T>(c)[e], ny = NY_of<T>(c)[e], l = L_of<T>(c)[e];
    const T GAM = gam_of<T>(c), IG1 = ig1_of<T>(c);
    const int c1 = c.ec1[e];
    const bool inner = edge_inner<SIDE>(c, e);
    const int c2 = inner ? c.ec2[e] : -1;
    Prim<T> qL{};
    DevBnd b{};
    T Tc = T(0), M = T(0), gm1 = T(0), Cv = T(0);
    T fb[4];
    {
        double m1[4], m2[4] = {0, 0, 0, 0};
        ld4(a.mu, c1, m1);
        if (inner) ld4(a.mu, c2, m2);
        const double lh = to_wide(l) * (RECON == RECON_NONE ? 1.0 : 0.5);
        for (int k = 0; k < 4; k++) fb[k] = to_face<T>((m2[k] - m1[k]) * lh);
    }
    if (!inner) {
        qL = load_prim(W_of<T>(c), c1);
        b = c.bnds[c.ebnd[e]];
        const MatT<T> mt = matT_of<T>(c, c1);
        gm1 = mt.gm1; Cv = mt.Cv; M = mt.M;
        Tc = temperature(qL, gm1, Cv);
    }
    Prim<T> q1b = zero_prim<T>(), q2b = zero_prim<T>(), gcb = zero_prim<T>();
    T g1b[8], g2b[8], bp[4];
#pragma unroll
    for (int k = 0; k < 8; k++) { g1b[k] = acc0<T>(); g2b[k] = acc0<T>(); }
#pragma unroll
    for (int k = 0; k < 4; k++) bp[k] = acc0<T>();
    T Tcb = acc0<T>();
    const unsigned bits = RECON == RECON_MINMOD ? r.bits[e] : 0u;
    const int ngp = RECON == RECON_NONE ? 1 : 2;
#pragma unroll 1
    for (int gp = 0; gp < ngp; gp++) {
        const T* v = static_cast<const T*>(r.v) + (size_t)(10 * gp) * ne + e;
        const Prim<T> pL{v[0], v[ne], v[2 * (size_t)ne], v[3 * (size_t)ne]};
        const Prim<T> pR{v[4 * (size_t)ne], v[5 * (size_t)ne], v[6 * (size_t)ne], v[7 * (size_t)ne]};
        const T cL = v[8 * (size_t)ne], cR = v[9 * (size_t)ne];
        T dxL = T(0), dyL = T(0), dxR = T(0), dyR = T(0);
        if (RECON != RECON_NONE) {
            dxL = DL[(4 * gp) * ne + e]; dyL = DL[(4 * gp + 1) * ne + e];
            if (inner) { dxR = DL[(4 * gp + 2) * ne + e]; dyR = DL[(4 * gp + 3) * ne + e]; }
        }
        Prim<T> pLb = zero_prim<T>(), pRb = zero_prim<T>();
        vjp_hllc_c(pL, pR, cL, cR, nx, ny, GAM, IG1, fb, pLb, pRb);
        if (!inner) vjp_ghost(b, pL, Tc, nx, ny, M, pRb, pLb, Tcb, bp);
        if (RECON == RECON_NONE) {
            q1b.r += pLb.r; q1b.u += pLb.u; q1b.v += pLb.v; q1b.p += pLb.p;
            if (inner) { q2b.r += pRb.r; q2b.u += pRb.u; q2b.v += pRb.v; q2b.p += pRb.p; }
        } else if (inner) {
            vjp_reconstruct_code<RECON>(bits >> (16 * gp), dxL, dyL, pLb, q1b, g1b, q2b);
            vjp_reconstruct_code<RECON>(bits >> (16 * gp + 8), dxR, dyR, pRb, q2b, g2b, q1b);
        } else {
            vjp_reconstruct_code<RECON>(bits >> (16 * gp), dxL, dyL, pLb, q1b, g1b, gcb);
        }
    }
    if (!inner) {
        if (RECON == RECON_MINMOD) vjp_ghost(b, qL, Tc, nx, ny, M, gcb, q1b, Tcb, bp);
        vjp_temperature(qL, gm1, Cv, Tcb, q1b);
        double* o = a.eb + 4 * (size_t)(e - c.n_int);
        o[0] += to_wide(bp[0]); o[1] += to_wide(bp[1]); o[2] += to_wide(bp[2]); o[3] += to_wide(bp[3]);
    }
    T* o = static_cast<T*>(a.eq) + 24 * (size_t)e;
    st4(o, 0, q1b.r, q1b.u, q1b.v, q1b.p);
    st8(o + 4, 0, g1b);
    st4(o + 12, 0, q2b.r, q2b.u, q2b.v, q2b.p);
    st8(o + 16, 0, g2b);
}

// The three faces' contributions summed exactly (SumAcc): the primitive adjoint is
// rounded once into FP64 (it is summed again in k_adj_cell), the gradient adjoint
// into the face precision and divided by the cell's area (it only enters products there).
template <typename T>
__global__ void __launch_bounds__(256) k_adj_gather(const DevCase c, const AdjCase a) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    SumAcc<T> q[4], g[8];
    const T* eq = static_cast<const T*>(a.eq);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const T* s = eq + 24 * (size_t)(f >> 1) + ((f & 1) ? 12 : 0);
        T v[12];
        ld4(s, 0, v);
        ld8(s + 4, 0, v + 4);
#pragma unroll
        for (int m = 0; m < 4; m++) q[m].add(v[m]);
#pragma unroll
        for (int m = 0; m < 8; m++) g[m].add(v[4 + m]);
    }
    st4(a.qbar, i, q[0].value(), q[1].value(), q[2].value(), q[3].value());
    // kept divided by the cell's area: the Green-Gauss VJP (k_adj_cell) then needs no
    // per-face weights of its own and no products by 1/S
    const T iSi = invS_of<T>(c)[i];
    T gv[8];
#pragma unroll
    for (int m = 0; m < 8; m++) gv[m] = g[m].face() * iSi;
    st8(static_cast<T*>(a.gbar), i, gv);
}

// coef_t / coef_acc: the scheme's stage algebra (the previous stage's t_bar and
// the step input's share); first: this is stage 0, write the step's lambda and,
// with (coef_t, coef_acc) the last stage's coefficients, start the step before it
// (t_bar, acc and mu from lambda: what k_adj_step_start does for the first step).
template <typename T>
__global__ void __launch_bounds__(256) k_adj_cell(const DevCase c, const AdjCase a, double coef_t, double coef_acc,
                                                  int first) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const MatT<T> mt = matT_of<T>(c, i);
    const Prim<T> q = load_prim(W_of<T>(c), i);
    // h = the gradient adjoints divided by the area (k_adj_gather)
    const T* h = static_cast<const T*>(a.gbar);
    // the cell's primitive adjoint: the gathered FP64 value plus the sum of the
    // Green-Gauss products (r, u, v, p)
    SumAcc<T> qs[4];
    T Tcb = acc0<T>();
    Prim<T> qb = zero_prim<T>();  // ghost-path contributions (boundary faces only)
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const int e = f >> 1;
        const bool side2 = f & 1;
        const T nx = NX_of<T>(c)[e], ny = NY_of<T>(c)[e], l = L_of<T>(c)[e];
        // d g_i / d (neighbour or ghost value) = +-(l/2) n / S_i with n outward from c1; the
        // neighbour's gradient takes q_i with the opposite sign and its own 1/S_j. The own
        // value's direct terms, (1/S_i) sum_k (l_k/2) n_out,k over the three faces, are the
        // outward normals of a closed triangle weighted by their lengths: zero, and left out.
        const T w = neg_if(T(0.5) * l, side2);
        const T wx = w * nx, wy = w * ny;
        const int j = side2 ? c.ec1[e] : c.ec2[e];
        if (j >= 0) {
            T hj[8];
            ld8(h, j, hj);
            qs[0].add(-madd(wx * hj[0], wy, hj[1]));
            qs[3].add(-madd(wx * hj[2], wy, hj[3]));
            qs[1].add(-madd(wx * hj[4], wy, hj[5]));
            qs[2].add(-madd(wx * hj[6], wy, hj[7]));
        } else {  // boundary face: the ghost of the unreconstructed centre state
            T hi[8];
            ld8(h, i, hi);
            const T s0 = madd(wx * hi[0], wy, hi[1]), s1 = madd(wx * hi[2], wy, hi[3]);
            const T s2 = madd(wx * hi[4], wy, hi[5]), s3 = madd(wx * hi[6], wy, hi[7]);
            const DevBnd b = c.bnds[c.ebnd[e]];
            const T Tc = temperature(q, mt.gm1, mt.Cv);
            Prim<T> ob;
            ob.r = s0; ob.p = s1; ob.u = s2; ob.v = s3;
            T bp[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()};
            vjp_ghost(b, q, Tc, nx, ny, mt.M, ob, qb, Tcb, bp);
            double* o = a.eb2 + 4 * (size_t)(e - c.n_int);
            o[0] += to_wide(bp[0]); o[1] += to_wide(bp[1]); o[2] += to_wide(bp[2]); o[3] += to_wide(bp[3]);
        }
    }
    if (Tcb != T(0.0)) vjp_temperature(q, mt.gm1, mt.Cv, Tcb, qb);
    {
        double q0[4];
        ld4(a.qbar, i, q0);  // r, u, v, p
        qs[0].add(qb.r); qs[1].add(qb.u); qs[2].add(qb.v); qs[3].add(qb.p);
        qb.r = to_face<T>(q0[0] + qs[0].value());
        qb.u = to_face<T>(q0[1] + qs[1].value());
        qb.v = to_face<T>(q0[2] + qs[2].value());
        qb.p = to_face<T>(q0[3] + qs[3].value());
    }
    T V[4] = {acc0<T>(), acc0<T>(), acc0<T>(), acc0<T>()};
    vjp_cons2prim_q(q, mt.gm1, qb, V);
    double ux[4];
    for (int k = 0; k < 4; k++) ux[k] = a.tb[k * nc + i] + to_wide(V[k]);
    if (first) {  // lambda of the step input, and (coef_t, coef_acc = the last stage's) the next step's start
        const double cf = c.cfl[i];
        double t[4];
        for (int k = 0; k < 4; k++) {
            const double l = a.acc[k * nc + i] + ux[k];
            a.lam[k * nc + i] = l;
            t[k] = coef_t * l;
            a.tb[k * nc + i] = t[k];
            a.acc[k * nc + i] = coef_acc * l;
        }
        st4(a.mu_out, i, cf * t[0], cf * t[1], cf * t[2], cf * t[3]);
    } else {
        const double cf = c.cfl[i];
        double t[4];
        for (int k = 0; k < 4; k++) {
            t[k] = coef_t * ux[k];
            a.tb[k * nc + i] = t[k];
            a.acc[k * nc + i] += coef_acc * ux[k];
        }
        st4(a.mu_out, i, cf * t[0], cf * t[1], cf * t[2], cf * t[3]);
    }
}

template <int FLUX>
void adj_flux_by_recon(const DevCase& c, const AdjCase& a, int recon, cudaStream_t s) {
    const int g = adj_nblk(c.ne, 128);
    if (recon == RECON_NONE) k_adj_flux<KT, FLUX, RECON_NONE><<<g, 128, 0, s>>>(c, a);
    else if (recon == RECON_LINEAR) k_adj_flux<KT, FLUX, RECON_LINEAR><<<g, 128, 0, s>>>(c, a);
    else k_adj_flux<KT, FLUX, RECON_MINMOD><<<g, 128, 0, s>>>(c, a);
}
}  // namespace

void KFN(adj_flux)(const DevCase& c, const AdjCase& a, int flux, int recon, cudaStream_t s) {
    if (flux == FLUX_HLLC) adj_flux_by_recon<FLUX_HLLC>(c, a, recon, s);
    else adj_flux_by_recon<FLUX_LAX>(c, a, recon, s);
}
void KFN(flux_rec)(const DevCase& c, int recon, const FluxRec& r, cudaStream_t s) {
    // 128-thread blocks: at ~164 registers a thread, 256-thread blocks leave one block (8
    // warps) per SM, 128-thread blocks three (12 warps)
    const int g = adj_nblk(c.ne, 128);
    if (recon == RECON_NONE) k_flux_rec<KT, RECON_NONE><<<g, 128, 0, s>>>(c, r);
    else if (recon == RECON_LINEAR) k_flux_rec<KT, RECON_LINEAR><<<g, 128, 0, s>>>(c, r);
    else k_flux_rec<KT, RECON_MINMOD><<<g, 128, 0, s>>>(c, r);
}
void KFN(adj_flux_rec)(const DevCase& c, const AdjCase& a, int recon, const FluxRec& r, cudaStream_t s) {
    const int g = adj_nblk(c.ne, 128);
    if (recon == RECON_NONE) k_adj_flux_rec<KT, RECON_NONE><<<g, 128, 0, s>>>(c, a, r);
    else if (recon == RECON_LINEAR) k_adj_flux_rec<KT, RECON_LINEAR><<<g, 128, 0, s>>>(c, a, r);
    else k_adj_flux_rec<KT, RECON_MINMOD><<<g, 128, 0, s>>>(c, a, r);
}
void KFN(adj_gather)(const DevCase& c, const AdjCase& a, cudaStream_t s) {
    k_adj_gather<KT><<<adj_nblk(c.nc, 128), 128, 0, s>>>(c, a);
}
void KFN(adj_cell)(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, int first, cudaStream_t s) {
    k_adj_cell<KT><<<adj_nblk(c.nc, 128), 128, 0, s>>>(c, a, coef_t, coef_acc, first);
}

}  // namespace cfd2d
