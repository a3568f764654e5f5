// Discrete adjoint of the FP64 step (built with -fmad=false, like the forward
// FP64 kernels, so every branch decision it recomputes matches the forward's).
//
// Per Runge-Kutta stage s, with stage input X_s and residual R(X_s), the
// forward computes t_s = X_s + cfl * R(X_s). Backward, given the adjoint t_bar
// of t_s and mu = cfl * t_bar:
//   k_adj_flux   per edge: F_bar = mu_c2 - mu_c1 (the reference's -=/+=), the
//                VJP of both Gauss-point fluxes, reconstructions and ghost
//                states -> adjoints of the two cells' primitives and gradients
//   k_adj_gather per cell: sum of its faces' contributions (fixed order)
//   k_adj_cell   per cell: VJP of the Green-Gauss gradients (own and the three
//                neighbours' gradient adjoints), of the boundary ghosts and of
//                convertConsToPar; X_bar = t_bar + (dR/dX)^T mu; the scheme's
//                stage algebra gives the previous stage's t_bar
// No atomics: every sum is a gather in a fixed order.
#include "adjoint.cuh"

namespace cfd2d {


namespace {

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ Prim<double> zero_prim() {
    Prim<double> z;
    z.r = 0; z.u = 0; z.v = 0; z.p = 0;
    return z;
}

template <int FLUX>
__device__ __forceinline__ void vjp_flux(const Prim<double>& L, const Prim<double>& R, double nx, double ny,
                                         double GAM, const double* fb, Prim<double>& Lb, Prim<double>& Rb) {
    if (FLUX == FLUX_HLLC) vjp_hllc(L, R, nx, ny, GAM, fb, Lb, Rb);
    else vjp_lax(L, R, nx, ny, GAM, fb, Lb, Rb);
}

template <int FLUX, int RECON>
__global__ void __launch_bounds__(256) k_adj_flux(const DevCase c, const AdjCase a) {
    const int ne = c.ne;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double* W = c.W64;
    const double* G = c.G64;
    const double* DL = c.dl;
    const double nx = c.nx[e], ny = c.ny[e], l = c.l[e];
    const double GAM = c.gam_flux;
    const int c1 = c.ec1[e];
    const bool inner = e < c.n_int;
    const int c2 = inner ? c.ec2[e] : -1;
    const Prim<double> qL = load_prim(W, c1);
    Prim<double> qR = qL, gc = qL;
    DevBnd b{};
    double Tc = 0, M = 0, gm1 = 0, Cv = 0;
    double fb[4];
    {
        double m1[4], m2[4] = {0, 0, 0, 0};
        ld4(a.mu, c1, m1);
        if (inner) ld4(a.mu, c2, m2);
        // F = (sum over Gauss points of f) * l/2; R_c1 -= F, R_c2 += F
        const double lh = l * 0.5 * (RECON == RECON_NONE ? 2.0 : 1.0);
        for (int k = 0; k < 4; k++) fb[k] = (m2[k] - m1[k]) * lh;
    }
    if (inner) {
        qR = load_prim(W, c2);
    } else {
        b = c.bnds[c.ebnd[e]];
        const DevMat mt = mat_of(c, c1);
        gm1 = mt.gm1; Cv = mt.Cv; M = mt.M;
        Tc = temperature(qL, gm1, Cv);
        if (RECON == RECON_MINMOD) gc = ghost_state(b, qL, Tc, nx, ny, M);
    }
    Prim<double> q1b = zero_prim(), q2b = zero_prim(), gcb = zero_prim();
    double g1b[8] = {0}, g2b[8] = {0}, bp[4] = {0, 0, 0, 0}, Tcb = 0;
    const int ngp = RECON == RECON_NONE ? 1 : 2;
#pragma unroll 1
    for (int gp = 0; gp < ngp; gp++) {
        Prim<double> pL = qL, pR = qR;
        double aL[4] = {0, 0, 0, 0}, aR[4] = {0, 0, 0, 0};
        double dxL = 0, dyL = 0, dxR = 0, dyR = 0;
        if (RECON != RECON_NONE) {
            double g[8];
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
        Prim<double> pLb = zero_prim(), pRb = zero_prim();
        vjp_flux<FLUX>(pL, pR, nx, ny, GAM, fb, pLb, pRb);
        if (!inner) vjp_ghost(b, pL, Tc, nx, ny, M, pRb, pLb, Tcb, bp);
        if (RECON == RECON_NONE) {
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
        o[0] += bp[0]; o[1] += bp[1]; o[2] += bp[2]; o[3] += bp[3];
    }
    double* o = a.eq + 24 * (size_t)e;
    o[0] = q1b.r; o[1] = q1b.u; o[2] = q1b.v; o[3] = q1b.p;
    for (int k = 0; k < 8; k++) o[4 + k] = g1b[k];
    o[12] = q2b.r; o[13] = q2b.u; o[14] = q2b.v; o[15] = q2b.p;
    for (int k = 0; k < 8; k++) o[16 + k] = g2b[k];
}

__global__ void __launch_bounds__(256) k_adj_gather(const DevCase c, const AdjCase a) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double q[4] = {0, 0, 0, 0}, g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const double* s = a.eq + 24 * (size_t)(f >> 1) + ((f & 1) ? 12 : 0);
        for (int m = 0; m < 4; m++) q[m] += s[m];
        for (int m = 0; m < 8; m++) g[m] += s[4 + m];
    }
    st4(a.qbar, i, q[0], q[1], q[2], q[3]);
    st8(a.gbar, i, g);
}

// coef_t / coef_acc: the scheme's stage algebra (the previous stage's t_bar and
// the step input's share); first: this is stage 0, write the step's lambda.
__global__ void __launch_bounds__(256) k_adj_cell(const DevCase c, const AdjCase a, double coef_t, double coef_acc,
                                                  int first) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const DevMat mt = mat_of(c, i);
    const double U[4] = {a.X[i], a.X[nc + i], a.X[2 * nc + i], a.X[3 * nc + i]};
    const Prim<double> q = load_prim(c.W64, i);
    double qbv[4];
    ld4(a.qbar, i, qbv);
    Prim<double> qb;
    qb.r = qbv[0]; qb.u = qbv[1]; qb.v = qbv[2]; qb.p = qbv[3];
    double gi[8];
    ld8(a.gbar, i, gi);
    const double iSi = c.invS[i];
    double Tcb = 0;
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i];
        const int e = f >> 1;
        const bool side2 = f & 1;
        const double nx = c.nx[e], ny = c.ny[e], l = c.l[e];
        const double wi = (side2 ? -0.5 : 0.5) * l * iSi;
        // d g_i / d q_i and d g_i / d (neighbour or ghost): the same weight
        const double s0 = wi * (nx * gi[0] + ny * gi[1]), s1 = wi * (nx * gi[2] + ny * gi[3]);
        const double s2 = wi * (nx * gi[4] + ny * gi[5]), s3 = wi * (nx * gi[6] + ny * gi[7]);
        qb.r += s0; qb.p += s1; qb.u += s2; qb.v += s3;
        const int j = side2 ? c.ec1[e] : c.ec2[e];
        if (j >= 0) {  // the neighbour's gradient uses this cell's value with the opposite orientation
            double gj[8];
            ld8(a.gbar, j, gj);
            const double wj = (side2 ? 0.5 : -0.5) * l * c.invS[j];
            qb.r += wj * (nx * gj[0] + ny * gj[1]);
            qb.p += wj * (nx * gj[2] + ny * gj[3]);
            qb.u += wj * (nx * gj[4] + ny * gj[5]);
            qb.v += wj * (nx * gj[6] + ny * gj[7]);
        } else {  // boundary face: the ghost of the unreconstructed centre state
            const DevBnd b = c.bnds[c.ebnd[e]];
            const double Tc = temperature(q, mt.gm1, mt.Cv);
            Prim<double> ob;
            ob.r = s0; ob.p = s1; ob.u = s2; ob.v = s3;
            double bp[4] = {0, 0, 0, 0};
            vjp_ghost(b, q, Tc, nx, ny, mt.M, ob, qb, Tcb, bp);
            double* o = a.eb2 + 4 * (size_t)(e - c.n_int);
            o[0] += bp[0]; o[1] += bp[1]; o[2] += bp[2]; o[3] += bp[3];
        }
    }
    if (Tcb != 0.0) vjp_temperature(q, mt.gm1, mt.Cv, Tcb, qb);
    double V[4] = {0, 0, 0, 0};
    vjp_cons2prim(U, mt.gm1, qb, V);
    double ux[4];
    for (int k = 0; k < 4; k++) ux[k] = a.tb[k * nc + i] + V[k];
    if (first) {
        for (int k = 0; k < 4; k++) a.lam[k * nc + i] = a.acc[k * nc + i] + ux[k];
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

// Start of a step backward: t_bar = coef_t * lambda, acc = coef_acc * lambda, mu = cfl t_bar.
__global__ void __launch_bounds__(256) k_adj_step_start(const DevCase c, const AdjCase a, double coef_t,
                                                        double coef_acc) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double cf = c.cfl[i];
    double t[4];
    for (int k = 0; k < 4; k++) {
        const double l = a.lam[k * nc + i];
        t[k] = coef_t * l;
        a.tb[k * nc + i] = t[k];
        a.acc[k * nc + i] = coef_acc * l;
    }
    st4(a.mu_out, i, cf * t[0], cf * t[1], cf * t[2], cf * t[3]);
}

// dbnd[b] = sum over boundary edges of boundary b of their running sums (flux and
// gradient paths, all stages and steps), in a fixed order.
__global__ void __launch_bounds__(256) k_adj_bnd_reduce(const DevCase c, const AdjCase a) {
    __shared__ double sh[4][256];
    const int nb = c.ne - c.n_int;
    for (int bi = 0; bi < a.n_bnd; bi++) {
        double s[4] = {0, 0, 0, 0};
        for (int k = threadIdx.x; k < nb; k += blockDim.x) {
            if (c.ebnd[c.n_int + k] != bi) continue;
            for (int m = 0; m < 4; m++) s[m] += a.eb[4 * (size_t)k + m] + a.eb2[4 * (size_t)k + m];
        }
        for (int m = 0; m < 4; m++) sh[m][threadIdx.x] = s[m];
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w)
                for (int m = 0; m < 4; m++) sh[m][threadIdx.x] += sh[m][threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0)
            for (int m = 0; m < 4; m++) a.dbnd[4 * bi + m] = sh[m][0];
        __syncthreads();
    }
}

// Objective J = sum_i w_i (p_i - p_ref)^2 (kind 0) or sum_i w_i rho_i^2 (kind 1):
// fixed-partition partial sums.
__global__ void __launch_bounds__(256) k_objective(const DevCase c, const double* __restrict__ w, int kind,
                                                   double p_ref, double* __restrict__ partial) {
    const int nc = c.nc;
    const long chunk = ((long)nc + gridDim.x - 1) / gridDim.x;
    const long b0 = blockIdx.x * chunk, b1 = min((long)nc, b0 + chunk);
    double s = 0.0;
    for (long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        if (w[i] == 0.0) continue;
        const DevMat mt = mat_of(c, (int)i);
        const Prim<double> q = cons2prim<double>(c.A[i], c.A[nc + i], c.A[2 * nc + i], c.A[3 * nc + i], mt.gm1);
        const double d = kind == 0 ? q.p - p_ref : q.r;
        s += w[i] * d * d;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(256) k_objective_grad(const DevCase c, const AdjCase a, const double* __restrict__ w,
                                                        int kind, double p_ref) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double V[4] = {0, 0, 0, 0};
    if (w[i] != 0.0) {
        const DevMat mt = mat_of(c, i);
        const double U[4] = {c.A[i], c.A[nc + i], c.A[2 * nc + i], c.A[3 * nc + i]};
        const Prim<double> q = cons2prim<double>(U[0], U[1], U[2], U[3], mt.gm1);
        Prim<double> qb = zero_prim();
        if (kind == 0) qb.p = 2.0 * w[i] * (q.p - p_ref);
        else qb.r = 2.0 * w[i] * q.r;
        vjp_cons2prim(U, mt.gm1, qb, V);
    }
    for (int k = 0; k < 4; k++) a.lam[k * nc + i] = V[k];
}

}  // namespace

void launch_adj_flux(const DevCase& c, const AdjCase& a, int flux, int recon, cudaStream_t s) {
    const int g = nblk(c.ne, 256);
    if (flux == FLUX_HLLC) {
        if (recon == RECON_NONE) k_adj_flux<FLUX_HLLC, RECON_NONE><<<g, 256, 0, s>>>(c, a);
        else if (recon == RECON_LINEAR) k_adj_flux<FLUX_HLLC, RECON_LINEAR><<<g, 256, 0, s>>>(c, a);
        else k_adj_flux<FLUX_HLLC, RECON_MINMOD><<<g, 256, 0, s>>>(c, a);
    } else {
        if (recon == RECON_NONE) k_adj_flux<FLUX_LAX, RECON_NONE><<<g, 256, 0, s>>>(c, a);
        else if (recon == RECON_LINEAR) k_adj_flux<FLUX_LAX, RECON_LINEAR><<<g, 256, 0, s>>>(c, a);
        else k_adj_flux<FLUX_LAX, RECON_MINMOD><<<g, 256, 0, s>>>(c, a);
    }
}
void launch_adj_gather(const DevCase& c, const AdjCase& a, cudaStream_t s) {
    k_adj_gather<<<nblk(c.nc, 256), 256, 0, s>>>(c, a);
}
void launch_adj_cell(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, int first, cudaStream_t s) {
    k_adj_cell<<<nblk(c.nc, 256), 256, 0, s>>>(c, a, coef_t, coef_acc, first);
}
void launch_adj_step_start(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, cudaStream_t s) {
    k_adj_step_start<<<nblk(c.nc, 256), 256, 0, s>>>(c, a, coef_t, coef_acc);
}
void launch_adj_bnd_reduce(const DevCase& c, const AdjCase& a, cudaStream_t s) {
    if (c.ne > c.n_int && a.n_bnd > 0) k_adj_bnd_reduce<<<1, 256, 0, s>>>(c, a);
}
void launch_objective(const DevCase& c, const double* w, int kind, double p_ref, double* partial, int nblocks,
                      cudaStream_t s) {
    k_objective<<<nblocks, 256, 0, s>>>(c, w, kind, p_ref, partial);
}
void launch_objective_grad(const DevCase& c, const AdjCase& a, const double* w, int kind, double p_ref,
                           cudaStream_t s) {
    k_objective_grad<<<nblk(c.nc, 256), 256, 0, s>>>(c, a, w, kind, p_ref);
}

}  // namespace cfd2d
