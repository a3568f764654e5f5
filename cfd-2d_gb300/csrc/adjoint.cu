// Discrete adjoint: the FP64-face kernels (built with -fmad=false, like the
// forward FP64 kernels, so every branch decision they recompute matches the
// forward's), the per-cell kernels shared by both face precisions, and the
// precision dispatch. adjoint_mixed.cu instantiates the FP32-face kernels.
#define KT double
#define KFN(name) launch_##name##_fp64
#include "adj_inst.cuh"

namespace cfd2d {

void launch_adj_flux_mixed(const DevCase&, const AdjCase&, int, int, cudaStream_t);
void launch_flux_rec_mixed(const DevCase&, int, const FluxRec&, cudaStream_t);
void launch_adj_flux_rec_mixed(const DevCase&, const AdjCase&, int, const FluxRec&, cudaStream_t);
void launch_adj_gather_mixed(const DevCase&, const AdjCase&, cudaStream_t);
void launch_adj_cell_mixed(const DevCase&, const AdjCase&, double, double, int, cudaStream_t);

namespace {

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

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
        Prim<double> qb = zero_prim<double>();
        if (kind == 0) qb.p = 2.0 * w[i] * (q.p - p_ref);
        else qb.r = 2.0 * w[i] * q.r;
        vjp_cons2prim(U, mt.gm1, qb, V);
    }
    for (int k = 0; k < 4; k++) a.lam[k * nc + i] = V[k];
}

}  // namespace

void launch_adj_flux(const DevCase& c, const AdjCase& a, int flux, int recon, int precision, cudaStream_t s) {
    if (precision == PREC_MIXED) launch_adj_flux_mixed(c, a, flux, recon, s);
    else launch_adj_flux_fp64(c, a, flux, recon, s);
}
void launch_flux_rec(const DevCase& c, int recon, const FluxRec& r, int precision, cudaStream_t s) {
    if (precision == PREC_MIXED) launch_flux_rec_mixed(c, recon, r, s);
    else launch_flux_rec_fp64(c, recon, r, s);
}
void launch_adj_flux_rec(const DevCase& c, const AdjCase& a, int recon, const FluxRec& r, int precision,
                         cudaStream_t s) {
    if (precision == PREC_MIXED) launch_adj_flux_rec_mixed(c, a, recon, r, s);
    else launch_adj_flux_rec_fp64(c, a, recon, r, s);
}
void launch_adj_gather(const DevCase& c, const AdjCase& a, int precision, cudaStream_t s) {
    if (precision == PREC_MIXED) launch_adj_gather_mixed(c, a, s);
    else launch_adj_gather_fp64(c, a, s);
}
void launch_adj_cell(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, int first, int precision,
                     cudaStream_t s) {
    if (precision == PREC_MIXED) launch_adj_cell_mixed(c, a, coef_t, coef_acc, first, s);
    else launch_adj_cell_fp64(c, a, coef_t, coef_acc, first, s);
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
