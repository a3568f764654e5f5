// GMRES on the implicit method's block system (the reference calls HYPRE's GMRES,
// src/methods/solvers/SolverHypreGmres.cpp: Krylov dimension 30, 20 iterations,
// relative tolerance 1e-7, x0 = 0, no preconditioner). Restarted GMRES with modified
// Gram-Schmidt and Givens rotations (Saad and Schultz 1986), stopping when the
// residual estimate |g_{j+1}| <= eps |b|, then checked against the true residual.
//
// One solve is a fixed sequence of kernels (captured in the step's CUDA graph): every
// kernel first reads the control block and returns at once when the Arnoldi loop has
// ended, so iterations past convergence cost a launch each and no memory traffic.
// Reductions are deterministic: kRedBlocks partial sums, added in a fixed order.
// Built with FMA contraction (the solver is not part of the bit-exact path).
#include <cuda_runtime.h>

#include "implicit.hpp"

namespace cfd2d {

namespace {

constexpr int kT = 256;  // threads of every grid-stride kernel

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    __syncthreads();
    return s;  // valid in thread 0
}

// sum of the kRedBlocks partials in a fixed order, by every block (thread 0's value broadcast)
__device__ __forceinline__ double total(const double* __restrict__ part, double* sh) {
    double v = 0.0;
    for (int k = threadIdx.x; k < kRedBlocks; k += blockDim.x) v += part[k];
    double s = block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = s;
    __syncthreads();
    s = sh[32];
    __syncthreads();
    return s;
}

__device__ __forceinline__ void put_partial(double v, double* part, double* sh) {
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// y = A x for the rows of cell i: the diagonal block, then the faces' blocks
__device__ __forceinline__ void row_matvec(const ImpCase& c, int i, const double* __restrict__ x, double y[4]) {
    const int nc = c.nc;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    const double2 a = x2[2 * (size_t)i], b = x2[2 * (size_t)i + 1];
    const double xi[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
    for (int r = 0; r < 4; r++) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 4; q++) s = fma(c.D[(size_t)(4 * r + q) * nc + i], xi[q], s);
        y[r] = s;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int f = c.face[k * nc + i], e = f >> 1;
        if (e >= c.n_int) continue;
        const int j = (f & 1) ? c.ec1[e] : c.ec2[e];
        const double2 p = x2[2 * (size_t)j], t = x2[2 * (size_t)j + 1];
        const double xj[4] = {p.x, p.y, t.x, t.y};
        const double* O = c.O + (size_t)(16 * k) * nc + i;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double s = y[r];
#pragma unroll
            for (int q = 0; q < 4; q++) s = fma(O[(size_t)(4 * r + q) * nc], xj[q], s);
            y[r] = s;
        }
    }
}

__device__ __forceinline__ double* Vk(const ImpCase& c, int k) { return c.V + (size_t)k * 4 * c.nc; }

// cycle start: counters, and |src|^2 partials (src = b on the first cycle, else r); x = 0 on the first
__global__ void k_gm_reset(const ImpCase c, int first) {
    GmresCtl* g = c.ctl;
    if (first) { g->it = 0; g->final_ = 0; g->status = 0; g->cycle = 0; }
    g->cols = 0; g->done = 0; g->restart = 0; g->cycle++;
}

__global__ void __launch_bounds__(kT) k_gm_src_norm(const ImpCase c, int first) {
    __shared__ double sh[33];
    const double* src = first ? c.b : c.r;
    const size_t n = 4 * (size_t)c.nc;
    double v = 0.0;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n; q += (size_t)gridDim.x * kT) {
        const double s = src[q];
        v = fma(s, s, v);
        if (first) c.x[q] = 0.0;
    }
    put_partial(v, c.part, sh);
}

__global__ void __launch_bounds__(kT) k_gm_v0(const ImpCase c, int first) {
    __shared__ double sh[33];
    GmresCtl* g = c.ctl;
    if (g->final_) return;
    const double beta = sqrt(total(c.part, sh));
    const double bnorm = first ? beta : g->bnorm;
    const double eps_abs = first ? c.eps * beta : g->eps_abs;
    const bool stop = beta <= eps_abs || g->it >= c.maxit;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (first) { g->bnorm = bnorm; g->eps_abs = eps_abs; }
        g->rnorm = beta;
        g->g[0] = beta;
        for (int k = 1; k <= c.kdim; k++) g->g[k] = 0.0;
        if (stop) {
            g->done = 1;
            if (first) {  // b = 0: x = 0 is the solution
                g->final_ = 1;
                g->rel = 0.0;
                g->status = 0;
            }
        }
    }
    if (stop) return;
    const double* src = first ? c.b : c.r;
    double* v0 = Vk(c, 0);
    const double ib = 1.0 / beta;
    const size_t n = 4 * (size_t)c.nc;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n; q += (size_t)gridDim.x * kT) v0[q] = src[q] * ib;
}

// w = V_{j+1} = A V_j, and the partials of <w, V_0>
__global__ void __launch_bounds__(kT) k_gm_spmv(const ImpCase c, int j) {
    __shared__ double sh[33];
    if (c.ctl->done) return;
    const double* vj = Vk(c, j);
    double* w = Vk(c, j + 1);
    const double* v0 = Vk(c, 0);
    double acc = 0.0;
    for (int i = blockIdx.x * kT + threadIdx.x; i < c.nc; i += gridDim.x * kT) {
        double y[4];
        row_matvec(c, i, vj, y);
        double2* w2 = reinterpret_cast<double2*>(w) + 2 * (size_t)i;
        w2[0] = make_double2(y[0], y[1]);
        w2[1] = make_double2(y[2], y[3]);
        const double2* a2 = reinterpret_cast<const double2*>(v0) + 2 * (size_t)i;
        const double2 a = a2[0], b = a2[1];
        acc = fma(y[0], a.x, acc); acc = fma(y[1], a.y, acc); acc = fma(y[2], b.x, acc); acc = fma(y[3], b.y, acc);
    }
    put_partial(acc, c.part, sh);
}

// modified Gram-Schmidt step i of column j: h = <w, V_i> (from the partials), w -= h V_i,
// then the partials of <w, V_{i+1}> (i < j) or of |w|^2 (i == j)
__global__ void __launch_bounds__(kT) k_gm_mgs(const ImpCase c, int i, int j) {
    __shared__ double sh[33];
    GmresCtl* g = c.ctl;
    if (g->done) return;
    const double* pin = c.part + (i & 1) * kRedBlocks;
    double* pout = c.part + ((i + 1) & 1) * kRedBlocks;
    const double h = total(pin, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0) g->H[i * c.kdim + j] = h;
    double2* w = reinterpret_cast<double2*>(Vk(c, j + 1));
    const double2* vi = reinterpret_cast<const double2*>(Vk(c, i));
    const double2* vn = reinterpret_cast<const double2*>(Vk(c, i < j ? i + 1 : j + 1));
    const size_t n2 = 2 * (size_t)c.nc;
    double acc = 0.0;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n2; q += (size_t)gridDim.x * kT) {
        double2 a = w[q];
        const double2 b = vi[q];
        a.x = fma(-h, b.x, a.x);
        a.y = fma(-h, b.y, a.y);
        w[q] = a;
        const double2 d = i < j ? vn[q] : a;
        acc = fma(a.x, d.x, acc);
        acc = fma(a.y, d.y, acc);
    }
    put_partial(acc, pout, sh);
}

// H[j+1][j] = |w|; V_{j+1} = w / |w|
__global__ void __launch_bounds__(kT) k_gm_normalize(const ImpCase c, int j) {
    __shared__ double sh[33];
    GmresCtl* g = c.ctl;
    if (g->done) return;
    const double hn = sqrt(total(c.part + ((j + 1) & 1) * kRedBlocks, sh));
    if (blockIdx.x == 0 && threadIdx.x == 0) g->H[(j + 1) * c.kdim + j] = hn;
    if (hn == 0.0) return;
    const double ih = 1.0 / hn;
    double* w = Vk(c, j + 1);
    const size_t n = 4 * (size_t)c.nc;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n; q += (size_t)gridDim.x * kT) w[q] *= ih;
}

// Givens rotations of column j, the residual estimate, the end of the Arnoldi loop
__global__ void k_gm_givens(const ImpCase c, int j) {
    GmresCtl* g = c.ctl;
    if (g->done) return;
    const int m = c.kdim;
    double* H = g->H;
    for (int i = 0; i < j; i++) {
        const double a = H[i * m + j], b = H[(i + 1) * m + j];
        H[i * m + j] = g->cs[i] * a + g->sn[i] * b;
        H[(i + 1) * m + j] = -g->sn[i] * a + g->cs[i] * b;
    }
    const double a = H[j * m + j], b = H[(j + 1) * m + j];
    const double r = sqrt(a * a + b * b);
    if (r == 0.0) { g->cs[j] = 1.0; g->sn[j] = 0.0; }
    else { g->cs[j] = a / r; g->sn[j] = b / r; }
    H[j * m + j] = g->cs[j] * a + g->sn[j] * b;
    H[(j + 1) * m + j] = 0.0;
    g->g[j + 1] = -g->sn[j] * g->g[j];
    g->g[j] = g->cs[j] * g->g[j];
    g->rnorm = fabs(g->g[j + 1]);
    g->it++;
    g->cols = j + 1;
    if (g->rnorm <= g->eps_abs || g->it >= c.maxit || g->cols == m) g->done = 1;
}

// back substitution H y = g over the cycle's columns
__global__ void k_gm_solve(const ImpCase c) {
    GmresCtl* g = c.ctl;
    if (g->final_) return;
    const int m = c.kdim, n = g->cols;
    for (int i = n - 1; i >= 0; i--) {
        double s = g->g[i];
        for (int k = i + 1; k < n; k++) s -= g->H[i * m + k] * g->y[k];
        g->y[i] = s / g->H[i * m + i];
    }
}

// x += V y
__global__ void __launch_bounds__(kT) k_gm_xupdate(const ImpCase c) {
    const GmresCtl* g = c.ctl;
    if (g->final_) return;
    const int n = g->cols;
    const size_t nv = 4 * (size_t)c.nc;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < nv; q += (size_t)gridDim.x * kT) {
        double s = c.x[q];
        for (int k = 0; k < n; k++) s = fma(g->y[k], c.V[(size_t)k * nv + q], s);
        c.x[q] = s;
    }
}

// r = b - A x and the partials of |r|^2
__global__ void __launch_bounds__(kT) k_gm_resid(const ImpCase c) {
    __shared__ double sh[33];
    if (c.ctl->final_) return;
    double acc = 0.0;
    for (int i = blockIdx.x * kT + threadIdx.x; i < c.nc; i += gridDim.x * kT) {
        double y[4];
        row_matvec(c, i, c.x, y);
        double2* r2 = reinterpret_cast<double2*>(c.r) + 2 * (size_t)i;
        const double2* b2 = reinterpret_cast<const double2*>(c.b) + 2 * (size_t)i;
        const double2 ba = b2[0], bb = b2[1];
        const double r0 = ba.x - y[0], r1 = ba.y - y[1], r2v = bb.x - y[2], r3 = bb.y - y[3];
        r2[0] = make_double2(r0, r1);
        r2[1] = make_double2(r2v, r3);
        acc = fma(r0, r0, acc); acc = fma(r1, r1, acc); acc = fma(r2v, r2v, acc); acc = fma(r3, r3, acc);
    }
    put_partial(acc, c.part, sh);
}

// the true residual decides: final (with MatrixSolver's status bits) or another cycle
__global__ void __launch_bounds__(kT) k_gm_finish(const ImpCase c) {
    __shared__ double sh[33];
    GmresCtl* g = c.ctl;
    if (g->final_) return;
    const double rn = sqrt(total(c.part, sh));
    if (threadIdx.x != 0) return;
    g->rnorm = rn;
    g->rel = g->bnorm > 0.0 ? rn / g->bnorm : 0.0;
    if (rn <= g->eps_abs || g->it >= c.maxit) {
        g->final_ = 1;
        g->restart = 0;
        int st = 0;
        if (g->it >= c.maxit) st |= SOLVE_MAX_ITER;
        if (!(g->rel < c.eps) || !isfinite(g->rel)) st |= SOLVE_CONVERG;
        g->status = st;
    } else {
        g->restart = 1;
    }
}

}  // namespace

void imp_launch_gmres_cycle(const ImpCase& c, bool first, cudaStream_t s) {
    const int f = first ? 1 : 0;
    k_gm_reset<<<1, 1, 0, s>>>(c, f);
    k_gm_src_norm<<<kRedBlocks, kT, 0, s>>>(c, f);
    k_gm_v0<<<kRedBlocks, kT, 0, s>>>(c, f);
    const int jmax = c.kdim < c.maxit ? c.kdim : c.maxit;
    for (int j = 0; j < jmax; j++) {
        k_gm_spmv<<<kRedBlocks, kT, 0, s>>>(c, j);
        for (int i = 0; i <= j; i++) k_gm_mgs<<<kRedBlocks, kT, 0, s>>>(c, i, j);
        k_gm_normalize<<<kRedBlocks, kT, 0, s>>>(c, j);
        k_gm_givens<<<1, 1, 0, s>>>(c, j);
    }
    k_gm_solve<<<1, 1, 0, s>>>(c);
    k_gm_xupdate<<<kRedBlocks, kT, 0, s>>>(c);
    k_gm_resid<<<kRedBlocks, kT, 0, s>>>(c);
    k_gm_finish<<<1, kT, 0, s>>>(c);
}

}  // namespace cfd2d
