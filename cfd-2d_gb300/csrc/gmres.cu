// GMRES on the implicit method's block system (the reference calls HYPRE's GMRES,
// src/methods/solvers/SolverHypreGmres.cpp: Krylov dimension 30, 20 iterations,
// relative tolerance 1e-7, x0 = 0, no preconditioner). Restarted GMRES with Givens
// rotations (Saad and Schultz 1986), stopping when the residual estimate
// |g_{j+1}| <= eps |b|, then checked against the true residual. The Arnoldi step
// orthogonalises with classical Gram-Schmidt: all inner products <w, v_i> in one pass
// over the basis, then w -= sum h_i v_i in a second, instead of modified Gram-Schmidt's
// j + 1 dependent passes (which the oracle and HYPRE use); in exact arithmetic both
// give the same Krylov iterate, and with the reference's at most 20 basis vectors the
// results agree with the oracle's to rounding. Krylov vectors are kept unscaled with
// their factors 1/|w|, so no normalisation pass runs.
//
// One solve is a fixed sequence of kernels (captured in the step's CUDA graph): every
// kernel first reads the control block and returns at once when the Arnoldi loop has
// ended, so iterations past convergence cost a launch each and no memory traffic.
// Reductions are deterministic: kRedBlocks partial sums, added in a fixed order.
// Built with FMA contraction (the solver is not part of the bit-exact path).
#include <cuda_runtime.h>

#include <algorithm>

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

// y = A x for the four rows of cell i: the diagonal block, then the faces' blocks in
// order, four independent accumulation chains. Every load is independent of the others
// but for the neighbours' x after their index; a boundary face's block is zero and
// points at the cell itself, so there is no branch. A block column (q) of the four rows
// is 32 contiguous bytes, so a warp's loads of it are one contiguous kilobyte.
__device__ __forceinline__ void row_matvec(const ImpCase& c, int i, const double* __restrict__ x, double y[4]) {
    const int nc = c.nc;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    int nb[4];
    nb[0] = i;
    nb[1] = __ldg(c.nbr + i);
    nb[2] = __ldg(c.nbr + nc + i);
    nb[3] = __ldg(c.nbr + 2 * nc + i);
    double2 blk[4][4][2];  // [block: D, O0, O1, O2][column q][rows 0-1, 2-3]
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double2* d = reinterpret_cast<const double2*>(c.D + dblk(nc, i, 0, q));
        blk[0][q][0] = __ldg(d);
        blk[0][q][1] = __ldg(d + 1);
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const double2* o = reinterpret_cast<const double2*>(c.O + oblk(nc, i, k, 0, q));
            blk[k + 1][q][0] = __ldg(o);
            blk[k + 1][q][1] = __ldg(o + 1);
        }
    double xv[4][4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double2 p = __ldg(x2 + 2 * (size_t)nb[k]), t = __ldg(x2 + 2 * (size_t)nb[k] + 1);
        xv[k][0] = p.x; xv[k][1] = p.y; xv[k][2] = t.x; xv[k][3] = t.y;
    }
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            s0 = fma(blk[k][q][0].x, xv[k][q], s0);
            s1 = fma(blk[k][q][0].y, xv[k][q], s1);
            s2 = fma(blk[k][q][1].x, xv[k][q], s2);
            s3 = fma(blk[k][q][1].y, xv[k][q], s3);
        }
    y[0] = s0; y[1] = s1; y[2] = s2; y[3] = s3;
}

__device__ __forceinline__ double* Vk(const ImpCase& c, int k) { return c.V + (size_t)k * 4 * c.nc; }

// Givens rotations of column j, the residual estimate, the end of the Arnoldi loop
__device__ void givens(const ImpCase& c, GmresCtl* g, int j) {
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
        g->s[0] = 1.0;
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

// w = V_{j+1} = A (s_j V_j): the Krylov vectors are kept unscaled with their factor
// 1/|w| in s (the scaling pass of every iteration is folded into its uses)
__global__ void __launch_bounds__(kT) k_gm_spmv(const ImpCase c, int j) {
    const GmresCtl* g = c.ctl;
    if (g->done) return;
    const double sj = g->s[j];
    const double* vj = Vk(c, j);
    double2* w = reinterpret_cast<double2*>(Vk(c, j + 1));
    for (int i = blockIdx.x * kT + threadIdx.x; i < c.nc; i += gridDim.x * kT) {
        double y[4];
        row_matvec(c, i, vj, y);
        w[2 * (size_t)i] = make_double2(y[0] * sj, y[1] * sj);
        w[2 * (size_t)i + 1] = make_double2(y[2] * sj, y[3] * sj);
    }
}

// the partials of <w, V_i>, i = i0 .. i0 + CNT - 1 (classical Gram-Schmidt: all inner
// products of the column in one pass over w), into part[i][block]
template <int CNT>
__global__ void __launch_bounds__(kT) k_gm_dots(const ImpCase c, int j, int i0) {
    __shared__ double sh[CNT][kT / 32];
    if (c.ctl->done) return;
    const double2* w = reinterpret_cast<const double2*>(Vk(c, j + 1));
    const double2* v0 = reinterpret_cast<const double2*>(Vk(c, i0));
    const size_t n2 = 2 * (size_t)c.nc;
    double acc[CNT];
#pragma unroll
    for (int u = 0; u < CNT; u++) acc[u] = 0.0;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n2; q += (size_t)gridDim.x * kT) {
        const double2 a = w[q];
        double2 b[CNT];
#pragma unroll
        for (int u = 0; u < CNT; u++) b[u] = v0[(size_t)u * n2 + q];
#pragma unroll
        for (int u = 0; u < CNT; u++) {
            acc[u] = fma(a.x, b[u].x, acc[u]);
            acc[u] = fma(a.y, b[u].y, acc[u]);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int u = 0; u < CNT; u++) {
        double v = acc[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[u][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < CNT) {
        double t = 0.0;
        for (int k = 0; k < kT / 32; k++) t += sh[threadIdx.x][k];
        c.part[(size_t)(i0 + threadIdx.x) * kRedBlocks + blockIdx.x] = t;
    }
}

// h_ij = s_i <w, V_i> from the partials (one warp per i, in a fixed order) into column j
// of H, and the coefficients h_ij s_i of the update
__global__ void __launch_bounds__(1024) k_gm_hcol(const ImpCase c, int j) {
    GmresCtl* g = c.ctl;
    if (g->done) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i <= j; i += 32) {
        const double* p = c.part + (size_t)i * kRedBlocks;
        double v = 0.0;
        for (int k = lane; k < kRedBlocks; k += 32) v += p[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) {
            const double h = g->s[i] * v;
            g->H[i * c.kdim + j] = h;
            g->coef[i] = h * g->s[i];
        }
    }
}

// w -= sum_i h_ij s_i V_i, and the partials of |w|^2
__global__ void __launch_bounds__(kT) k_gm_orth(const ImpCase c, int j) {
    __shared__ double sh[33];
    __shared__ double hs[kGmresMaxKdim];
    GmresCtl* g = c.ctl;
    if (g->done) return;
    for (int i = threadIdx.x; i <= j; i += kT) hs[i] = g->coef[i];
    __syncthreads();
    double2* w = reinterpret_cast<double2*>(Vk(c, j + 1));
    const size_t n2 = 2 * (size_t)c.nc;
    double acc = 0.0;
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n2; q += (size_t)gridDim.x * kT) {
        double2 a = w[q];
        for (int i = 0; i <= j; i++) {
            const double2 b = reinterpret_cast<const double2*>(Vk(c, i))[q];
            a.x = fma(-hs[i], b.x, a.x);
            a.y = fma(-hs[i], b.y, a.y);
        }
        w[q] = a;
        acc = fma(a.x, a.x, acc);
        acc = fma(a.y, a.y, acc);
    }
    put_partial(acc, c.part, sh);
}

// H[j+1][j] = |w|, s_{j+1} = 1/|w|, the Givens rotations of column j, the residual
// estimate and the end of the Arnoldi loop
__global__ void __launch_bounds__(kT) k_gm_givens(const ImpCase c, int j) {
    __shared__ double sh[33];
    GmresCtl* g = c.ctl;
    if (g->done) return;
    const double hn = sqrt(total(c.part, sh));
    if (threadIdx.x != 0) return;
    g->H[(j + 1) * c.kdim + j] = hn;
    g->s[j + 1] = hn != 0.0 ? 1.0 / hn : 0.0;
    givens(c, g, j);
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

// x += sum_k y_k s_k V_k
__global__ void __launch_bounds__(kT) k_gm_xupdate(const ImpCase c) {
    __shared__ double ys[kGmresMaxKdim];
    const GmresCtl* g = c.ctl;
    if (g->final_) return;
    const int n = g->cols;
    for (int k = threadIdx.x; k < n; k += kT) ys[k] = g->y[k] * g->s[k];
    __syncthreads();
    const size_t n2 = 2 * (size_t)c.nc;
    double2* x = reinterpret_cast<double2*>(c.x);
    const double2* V = reinterpret_cast<const double2*>(c.V);
    for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n2; q += (size_t)gridDim.x * kT) {
        double2 s = x[q];
        for (int k = 0; k < n; k++) {
            const double2 v = V[(size_t)k * n2 + q];
            s.x = fma(ys[k], v.x, s.x);
            s.y = fma(ys[k], v.y, s.y);
        }
        x[q] = s;
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
        for (int k = 0; k < 4; k++) {
            const double r = c.b[4 * (size_t)i + k] - y[k];
            c.r[4 * (size_t)i + k] = r;
            acc = fma(r, r, acc);
        }
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

constexpr int kDotChunk = 12;  // inner products per pass over w (registers: 2 x 12 doubles of V)

template <int N>
void dots_n(const ImpCase& c, int j, int i0, int cnt, cudaStream_t s) {
    if constexpr (N > 0) {
        if (cnt == N) k_gm_dots<N><<<kRedBlocks, kT, 0, s>>>(c, j, i0);
        else dots_n<N - 1>(c, j, i0, cnt, s);
    }
}
void launch_dots(const ImpCase& c, int j, int i0, int cnt, cudaStream_t s) { dots_n<kDotChunk>(c, j, i0, cnt, s); }

}  // namespace

void imp_launch_gmres_cycle(const ImpCase& c, bool first, cudaStream_t s) {
    const int f = first ? 1 : 0;
    k_gm_reset<<<1, 1, 0, s>>>(c, f);
    k_gm_src_norm<<<kRedBlocks, kT, 0, s>>>(c, f);
    k_gm_v0<<<kRedBlocks, kT, 0, s>>>(c, f);
    const int jmax = c.kdim < c.maxit ? c.kdim : c.maxit;
    for (int j = 0; j < jmax; j++) {
        k_gm_spmv<<<kRedBlocks, kT, 0, s>>>(c, j);
        for (int i0 = 0; i0 <= j; i0 += kDotChunk) launch_dots(c, j, i0, std::min(kDotChunk, j + 1 - i0), s);
        k_gm_hcol<<<1, 1024, 0, s>>>(c, j);
        k_gm_orth<<<kRedBlocks, kT, 0, s>>>(c, j);
        k_gm_givens<<<1, kT, 0, s>>>(c, j);
    }
    k_gm_solve<<<1, 1, 0, s>>>(c);
    k_gm_xupdate<<<kRedBlocks, kT, 0, s>>>(c);
    k_gm_resid<<<kRedBlocks, kT, 0, s>>>(c);
    k_gm_finish<<<1, kT, 0, s>>>(c);
}

}  // namespace cfd2d
