// Precision dispatch and the precision-independent kernels (time step,
// permutations, conservation sums). Built with -fmad=false.
#include "kernels.cuh"

namespace cfd2d {

void launch_grad_fp64(const DevCase&, cudaStream_t);
void launch_flux_fp64(const DevCase&, int, int, cudaStream_t);
void launch_update_fp64(const DevCase&, int, int, cudaStream_t);
void launch_remediate_fp64(const DevCase&, cudaStream_t);
void launch_prims_fp64(const DevCase&, cudaStream_t);
void launch_residual_fp64(const DevCase&, double*, cudaStream_t);
void launch_grad_mixed(const DevCase&, cudaStream_t);
void launch_flux_mixed(const DevCase&, int, int, cudaStream_t);
void launch_update_mixed(const DevCase&, int, int, cudaStream_t);
void launch_remediate_mixed(const DevCase&, cudaStream_t);
void launch_prims_mixed(const DevCase&, cudaStream_t);
void launch_residual_mixed(const DevCase&, double*, cudaStream_t);

void launch_grad(const DevCase& c, int p, cudaStream_t s) {
    p == PREC_MIXED ? launch_grad_mixed(c, s) : launch_grad_fp64(c, s);
}
void launch_flux(const DevCase& c, int p, int flux, int recon, cudaStream_t s) {
    p == PREC_MIXED ? launch_flux_mixed(c, flux, recon, s) : launch_flux_fp64(c, flux, recon, s);
}
void launch_update(const DevCase& c, int p, int scheme, int stage, cudaStream_t s) {
    p == PREC_MIXED ? launch_update_mixed(c, scheme, stage, s) : launch_update_fp64(c, scheme, stage, s);
}
void launch_remediate(const DevCase& c, int p, cudaStream_t s) {
    p == PREC_MIXED ? launch_remediate_mixed(c, s) : launch_remediate_fp64(c, s);
}
void launch_prims(const DevCase& c, int p, cudaStream_t s) {
    p == PREC_MIXED ? launch_prims_mixed(c, s) : launch_prims_fp64(c, s);
}
void launch_residual(const DevCase& c, int p, double* R, cudaStream_t s) {
    p == PREC_MIXED ? launch_residual_mixed(c, R, s) : launch_residual_fp64(c, R, s);
}

namespace {
inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

// CFL*S/max(|u|+c, |v|+c) per cell (calcTimeStep, src/methods/fvm_tvd.cpp:227-234);
// the minimum over cells is order-independent, so an atomic min on the bit
// pattern of the positive doubles is deterministic.
__global__ void __launch_bounds__(256) k_dt_min(const DevCase c, unsigned long long* out) {
    const int nc = c.nc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double t = __longlong_as_double(0x7ff0000000000000ll);  // +inf
    if (i < nc) {
        const DevMat mt = mat_of(c, i);
        const Prim<double> q = cons2prim<double>(c.A[i], c.A[nc + i], c.A[2 * nc + i], c.A[3 * nc + i], mt.gm1);
        const double cz = sqrt(mt.gam * q.p / q.r);
        t = c.cfl_number * c.S[i] / t_max(fabs(q.u) + cz, fabs(q.v) + cz);
        if (!(t >= 0.0)) t = __longlong_as_double(0x7ff0000000000000ll);
    }
    for (int o = 16; o > 0; o >>= 1) t = fmin(t, __shfl_xor_sync(0xffffffffu, t, o));
    __shared__ double w[8];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) t = fmin(t, w[k]);
        atomicMin(out, (unsigned long long)__double_as_longlong(t));
    }
}

__global__ void k_fill_cfl(const DevCase c, double tau) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nc) return;
    c.ctau[i] = tau;
    c.cfl[i] = tau / c.S[i];
}

__global__ void k_gather_state(const DevCase c, const double* __restrict__ src, double* __restrict__ dst) {
    const int nc = c.nc;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;  // original cell
    if (o >= nc) return;
    const int i = c.iperm[o];
#pragma unroll
    for (int k = 0; k < 4; k++) dst[(size_t)k * nc + i] = src[(size_t)k * nc + o];
}

__global__ void k_scatter_state(const DevCase c, const double* __restrict__ src, double* __restrict__ dst) {
    const int nc = c.nc;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nc) return;
    const int i = c.iperm[o];
#pragma unroll
    for (int k = 0; k < 4; k++) dst[(size_t)k * nc + o] = src[(size_t)k * nc + i];
}

// The state straight from / to four host arrays the device addresses (pinned memory,
// or pageable memory where the system gives the GPU coherent access to it): one pass
// over the host link, permuted on the way, no staging copy in HBM.
__global__ void k_gather_state_host(const DevCase c, HostArrays4 src, double* __restrict__ dst) {
    const int nc = c.nc;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nc) return;
    const int i = c.iperm[o];
#pragma unroll
    for (int k = 0; k < 4; k++) dst[(size_t)k * nc + i] = src.p[k][o];
}

__global__ void k_scatter_state_host(const DevCase c, const double* __restrict__ src, HostArrays4 dst) {
    const int nc = c.nc;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nc) return;
    const int i = c.iperm[o];
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (dst.p[k]) dst.p[k][o] = src[(size_t)k * nc + i];
}

__global__ void k_permute_scalar(const DevCase c, const double* __restrict__ src, double* __restrict__ dst) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.nc) return;
    dst[o] = src[c.iperm[o]];
}

__global__ void k_permute_flags(const DevCase c, const unsigned* __restrict__ src, unsigned* __restrict__ dst) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.nc) return;
    dst[o] = src[c.iperm[o]];
}

// Sums of S*U over a fixed partition of the cells: block b takes a contiguous
// chunk and reduces it in a fixed tree, so the result does not depend on timing.
__global__ void __launch_bounds__(256) k_conservation(const DevCase c, double* __restrict__ partial) {
    const int nc = c.nc;
    const long chunk = ((long)nc + gridDim.x - 1) / gridDim.x;
    const long b0 = blockIdx.x * chunk, b1 = min((long)nc, b0 + chunk);
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const double s = c.S[i];
        for (int k = 0; k < 4; k++) a[k] += s * c.A[(size_t)k * nc + i];
    }
    __shared__ double sh[4][256];
    for (int k = 0; k < 4; k++) sh[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) partial[4 * blockIdx.x + k] = sh[k][0];
}
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {  // splitmix64 finaliser
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void k_selftest(int which, long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r1 = mix64(seed ^ (2 * k)), r2 = mix64(seed ^ (2 * k + 1));
        if (which == 0) {  // quotients of random doubles over a wide exponent range, by the reciprocal form
            const double a = __longlong_as_double((long long)(((r1 % 1400) + 324ull) << 52 | (r2 & 0xfffffffffffffull) |
                                                              (r1 & 0x8000000000000000ull)));
            const double b = __longlong_as_double((long long)((((r2 >> 52) % 1400) + 324ull) << 52 |
                                                              (mix64(r1) & 0xfffffffffffffull)));
            double a2 = a, b2 = b;
            if ((r1 & 0xf0) == 0) a2 = (r1 & 0x100) ? -0.0 : 0.0;      // zero dividends, both signs
            if ((r2 & 0xf00) == 0) b2 = __longlong_as_double((long long)(r2 & 0xfff0000000000000ull));  // any exponent
            const double y = 1.0 / b2;
            const double q1 = div_rn(a2, b2, y), q2 = a2 / b2;
            local += __double_as_longlong(q1) != __double_as_longlong(q2);
        } else if (which == 1) {  // widening of random normal floats
            const float f = __uint_as_float((unsigned)(((r1 % 254) + 1) << 23) | (unsigned)(r2 & 0x807fffffu));
            local += __double_as_longlong(widen(f)) != __double_as_longlong((double)f);
        } else if (which == 3) {  // minmod against the reference's a*b > 0 ? (|a|<|b| ? a : b) : 0
            // exponent fields over the whole range (zero, subnormal, normal, inf/NaN), with extra
            // weight near the product's underflow threshold (sum of fields ~ 972)
            const unsigned long long ex1 = (r1 & 3) == 0 ? (r1 >> 8) % 2048 : 300 + (r1 >> 8) % 400;
            const unsigned long long ex2 = (r2 & 3) == 0 ? (r2 >> 8) % 2048 : 972 - ex1 + (long long)((r2 >> 8) % 9) - 4;
            const unsigned long long m1 = (r1 & 12) == 0 ? 0 : mix64(r2) & 0xfffffffffffffull;
            const unsigned long long m2 = (r2 & 12) == 0 ? 0 : mix64(r1) & 0xfffffffffffffull;
            const double a = __longlong_as_double((long long)((r1 & 0x8000000000000000ull) | (ex1 & 0x7ff) << 52 | m1));
            const double b = __longlong_as_double((long long)(((r2 << 1) & 0x8000000000000000ull) | (ex2 & 0x7ff) << 52 | m2));
            const double ref = a * b > 0.0 ? (fabs(a) < fabs(b) ? a : b) : 0.0;
            local += __double_as_longlong(minmod(a, b)) != __double_as_longlong(ref);
        } else {  // narrowing of random doubles in float range: within 1 ulp of the hardware's
            const double d = __longlong_as_double((long long)(((r1 % 250) + 1023 - 124) << 52 | (r2 & 0x800fffffffffffffull)));
            const int u1 = __float_as_int(narrow(d)), u2 = __float_as_int((float)d);
            local += (u1 - u2 > 1 || u2 - u1 > 1);
        }
    }
    if (local) atomicAdd(bad, local);
}
}  // namespace

long long selftest_arith(int which, long long n, unsigned long long seed) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return -1;
    cudaMemset(d, 0, sizeof *d);
    k_selftest<<<1216, 256>>>(which, n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? (long long)h : -1;
}

void launch_dt_min(const DevCase& c, unsigned long long* out, cudaStream_t s) {
    k_dt_min<<<nblk(c.nc, 256), 256, 0, s>>>(c, out);
}
void launch_fill_cfl(const DevCase& c, double tau, cudaStream_t s) {
    k_fill_cfl<<<nblk(c.nc, 256), 256, 0, s>>>(c, tau);
}
void launch_gather_state(const DevCase& c, const double* src, double* dst, cudaStream_t s) {
    k_gather_state<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_scatter_state(const DevCase& c, const double* src, double* dst, cudaStream_t s) {
    k_scatter_state<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_gather_state_host(const DevCase& c, const HostArrays4& src, double* dst, cudaStream_t s) {
    k_gather_state_host<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_scatter_state_host(const DevCase& c, const double* src, const HostArrays4& dst, cudaStream_t s) {
    k_scatter_state_host<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_permute_scalar(const DevCase& c, const double* src, double* dst, cudaStream_t s) {
    k_permute_scalar<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_permute_flags(const DevCase& c, const unsigned* src, unsigned* dst, cudaStream_t s) {
    k_permute_flags<<<nblk(c.nc, 256), 256, 0, s>>>(c, src, dst);
}
void launch_conservation(const DevCase& c, double* partial, int nblocks, cudaStream_t s) {
    k_conservation<<<nblocks, 256, 0, s>>>(c, partial);
}

}  // namespace cfd2d
