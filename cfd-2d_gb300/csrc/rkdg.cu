// Device code of FEM_RKDG (src/methods/fem_rkdg.cpp). Built with -fmad=false: every
// product and sum rounds on its own, in the reference's order, so the FP64 results equal
// the reference's bit for bit (the quotients by the density and the cell sizes are
// correctly rounded, div_rn; the polynomial sums start from +0 as VECTOR::SCALAR_PROD's).
#include "rkdg.hpp"

#include "kernels.cuh"

namespace cfd2d {
namespace {

// 0 + x in round-to-nearest: x, except -0 -> +0 (an integer select, no FP64 add)
__device__ __forceinline__ double pz(double x) {
    const long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

__device__ __forceinline__ DgMat dmat(const DgCase& c, int cell) { return c.cmat ? c.mats[c.cmat[cell]] : c.mat0; }

__device__ __forceinline__ void load12(const double* __restrict__ U, int i, double* a) {
    const double2* p = reinterpret_cast<const double2*>(U + 12 * (size_t)i);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double2 t = __ldg(p + k);
        a[2 * k] = t.x;
        a[2 * k + 1] = t.y;
    }
}
__device__ __forceinline__ void store12(double* __restrict__ U, int i, const double* a) {
    double2* p = reinterpret_cast<double2*>(U + 12 * (size_t)i);
#pragma unroll
    for (int k = 0; k < 6; k++) p[k] = make_double2(a[2 * k], a[2 * k + 1]);
}

struct DgPar { double r, u, v, E, p, y; };

// convertConsToPar (:1420-1430) through URS(0)'s pressure: each variable's polynomial at a
// point (SCALAR_PROD from s = 0 with the basis (1, F1, F2), src/global.h:128-135), u, v, E
// by r (:1422-1425), e, p = r e (gam - 1) (src/global.cpp:15-17). y = RN(1/r).
__device__ __forceinline__ DgPar dg_eval(const double* a, double F1, double F2, double gm1) {
    double s[4];
#pragma unroll
    for (int v = 0; v < 4; v++) {
        double t = pz(a[3 * v]);  // 0 + a0 * 1.0
        t = t + a[3 * v + 1] * F1;
        t = t + a[3 * v + 2] * F2;
        s[v] = t;
    }
    DgPar q;
    q.r = s[0];
    q.y = 1.0 / q.r;
    q.u = div_rn(s[1], q.r, q.y);
    q.v = div_rn(s[2], q.r, q.y);
    q.E = div_rn(s[3], q.r, q.y);
    const double e = q.E - 0.5 * (q.u * q.u + q.v * q.v);
    q.p = q.r * e * gm1;
    return q;
}

// calcConvectionSurf (:995-1122), one thread per edge: both sides at each Gauss point, the
// flux (calcFlux :918-960; boundaryCond :1324-1343 for a boundary edge), the sides'
// integrals sum_g (F w) f in Gauss-point order, times edgeJ.
template <int FLUX, int GE>
__global__ void __launch_bounds__(128) k_dg_edge(const DgCase c, const double* __restrict__ U) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= c.ne) return;
    const int c1 = c.ec1[e], c2 = c.ec2[e];
    const bool inner = c2 >= 0;
    double a1[12], a2[12];
    load12(U, c1, a1);
    if (inner) load12(U, c2, a2);
    const DgMat m1 = dmat(c, c1);
    const double gm2 = inner ? dmat(c, c2).gm1 : 0.0;
    const double nx = c.enx[e], ny = c.eny[e];
    double i1[12], i2[12];
    bool hit = false;
#pragma unroll
    for (int g = 0; g < GE; g++) {
        const double2* Fp = reinterpret_cast<const double2*>(c.eF + ((size_t)e * GE + g) * 4);
        const double2 Fa = __ldg(Fp), Fb = __ldg(Fp + 1);
        const DgPar L = dg_eval(a1, Fa.x, Fa.y, m1.gm1);
        const Prim<double> qL{L.r, L.u, L.v, L.p};
        Prim<double> qR;
        double yR;
        if (inner) {
            const DgPar R = dg_eval(a2, Fb.x, Fb.y, gm2);
            qR = Prim<double>{R.r, R.u, R.v, R.p};
            yR = R.y;
        } else {
            // URS(1) of pL (:1428) gives the temperature an outlet or wall ghost carries
            const double Tc = temperature(qL, m1.gm1, m1.Cv);
            qR = ghost_state(c.bnds[c.ebnd[e]], qL, Tc, nx, ny, m1.M);
            yR = 1.0 / qR.r;
        }
        double f[4];
        if (FLUX == FLUX_GODUNOV) hit |= flux_godunov<double, true>(f, qL, qR, nx, ny, m1.rg, c.newton_cap, L.y, yR);
        else flux_lax<double, true>(f, qL, qR, nx, ny, m1.gam, m1.ig1, L.y, yR);
        const double w = c.egw[g];
        const double w1[3] = {w, GE == 2 ? Fa.x : Fa.x * w, GE == 2 ? Fa.y : Fa.y * w};  // getF(c1, pt) * w (w = 1 for 2 points)
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const double t = w1[k] * f[v];
                i1[3 * v + k] = g == 0 ? pz(t) : i1[3 * v + k] + t;
            }
        if (inner) {
            const double w2[3] = {w, GE == 2 ? Fb.x : Fb.x * w, GE == 2 ? Fb.y : Fb.y * w};
#pragma unroll
            for (int v = 0; v < 4; v++)
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const double t = w2[k] * f[v];
                    i2[3 * v + k] = g == 0 ? pz(t) : i2[3 * v + k] + t;
                }
        }
    }
    const double J = c.edgeJ[e];
#pragma unroll
    for (int k = 0; k < 12; k++) i1[k] = i1[k] * J;
    store12(c.E1, e, i1);
    if (inner) {
#pragma unroll
        for (int k = 0; k < 12; k++) i2[k] = i2[k] * J;
        store12(c.E2, e, i2);
    }
    if (hit) atomicOr(c.err, ERRBIT_NEWTON_CAP);
}

// max over a warp's non-negative doubles (as ordered bits), then one atomic per warp
__device__ __forceinline__ void warp_max_bits(unsigned long long v, unsigned long long* dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}
__device__ __forceinline__ void warp_min_bits(unsigned long long v, unsigned long long* dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(dst, v);
}
// a value a "max > x" test would keep: positive and not NaN, else 0
__device__ __forceinline__ unsigned long long pos_bits(double x) {
    const long long b = __double_as_longlong(x);
    return (b > 0 && b <= 0x7ff0000000000000ll) ? (unsigned long long)b : 0ull;
}

// One thread per cell: calcConvectionVol (:1124-1210) at the cell's Gauss points, the
// edges' integrals in ascending original edge number (c1: -=, c2: +=, :1076-1084), then
// calcNewFields (:1216-1242) / calcNewFields2 (:1244-1284). Stage 1 reads A and writes B;
// stage 2 reads B (and A) and writes A.
template <int GC>
__global__ void __launch_bounds__(128) k_dg_cell(const DgCase c, int stage, int with_res) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < c.nc;
    unsigned long long rb[4] = {0, 0, 0, 0};
    if (live) {
        double a[12];
        load12(stage == 1 ? c.A : c.B, i, a);
        const DgMat m = dmat(c, i);
        const double ihx = c.ih[2 * (size_t)i], ihy = c.ih[2 * (size_t)i + 1];
        double in[12];
#pragma unroll
        for (int g = 0; g < GC; g++) {
            const double2 F = __ldg(reinterpret_cast<const double2*>(c.cF) + (size_t)i * GC + g);
            const DgPar q = dg_eval(a, F.x, F.y, m.gm1);
            const double fr = q.r * q.u;
            const double fu = fr * q.u + q.p;
            const double fv = fr * q.v;
            const double fe = q.u * (q.r * q.E + q.p);
            const double gr = q.r * q.v;
            const double gu = gr * q.u;
            const double gv = gr * q.v + q.p;
            const double ge = q.v * (q.r * q.E + q.p);
            const double fx[4] = {fr, fu, fv, fe}, gy[4] = {gr, gu, gv, ge};
            const double w = c.cgw[g];
            // tmpInt = 0; += getDFDX * f = (0, 1/HX, 0) f; += getDFDY * g = (0, 0, 1/HY) g; *= w.
            // With finite fluxes the products by 0 are +-0 and every sum with them is exact:
            // component 1 is 0 + f/HX (pz), component 2 is 0 + g/HY, component 0 is +-0 after
            // the weight, which leaves the running sum as it is (+0 from the first point on,
            // or the NaN / inf an earlier point left). Non-finite fluxes take the literal form.
            bool finite = true;
#pragma unroll
            for (int v = 0; v < 4; v++)
                finite = finite && ((__double2hiint(fx[v]) & 0x7ff00000) != 0x7ff00000) &&
                         ((__double2hiint(gy[v]) & 0x7ff00000) != 0x7ff00000);
            if (finite) {
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const double t1 = pz(ihx * fx[v]) * w;
                    const double t2 = pz(ihy * gy[v]) * w;
                    if (g == 0) in[3 * v] = 0.0;
                    in[3 * v + 1] = g == 0 ? pz(t1) : in[3 * v + 1] + t1;
                    in[3 * v + 2] = g == 0 ? pz(t2) : in[3 * v + 2] + t2;
                }
            } else {
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    double t0 = 0.0 + 0.0 * fx[v];
                    double t1 = 0.0 + ihx * fx[v];
                    double t2 = 0.0 + 0.0 * fx[v];
                    t0 = t0 + 0.0 * gy[v];
                    t1 = t1 + 0.0 * gy[v];
                    t2 = t2 + ihy * gy[v];
                    t0 = t0 * w; t1 = t1 * w; t2 = t2 * w;
                    in[3 * v] = g == 0 ? pz(t0) : in[3 * v] + t0;
                    in[3 * v + 1] = g == 0 ? pz(t1) : in[3 * v + 1] + t1;
                    in[3 * v + 2] = g == 0 ? pz(t2) : in[3 * v + 2] + t2;
                }
            }
        }
        const double J = c.cellJ[i];
        double R[12];
#pragma unroll
        for (int k = 0; k < 12; k++) R[k] = pz(in[k] * J);  // ro_int (0) += intRO * cellJ
#pragma unroll
        for (int f = 0; f < 3; f++) {
            const int fw = c.face[(size_t)f * c.nc + i];
            const int e = fw >> 3;
            double s[12];
            if (fw & 1) {
                load12(c.E2, e, s);
#pragma unroll
                for (int k = 0; k < 12; k++) R[k] = R[k] + s[k];
            } else {
                load12(c.E1, e, s);
#pragma unroll
                for (int k = 0; k < 12; k++) R[k] = R[k] - s[k];
            }
        }
        const double* Mi = c.invA + 9 * (size_t)i;
        double M[9];
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = __ldg(Mi + k);
        const double ct = c.ctau[i];
        double out[12];
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int r = 0; r < 3; r++) {
                double t = pz(M[3 * r] * R[3 * v]);  // VECTOR *= matr: tmp = 0; += m_rj e_j
                t = t + M[3 * r + 1] * R[3 * v + 1];
                t = t + M[3 * r + 2] * R[3 * v + 2];
                t = t * ct;
                out[3 * v + r] = a[3 * v + r] + t;
            }
        if (stage == 1) {
            store12(c.B, i, out);
        } else {
            const bool shared = c.rk_mode == DG_RK_REFERENCE && (c.cflag[i] & 1);
            double old[12];
            if (c.rk_mode == DG_RK_HEUN) load12(c.A, i, old);
            else
#pragma unroll
                for (int k = 0; k < 12; k++) old[k] = a[k];  // the first stage's result (zeroIntegrals)
            double res[12];
#pragma unroll
            for (int k = 0; k < 12; k++) {
                const double o = shared ? out[k] : old[k];
                res[k] = (out[k] + o) * 0.5;
            }
            store12(c.A, i, res);
            // a non-positive or NaN cell-mean density or energy is reported (the state is
            // still advanced, as the reference would): bit tests on the integer pipe
            const long long br = __double_as_longlong(res[0]), be = __double_as_longlong(res[9]);
            if (br <= 0 || br >= 0x7ff0000000000000ll || be <= 0 || be >= 0x7ff0000000000000ll)
                atomicOr(c.err, ERRBIT_NONPHYSICAL);
            if (with_res) {  // calcResiduals, :1286-1319: | U - ro_old |, ro_old the cell's own for shared cells
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const double u = res[3 * v + k];
                        const double x = fabs(u - (shared ? u : old[3 * v + k]));
                        s = s + x * x;
                    }
                    rb[v] = pos_bits(sqrt(s));
                }
            }
        }
    }
    if (with_res && stage == 2)
#pragma unroll
        for (int v = 0; v < 4; v++) warp_max_bits(rb[v], c.res + v);
}

// calcTimeStep (:382-447): the largest |u| + c over the cell's Gauss points, its edges'
// Gauss points (the reference reads edgeGP[edge][slot]; HEUN: all of them) and the centre.
template <int GC, int GE>
__global__ void __launch_bounds__(128) k_dg_tstep(const DgCase c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < c.nc;
    unsigned long long tb = 0x7ff0000000000000ull;  // +inf: neutral for the minimum
    if (live) {
        double a[12];
        load12(c.A, i, a);
        const DgMat m = dmat(c, i);
        double maxU = 0.0;
        auto visit = [&](double F1, double F2) {
            const DgPar q = dg_eval(a, F1, F2, m.gm1);
            const double cz = sqrt(div_rn(m.gam * q.p, q.r, q.y));  // URS(0)
            const double Uv = sqrt(q.u * q.u + q.v * q.v) + cz;    // magU() + cz
            if (maxU < Uv) maxU = Uv;
        };
#pragma unroll
        for (int g = 0; g < GC; g++) {
            const double2 F = __ldg(reinterpret_cast<const double2*>(c.cF) + (size_t)i * GC + g);
            visit(F.x, F.y);
        }
#pragma unroll
        for (int f = 0; f < 3; f++) {
            const int fw = c.face[(size_t)f * c.nc + i];
            const int e = fw >> 3, slot = (fw >> 1) & 3, side = fw & 1;
            if (c.rk_mode == DG_RK_REFERENCE) {
                if (slot < GE) {
                    const double2 F = __ldg(reinterpret_cast<const double2*>(c.eF) + ((size_t)e * GE + slot) * 2 + side);
                    visit(F.x, F.y);
                }
            } else {
#pragma unroll
                for (int g = 0; g < GE; g++) {
                    const double2 F = __ldg(reinterpret_cast<const double2*>(c.eF) + ((size_t)e * GE + g) * 2 + side);
                    visit(F.x, F.y);
                }
            }
        }
        visit(c.fc[2 * (size_t)i], c.fc[2 * (size_t)i + 1]);
        if (c.steady) {
            c.ctau[i] = c.cfl * c.S[i] / maxU;
        } else {
            const double tmp = c.S[i] / maxU;
            const long long b = __double_as_longlong(tmp);
            if (b >= 0 && b <= 0x7ff0000000000000ll) tb = (unsigned long long)b;  // NaN never wins "tmp < tau"
        }
    }
    if (!c.steady) warp_min_bits(tb, c.tmin);
}

__global__ void k_dg_fill(double* dst, double v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}

__global__ void k_dg_gather(const int* __restrict__ iperm, const double* __restrict__ src, double* __restrict__ dst,
                            int nc) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 12ll * nc) return;
    const int i = (int)(t / 12), k = (int)(t % 12);
    dst[12 * (size_t)iperm[i] + k] = src[t];
}
__global__ void k_dg_scatter(const int* __restrict__ iperm, const double* __restrict__ src, double* __restrict__ dst,
                             int nc) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 12ll * nc) return;
    const int i = (int)(t / 12), k = (int)(t % 12);
    dst[t] = src[12 * (size_t)iperm[i] + k];
}

inline int blocks(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

void dg_launch_edges(const DgCase& c, int flux, const double* U, cudaStream_t s) {
    const int nb = blocks(c.ne, 128);
    if (flux == FLUX_LAX) {
        if (c.ge == 3) k_dg_edge<FLUX_LAX, 3><<<nb, 128, 0, s>>>(c, U);
        else k_dg_edge<FLUX_LAX, 2><<<nb, 128, 0, s>>>(c, U);
    } else {
        if (c.ge == 3) k_dg_edge<FLUX_GODUNOV, 3><<<nb, 128, 0, s>>>(c, U);
        else k_dg_edge<FLUX_GODUNOV, 2><<<nb, 128, 0, s>>>(c, U);
    }
}

void dg_launch_cells(const DgCase& c, int stage, bool with_res, cudaStream_t s) {
    const int nb = blocks(c.nc, 128);
    if (c.gc == 4) k_dg_cell<4><<<nb, 128, 0, s>>>(c, stage, with_res ? 1 : 0);
    else k_dg_cell<3><<<nb, 128, 0, s>>>(c, stage, with_res ? 1 : 0);
}

void dg_launch_time_step(const DgCase& c, cudaStream_t s) {
    const int nb = blocks(c.nc, 128);
    if (c.gc == 4) {
        if (c.ge == 3) k_dg_tstep<4, 3><<<nb, 128, 0, s>>>(c);
        else k_dg_tstep<4, 2><<<nb, 128, 0, s>>>(c);
    } else {
        if (c.ge == 3) k_dg_tstep<3, 3><<<nb, 128, 0, s>>>(c);
        else k_dg_tstep<3, 2><<<nb, 128, 0, s>>>(c);
    }
}

void dg_launch_fill(double* dst, double v, int n, cudaStream_t s) {
    k_dg_fill<<<blocks(n, 256), 256, 0, s>>>(dst, v, n);
}

void dg_launch_gather(const DgCase& c, const double* src_orig, double* dst_store, cudaStream_t s) {
    k_dg_gather<<<blocks(12ll * c.nc, 256), 256, 0, s>>>(c.iperm, src_orig, dst_store, c.nc);
}
void dg_launch_scatter(const DgCase& c, const double* src_store, double* dst_orig, cudaStream_t s) {
    k_dg_scatter<<<blocks(12ll * c.nc, 256), 256, 0, s>>>(c.iperm, src_store, dst_orig, c.nc);
}

}  // namespace cfd2d
