// cfd2d_residual_first_order_static: the first-order residual (edge fluxes at
// the cell-centre states, gathered onto the cells) with its scratch in a fixed
// device array instead of memory the library allocates.
//
// Who needs it: callers that must not allocate device memory at the moment they
// call in, for example code recording a CUDA graph (cudaMalloc is not allowed
// while a stream is being captured), hosts that run the solver inside another
// framework whose memory pool owns the whole device budget, or real-time
// loops that forbid allocation after start-up. They pass their own device
// buffers for the mesh, the state and the result; the only scratch, one FP64
// flux per edge and component, lives in g_static_edge_flux below.
//
// The array is CFD2D_STATIC_MAX_EDGES x 4 doubles (8 MiB). Every GPU that
// loads this library holds it until the process exits. Every call shares it
// and it keeps the last call's contents; each call writes every edge slot it
// reads, so nothing has to start at zero. Two calls whose kernels overlap on
// the GPU (different streams, or different host threads on one device) race
// on the array: order them on one stream.
//
// Built with -fmad=false, like the FP64 solver kernels, so the result equals
// cfd2d_residual of a solver created with RECONSTRUCTION NONE bit for bit.
#include <cuda_runtime.h>

#include <mutex>

#include "cfd2d.h"
#include "kernels.cuh"

namespace cfd2d {
namespace {

constexpr int kMaxBnd = 16;

__device__ __align__(256) double g_static_edge_flux[4 * (size_t)CFD2D_STATIC_MAX_EDGES];

struct StaticArgs {
    int nc, ne, nbnd;
    const int* cell_edges;
    const int* c12;
    const double* n;
    const double* l;
    const int* bnd;
    DevBnd b[kMaxBnd];
    DevMat mat;
    double gam;
    const double* U;
    double* R;
    double* F;  // device address of g_static_edge_flux
};

template <int FLUX>
__global__ void __launch_bounds__(256) k_static_edge_flux(const StaticArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.ne) return;
    const int nc = a.nc, ne = a.ne;
    const int c1 = a.c12[2 * e], c2 = a.c12[2 * e + 1];
    // the boundary index is read and checked on boundary edges only: a mesh without
    // boundary conditions (n_bnd == 0) is valid as long as no edge needs one
    const int bi = c2 >= 0 ? 0 : (a.bnd ? a.bnd[e] : -1);
    const bool bad_bnd = c2 < 0 && (bi < 0 || bi >= a.nbnd);
    if (c1 < 0 || c1 >= nc || c2 >= nc || c2 < -1 || bad_bnd) {  // inconsistent mesh: NaN, no access
        for (int k = 0; k < 4; k++) a.F[(size_t)k * ne + e] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    const double nx = a.n[2 * e], ny = a.n[2 * e + 1], l = a.l[e];
    const Prim<double> qL = cons2prim<double>(a.U[c1], a.U[nc + c1], a.U[2 * nc + c1], a.U[3 * nc + c1], a.mat.gm1);
    Prim<double> qR;
    if (c2 >= 0) {
        qR = cons2prim<double>(a.U[c2], a.U[nc + c2], a.U[2 * nc + c2], a.U[3 * nc + c2], a.mat.gm1);
    } else {
        const double Tc = temperature(qL, a.mat.gm1, a.mat.Cv);
        qR = ghost_state(a.b[bi], qL, Tc, nx, ny, a.mat.M);
    }
    double f[4];
    num_flux<double, FLUX>(f, qL, qR, nx, ny, a.gam, 1.0 / (a.gam - 1.0), 100);
    const double lh = l * 0.5;
    for (int k = 0; k < 4; k++) {  // both Gauss points see the same states
        double s = 0.0;
        s = s + f[k];
        s = s + f[k];
        a.F[(size_t)k * ne + e] = s * lh;
    }
}

__global__ void __launch_bounds__(256) k_static_gather(const StaticArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nc) return;
    const int nc = a.nc, ne = a.ne;
    double r[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < 3; k++) {  // ascending edge numbers: the reference's accumulation order
        const int e = a.cell_edges[3 * i + k];
        const bool bad = e < 0 || e >= ne;
        const bool side2 = !bad && a.c12[2 * e] != i;
        for (int q = 0; q < 4; q++) {
            const double v = bad ? __longlong_as_double(0x7ff8000000000000ll) : a.F[(size_t)q * ne + e];
            r[q] = side2 ? r[q] + v : r[q] - v;
        }
    }
    for (int q = 0; q < 4; q++) a.R[(size_t)q * nc + i] = r[q];
}

// Device address of the scratch array, looked up once per device with that
// device current (the host-side symbol is only a stand-in, not a device address).
// A cudaDeviceReset ends the context that address belongs to; cfd2d_static_reset
// forgets the cached addresses so that the next call looks them up again.
std::mutex g_mu;
void* g_scratch_dev[64] = {nullptr};

}  // namespace
}  // namespace cfd2d

extern "C" int cfd2d_residual_first_order_static(int n_cells, int n_edges, const int* cell_edges,
                                                 const int* edge_c12, const double* edge_n, const double* edge_l,
                                                 const int* edge_bnd, int n_bnd, const int* bnd_kind,
                                                 const double* bnd_par, double M, double Cp, int flux,
                                                 const double* U, double* R, void* stream) {
    using namespace cfd2d;
    if (n_cells <= 0 || n_edges <= 0 || !cell_edges || !edge_c12 || !edge_n || !edge_l || !U || !R ||
        (n_bnd > 0 && (!edge_bnd || !bnd_kind || !bnd_par)) || n_bnd < 0 || flux < 0 || flux > 3)
        return CFD2D_ERR_INVALID_ARG;
    if (n_edges > CFD2D_STATIC_MAX_EDGES || n_bnd > kMaxBnd) return CFD2D_ERR_CAPACITY;
    for (int k = 0; k < n_bnd; k++)
        if (bnd_kind[k] < BND_INLET || bnd_kind[k] > BND_WALL_NO_SLIP) return CFD2D_ERR_INVALID_ARG;
    // an error some earlier, unrelated CUDA work left pending is not this call's: it is
    // reported before anything runs and left pending for its owner
    if (cudaPeekAtLastError() != cudaSuccess) return CFD2D_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CFD2D_ERR_NO_DEVICE;
    void* scratch;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_dev[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_static_edge_flux) != cudaSuccess || !p) return CFD2D_ERR_CUDA;
            g_scratch_dev[dev] = p;
        }
        scratch = g_scratch_dev[dev];
    }
    StaticArgs a{};
    a.nc = n_cells;
    a.ne = n_edges;
    a.nbnd = n_bnd;
    a.cell_edges = cell_edges;
    a.c12 = edge_c12;
    a.n = edge_n;
    a.l = edge_l;
    a.bnd = edge_bnd;
    for (int k = 0; k < n_bnd; k++) {
        a.b[k].kind = bnd_kind[k];
        a.b[k].u = bnd_par[4 * k];
        a.b[k].v = bnd_par[4 * k + 1];
        a.b[k].T = bnd_par[4 * k + 2];
        a.b[k].p = bnd_par[4 * k + 3];
    }
    a.mat.M = M;
    a.mat.Cp = Cp;
    a.mat.Cv = Cp - GAS_R / M;
    a.mat.gam = Cp / a.mat.Cv;
    a.mat.gm1 = a.mat.gam - 1;
    a.gam = 1.4;  // FVM_TVD::run's flux gamma, src/methods/fvm_tvd.cpp:345
    a.U = U;
    a.R = R;
    a.F = static_cast<double*>(scratch);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int ge = (n_edges + 255) / 256, gc = (n_cells + 255) / 256;
    switch (flux) {
    case FLUX_LAX: k_static_edge_flux<FLUX_LAX><<<ge, 256, 0, s>>>(a); break;
    case FLUX_ROE: k_static_edge_flux<FLUX_ROE><<<ge, 256, 0, s>>>(a); break;
    case FLUX_HLLC: k_static_edge_flux<FLUX_HLLC><<<ge, 256, 0, s>>>(a); break;
    default: k_static_edge_flux<FLUX_GODUNOV><<<ge, 256, 0, s>>>(a); break;
    }
    if (cudaGetLastError() != cudaSuccess) return CFD2D_ERR_CUDA;  // the flux launch
    k_static_gather<<<gc, 256, 0, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? CFD2D_OK : CFD2D_ERR_CUDA;  // the gather launch
}

extern "C" int cfd2d_static_reset(void) {
    using namespace cfd2d;
    std::lock_guard<std::mutex> lk(g_mu);
    for (void*& p : g_scratch_dev) p = nullptr;
    return CFD2D_OK;
}
