// The implicit method FVM_TVD_IMPLICIT (src/methods/fvm_tvd_implicit.cpp) on the GPU.
//
// Per step: primitives and Green-Gauss gradients of the cell-centre states, the edge
// fluxes at two Gauss points, then one kernel per cell that gathers its right-hand side
// and its block row of the Roe-linearised system
//     (S/cTau I + sum_faces l A+(n_f)) dU_i + sum_faces l A-(n_f) dU_nb(f) = -sum_faces F_f l/2,
// GMRES on that block system, smoothing, the update with limits, remediation and the
// limited-cell count; the host applies the CFL rules. One CUDA graph per step.
//
// Layout in HBM (storage = RCM cell order, faces of a cell in ascending original edge
// order as Cell::edgesInd lists them): diagonal blocks D[column][nc][row] and face
// blocks O[face][column][nc][row] (the matrix-vector product runs four threads per
// cell, one per row, and every load of a block column is one contiguous run across a
// warp), right-hand side and every Krylov vector as [nc][4] (x[4c + k], the
// reference's numbering of unknowns).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.hpp"
#include "mesh.hpp"
#include "task.hpp"

namespace cfd2d {

// entry (row r, column q) of cell i's diagonal block and of its face k's block
__host__ __device__ inline size_t dblk(int nc, int i, int r, int q) { return ((size_t)q * nc + i) * 4 + r; }
__host__ __device__ inline size_t oblk(int nc, int i, int k, int r, int q) {
    return ((size_t)(4 * k + q) * nc + i) * 4 + r;
}

// Boundary kinds of the implicit method (Boundary::BOUND_*, src/global.h:233-235).
enum ImpBndKind { IBND_INLET = 1, IBND_OUTLET = 2, IBND_WALL = 3 };
// MatrixSolver::RESULT_* (src/methods/solvers/MatrixSolver.h:13-16)
enum : int { SOLVE_OK = 0, SOLVE_MAX_ITER = 0x2, SOLVE_CONVERG = 0x4 };

constexpr int kGmresMaxKdim = 64;   // Krylov dimension bound of the device control block
constexpr int kRedBlocks = 608;     // blocks of every reduction kernel (4 per SM)

// GMRES state shared by the kernels of one solve (device memory).
struct GmresCtl {
    double bnorm, eps_abs, rnorm, rel;
    double H[(kGmresMaxKdim + 1) * kGmresMaxKdim];  // H[i * kdim + j]
    double cs[kGmresMaxKdim], sn[kGmresMaxKdim], g[kGmresMaxKdim + 1], y[kGmresMaxKdim];
    double s[kGmresMaxKdim + 1];     // Krylov vector k is s[k] V_k (V_k stored unscaled)
    double coef[kGmresMaxKdim];      // h_ij s_i of the column being orthogonalised
    int it;        // iterations over all cycles
    int cols;      // columns of the current cycle
    int done;      // the cycle's Arnoldi loop has ended
    int status;    // SOLVE_* bits once final
    int restart;   // the true residual asks for another cycle
    int final_;    // the solve has ended (converged, failed or out of iterations)
    int n_lim;     // limited cells after the update (getLimitedCellsCount)
    int cycle;     // cycle counter
};

// Everything the implicit kernels read; passed by value.
struct ImpCase {
    int nc, ne, n_int;
    int flux;                 // FLUX_GODUNOV or FLUX_LAX
    int steady, smoothing, newton_cap;
    int kdim, maxit;
    double eps;               // GMRES relative tolerance
    double smoothing_par;
    double tau_xml;
    double gam_flux, ig1_flux;
    RimGas<double> rg_flux;   // the exact Riemann solver's constants of gam_flux
    double lim_rmin, lim_rmax, lim_pmin, lim_pmax, lim_umax;
    // geometry (storage order)
    const int* face;          // 3*nc: (edge << 1) | side (side 1: the cell is c2)
    const int* ec1;           // ne
    const int* ec2;
    const int* ebnd;
    const double* nx;
    const double* ny;
    const double* l;
    const double* dl;         // 8*ne Gauss-point offsets (gp0: dxL dyL dxR dyR, gp1: ...)
    const double* S;          // nc
    const double* invS;       // nc, RN(1/S)
    const int* nbr;           // 3*nc the cell across each face (storage), or the cell itself on the boundary
    const int* iperm;         // original -> storage
    const uint8_t* cmat;      // nc or nullptr
    const DevMat* mats;
    const DevBnd* bnds;       // kind = ImpBndKind, (u, v, T, p) = (Vx, Vy, T, P)
    DevMat mat0;
    // state
    double* A;                // 4*nc conserved (SoA)
    double* W;                // nc x 4 primitives r, u, v, p
    double* G;                // nc x 8 gradients
    double* F;                // ne x 4 edge fluxes times l/2
    double* R;                // ne x 4 Roe state of the edge's centre states: u, v, c, H
    double* ctau;             // nc
    double* cfl;              // 1: the CFL number of the steady rules
    unsigned* flags;          // nc
    unsigned* err;            // 1
    // block system
    double* D;                // 16*nc
    double* O;                // 48*nc
    double* b;                // 4*nc
    double* x;                // 4*nc
    double* x2;               // 4*nc (smoothing output)
    double* V;                // (kdim + 1) * 4*nc Krylov basis
    double* r;                // 4*nc residual of a restart
    double* part;             // (kGmresMaxKdim + 1) x kRedBlocks partial sums of the reductions
    GmresCtl* ctl;
    int* n_lim;               // 1
};

// ---- kernels (implicit.cu: FP64 assembly, parity with the reference; gmres.cu: the solver)
void imp_launch_prims(const ImpCase& c, cudaStream_t s);
void imp_launch_grad(const ImpCase& c, cudaStream_t s);
void imp_launch_flux(const ImpCase& c, cudaStream_t s);
void imp_launch_assemble(const ImpCase& c, cudaStream_t s);
void imp_launch_post(const ImpCase& c, cudaStream_t s);   // smoothing, update + limits, remediation, count
void imp_launch_gmres_cycle(const ImpCase& c, bool first, cudaStream_t s);
void imp_launch_permute_blocks(const ImpCase& c, double* dst, int which, cudaStream_t s);

class ImplicitSolver {
public:
    ImplicitSolver(const TaskConfig& t, Topo&& topo, const std::vector<int>& cell_region,
                   const std::vector<int>& edge_bnd);
    ~ImplicitSolver();
    ImplicitSolver(const ImplicitSolver&) = delete;
    ImplicitSolver& operator=(const ImplicitSolver&) = delete;

    int step(int n);          // CFD2D_OK or a warning code
    int run();
    void get_state(double* ro, double* ru, double* rv, double* re);
    void set_state(const double* ro, const double* ru, const double* rv, const double* re);
    void get_ctau(double* out);
    void get_flags(unsigned* out);
    // the block system of the current state (reference cell order, faces in Cell::edgesInd order)
    void system(double* diag, double* off, double* rhs, double* ctau);
    void save_vtk(int step);
    // restart files: state, cTau, flags, step counter, time, CFL number, solver status
    void save_state(const char* path);
    void load_state(const char* path);
    double timed_steps(int n);
    // n steps launched phase by phase with CUDA events around each phase: ms and launch
    // counts of 0 primitives + gradients, 1 Gauss-point fluxes + Roe states, 2 block-row
    // assembly, 3 GMRES + update (the steps are taken)
    void profile_steps(int n, double ms[4], int launches[4]);

    const TaskConfig& task() const { return task_; }
    const Topo& topo() const { return topo_; }
    const Layout& layout() const { return lay_; }
    int n_steps() const { return steps_; }
    double time() const { return t_; }
    double cfl() const { return cfl_; }
    int last_iters() const { return last_.it; }
    double last_rel() const { return last_.rel; }
    int last_status() const { return last_.status; }
    int last_n_lim() const { return last_.n_lim; }
    size_t device_bytes() const { return bytes_; }

private:
    template <typename T> T* dalloc(size_t n);
    template <typename T> T* upload(const std::vector<T>& v);
    void build_graphs();
    void assemble_only();
    void one_step();
    int read_status();
    void use_device() const { cudaSetDevice(dev_); }

    TaskConfig task_;
    Topo topo_;
    Layout lay_;
    int dev_ = 0;
    ImpCase ic_{};
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t g_step_ = nullptr;     // assembly + first GMRES cycle + post
    cudaGraphExec_t g_restart_ = nullptr;  // another GMRES cycle + post
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
    double* stage_ = nullptr;              // 48*nc staging for permutations
    GmresCtl* ctl_host_ = nullptr;         // pinned copy of the control block
    GmresCtl last_{};
    double t_ = 0, cfl_ = 0;
    int steps_ = 0;
    int solver_err_ = 0;
    int failed_in_row_ = 0;                // consecutive failed solves
    static constexpr int kMaxFailedSolves = 1000;
};

}  // namespace cfd2d
