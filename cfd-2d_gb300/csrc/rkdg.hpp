// The explicit discontinuous Galerkin method FEM_RKDG (src/methods/fem_rkdg.cpp) on the GPU.
//
// P1 basis per triangle (1, (x-xc)/HX, (y-yc)/HY), cell quadrature of 3 or 4 points, edge
// quadrature of 2 or 3 points, two Runge-Kutta stages. Per stage two kernels: one thread
// per edge evaluates both sides' polynomials at the edge's Gauss points, the Riemann flux
// (GODUNOV or LAX) and the two sides' surface integrals; one thread per cell evaluates the
// volume integral at the cell's Gauss points, gathers its three edges' integrals in
// ascending original edge number (the order of the reference's edge loop), multiplies by
// the inverse mass matrix and cTau and forms the stage result. One CUDA graph per step.
//
// Layout in HBM (storage = RCM cell order; edges sorted by their lower storage cell,
// boundary edges last):
//   cells:  coefficients A, B [nc][12] (ro[3] ru[3] rv[3] re[3], 96 B, one record per
//           gather), basis values at the cell's Gauss points cF [nc][gc][2], 1/HX and 1/HY
//           ih [nc][2], the centre's basis values fc [nc][2], cellJ, S, cTau [nc],
//           inverse mass matrix invA [nc][9], faces face[3][nc] = (edge << 3) | (slot << 1)
//           | side in ascending original edge order (slot: the edge's place in the cell's
//           node order, the time step's Gauss-point index as the reference reads it).
//   edges:  c1, c2, boundary index [ne], normal and edgeJ [ne], basis values of both sides
//           at the Gauss points eF [ne][ge][4], the sides' surface integrals E1, E2 [ne][12]
//           (already times edgeJ).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.hpp"
#include "task.hpp"

namespace cfd2d {

enum DgRkMode { DG_RK_REFERENCE = 0, DG_RK_HEUN = 1 };

// A material with the constants the method derives from it (Material::URS, getGamma).
struct DgMat {
    double M, Cv, gam, gm1, ig1, iCv;  // ig1 = RN(1/(gam-1)), iCv = RN(1/Cv)
    RimGas<double> rg;                 // the exact Riemann solver's constants of gam
};

// Everything the kernels read; passed by value.
struct DgCase {
    int nc, ne, n_int, gc, ge;
    int steady, rk_mode, newton_cap;
    double cfl;
    double cgw[4];            // cell Gauss weights (calcGaussPar)
    double egw[3];            // edge Gauss weights
    // cells (storage order)
    const int* face;          // 3*nc
    const double* cF;         // nc x gc x 2
    const double* ih;         // nc x 2
    const double* fc;         // nc x 2
    const double* cellJ;      // nc
    const double* S;          // nc
    const double* invA;       // nc x 9
    const uint8_t* cmat;      // nc or nullptr (one material)
    const uint8_t* cflag;     // nc: bit 0 = the reference's ro_old shares the cell's coefficients
    const int* iperm;         // original -> storage
    // edges (storage order)
    const int* ec1;
    const int* ec2;
    const int* ebnd;
    const double* enx;
    const double* eny;
    const double* edgeJ;
    const double* eF;         // ne x ge x 4: F1, F2 of c1, then of c2
    const DgMat* mats;
    DgMat mat0;
    const DevBnd* bnds;
    // state
    double* A;                // nc x 12: U^n and the step's result
    double* B;                // nc x 12: the first stage's result
    double* E1;               // ne x 12
    double* E2;               // ne x 12
    double* ctau;             // nc
    unsigned long long* tmin; // 1: min over cells of S/maxU (bits of a non-negative double)
    unsigned long long* res;  // 4: residual maxima (bits)
    unsigned* err;            // 1
};

// ---- kernels (rkdg.cu, -fmad=false: every product and sum rounds on its own)
void dg_launch_edges(const DgCase& c, int flux, const double* U, cudaStream_t s);
// stage 1: B = A + cTau invA R(A); stage 2: A = average of (B + cTau invA R(B)) with the
// old state, residual maxima into c.res when with_res
void dg_launch_cells(const DgCase& c, int stage, bool with_res, cudaStream_t s);
// calcTimeStep: steady -> cTau per cell; unsteady -> c.tmin
void dg_launch_time_step(const DgCase& c, cudaStream_t s);
void dg_launch_fill(double* dst, double v, int n, cudaStream_t s);
// coefficient permutation between caller order (original cells, 12 per cell) and storage
void dg_launch_gather(const DgCase& c, const double* src_orig, double* dst_store, cudaStream_t s);
void dg_launch_scatter(const DgCase& c, const double* src_store, double* dst_orig, cudaStream_t s);

// A .proc mesh part (Grid::readMeshFiles, src/mesh/grid.cpp:275-420) or mesh arrays.
struct DgMesh {
    int nn = 0, nc = 0, ne = 0;
    int nn_own = 0;                  // the part's own nodes (nCount), written to the VTU file
    std::vector<double> xy;          // 2*nn
    std::vector<int> tri;            // 3*nc
    std::vector<std::string> names;  // distinct cell type names
    std::vector<int> cell_name;      // nc, index into names
    std::vector<int> en;             // 2*ne
    std::vector<int> etype;          // ne: 0 inside, 0x100 named, else the edgeType number
    std::vector<std::string> ename;  // ne
};
DgMesh read_proc_mesh(const std::string& path);
// Mesh arrays: edges numbered by first appearance over the cells' sides (t0,t1), (t1,t2),
// (t2,t0), oriented as first seen; boundary edges take the boundary of their segment.
DgMesh dg_mesh_from_arrays(int nn, const double* xy, int nc, const int* tri, const int* cell_region,
                           const std::vector<std::string>& region_names, int nb, const int* bseg,
                           const int* bseg_bnd, const std::vector<TaskBound>& bnds);

class RkdgSolver {
public:
    RkdgSolver(const TaskConfig& t, DgMesh&& mesh);
    ~RkdgSolver();
    RkdgSolver(const RkdgSolver&) = delete;
    RkdgSolver& operator=(const RkdgSolver&) = delete;

    int step(int n);
    int run();
    // coefficients in caller order, 12 per cell (ro[3] ru[3] rv[3] re[3]); any device-
    // addressable or pageable host buffer
    void get_coeffs(double* out);
    // sets the coefficients and redoes the time step from the XML TAU, as init does
    void set_coeffs(const double* in);
    // cell-centre conserved values (the polynomial at the centre), caller order
    void get_state(double* ro, double* ru, double* rv, double* re);
    // piecewise-constant state: coefficients (value, 0, 0) per variable, as init forms
    // them from the regions (convertParToCons), then the time step as set_coeffs
    void set_state(const double* ro, const double* ru, const double* rv, const double* re);
    void get_ctau(double* out);
    void set_tau(double tau);        // impose a time step (every cell)
    void residuals(double out[4]);   // of the last step
    void save_vtu(int step);
    // restart files: coefficients, cTau, step counter, time and TAU
    void save_state(const char* path);
    void load_state(const char* path);
    double timed_steps(int n);      // device ms of n steps (graph replays between CUDA events)
    // n steps launched kernel by kernel with events: ms of 0 edge kernels, 1 cell kernels,
    // 2 time step (steady), launches per step in launches[0..2]
    void profile_steps(int n, double ms[3], int launches[3]);

    const TaskConfig& task() const { return task_; }
    int nc() const { return mesh_.nc; }
    int ne() const { return mesh_.ne; }
    int n_nodes() const { return mesh_.nn; }
    int n_boundary_edges() const { return c_.ne - c_.n_int; }
    int n_steps() const { return steps_; }
    double time() const { return t_; }
    double tau() const { return tau_; }
    size_t device_bytes() const { return bytes_; }

private:
    template <typename T> T* dalloc(size_t n);
    template <typename T> T* upload(const std::vector<T>& v);
    void build_graphs();
    void time_step();
    void one_step(bool with_res);
    int read_status();
    void use_device() const { cudaSetDevice(dev_); }

    TaskConfig task_;
    DgMesh mesh_;
    int dev_ = 0;
    DgCase c_{};
    double centre_value(const double* a, int i) const;

    std::vector<int> perm_;           // storage -> original
    std::vector<int> iperm_;          // original -> storage
    std::vector<double> fc_;          // 2*nc basis values at the centres, original order
    std::vector<int> cmat_orig_;
    std::vector<DgMat> mats_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t g_step_ = nullptr;      // two stages
    cudaGraphExec_t g_step_res_ = nullptr;  // two stages + residuals
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
    double* stage_ = nullptr;               // 12*nc staging for permutations
    unsigned long long* host_bits_ = nullptr;  // pinned: tmin, res[4]
    double t_ = 0, tau_ = 0;
    int steps_ = 0;
    bool res_valid_ = false;
};

}  // namespace cfd2d
