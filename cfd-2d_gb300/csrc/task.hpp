// task.xml of the FVM_TVD method (src/methods/fvm_tvd.cpp:26-128, src/bnd_cond.cpp:10-72),
// of FVM_TVD_IMPLICIT (src/methods/fvm_tvd_implicit.cpp:13-184) and of FEM_RKDG
// (src/methods/fem_rkdg.cpp:23-235).
#pragma once
#include <string>
#include <vector>

#include "kernels.hpp"
#include "mesh.hpp"

namespace cfd2d {

struct TaskMaterial { std::string name; int id = 0; double M = 0, Cp = 0, K = 0, ML = 0; };
struct TaskRegion { int id = 0, matId = 0, cellType = 0; std::string name; double u = 0, v = 0, T = 0, p = 0; };
struct TaskBound { int edgeType = 0; int kind = 0; std::string name; double par[4] = {0, 0, 0, 0}; };

enum MethodKind { METHOD_FVM_TVD = 0, METHOD_FVM_TVD_IMPLICIT = 1, METHOD_FEM_RKDG = 2 };

struct TaskConfig {
    std::string path, dir;
    int method = METHOD_FVM_TVD;
    int steady = 1;
    double tau = 0, tmax = 0, cfl = 0;
    int step_max = 0, file_step = 1, print_step = 1;
    double lim_rmin = 0, lim_rmax = 0, lim_pmin = 0, lim_pmax = 0, lim_umax = 0;
    std::vector<TaskMaterial> mats;
    std::vector<TaskRegion> regions;
    std::vector<TaskBound> bnds;
    std::string mesh_name, mesh_type;
    int gauss_points = -1;    // <mesh><gaussPoints>: Triangle meshes get 1 point (no flux) unless 2
    // method selections; absent elements give the reference's method
    int flux = FLUX_GODUNOV, recon = RECON_LINEAR, scheme = TIME_HEUN, precision = PREC_FP64;
    int reorder = -1;         // cell order: 0 file order, 1 RCM, 2 Hilbert; -1: RCM (Hilbert with the fused stage)
    int fused = -1;           // mixed form (-1: 3), 0 per-kernel stages; SSP-RK3 / Heun: 1 one tiled kernel per stage (gradients, fluxes,
                              // update), 2 gradients then one tiled flux-and-update kernel per stage,
                              // 3 the flux kernel forms the two cells' gradients (no gradient kernel)
    int adj_store = -1;       // adjoint segment store: 0 states only, 1 + primitives, 2 + gradients,
                              // 3 + HLLC flux records, -1 by memory
    double adj_memory = 0.0;  // device-memory budget of the handle for the adjoint (bytes; 0: 80% of the free memory)
    int newton_cap = 100;     // iteration cap of the exact Riemann solver
    int flux_pipe = 1;        // mixed form: the software-pipelined flux kernel (0: one thread per edge)
    // FVM_TVD_IMPLICIT (src/methods/fvm_tvd_implicit.cpp:13-184): <CFL> start (in cfl),
    // scale, max, step, max_limited_cells; <smoothing>; the matrix solver's parameters
    // (run() hard-codes 20 iterations and 1e-7, SolverHypreGmres.h the Krylov dimension 30)
    double cfl_scale = 1.0, cfl_max = 1.0, max_lim_cells = 0.0;
    int cfl_step = 1;
    int smoothing = 0;
    double smoothing_par = 0.0;
    double gmres_eps = 1.0e-7;
    int gmres_maxit = 20, gmres_kdim = 30;
    // FEM_RKDG (src/methods/fem_rkdg.cpp:23-60): BASE_FUNC_COUNT, GP_CELL_COUNT, GP_EDGE_COUNT;
    // RK_MODE (an extension): 0 the reference's stages as written, 1 Heun's average with U^n
    int dg_func_count = 3, dg_gp_cell = 4, dg_gp_edge = 3, dg_rk = 0;
};

TaskConfig parse_task(const std::string& path);

// Region initial state exactly as init forms it: URS(2), URS(1), convertParToCons.
void region_state(const TaskMaterial& m, const TaskRegion& r, double U[4]);

// Bind a raw mesh to the task: region per cell (by name) and boundary per
// boundary edge (by name for UNV groups, by edgeType for Triangle markers).
void bind_mesh(const TaskConfig& t, const RawMesh& raw, const Topo& topo, std::vector<int>& cell_region,
               std::vector<int>& edge_bnd);
// FVM_TVD_IMPLICIT's binding: region by the cell's integer type (the .ele attribute,
// getRegionByCellType, :1027-1036), boundary by the edge's type (the .poly marker, -1
// for a boundary edge the .poly does not list; boundaryCond, :963-975).
void bind_mesh_implicit(const TaskConfig& t, const RawMesh& raw, const Topo& topo, std::vector<int>& cell_region,
                        std::vector<int>& edge_bnd);

}  // namespace cfd2d
