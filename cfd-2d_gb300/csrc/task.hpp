// task.xml of the FVM_TVD method (src/methods/fvm_tvd.cpp:26-128, src/bnd_cond.cpp:10-72).
#pragma once
#include <string>
#include <vector>

#include "kernels.hpp"
#include "mesh.hpp"

namespace cfd2d {

struct TaskMaterial { std::string name; int id = 0; double M = 0, Cp = 0, K = 0, ML = 0; };
struct TaskRegion { int id = 0, matId = 0, cellType = 0; std::string name; double u = 0, v = 0, T = 0, p = 0; };
struct TaskBound { int edgeType = 0; int kind = 0; std::string name; double par[4] = {0, 0, 0, 0}; };

struct TaskConfig {
    std::string path, dir;
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
    int fused = -1;           // mixed form, SSP-RK3 / Heun: 1 runs one tiled kernel per stage (opt-in)
    int adj_store = -1;       // adjoint segment store: 0 states only, 1 + primitives, 2 + gradients, -1 by memory
    int newton_cap = 100;     // iteration cap of the exact Riemann solver
};

TaskConfig parse_task(const std::string& path);

// Region initial state exactly as init forms it: URS(2), URS(1), convertParToCons.
void region_state(const TaskMaterial& m, const TaskRegion& r, double U[4]);

// Bind a raw mesh to the task: region per cell (by name) and boundary per
// boundary edge (by name for UNV groups, by edgeType for Triangle markers).
void bind_mesh(const TaskConfig& t, const RawMesh& raw, const Topo& topo, std::vector<int>& cell_region,
               std::vector<int>& edge_bnd);

}  // namespace cfd2d
