// Batches of independent instances in one solver, per-instance time steps, and
// the launch-shape autotuner.
//
// A batch is the disjoint union of its instances' meshes: cell, edge, node,
// region, material and boundary numbers are offset per instance, so every
// kernel of the single-instance path runs unchanged over all instances at once
// (one launch per kernel kind and stage, one CUDA graph per step). The only
// per-instance quantity of the step, the global time step TAU of STEADY=0, is
// already a per-cell factor (cfl = TAU / S), so each instance keeps its own.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

#include "cfd2d.h"
#include "solver.hpp"

namespace cfd2d {

Batch merge_batch(std::vector<TaskConfig>& tasks, std::vector<Topo>& topos, std::vector<std::vector<int>>& cregs,
                  std::vector<std::vector<int>>& ebnds) {
    const size_t n = tasks.size();
    if (n == 0) throw Error(CFD2D_ERR_INVALID_ARG, "empty batch");
    Batch b;
    b.task = tasks[0];
    b.task.mats.clear();
    b.task.regions.clear();
    b.task.bnds.clear();
    Topo& u = b.topo;
    int node_off = 0, cell_off = 0, edge_off = 0, reg_off = 0, bnd_off = 0;
    for (size_t k = 0; k < n; k++) {
        const TaskConfig& t = tasks[k];
        if (t.flux != b.task.flux || t.recon != b.task.recon || t.scheme != b.task.scheme ||
            t.precision != b.task.precision || t.steady != b.task.steady)
            throw Error(CFD2D_ERR_INVALID_ARG, "batch instances must share FLUX, RECONSTRUCTION, TIME_SCHEME, "
                                               "PRECISION and STEADY");
        if (t.steady && t.cfl != b.task.cfl)
            throw Error(CFD2D_ERR_INVALID_ARG, "batch instances with local time steps must share CFL");
        const Topo& s = topos[k];
        Instance in;
        in.cell_off = cell_off;
        in.nc = s.nc;
        in.tau_xml = t.tau;
        in.cfl = t.cfl;
        b.inst.push_back(in);
        // identical materials (same M, Cp, K, ML) are stored once
        std::vector<int> mat_map(t.mats.size());
        for (size_t q = 0; q < t.mats.size(); q++) {
            const TaskMaterial& m = t.mats[q];
            int found = -1;
            for (size_t r = 0; r < b.task.mats.size(); r++) {
                const TaskMaterial& o = b.task.mats[r];
                if (o.M == m.M && o.Cp == m.Cp && o.K == m.K && o.ML == m.ML) { found = (int)r; break; }
            }
            if (found < 0) {
                found = (int)b.task.mats.size();
                b.task.mats.push_back(m);
            }
            mat_map[q] = found;
        }
        for (auto r : t.regions) {
            r.matId = mat_map[r.matId];
            b.task.regions.push_back(r);
        }
        for (auto& bc : t.bnds) b.task.bnds.push_back(bc);
        for (int v : cregs[k]) b.cell_region.push_back(v + reg_off);
        for (int v : ebnds[k]) b.edge_bnd.push_back(v >= 0 ? v + bnd_off : -1);
        u.xy.insert(u.xy.end(), s.xy.begin(), s.xy.end());
        for (int v : s.tri) u.tri.push_back(v + node_off);
        for (int v : s.cedges) u.cedges.push_back(v + edge_off);
        u.S.insert(u.S.end(), s.S.begin(), s.S.end());
        u.cx.insert(u.cx.end(), s.cx.begin(), s.cx.end());
        u.cy.insert(u.cy.end(), s.cy.begin(), s.cy.end());
        for (int e = 0; e < s.ne; e++) {
            u.n1.push_back(s.n1[e] + node_off);
            u.n2.push_back(s.n2[e] + node_off);
            u.c1.push_back(s.c1[e] + cell_off);
            u.c2.push_back(s.c2[e] >= 0 ? s.c2[e] + cell_off : -1);
            u.npts.push_back(s.npts[e]);
            u.bseg_of_edge.push_back(-1);
        }
        u.nx.insert(u.nx.end(), s.nx.begin(), s.nx.end());
        u.ny.insert(u.ny.end(), s.ny.begin(), s.ny.end());
        u.l.insert(u.l.end(), s.l.begin(), s.l.end());
        u.pts.insert(u.pts.end(), s.pts.begin(), s.pts.end());
        node_off += s.nn;
        cell_off += s.nc;
        edge_off += s.ne;
        reg_off += (int)t.regions.size();
        bnd_off += (int)t.bnds.size();
        topos[k] = Topo();  // free as we go
    }
    if (b.task.mats.size() > 255) throw Error(CFD2D_ERR_INVALID_ARG, "a batch holds at most 255 materials");
    u.nn = node_off;
    u.nc = cell_off;
    u.ne = edge_off;
    return b;
}

// calcTimeStep's STEADY=0 branch per instance: TAU_k = min(TAU_xml_k, min over its
// cells of CFL_k S / max(|u|+c, |v|+c)), computed on the host from the state
// with the expressions the device uses (correctly rounded sqrt and division).
void Solver::compute_tau_batch() {
    const int nc = dc_.nc;
    std::vector<double> U(4 * (size_t)nc);
    CUDA_CHECK(cudaMemcpyAsync(U.data(), dc_.A, U.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    std::vector<int> inst_of(nc);
    for (size_t k = 0; k < inst_.size(); k++)
        for (int o = inst_[k].cell_off; o < inst_[k].cell_off + inst_[k].nc; o++) inst_of[o] = (int)k;
    std::vector<double> tmin(inst_.size());
    for (size_t k = 0; k < inst_.size(); k++) tmin[k] = inst_[k].tau_xml;
    for (int i = 0; i < nc; i++) {
        const int k = inst_of[lay_.perm[i]];
        const TaskMaterial& m = task_.mats[cell_mat_[lay_.perm[i]]];
        const double Cv = m.Cp - GAS_R / m.M, gam = m.Cp / Cv;
        const double ro = U[i], u = U[nc + i] / ro, v = U[2 * (size_t)nc + i] / ro, E = U[3 * (size_t)nc + i] / ro;
        const double e = E - 0.5 * (u * u + v * v);
        const double p = ro * e * (gam - 1);
        const double cz = std::sqrt(gam * p / ro);
        const double a = std::fabs(u) + cz, b = std::fabs(v) + cz;
        const double t = inst_[k].cfl * lay_.S[i] / (a > b ? a : b);
        if (tmin[k] > t) tmin[k] = t;
    }
    std::vector<double> ct(nc), cf(nc);
    for (size_t k = 0; k < inst_.size(); k++) inst_[k].tau = tmin[k];
    for (int i = 0; i < nc; i++) {
        ct[i] = inst_[inst_of[lay_.perm[i]]].tau;
        cf[i] = ct[i] / lay_.S[i];
    }
    tau_ = inst_[0].tau;
    CUDA_CHECK(cudaMemcpyAsync(dc_.ctau, ct.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaMemcpyAsync(dc_.cfl, cf.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::rebuild_graph() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (graph_) cudaGraphDestroy(graph_);
    gexec_ = nullptr;
    graph_ = nullptr;
    build_graph();
}

// Launch-shape autotuner. For each kernel kind (gradients, edge fluxes, stage
// update) it times block sizes {64, 128, 256} x grids {one thread per item,
// 1, 2, 4, 8 blocks per SM (a persistent grid striding over the items)} with
// CUDA events on the solver's stream, on the solver's own mesh and state, and
// keeps the fastest. The update kernel is timed in a stage that writes only
// the stage buffer; the primitives are restored afterwards. The shapes change
// no arithmetic, so results are bit-identical for every choice.
void Solver::autotune(const char* json_path, int reps) {
    use_device();
    int dev = 0, sms = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaDeviceProp prop{};
    CUDA_CHECK(cudaGetDeviceProperties(&prop, dev));
    const int p = task_.precision;
    const int blocks[3] = {64, 128, 256};
    const int grids[5] = {0, 1, 2, 4, 8};
    cudaEvent_t a, b;
    CUDA_CHECK(cudaEventCreate(&a));
    CUDA_CHECK(cudaEventCreate(&b));
    double best_ms[N_TUNED_KINDS];
    const char* names[N_TUNED_KINDS] = {"grad", "flux", "update"};
    for (int kind = 0; kind < N_TUNED_KINDS; kind++) {
        if (kind == KIND_GRAD && (task_.recon == RECON_NONE || gauss_points_ == 0)) {
            best_ms[kind] = 0;
            continue;
        }
        LaunchShape best = dc_.shape[kind];
        best_ms[kind] = 1e30;
        for (int bs : blocks)
            for (int gm : grids) {
                dc_.shape[kind].block = bs;
                dc_.shape[kind].grid = gm * sms;
                auto run = [&] {
                    if (kind == KIND_GRAD) launch_grad(dc_, p, stream_);
                    else if (kind == KIND_FLUX) launch_flux(dc_, p, task_.flux, task_.recon, stream_);
                    else launch_update(dc_, p, TIME_HEUN, 0, stream_);
                };
                run();  // warm-up
                CUDA_CHECK(cudaEventRecord(a, stream_));
                for (int r = 0; r < reps; r++) run();
                CUDA_CHECK(cudaEventRecord(b, stream_));
                CUDA_CHECK(cudaEventSynchronize(b));
                float ms = 0;
                CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
                if (ms / reps < best_ms[kind]) {
                    best_ms[kind] = ms / reps;
                    best = dc_.shape[kind];
                }
            }
        dc_.shape[kind] = best;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    launch_prims(dc_, p, stream_);
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    rebuild_graph();
    if (json_path && *json_path) {
        FILE* f = std::fopen(json_path, "w");
        if (!f) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + json_path + "' opening error.");
        std::fprintf(f, "{\"device\": \"%s\", \"sms\": %d, \"cells\": %d, \"edges\": %d, \"precision\": %d, "
                        "\"flux\": %d, \"recon\": %d, \"instances\": %d",
                     prop.name, sms, dc_.nc, dc_.ne, p, task_.flux, task_.recon, n_instances());
        for (int kind = 0; kind < N_TUNED_KINDS; kind++)
            std::fprintf(f, ", \"%s\": {\"block\": %d, \"grid\": %d, \"ms\": %.6f}", names[kind],
                         dc_.shape[kind].block, dc_.shape[kind].grid, best_ms[kind]);
        std::fprintf(f, "}\n");
        std::fclose(f);
    }
}

void Solver::load_tuning(const char* json_path) {
    use_device();
    std::ifstream in(json_path);
    if (!in) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + json_path + "' opening error.");
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string s = ss.str();
    const char* names[N_TUNED_KINDS] = {"grad", "flux", "update"};
    for (int kind = 0; kind < N_TUNED_KINDS; kind++) {
        const size_t k = s.find(std::string("\"") + names[kind] + "\"");
        if (k == std::string::npos) continue;
        int bs = 0, gr = 0;
        const size_t pb = s.find("\"block\":", k), pg = s.find("\"grid\":", k);
        if (pb == std::string::npos || pg == std::string::npos) continue;
        bs = std::atoi(s.c_str() + pb + 8);
        gr = std::atoi(s.c_str() + pg + 7);
        if (bs != 64 && bs != 128 && bs != 256) throw Error(CFD2D_ERR_INVALID_ARG, "tuning file: bad block size");
        if (gr < 0) throw Error(CFD2D_ERR_INVALID_ARG, "tuning file: bad grid");
        dc_.shape[kind].block = bs;
        dc_.shape[kind].grid = gr;
    }
    rebuild_graph();
}

}  // namespace cfd2d
