// extern "C" entry points (include/cfd2d.h). Every call catches everything and
// returns a status code; the message of the last failure is kept per thread.
#include <sys/stat.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "cfd2d.h"
#include "implicit.hpp"
#include "rkdg.hpp"
#include "mesh.hpp"
#include "solver.hpp"
#include "task.hpp"

// One handle: the explicit solver (s) or the implicit one (imp).
struct cfd2d_solver {
    std::unique_ptr<cfd2d::Solver> s;
    std::unique_ptr<cfd2d::ImplicitSolver> imp;
    std::unique_ptr<cfd2d::RkdgSolver> dg;
};

struct cfd2d_mesh {
    cfd2d::Topo topo;
    std::vector<int> edge_bnd;
};

namespace {

thread_local std::string g_err;

// An NVTX range around each entry point that does GPU work (visible to Nsight
// Systems / Compute; without a tool attached NVTX calls are no-ops).
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

template <typename F>
int guarded(F&& f) {
    try {
        g_err.clear();
        return f();
    } catch (const cfd2d::Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(CFD2D_ERR_CAPACITY, "host memory exhausted");
    } catch (const std::exception& e) {
        return fail(CFD2D_ERR_INVALID_ARG, e.what());
    } catch (...) {
        return fail(CFD2D_ERR_INVALID_ARG, "unknown error");
    }
}

bool file_exists(const std::string& p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

std::string resolve(const cfd2d::TaskConfig& t, const std::string& name, const char* probe_ext) {
    if (name.empty() || name[0] == '/') return name;
    if (file_exists(name + probe_ext)) return name;
    std::string alt = t.dir + "/" + name;
    if (file_exists(alt + probe_ext)) return alt;
    return name;
}

// Read the task's mesh and bind it (MeshReader::create + the binding in FVM_TVD::init).
void load_task_mesh(const cfd2d::TaskConfig& t, cfd2d::Topo& topo, std::vector<int>& cell_region,
                    std::vector<int>& edge_bnd, int& gauss_points) {
    cfd2d::RawMesh raw;
    if (t.method == cfd2d::METHOD_FVM_TVD_IMPLICIT) {  // Grid::initFromFiles, src/mesh/grid.cpp:51-252
        raw = cfd2d::read_triangle(resolve(t, t.mesh_name, ".node"));
        gauss_points = 2;
        topo = cfd2d::build_topology(raw.nn(), raw.xy.data(), raw.nc(), raw.tri.data(), raw.neigh.data(),
                                     (int)raw.bseg.size() / 2, raw.bseg.data(), false, 2);
        cfd2d::bind_mesh_implicit(t, raw, topo, cell_region, edge_bnd);
        return;
    }
    if (t.mesh_type == "salome_unv") {
        raw = cfd2d::read_unv(resolve(t, t.mesh_name, ""));
        gauss_points = 2;
    } else {
        raw = cfd2d::read_triangle(resolve(t, t.mesh_name, ".node"));
        // the reference's Triangle reader gives every edge one point, so its
        // Gauss-point loop never runs (src/mesh/MeshReaderBerkleyTriangle.cpp:102)
        gauss_points = t.gauss_points == 2 ? 2 : 0;
        if (gauss_points == 0)
            cfd2d::log_line("WARNING: berkeley_triangle mesh: edges carry one point as in the reference, "
                            "so no flux is computed; set <mesh><gaussPoints value=\"2\"/> for two Gauss points\n");
    }
    topo = cfd2d::build_topology(raw.nn(), raw.xy.data(), raw.nc(), raw.tri.data(),
                                 raw.berkeley ? raw.neigh.data() : nullptr, (int)raw.bseg.size() / 2,
                                 raw.bseg.data(), !raw.berkeley, gauss_points);
    cfd2d::bind_mesh(t, raw, topo, cell_region, edge_bnd);
}

// Neighbours as the Triangle generator's .neigh lists them (neighbour j across the
// edge opposite node j, -2 for none after the loader's decrement), from the triangles.
std::vector<int> triangle_neigh(int nc, const int* tri) {
    std::vector<std::pair<long long, int>> keys(3 * (size_t)nc);
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            long long a = tri[3 * i + (j + 1) % 3], b = tri[3 * i + (j + 2) % 3];
            keys[3 * (size_t)i + j] = {std::min(a, b) * (1ll << 32) + std::max(a, b), 3 * i + j};
        }
    std::sort(keys.begin(), keys.end());
    std::vector<int> nb(3 * (size_t)nc, -2);
    for (size_t q = 0; q + 1 < keys.size(); q++)
        if (keys[q].first == keys[q + 1].first) {
            nb[keys[q].second] = keys[q + 1].second / 3;
            nb[keys[q + 1].second] = keys[q].second / 3;
        }
    return nb;
}

void check_desc(const cfd2d_mesh_desc* m) {
    if (!m || m->n_nodes <= 0 || m->n_cells <= 0 || !m->xy || !m->tri || m->n_bsegs < 0 ||
        (m->n_bsegs > 0 && (!m->bseg || !m->bseg_bnd)))
        throw cfd2d::Error(CFD2D_ERR_INVALID_ARG, "mesh description is incomplete");
}

cfd2d::Topo topo_from_desc(const cfd2d_mesh_desc* m, const int* berkeley_neigh, int gauss_points) {
    return cfd2d::build_topology(m->n_nodes, m->xy, m->n_cells, m->tri, berkeley_neigh, m->n_bsegs, m->bseg,
                                 berkeley_neigh == nullptr, gauss_points);
}

std::vector<int> edge_bnd_from_desc(const cfd2d_mesh_desc* m, const cfd2d::Topo& t, int nbnd) {
    std::vector<int> eb(t.ne, -1);
    for (int e = 0; e < t.ne; e++) {
        if (t.c2[e] >= 0) continue;
        int s = t.bseg_of_edge[e];
        int b = s >= 0 ? m->bseg_bnd[s] : -1;
        if (b < 0 || (nbnd >= 0 && b >= nbnd))
            throw cfd2d::Error(CFD2D_ERR_EDGE_UNKNOWN,
                               "ERROR (boundary condition): unknown edge type of edge " + std::to_string(e) + "...");
        eb[e] = b;
    }
    return eb;
}

// The explicit solver of a handle; entry points of the explicit method only fail on
// an implicit handle.
cfd2d::Solver& ex(const cfd2d_t* h) {
    if (!h->s)
        throw cfd2d::Error(CFD2D_ERR_INVALID_ARG,
                           h->dg ? "not available for the FEM_RKDG method" : "not available for the FVM_TVD_IMPLICIT method");
    return *h->s;
}

cfd2d::RkdgSolver& dgs(const cfd2d_t* h) {
    if (!h->dg) throw cfd2d::Error(CFD2D_ERR_INVALID_ARG, "not a FEM_RKDG handle");
    return *h->dg;
}

}  // namespace

extern "C" {

int cfd2d_create(const char* task_xml_path, cfd2d_t** out) {
    Range r("cfd2d_create");
    return guarded([&] {
        if (!task_xml_path || !out) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        *out = nullptr;
        cfd2d::TaskConfig t = cfd2d::parse_task(task_xml_path);
        auto h = std::make_unique<cfd2d_solver>();
        if (t.method == cfd2d::METHOD_FEM_RKDG) {  // Grid::readMeshFiles: mesh/mesh.0000.proc
            cfd2d::DgMesh m = cfd2d::read_proc_mesh(resolve(t, t.mesh_name, ""));
            h->dg = std::make_unique<cfd2d::RkdgSolver>(t, std::move(m));
            *out = h.release();
            return CFD2D_OK;
        }
        cfd2d::Topo topo;
        std::vector<int> cr, eb;
        int gp = 2;
        load_task_mesh(t, topo, cr, eb, gp);
        if (t.method == cfd2d::METHOD_FVM_TVD_IMPLICIT)
            h->imp = std::make_unique<cfd2d::ImplicitSolver>(t, std::move(topo), cr, eb);
        else
            h->s = std::make_unique<cfd2d::Solver>(t, std::move(topo), cr, eb, gp);
        *out = h.release();
        return CFD2D_OK;
    });
}

int cfd2d_create_with_mesh(const char* task_xml_path, const cfd2d_mesh_desc* mesh, cfd2d_t** out) {
    Range r("cfd2d_create_with_mesh");
    return guarded([&] {
        if (!task_xml_path || !out) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        *out = nullptr;
        check_desc(mesh);
        if (!mesh->cell_region) return fail(CFD2D_ERR_INVALID_ARG, "cell_region is required");
        cfd2d::TaskConfig t = cfd2d::parse_task(task_xml_path);
        if (t.method == cfd2d::METHOD_FEM_RKDG) {
            std::vector<std::string> names;
            for (auto& r : t.regions) names.push_back(r.name);
            cfd2d::DgMesh m = cfd2d::dg_mesh_from_arrays(mesh->n_nodes, mesh->xy, mesh->n_cells, mesh->tri,
                                                         mesh->cell_region, names, mesh->n_bsegs, mesh->bseg,
                                                         mesh->bseg_bnd, t.bnds);
            auto h = std::make_unique<cfd2d_solver>();
            h->dg = std::make_unique<cfd2d::RkdgSolver>(t, std::move(m));
            *out = h.release();
            return CFD2D_OK;
        }
        const bool imp = t.method == cfd2d::METHOD_FVM_TVD_IMPLICIT;
        std::vector<int> tn;
        if (imp) tn = triangle_neigh(mesh->n_cells, mesh->tri);
        cfd2d::Topo topo = topo_from_desc(mesh, imp ? tn.data() : nullptr, 2);
        std::vector<int> cr(mesh->cell_region, mesh->cell_region + mesh->n_cells);
        for (int r : cr)
            if (r < 0 || r >= (int)t.regions.size())
                return fail(CFD2D_ERR_REGION_UNKNOWN, "cell_region refers to a missing region");
        std::vector<int> eb = edge_bnd_from_desc(mesh, topo, (int)t.bnds.size());
        auto h = std::make_unique<cfd2d_solver>();
        if (imp) {
            h->imp = std::make_unique<cfd2d::ImplicitSolver>(t, std::move(topo), cr, eb);
            *out = h.release();
            return CFD2D_OK;
        }
        h->s = std::make_unique<cfd2d::Solver>(t, std::move(topo), cr, eb, 2);
        *out = h.release();
        return CFD2D_OK;
    });
}

int cfd2d_batch_create(int n, const char* const* task_xml_paths, const cfd2d_mesh_desc* meshes, cfd2d_t** out) {
    Range r("cfd2d_batch_create");
    return guarded([&] {
        if (n < 1 || !task_xml_paths || !out) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        *out = nullptr;
        std::vector<cfd2d::TaskConfig> tasks;
        std::vector<cfd2d::Topo> topos(n);
        std::vector<std::vector<int>> cregs(n), ebnds(n);
        for (int k = 0; k < n; k++) {
            if (!task_xml_paths[k]) return fail(CFD2D_ERR_INVALID_ARG, "null task path");
            tasks.push_back(cfd2d::parse_task(task_xml_paths[k]));
            if (meshes) {
                const cfd2d_mesh_desc* m = meshes + k;
                check_desc(m);
                if (!m->cell_region) return fail(CFD2D_ERR_INVALID_ARG, "cell_region is required");
                topos[k] = topo_from_desc(m, nullptr, 2);
                cregs[k].assign(m->cell_region, m->cell_region + m->n_cells);
                for (int r : cregs[k])
                    if (r < 0 || r >= (int)tasks[k].regions.size())
                        return fail(CFD2D_ERR_REGION_UNKNOWN, "cell_region refers to a missing region");
                ebnds[k] = edge_bnd_from_desc(m, topos[k], (int)tasks[k].bnds.size());
            } else {
                int gp = 2;
                load_task_mesh(tasks[k], topos[k], cregs[k], ebnds[k], gp);
                if (gp != 2) return fail(CFD2D_ERR_INVALID_ARG, "batch instances need two-point edges");
            }
        }
        cfd2d::Batch b = cfd2d::merge_batch(tasks, topos, cregs, ebnds);
        auto h = std::make_unique<cfd2d_solver>();
        h->s = std::make_unique<cfd2d::Solver>(b.task, std::move(b.topo), b.cell_region, b.edge_bnd, 2, b.inst);
        *out = h.release();
        return CFD2D_OK;
    });
}

int cfd2d_batch_instance(const cfd2d_t* h, int k, int* cell_offset, int* n_cells, double* tau, double* time) {
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        if (h->imp) {
            if (k != 0) return fail(CFD2D_ERR_INVALID_ARG, "instance out of range");
            if (cell_offset) *cell_offset = 0;
            if (n_cells) *n_cells = h->imp->topo().nc;
            if (tau) *tau = h->imp->task().tau;
            if (time) *time = h->imp->time();
            return CFD2D_OK;
        }
        const cfd2d::Solver& s = *h->s;
        if (k < 0 || k >= s.n_instances()) return fail(CFD2D_ERR_INVALID_ARG, "instance out of range");
        if (!s.is_batch()) {
            if (cell_offset) *cell_offset = 0;
            if (n_cells) *n_cells = s.topo().nc;
            if (tau) *tau = s.tau();
            if (time) *time = s.time();
            return CFD2D_OK;
        }
        const cfd2d::Instance& in = s.instance(k);
        if (cell_offset) *cell_offset = in.cell_off;
        if (n_cells) *n_cells = in.nc;
        if (tau) *tau = in.tau;
        if (time) *time = in.t;
        return CFD2D_OK;
    });
}

int cfd2d_autotune(cfd2d_t* h, const char* json_path) {
    Range r("cfd2d_autotune");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        ex(h).autotune(json_path, 5);
        return CFD2D_OK;
    });
}

int cfd2d_load_tuning(cfd2d_t* h, const char* json_path) {
    return guarded([&] {
        if (!h || !json_path) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        ex(h).load_tuning(json_path);
        return CFD2D_OK;
    });
}

int cfd2d_step(cfd2d_t* h, int nsteps) {
    Range r("cfd2d_step");
    return guarded([&] {
        if (!h || nsteps < 0) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        int s = h->dg ? h->dg->step(nsteps) : h->imp ? h->imp->step(nsteps) : ex(h).step(nsteps);
        if (s != CFD2D_OK) g_err = s == CFD2D_ERR_NEWTON_CAP ? "exact Riemann solver hit its iteration cap"
                                                            : "non-positive or NaN density/pressure";
        return s;
    });
}

int cfd2d_run(cfd2d_t* h) {
    Range r("cfd2d_run");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        return h->dg ? h->dg->run() : h->imp ? h->imp->run() : ex(h).run();
    });
}

int cfd2d_destroy(cfd2d_t* h) {
    return guarded([&] {
        delete h;
        return CFD2D_OK;
    });
}

int cfd2d_get_info(const cfd2d_t* h, cfd2d_info_t* info) {
    return guarded([&] {
        if (!h || !info) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        std::memset(info, 0, sizeof *info);
        if (h->dg) {
            const cfd2d::RkdgSolver& m = *h->dg;
            info->n_cells = m.nc();
            info->n_edges = m.ne();
            info->n_boundary_edges = m.n_boundary_edges();
            info->n_nodes = m.n_nodes();
            info->step = m.n_steps();
            info->flux = m.task().flux;
            info->recon = -1;
            info->scheme = -1;
            info->precision = m.task().precision;
            info->steady = m.task().steady;
            info->time = m.time();
            info->tau = m.tau();
            info->device_bytes = m.device_bytes();
            info->n_instances = 1;
            return CFD2D_OK;
        }
        if (h->imp) {
            const cfd2d::ImplicitSolver& m = *h->imp;
            info->n_cells = m.topo().nc;
            info->n_edges = m.topo().ne;
            info->n_boundary_edges = m.layout().ne - m.layout().n_int;
            info->n_nodes = m.topo().nn;
            info->step = m.n_steps();
            info->flux = m.task().flux;
            info->recon = m.task().recon;
            info->scheme = m.task().scheme;
            info->precision = m.task().precision;
            info->steady = m.task().steady;
            info->time = m.time();
            info->tau = m.task().tau;
            info->device_bytes = m.device_bytes();
            info->n_instances = 1;
            return CFD2D_OK;
        }
        const cfd2d::Solver& s = *h->s;
        info->n_cells = s.topo().nc;
        info->n_edges = s.topo().ne;
        info->n_boundary_edges = s.layout().ne - s.layout().n_int;
        info->n_nodes = s.topo().nn;
        info->step = s.n_steps();
        info->flux = s.task().flux;
        info->recon = s.task().recon;
        info->scheme = s.task().scheme;
        info->precision = s.task().precision;
        info->steady = s.task().steady;
        info->time = s.time();
        info->tau = s.tau();
        info->device_bytes = s.device_bytes();
        info->n_instances = s.n_instances();
        return CFD2D_OK;
    });
}

int cfd2d_get_state(cfd2d_t* h, double* ro, double* ru, double* rv, double* re) {
    Range r("cfd2d_get_state");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        if (h->dg) h->dg->get_state(ro, ru, rv, re);
        else if (h->imp) h->imp->get_state(ro, ru, rv, re);
        else ex(h).get_state(ro, ru, rv, re);
        return CFD2D_OK;
    });
}

int cfd2d_set_state(cfd2d_t* h, const double* ro, const double* ru, const double* rv, const double* re,
                    int reset_time_step) {
    Range r("cfd2d_set_state");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        if (h->dg) h->dg->set_state(ro, ru, rv, re);
        else if (h->imp) h->imp->set_state(ro, ru, rv, re);
        else ex(h).set_state(ro, ru, rv, re, reset_time_step != 0);
        return CFD2D_OK;
    });
}

int cfd2d_get_time_step(cfd2d_t* h, double* ctau) {
    return guarded([&] {
        if (!h || !ctau) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        if (h->dg) h->dg->get_ctau(ctau);
        else if (h->imp) h->imp->get_ctau(ctau);
        else ex(h).get_ctau(ctau);
        return CFD2D_OK;
    });
}

int cfd2d_get_flags(cfd2d_t* h, unsigned* flags) {
    return guarded([&] {
        if (!h || !flags) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        if (h->imp) h->imp->get_flags(flags);
        else ex(h).get_flags(flags);
        return CFD2D_OK;
    });
}

int cfd2d_residual(cfd2d_t* h, double* R) {
    Range r("cfd2d_residual");
    return guarded([&] {
        if (!h || !R) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        ex(h).residual(R);
        return CFD2D_OK;
    });
}

int cfd2d_conservation(cfd2d_t* h, double sums[4]) {
    return guarded([&] {
        if (!h || !sums) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        ex(h).conservation(sums);
        return CFD2D_OK;
    });
}

int cfd2d_save_vtk(cfd2d_t* h, int step) {
    Range r("cfd2d_save_vtk");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        if (h->dg) h->dg->save_vtu(step);
        else if (h->imp) h->imp->save_vtk(step);
        else ex(h).save_vtk(step);
        return CFD2D_OK;
    });
}

int cfd2d_save_state(cfd2d_t* h, const char* path) {
    Range r("cfd2d_save_state");
    return guarded([&] {
        if (!h || !path) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        if (h->dg) h->dg->save_state(path);
        else if (h->imp) h->imp->save_state(path);
        else ex(h).save_state(path);
        return CFD2D_OK;
    });
}

int cfd2d_load_state(cfd2d_t* h, const char* path) {
    Range r("cfd2d_load_state");
    return guarded([&] {
        if (!h || !path) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        if (h->dg) h->dg->load_state(path);
        else if (h->imp) h->imp->load_state(path);
        else ex(h).load_state(path);
        return CFD2D_OK;
    });
}

int cfd2d_set_objective(cfd2d_t* h, int kind, const double* weights, double p_ref) {
    return guarded([&] {
        if (!h || !weights) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        ex(h).set_objective(kind, weights, p_ref);
        return CFD2D_OK;
    });
}

int cfd2d_forward(cfd2d_t* h, int nsteps, int checkpoint_every, double* J) {
    Range r("cfd2d_forward");
    return guarded([&] {
        if (!h || !J) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        int st = CFD2D_OK;
        *J = ex(h).forward(nsteps, checkpoint_every, &st);
        return st;
    });
}

int cfd2d_backward(cfd2d_t* h, double* dJdU0, double* dJdbnd) {
    Range r("cfd2d_backward");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        ex(h).backward(dJdU0, dJdbnd);
        return CFD2D_OK;
    });
}

int cfd2d_set_boundary(cfd2d_t* h, int b, const double par[4]) {
    return guarded([&] {
        if (!h || !par) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        ex(h).set_boundary_params(b, par);
        return CFD2D_OK;
    });
}

int cfd2d_timed_steps(cfd2d_t* h, int nsteps, double* device_ms) {
    Range r("cfd2d_timed_steps");
    return guarded([&] {
        if (!h || !device_ms || nsteps < 0) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        *device_ms = h->dg    ? h->dg->timed_steps(nsteps)
                     : h->imp ? h->imp->timed_steps(nsteps)
                              : ex(h).timed_steps(nsteps);
        return CFD2D_OK;
    });
}

int cfd2d_profile_steps(cfd2d_t* h, int nsteps, double kernel_ms[4], int kernel_launches[4]) {
    Range r("cfd2d_profile_steps");
    return guarded([&] {
        if (!h || !kernel_ms || !kernel_launches || nsteps < 0) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        if (h->dg) {
            h->dg->profile_steps(nsteps, kernel_ms, kernel_launches);
            kernel_ms[3] = 0.0;
            kernel_launches[3] = 0;
        } else if (h->imp) {
            h->imp->profile_steps(nsteps, kernel_ms, kernel_launches);
        } else {
            ex(h).profile_steps(nsteps, kernel_ms, kernel_launches);
        }
        return CFD2D_OK;
    });
}

int cfd2d_implicit_system(cfd2d_t* h, double* diag, double* off, double* rhs, double* ctau) {
    Range r("cfd2d_implicit_system");
    return guarded([&] {
        if (!h) return fail(CFD2D_ERR_INVALID_ARG, "null handle");
        if (!h->imp) return fail(CFD2D_ERR_INVALID_ARG, "not an FVM_TVD_IMPLICIT handle");
        h->imp->system(diag, off, rhs, ctau);
        return CFD2D_OK;
    });
}

int cfd2d_implicit_stats(const cfd2d_t* h, cfd2d_implicit_stats_t* st) {
    return guarded([&] {
        if (!h || !st) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        if (!h->imp) return fail(CFD2D_ERR_INVALID_ARG, "not an FVM_TVD_IMPLICIT handle");
        std::memset(st, 0, sizeof *st);
        st->iterations = h->imp->last_iters();
        st->status = h->imp->last_status();
        st->n_limited = h->imp->last_n_lim();
        st->rel_residual = h->imp->last_rel();
        st->cfl = h->imp->cfl();
        return CFD2D_OK;
    });
}

int cfd2d_dg_get_coeffs(cfd2d_t* h, double* coeffs) {
    Range r("cfd2d_dg_get_coeffs");
    return guarded([&] {
        if (!h || !coeffs) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        dgs(h).get_coeffs(coeffs);
        return CFD2D_OK;
    });
}

int cfd2d_dg_set_coeffs(cfd2d_t* h, const double* coeffs) {
    Range r("cfd2d_dg_set_coeffs");
    return guarded([&] {
        if (!h || !coeffs) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        dgs(h).set_coeffs(coeffs);
        return CFD2D_OK;
    });
}

int cfd2d_dg_set_time_step(cfd2d_t* h, double tau) {
    return guarded([&] {
        if (!h || !(tau > 0)) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        dgs(h).set_tau(tau);
        return CFD2D_OK;
    });
}

int cfd2d_dg_residuals(cfd2d_t* h, double res[4]) {
    return guarded([&] {
        if (!h || !res) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        dgs(h).residuals(res);
        return CFD2D_OK;
    });
}

int cfd2d_selftest(int which, long long n, unsigned long long seed, long long* mismatches) {
    return guarded([&] {
        if (!mismatches || which < 0 || which > 3 || n < 0) return fail(CFD2D_ERR_INVALID_ARG, "bad argument");
        long long r = cfd2d::selftest_arith(which, n, seed);
        if (r < 0) return fail(CFD2D_ERR_CUDA, "self-test launch failed");
        *mismatches = r;
        return CFD2D_OK;
    });
}

int cfd2d_set_device(int device) {
    return guarded([&] {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return fail(e == cudaErrorNoDevice ? CFD2D_ERR_NO_DEVICE : CFD2D_ERR_CUDA,
                                          std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        return CFD2D_OK;
    });
}

int cfd2d_last_error(char* buf, size_t n) {
    if (!buf || n == 0) return CFD2D_ERR_INVALID_ARG;
    std::strncpy(buf, g_err.c_str(), n - 1);
    buf[n - 1] = 0;
    return CFD2D_OK;
}

int cfd2d_set_verbosity(int level) {
    cfd2d::set_verbosity(level);
    return CFD2D_OK;
}

int cfd2d_set_log_file(const char* path) {
    return guarded([&] {
        cfd2d::set_log_file(path);
        return CFD2D_OK;
    });
}

int cfd2d_mesh_load(const char* task_xml_path, cfd2d_mesh_t** out) {
    return guarded([&] {
        if (!task_xml_path || !out) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        *out = nullptr;
        cfd2d::TaskConfig t = cfd2d::parse_task(task_xml_path);
        auto m = std::make_unique<cfd2d_mesh>();
        std::vector<int> cr;
        int gp = 2;
        load_task_mesh(t, m->topo, cr, m->edge_bnd, gp);
        *out = m.release();
        return CFD2D_OK;
    });
}

int cfd2d_mesh_build(const cfd2d_mesh_desc* mesh, const int* berkeley_neigh, cfd2d_mesh_t** out) {
    return guarded([&] {
        if (!out) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        *out = nullptr;
        check_desc(mesh);
        auto m = std::make_unique<cfd2d_mesh>();
        m->topo = topo_from_desc(mesh, berkeley_neigh, berkeley_neigh ? 0 : 2);
        m->edge_bnd.assign(m->topo.ne, -1);
        for (int e = 0; e < m->topo.ne; e++) {
            int s = m->topo.bseg_of_edge[e];
            if (m->topo.c2[e] < 0 && s >= 0) m->edge_bnd[e] = mesh->bseg_bnd[s];
        }
        *out = m.release();
        return CFD2D_OK;
    });
}

int cfd2d_mesh_sizes(const cfd2d_mesh_t* m, int* n_cells, int* n_edges) {
    if (!m) return fail(CFD2D_ERR_INVALID_ARG, "null mesh");
    if (n_cells) *n_cells = m->topo.nc;
    if (n_edges) *n_edges = m->topo.ne;
    return CFD2D_OK;
}

int cfd2d_mesh_export(const cfd2d_mesh_t* m, int* cell_edges, double* cell_S, double* cell_c, int* edge_n12,
                      int* edge_c12, int* edge_bnd, int* edge_npts, double* edge_n, double* edge_l,
                      double* edge_pts) {
    return guarded([&] {
        if (!m) return fail(CFD2D_ERR_INVALID_ARG, "null mesh");
        const cfd2d::Topo& t = m->topo;
        for (int i = 0; i < t.nc; i++) {
            for (int k = 0; k < 3; k++)
                if (cell_edges) cell_edges[3 * i + k] = t.cedges[3 * i + k];
            if (cell_S) cell_S[i] = t.S[i];
            if (cell_c) { cell_c[2 * i] = t.cx[i]; cell_c[2 * i + 1] = t.cy[i]; }
        }
        for (int e = 0; e < t.ne; e++) {
            if (edge_n12) { edge_n12[2 * e] = t.n1[e]; edge_n12[2 * e + 1] = t.n2[e]; }
            if (edge_c12) { edge_c12[2 * e] = t.c1[e]; edge_c12[2 * e + 1] = t.c2[e]; }
            if (edge_bnd) edge_bnd[e] = m->edge_bnd[e];
            if (edge_npts) edge_npts[e] = t.npts[e];
            if (edge_n) { edge_n[2 * e] = t.nx[e]; edge_n[2 * e + 1] = t.ny[e]; }
            if (edge_l) edge_l[e] = t.l[e];
            if (edge_pts)
                for (int k = 0; k < 6; k++) edge_pts[6 * e + k] = t.pts[6 * (size_t)e + k];
        }
        return CFD2D_OK;
    });
}

int cfd2d_mesh_order(const cfd2d_mesh_t* m, int rcm, int* perm) {
    return guarded([&] {
        if (!m || !perm) return fail(CFD2D_ERR_INVALID_ARG, "null argument");
        std::vector<int> p;
        if (rcm) p = cfd2d::rcm_order(m->topo);
        else for (int i = 0; i < m->topo.nc; i++) p.push_back(i);
        std::copy(p.begin(), p.end(), perm);
        return CFD2D_OK;
    });
}

int cfd2d_mesh_free(cfd2d_mesh_t* m) {
    delete m;
    return CFD2D_OK;
}

}  // extern "C"
