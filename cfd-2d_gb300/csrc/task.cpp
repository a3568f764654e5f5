#include "task.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>

#include "cfd2d.h"
#include "xml.hpp"

namespace cfd2d {

namespace {

const XmlNode* need(const XmlNode* n, const char* name, const char* where) {
    const XmlNode* c = n ? n->child(name) : nullptr;
    if (!c) throw Error(CFD2D_ERR_TASK, std::string("task.xml: missing <") + name + "> in <" + where + ">");
    return c;
}

// TiXmlElement::Attribute(name, double*) / (name, int*): atof / atoi of the value.
double attr_d(const XmlNode* n, const char* a) {
    const char* v = n->attr(a);
    if (!v) throw Error(CFD2D_ERR_TASK, "task.xml: <" + n->name + "> has no attribute '" + a + "'");
    return std::atof(v);
}
int attr_i(const XmlNode* n, const char* a) {
    const char* v = n->attr(a);
    if (!v) throw Error(CFD2D_ERR_TASK, "task.xml: <" + n->name + "> has no attribute '" + a + "'");
    return std::atoi(v);
}

int pick(const XmlNode* ctl, const char* tag, std::initializer_list<std::pair<const char*, int>> opts, int dflt) {
    const XmlNode* n = ctl->child(tag);
    if (!n) return dflt;
    const char* v = n->attr("value");
    if (!v) throw Error(CFD2D_ERR_TASK, std::string("task.xml: <") + tag + "> has no value");
    for (auto& o : opts)
        if (std::strcmp(v, o.first) == 0) return o.second;
    throw Error(CFD2D_ERR_TASK, std::string("task.xml: unknown ") + tag + " '" + v + "'");
}

void parse_limits(TaskConfig& t, const XmlNode* task) {
    const XmlNode* lim = need(task, "limits", "task");
    t.lim_rmin = attr_d(need(lim, "ro", "limits"), "min");
    t.lim_rmax = attr_d(need(lim, "ro", "limits"), "max");
    t.lim_pmin = attr_d(need(lim, "p", "limits"), "min");
    t.lim_pmax = attr_d(need(lim, "p", "limits"), "max");
    t.lim_umax = attr_d(need(lim, "u", "limits"), "max");
}

int parse_materials(TaskConfig& t, const XmlNode* task) {
    const XmlNode* mats = need(task, "materials", "task");
    int nm = attr_i(mats, "count");
    auto mlist = mats->children_named("material");
    if (nm < 1 || nm > (int)mlist.size()) throw Error(CFD2D_ERR_TASK, "task.xml: <materials count> does not match");
    if (nm > 255) throw Error(CFD2D_ERR_TASK, "task.xml: more than 255 materials");
    for (int i = 0; i < nm; i++) {
        TaskMaterial m;
        m.id = attr_i(mlist[i], "id");
        m.name = need(mlist[i], "name", "material")->text;
        const XmlNode* p = need(mlist[i], "parameters", "material");
        m.M = attr_d(need(p, "M", "parameters"), "value");
        m.Cp = attr_d(need(p, "Cp", "parameters"), "value");
        m.K = attr_d(need(p, "K", "parameters"), "value");
        m.ML = attr_d(need(p, "ML", "parameters"), "value");
        t.mats.push_back(m);
    }
    return nm;
}

// <regions> with names (FVM_TVD::init :71-95, FEM_RKDG::init :80-107)
void parse_regions(TaskConfig& t, const XmlNode* task, int nm) {
    const XmlNode* regs = need(task, "regions", "task");
    int nr = attr_i(regs, "count");
    auto rlist = regs->children_named("region");
    if (nr < 1 || nr > (int)rlist.size()) throw Error(CFD2D_ERR_TASK, "task.xml: <regions count> does not match");
    for (int i = 0; i < nr; i++) {
        TaskRegion r;
        r.id = attr_i(rlist[i], "id");
        r.matId = attr_i(need(rlist[i], "material", "region"), "id");
        r.cellType = attr_i(need(rlist[i], "cell", "region"), "type");
        r.name = need(rlist[i], "name", "region")->text;
        const XmlNode* p = need(rlist[i], "parameters", "region");
        r.u = attr_d(need(p, "Vx", "parameters"), "value");
        r.v = attr_d(need(p, "Vy", "parameters"), "value");
        r.T = attr_d(need(p, "T", "parameters"), "value");
        r.p = attr_d(need(p, "P", "parameters"), "value");
        if (r.matId < 0 || r.matId >= nm) throw Error(CFD2D_ERR_TASK, "task.xml: region refers to a missing material");
        t.regions.push_back(r);
    }

}

// <boundaries>: every <boundCond>, CFDBoundary::create (src/bnd_cond.cpp:10-72)
void parse_cfd_boundaries(TaskConfig& t, const XmlNode* task) {
    const XmlNode* bnds = need(task, "boundaries", "task");
    for (const XmlNode* b : bnds->children_named("boundCond")) {  // CFDBoundary::create, src/bnd_cond.cpp:10-72
        TaskBound tb;
        const char* type = need(b, "type", "boundCond")->text.c_str();
        if (std::strcmp(type, "BOUND_INLET") == 0) {
            tb.kind = BND_INLET;
            const XmlNode* p = b->child("parameters");
            const char* names[4] = {"Vx", "Vy", "T", "P"};
            for (int k = 0; k < 4; k++) {
                const XmlNode* n = p ? p->child(names[k]) : nullptr;
                if (!n) throw Error(CFD2D_ERR_BOUND_NOPAR, std::string("Parameter '") + names[k] +
                                                               "' isn't specified  for BOUND_INLET.");
                tb.par[k] = attr_d(n, "value");
            }
        } else if (std::strcmp(type, "BOUND_OUTLET") == 0) {
            tb.kind = BND_OUTLET;
        } else if (std::strcmp(type, "BOUND_WALL_NO_SLIP") == 0) {
            tb.kind = BND_WALL_NO_SLIP;
        } else if (std::strcmp(type, "BOUND_WALL_SLIP") == 0) {
            tb.kind = BND_WALL_SLIP;
        } else {
            throw Error(CFD2D_ERR_BOUND_UNKNOWN, std::string("Unknown boundary type '") + type + "' specified.");
        }
        tb.edgeType = attr_i(b, "edgeType");
        tb.name = need(b, "name", "boundCond")->text;
        t.bnds.push_back(tb);
    }
}

// FVM_TVD_IMPLICIT::init, src/methods/fvm_tvd_implicit.cpp:13-184
void parse_implicit(TaskConfig& t, const XmlNode* task) {
    t.method = METHOD_FVM_TVD_IMPLICIT;
    const XmlNode* ctl = need(task, "control", "task");
    t.steady = attr_i(need(ctl, "STEADY", "control"), "value") == 0 ? 0 : 1;
    t.tau = attr_d(need(ctl, "TAU", "control"), "value");
    t.tmax = attr_d(need(ctl, "TMAX", "control"), "value");
    t.step_max = attr_i(need(ctl, "STEP_MAX", "control"), "value");
    t.file_step = attr_i(need(ctl, "FILE_OUTPUT_STEP", "control"), "value");
    t.print_step = attr_i(need(ctl, "LOG_OUTPUT_STEP", "control"), "value");
    const char* flx = need(ctl, "FLUX", "control")->attr("value");
    t.flux = flx && std::strcmp(flx, "LAX") == 0 ? FLUX_LAX : FLUX_GODUNOV;  // anything else: GODUNOV
    t.recon = RECON_LINEAR;
    t.scheme = TIME_EULER;
    t.precision = pick(ctl, "PRECISION", {{"FP64", PREC_FP64}}, PREC_FP64);
    t.reorder = pick(ctl, "REORDER", {{"NONE", 0}, {"RCM", 1}, {"HILBERT", 2}}, -1);
    if (const XmlNode* n = ctl->child("NEWTON_CAP")) t.newton_cap = std::max(1, attr_i(n, "value"));
    // the matrix solver's parameters (an extension; absent: the reference's, run() and
    // SolverHypreGmres.h: Krylov dimension 30, 20 iterations, relative tolerance 1e-7)
    if (const XmlNode* g = ctl->child("GMRES")) {
        if (g->attr("krylov")) t.gmres_kdim = attr_i(g, "krylov");
        if (g->attr("max_iter")) t.gmres_maxit = attr_i(g, "max_iter");
        if (g->attr("tolerance")) t.gmres_eps = attr_d(g, "tolerance");
        if (t.gmres_kdim < 1 || t.gmres_maxit < 1 || !(t.gmres_eps > 0))
            throw Error(CFD2D_ERR_TASK, "task.xml: <GMRES> needs krylov >= 1, max_iter >= 1, tolerance > 0");
    }
    if (t.steady) {
        const XmlNode* c = need(ctl, "CFL", "control");
        t.cfl = attr_d(need(c, "start", "CFL"), "value");
        t.cfl_scale = attr_d(need(c, "scale", "CFL"), "value");
        t.cfl_max = attr_d(need(c, "max", "CFL"), "value");
        t.cfl_step = attr_i(need(c, "step", "CFL"), "value");
        t.max_lim_cells = attr_d(need(c, "max_limited_cells", "CFL"), "value");
    }
    const XmlNode* sm = need(task, "smoothing", "task");
    t.smoothing = attr_i(need(sm, "using", "smoothing"), "value") == 1 ? 1 : 0;
    t.smoothing_par = attr_d(need(sm, "coefficient", "smoothing"), "value");
    parse_limits(t, task);
    const int nm = parse_materials(t, task);
    const XmlNode* regs = need(task, "regions", "task");
    int nr = attr_i(regs, "count");
    auto rlist = regs->children_named("region");
    if (nr < 1 || nr > (int)rlist.size()) throw Error(CFD2D_ERR_TASK, "task.xml: <regions count> does not match");
    for (int i = 0; i < nr; i++) {
        TaskRegion r;
        r.id = attr_i(rlist[i], "id");
        r.matId = attr_i(need(rlist[i], "material", "region"), "id");
        r.cellType = attr_i(need(rlist[i], "cell", "region"), "type");
        const XmlNode* p = need(rlist[i], "parameters", "region");
        r.u = attr_d(need(p, "Vx", "parameters"), "value");
        r.v = attr_d(need(p, "Vy", "parameters"), "value");
        r.T = attr_d(need(p, "T", "parameters"), "value");
        r.p = attr_d(need(p, "P", "parameters"), "value");
        if (r.matId < 0 || r.matId >= nm) throw Error(CFD2D_ERR_TASK, "task.xml: region refers to a missing material");
        t.regions.push_back(r);
    }
    const XmlNode* bnds = need(task, "boundaries", "task");
    int nb = attr_i(bnds, "count");
    auto blist = bnds->children_named("boundCond");
    if (nb < 0 || nb > (int)blist.size()) throw Error(CFD2D_ERR_TASK, "task.xml: <boundaries count> does not match");
    for (int i = 0; i < nb; i++) {
        TaskBound tb;
        tb.edgeType = attr_i(blist[i], "edgeType");
        const char* type = need(blist[i], "type", "boundCond")->text.c_str();
        if (std::strcmp(type, "BOUND_WALL") == 0) {
            tb.kind = 3;
        } else if (std::strcmp(type, "BOUND_OUTLET") == 0) {
            tb.kind = 2;
        } else if (std::strcmp(type, "BOUND_INLET") == 0) {
            tb.kind = 1;
            const XmlNode* p = need(blist[i], "parameters", "boundCond");
            tb.par[2] = attr_d(need(p, "T", "parameters"), "value");  // par = (Vx, Vy, T, P)
            tb.par[3] = attr_d(need(p, "P", "parameters"), "value");
            tb.par[0] = attr_d(need(p, "Vx", "parameters"), "value");
            tb.par[1] = attr_d(need(p, "Vy", "parameters"), "value");
        } else {
            throw Error(CFD2D_ERR_BOUND_UNKNOWN, std::string("ERROR: unsupported boundary condition type '") + type + "'");
        }
        t.bnds.push_back(tb);
    }
    const XmlNode* mesh = need(task, "mesh", "task");
    const char* mn = need(mesh, "name", "mesh")->attr("value");
    if (!mn) throw Error(CFD2D_ERR_TASK, "task.xml: <mesh> needs a name value");
    t.mesh_name = mn;
    t.mesh_type = "berkeley_triangle";  // Grid::initFromFiles, src/mesh/grid.cpp:51-252
    t.gauss_points = 2;                 // with the midpoint and two Gauss points per edge
}

// FEM_RKDG::init, src/methods/fem_rkdg.cpp:23-235 (the mesh part is read separately)
void parse_rkdg(TaskConfig& t, const XmlNode* task) {
    t.method = METHOD_FEM_RKDG;
    const XmlNode* ctl = need(task, "control", "task");
    t.steady = attr_i(need(ctl, "STEADY", "control"), "value") == 0 ? 0 : 1;
    t.tau = attr_d(need(ctl, "TAU", "control"), "value");
    t.tmax = attr_d(need(ctl, "TMAX", "control"), "value");
    t.cfl = attr_d(need(ctl, "CFL", "control"), "value");
    t.file_step = attr_i(need(ctl, "FILE_OUTPUT_STEP", "control"), "value");
    t.print_step = attr_i(need(ctl, "LOG_OUTPUT_STEP", "control"), "value");
    t.dg_func_count = attr_i(need(ctl, "BASE_FUNC_COUNT", "control"), "value");
    t.dg_gp_cell = attr_i(need(ctl, "GP_CELL_COUNT", "control"), "value");
    t.dg_gp_edge = attr_i(need(ctl, "GP_EDGE_COUNT", "control"), "value");
    const char* flx = need(ctl, "FLUX", "control")->attr("value");
    t.flux = flx && std::strcmp(flx, "LAX") == 0 ? FLUX_LAX : FLUX_GODUNOV;  // anything else: GODUNOV
    // the reference's mass-matrix inverse is the 3x3 cofactor formula (src/global.cpp:444-470)
    // and its quadratures exist for these counts only (calcGaussPar, :470-598)
    if (t.dg_func_count != 3)
        throw Error(CFD2D_ERR_TASK, "task.xml: BASE_FUNC_COUNT must be 3 (the reference inverts 3x3 mass matrices)");
    if (t.dg_gp_cell != 3 && t.dg_gp_cell != 4) throw Error(CFD2D_ERR_TASK, "task.xml: GP_CELL_COUNT must be 3 or 4");
    if (t.dg_gp_edge != 2 && t.dg_gp_edge != 3) throw Error(CFD2D_ERR_TASK, "task.xml: GP_EDGE_COUNT must be 2 or 3");
    t.dg_rk = pick(ctl, "RK_MODE", {{"REFERENCE", 0}, {"HEUN", 1}}, 0);
    t.reorder = pick(ctl, "REORDER", {{"NONE", 0}, {"RCM", 1}}, -1);
    t.precision = pick(ctl, "PRECISION", {{"FP64", PREC_FP64}}, PREC_FP64);
    if (const XmlNode* n = ctl->child("NEWTON_CAP")) t.newton_cap = std::max(1, attr_i(n, "value"));
    const int nm = parse_materials(t, task);
    parse_regions(t, task, nm);
    parse_cfd_boundaries(t, task);
    t.mesh_name = "mesh/mesh.0000.proc";  // Grid::readMeshFiles, src/mesh/grid.cpp:279-281 (process 0)
    t.mesh_type = "proc";
}

}  // namespace

TaskConfig parse_task(const std::string& path) {
    TaskConfig t;
    t.path = path;
    size_t slash = path.find_last_of('/');
    t.dir = slash == std::string::npos ? std::string(".") : path.substr(0, slash);
    std::unique_ptr<XmlNode> doc;
    try {
        doc = xml_load(path);
    } catch (const std::exception& e) {
        throw Error(CFD2D_ERR_XML, std::string("ERROR: ") + e.what());
    }
    const XmlNode* task = doc->child("task");
    if (!task) throw Error(CFD2D_ERR_TASK, "task.xml: no <task> element");
    const char* method = task->attr("method");
    if (method && std::strcmp(method, "FVM_TVD_IMPLICIT") == 0) {
        parse_implicit(t, task);
        return t;
    }
    if (method && std::strcmp(method, "FEM_RKDG") == 0) {
        parse_rkdg(t, task);
        return t;
    }
    if (method && std::strcmp(method, "FVM_TVD") != 0 && std::strcmp(method, "FVM_TVD_GPU") != 0)
        throw Error(CFD2D_ERR_TASK, std::string("ERROR: method '") + method + "' is not served by this library.");

    const XmlNode* ctl = need(task, "control", "task");
    t.steady = attr_i(need(ctl, "STEADY", "control"), "value") == 0 ? 0 : 1;
    t.tau = attr_d(need(ctl, "TAU", "control"), "value");
    t.tmax = attr_d(need(ctl, "TMAX", "control"), "value");
    t.cfl = attr_d(need(ctl, "CFL", "control"), "value");
    t.step_max = attr_i(need(ctl, "STEP_MAX", "control"), "value");
    t.file_step = attr_i(need(ctl, "FILE_OUTPUT_STEP", "control"), "value");
    t.print_step = attr_i(need(ctl, "LOG_OUTPUT_STEP", "control"), "value");
    t.flux = pick(ctl, "FLUX", {{"GODUNOV", FLUX_GODUNOV}, {"LAX", FLUX_LAX}, {"ROE", FLUX_ROE}, {"HLLC", FLUX_HLLC}},
                  FLUX_GODUNOV);
    t.recon = pick(ctl, "RECONSTRUCTION",
                   {{"NONE", RECON_NONE}, {"FIRST_ORDER", RECON_NONE}, {"LINEAR", RECON_LINEAR}, {"MINMOD", RECON_MINMOD}},
                   RECON_LINEAR);
    t.scheme = pick(ctl, "TIME_SCHEME", {{"EULER", TIME_EULER}, {"HEUN", TIME_HEUN}, {"SSPRK3", TIME_SSPRK3}}, TIME_HEUN);
    t.precision = pick(ctl, "PRECISION", {{"FP64", PREC_FP64}, {"MIXED", PREC_MIXED}}, PREC_FP64);
    t.reorder = pick(ctl, "REORDER", {{"NONE", 0}, {"RCM", 1}, {"HILBERT", 2}}, -1);
    t.fused = pick(ctl, "FUSED_STAGE", {{"0", 0}, {"1", 1}, {"2", 2}, {"3", 3}, {"OFF", 0}, {"ON", 1},
                                        {"FLUX_UPDATE", 2}, {"GRAD_IN_FLUX", 3}}, -1);
    t.adj_store = pick(ctl, "ADJOINT_STORE",
                       {{"AUTO", -1}, {"NONE", 0}, {"PRIMITIVES", 1}, {"ALL", 2}, {"FLUXES", 3}}, -1);
    if (const XmlNode* n = ctl->child("ADJOINT_MEMORY")) t.adj_memory = attr_d(n, "value");
    if (!(t.adj_memory >= 0.0)) throw Error(CFD2D_ERR_TASK, "ERROR: ADJOINT_MEMORY must be a byte count >= 0.");
    t.flux_pipe = pick(ctl, "FLUX_PIPELINE", {{"0", 0}, {"1", 1}, {"OFF", 0}, {"ON", 1}}, 1);
    if (const XmlNode* n = ctl->child("NEWTON_CAP")) t.newton_cap = attr_i(n, "value");
    if (t.newton_cap < 1) t.newton_cap = 1;

    parse_limits(t, task);
    const int nm = parse_materials(t, task);

    parse_regions(t, task, nm);
    parse_cfd_boundaries(t, task);

    const XmlNode* mesh = need(task, "mesh", "task");
    const char* mn = need(mesh, "name", "mesh")->attr("value");
    const char* mt = need(mesh, "filesType", "mesh")->attr("value");
    if (!mn || !mt) throw Error(CFD2D_ERR_TASK, "task.xml: <mesh> needs name and filesType values");
    t.mesh_name = mn;
    t.mesh_type = mt;
    if (t.mesh_type != "berkeley_triangle" && t.mesh_type != "salome_unv")
        throw Error(CFD2D_ERR_MESH_WRONG_NAME, "Wrong mesh type.");
    if (const XmlNode* g = mesh->child("gaussPoints")) t.gauss_points = attr_i(g, "value");
    return t;
}

void region_state(const TaskMaterial& m, const TaskRegion& r, double U[4]) {
    double Cv = m.Cp - GAS_R / m.M;     // Material::URS, src/global.cpp:9-30
    double gam = m.Cp / Cv;
    double p = r.p, T = r.T, u = r.u, v = r.v;
    double ro = p * m.M / (T * GAS_R);  // URS(2)
    double e = p / (ro * (gam - 1));     // URS(1)
    U[0] = ro;                           // convertParToCons, src/methods/fvm_tvd.cpp:795-801
    U[1] = ro * u;
    U[2] = ro * v;
    U[3] = ro * (e + 0.5 * (u * u + v * v));
}

void bind_mesh(const TaskConfig& t, const RawMesh& raw, const Topo& topo, std::vector<int>& cell_region,
               std::vector<int>& edge_bnd) {
    const int nc = topo.nc, ne = topo.ne;
    cell_region.assign(nc, -1);
    std::vector<int> region_of_name(raw.names.size(), -1);  // getRegion(typeName), src/methods/fvm_tvd.cpp:773-786
    for (size_t n = 0; n < raw.names.size(); n++)
        for (size_t r = 0; r < t.regions.size(); r++)
            if (t.regions[r].name == raw.names[n]) { region_of_name[n] = (int)r; break; }
    for (int i = 0; i < nc; i++) {
        cell_region[i] = region_of_name[raw.cell_name[i]];
        if (cell_region[i] < 0)
            throw Error(CFD2D_ERR_REGION_UNKNOWN,
                        "ERROR: unknown cell name '" + raw.names[raw.cell_name[i]] + "' of cell " + std::to_string(i));
    }
    edge_bnd.assign(ne, -1);
    std::map<long long, int> marker;  // Triangle: a later .poly line for the same edge wins (findEdge, src/mesh/grid.cpp:38-48)
    if (raw.berkeley)
        for (size_t s = 0; s < raw.bseg_marker.size(); s++) {
            long long a = raw.bseg[2 * s], b = raw.bseg[2 * s + 1];
            marker[std::min(a, b) * (1ll << 32) + std::max(a, b)] = raw.bseg_marker[s];
        }
    for (int e = 0; e < ne; e++) {  // boundary binding, src/methods/fvm_tvd.cpp:131-174
        if (topo.c2[e] >= 0) continue;
        int s = topo.bseg_of_edge[e];
        int b = -1;
        if (!raw.berkeley) {
            const std::string nm = s >= 0 ? raw.names[raw.bseg_name[s]] : std::string();
            for (size_t k = 0; k < t.bnds.size(); k++)
                if (!nm.empty() && t.bnds[k].name == nm) { b = (int)k; break; }
        } else {
            long long a = topo.n1[e], c = topo.n2[e];
            auto it = marker.find(std::min(a, c) * (1ll << 32) + std::max(a, c));
            int type = it != marker.end() ? it->second : -1;
            for (size_t k = 0; k < t.bnds.size(); k++)
                if (type != 0 && t.bnds[k].edgeType == type) { b = (int)k; break; }
        }
        if (b < 0)
            throw Error(CFD2D_ERR_EDGE_UNKNOWN,
                        "ERROR (boundary condition): unknown edge type of edge " + std::to_string(e) + "...");
        edge_bnd[e] = b;
    }
}

void bind_mesh_implicit(const TaskConfig& t, const RawMesh& raw, const Topo& topo, std::vector<int>& cell_region,
                        std::vector<int>& edge_bnd) {
    const int nc = topo.nc, ne = topo.ne;
    cell_region.assign(nc, -1);
    std::vector<int> region_of_name(raw.names.size(), -1);
    for (size_t n = 0; n < raw.names.size(); n++) {
        const int type = std::atoi(raw.names[n].c_str());  // the .ele attribute
        for (size_t r = 0; r < t.regions.size(); r++)
            if (t.regions[r].cellType == type) { region_of_name[n] = (int)r; break; }
    }
    for (int i = 0; i < nc; i++) {
        cell_region[i] = region_of_name[raw.cell_name[i]];
        if (cell_region[i] < 0)
            throw Error(CFD2D_ERR_REGION_UNKNOWN, "ERROR: unknown cell type " + raw.names[raw.cell_name[i]] + "...");
    }
    edge_bnd.assign(ne, -1);
    std::map<long long, int> marker;  // a later .poly line for the same edge wins (src/mesh/grid.cpp:214-221)
    for (size_t s = 0; s < raw.bseg_marker.size(); s++) {
        long long a = raw.bseg[2 * s], b = raw.bseg[2 * s + 1];
        marker[std::min(a, b) * (1ll << 32) + std::max(a, b)] = raw.bseg_marker[s];
    }
    for (int e = 0; e < ne; e++) {
        if (topo.c2[e] >= 0) continue;
        long long a = topo.n1[e], c = topo.n2[e];
        auto it = marker.find(std::min(a, c) * (1ll << 32) + std::max(a, c));
        const int type = it != marker.end() ? it->second : -1;
        int b = -1;
        for (size_t k = 0; k < t.bnds.size(); k++)
            if (t.bnds[k].edgeType == type) { b = (int)k; break; }
        if (b < 0)
            throw Error(CFD2D_ERR_EDGE_UNKNOWN,
                        "ERROR (boundary condition): unknown edge type of edge " + std::to_string(e) + "...");
        edge_bnd[e] = b;
    }
}

}  // namespace cfd2d
