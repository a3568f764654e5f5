// Host driver of FEM_RKDG on the GPU (src/methods/fem_rkdg.cpp): the mesh part, the
// geometry and quadrature (computed here once, in the reference's operation order), the
// binding of regions and boundaries, the device layout, the step graph, run(), the VTU
// output and the state exchange.
#include "rkdg.hpp"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cctype>
#include <sys/stat.h>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>

#include "cfd2d.h"
#include "mesh.hpp"
#include "solver.hpp"

namespace cfd2d {

// ------------------------------------------------------------------ mesh part

namespace {

struct Tokens {
    std::string buf;
    size_t pos = 0;
    bool next(const char*& s, size_t& n) {
        while (pos < buf.size() && std::isspace((unsigned char)buf[pos])) pos++;
        if (pos >= buf.size()) return false;
        size_t b = pos;
        while (pos < buf.size() && !std::isspace((unsigned char)buf[pos])) pos++;
        s = buf.data() + b;
        n = pos - b;
        return true;
    }
    std::string word(const char* what) {
        const char* s; size_t n;
        if (!next(s, n)) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("mesh part: missing ") + what);
        return std::string(s, n);
    }
    long long ival(const char* what) {  // fscanf "%d"
        const std::string w = word(what);
        char* end = nullptr;
        long long v = std::strtoll(w.c_str(), &end, 10);
        if (end == w.c_str()) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("mesh part: bad ") + what);
        return v;
    }
    double dval(const char* what) {     // fscanf "%lf": strtod, correctly rounded
        const std::string w = word(what);
        char* end = nullptr;
        double v = std::strtod(w.c_str(), &end);
        if (end == w.c_str()) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("mesh part: bad ") + what);
        return v;
    }
};

int name_index(std::vector<std::string>& names, std::unordered_map<std::string, int>& idx, const std::string& s) {
    auto it = idx.find(s);
    if (it != idx.end()) return it->second;
    const int k = (int)names.size();
    names.push_back(s);
    idx.emplace(s, k);
    return k;
}

}  // namespace

// Grid::readMeshFiles, src/mesh/grid.cpp:275-420, for a single-process part
DgMesh read_proc_mesh(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(CFD2D_ERR_FILE_OPENING, "Can not open file '" + path + "'");
    Tokens t;
    {
        std::ostringstream ss;
        ss << f.rdbuf();
        t.buf = ss.str();
    }
    log_line("Reading mesh part structure:\n");
    DgMesh m;
    log_line("\t- nodes;\n");
    const long long nn = t.ival("node count"), nnx = t.ival("node count");
    if (nn < 0 || nnx < nn || nnx > (1ll << 30)) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: bad node counts");
    m.nn = (int)nnx;
    m.nn_own = (int)nn;
    m.xy.resize(2 * (size_t)nnx);
    for (long long i = 0; i < nnx; i++) {
        t.ival("node number");
        m.xy[2 * i] = t.dval("x");
        m.xy[2 * i + 1] = t.dval("y");
    }
    log_line("\t- cells;\n");
    const long long nc = t.ival("cell count"), ncx = t.ival("cell count");
    if (nc <= 0 || ncx != nc || nc > (1ll << 30))
        throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: cell counts (a part with ghost cells belongs to a "
                                           "multi-process decomposition; this library runs one part)");
    m.nc = (int)nc;
    m.tri.resize(3 * (size_t)nc);
    m.cell_name.resize(nc);
    std::unordered_map<std::string, int> idx;
    for (long long i = 0; i < nc; i++) {
        t.ival("cell number");
        for (int k = 0; k < 3; k++) {
            const long long v = t.ival("cell node");
            if (v < 0 || v >= nnx) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: cell node out of range");
            m.tri[3 * i + k] = (int)v;
        }
        m.cell_name[i] = name_index(m.names, idx, t.word("cell type"));
    }
    log_line("\t- edges;\n");
    const long long ne = t.ival("edge count"), nex = t.ival("edge count");
    if (ne <= 0 || nex != ne || ne > (1ll << 30)) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: bad edge counts");
    m.ne = (int)ne;
    m.en.resize(2 * (size_t)ne);
    m.etype.resize(ne);
    m.ename.resize(ne);
    for (long long e = 0; e < ne; e++) {
        t.ival("edge number");
        for (int k = 0; k < 2; k++) {
            const long long v = t.ival("edge node");
            if (v < 0 || v >= nnx) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: edge node out of range");
            m.en[2 * e + k] = (int)v;
        }
        m.etype[e] = (int)t.ival("edge type");
        if (m.etype[e] != 0) m.ename[e] = t.word("edge type name");
    }
    log_line("  complete...\n");
    return m;
}

DgMesh dg_mesh_from_arrays(int nn, const double* xy, int nc, const int* tri, const int* cell_region,
                           const std::vector<std::string>& region_names, int nb, const int* bseg,
                           const int* bseg_bnd, const std::vector<TaskBound>& bnds) {
    DgMesh m;
    m.nn = nn;
    m.nn_own = nn;
    m.nc = nc;
    m.xy.assign(xy, xy + 2 * (size_t)nn);
    m.tri.assign(tri, tri + 3 * (size_t)nc);
    m.names = region_names;
    m.cell_name.assign(cell_region, cell_region + nc);
    for (int i = 0; i < nc; i++)
        if (m.cell_name[i] < 0 || m.cell_name[i] >= (int)region_names.size())
            throw Error(CFD2D_ERR_INVALID_ARG, "mesh arrays: region index out of range");
    std::unordered_map<long long, int> edge_of;
    edge_of.reserve(3 * (size_t)nc);
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            const int a = tri[3 * i + j], b = tri[3 * i + (j + 1) % 3];
            if (a < 0 || a >= nn || b < 0 || b >= nn) throw Error(CFD2D_ERR_INVALID_ARG, "mesh arrays: node out of range");
            const long long key = (long long)std::min(a, b) * (1ll << 31) + std::max(a, b);
            if (edge_of.emplace(key, m.ne).second) {
                m.en.push_back(a);
                m.en.push_back(b);
                m.ne++;
            }
        }
    m.etype.assign(m.ne, 0);
    m.ename.assign(m.ne, std::string());
    for (int s = 0; s < nb; s++) {
        const int a = bseg[2 * s], b = bseg[2 * s + 1];
        auto it = edge_of.find((long long)std::min(a, b) * (1ll << 31) + std::max(a, b));
        if (it == edge_of.end()) throw Error(CFD2D_ERR_INVALID_ARG, "mesh arrays: boundary segment is no cell side");
        const int k = bseg_bnd[s];
        if (k < 0 || k >= (int)bnds.size()) throw Error(CFD2D_ERR_INVALID_ARG, "mesh arrays: boundary index out of range");
        m.etype[it->second] = 0x100;  // Edge::TYPE_NAMED
        m.ename[it->second] = bnds[k].name;
    }
    return m;
}

// ------------------------------------------------------------------ solver

template <typename T>
T* RkdgSolver::dalloc(size_t n) {
    void* p = nullptr;
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    CUDA_CHECK(cudaMalloc(&p, b));
    allocs_.push_back(p);
    bytes_ += b;
    return static_cast<T*>(p);
}

template <typename T>
T* RkdgSolver::upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) CUDA_CHECK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
    return p;
}

namespace {
constexpr double kGR = GAS_R;  // Material::gR, src/global.cpp:6

struct Par { double r, u, v, E, e, p, cz, T; };

// Material::URS, src/global.cpp:9-30
void urs(const TaskMaterial& mt, Par& par, int flag) {
    const double Cv = mt.Cp - kGR / mt.M;
    const double gam = mt.Cp / Cv;
    switch (flag) {
    case 0: par.p = par.r * par.e * (gam - 1); par.cz = std::sqrt(gam * par.p / par.r); break;
    case 1: par.e = par.p / (par.r * (gam - 1)); par.T = par.e / Cv; break;
    case 2: par.r = par.p * mt.M / (par.T * kGR); par.cz = std::sqrt(gam * par.p / par.r); break;
    }
}
}  // namespace

RkdgSolver::RkdgSolver(const TaskConfig& t, DgMesh&& mesh) : task_(t), mesh_(std::move(mesh)) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(CFD2D_ERR_NO_DEVICE, "no CUDA device");
    CUDA_CHECK(cudaGetDevice(&dev_));
    const int nc = mesh_.nc, ne = mesh_.ne, gc = task_.dg_gp_cell, ge = task_.dg_gp_edge;
    const std::vector<double>& xy = mesh_.xy;
    const std::vector<int>& tri = mesh_.tri;

    // ---- binding (init :196-248 and getRegion by name :1382-1401)
    std::vector<int> region_of_name(mesh_.names.size(), -1);
    for (size_t n = 0; n < mesh_.names.size(); n++)
        for (size_t r = 0; r < task_.regions.size(); r++)
            if (task_.regions[r].name == mesh_.names[n]) { region_of_name[n] = (int)r; break; }
    std::vector<int> creg(nc);
    for (int i = 0; i < nc; i++) {
        creg[i] = region_of_name[mesh_.cell_name[i]];
        if (creg[i] < 0)
            throw Error(CFD2D_ERR_REGION_UNKNOWN, "ERROR: unknown cell name '" + mesh_.names[mesh_.cell_name[i]] + "'...");
    }
    std::vector<int> ebnd(ne, -1);
    for (int e = 0; e < ne; e++) {
        if (mesh_.etype[e] == 0) continue;
        int b = -1;
        for (size_t k = 0; k < task_.bnds.size(); k++) {
            const bool hit = mesh_.etype[e] == 0x100 ? task_.bnds[k].name == mesh_.ename[e]
                                                      : task_.bnds[k].edgeType == mesh_.etype[e];
            if (hit) { b = (int)k; break; }
        }
        if (b < 0)
            throw Error(CFD2D_ERR_EDGE_UNKNOWN,
                        "ERROR (boundary condition): unknown edge type of edge " + std::to_string(e) + "...");
        ebnd[e] = b;
    }
    cmat_orig_.resize(nc);
    for (int i = 0; i < nc; i++) cmat_orig_[i] = task_.regions[creg[i]].matId;

    // ---- geometry, original order (readMeshFiles :306-392, calcGaussPar :470-598)
    std::vector<double> cx(nc), cy(nc), HX(nc), HY(nc), S(nc), cellJ(nc);
    for (int i = 0; i < nc; i++) {
        const int* q = &tri[3 * (size_t)i];
        const double x0 = xy[2 * q[0]], x1 = xy[2 * q[1]], x2 = xy[2 * q[2]];
        const double y0 = xy[2 * q[0] + 1], y1 = xy[2 * q[1] + 1], y2 = xy[2 * q[2] + 1];
        cx[i] = (x0 + x1 + x2) / 3.0;
        cy[i] = (y0 + y1 + y2) / 3.0;
        auto mx3 = [](double a, double b, double c) { const double bc = b > c ? b : c; return a > bc ? a : bc; };
        HX[i] = mx3(std::fabs(x0 - x1), std::fabs(x1 - x2), std::fabs(x0 - x2));
        HY[i] = mx3(std::fabs(y0 - y1), std::fabs(y1 - y2), std::fabs(y0 - y2));
    }
    std::vector<int> cedge(3 * (size_t)nc), c1(ne, -1), c2(ne, -1), ncell(ne, 0);
    {
        std::unordered_map<long long, int> edge_of;
        edge_of.reserve(2 * (size_t)ne);
        for (int e = 0; e < ne; e++) {
            const int a = mesh_.en[2 * e], b = mesh_.en[2 * e + 1];
            edge_of[(long long)std::min(a, b) * (1ll << 31) + std::max(a, b)] = e;  // the file's last wins
        }
        for (int i = 0; i < nc; i++)
            for (int j = 0; j < 3; j++) {
                const int a = tri[3 * (size_t)i + j], b = tri[3 * (size_t)i + (j + 1) % 3];
                auto it = edge_of.find((long long)std::min(a, b) * (1ll << 31) + std::max(a, b));
                if (it == edge_of.end())
                    throw Error(CFD2D_ERR_MESH_FORMAT, "mesh part: a cell side is not among the edges");
                const int e = it->second;
                cedge[3 * (size_t)i + j] = e;
                if (ncell[e] == 0) c1[e] = i;
                else if (ncell[e] == 1) c2[e] = i;
                ncell[e]++;
            }
        for (int e = 0; e < ne; e++)
            if (ncell[e] < 1 || ncell[e] > 2)
                throw Error(CFD2D_ERR_MESH_FORMAT, "ERROR: edge #" + std::to_string(e) + " is not assigned to any cell.");
    }
    std::vector<double> enx(ne), eny(ne), el(ne), edgeJ(ne), egp(2 * (size_t)ge * ne), egw(ge);
    for (int e = 0; e < ne; e++) {
        const int na = mesh_.en[2 * e], nb = mesh_.en[2 * e + 1];
        const double xa = xy[2 * na], ya = xy[2 * na + 1], xb = xy[2 * nb], yb = xy[2 * nb + 1];
        const double mx = (xa + xb) / 2.0, my = (ya + yb) / 2.0;
        double nx = yb - ya, ny = xa - xb;
        const double l = std::sqrt(nx * nx + ny * ny);
        nx /= l;
        ny /= l;
        const double vx = cx[c1[e]] - mx, vy = cy[c1[e]] - my;
        if (vx * nx + vy * ny > 0) { nx *= -1; ny *= -1; }
        enx[e] = nx; eny[e] = ny; el[e] = l;
        double* gp = &egp[2 * (size_t)ge * e];
        if (ge == 3) {
            const double g1 = -3.0 / 5.0, g3 = 3.0 / 5.0;
            gp[0] = ((xa + xb) + g1 * (xb - xa)) / 2.0; gp[1] = ((ya + yb) + g1 * (yb - ya)) / 2.0;
            gp[2] = (xa + xb) / 2.0;                   gp[3] = (ya + yb) / 2.0;
            gp[4] = ((xa + xb) + g3 * (xb - xa)) / 2.0; gp[5] = ((ya + yb) + g3 * (yb - ya)) / 2.0;
        } else {
            const double s3 = 1.0 / std::sqrt(3.0);
            gp[0] = ((xa + xb) - s3 * (xb - xa)) * 0.5; gp[1] = ((ya + yb) - s3 * (yb - ya)) * 0.5;
            gp[2] = ((xa + xb) + s3 * (xb - xa)) * 0.5; gp[3] = ((ya + yb) + s3 * (yb - ya)) * 0.5;
        }
        edgeJ[e] = std::sqrt((xb - xa) * (xb - xa) + (yb - ya) * (yb - ya)) * 0.5;
    }
    if (ge == 3) { egw[0] = 5.0 / 9.0; egw[1] = 8.0 / 9.0; egw[2] = 5.0 / 9.0; }
    else { egw[0] = 1.0; egw[1] = 1.0; }
    for (int i = 0; i < nc; i++) {  // Heron in edgesInd order
        const double a = el[cedge[3 * (size_t)i]], b = el[cedge[3 * (size_t)i + 1]], c = el[cedge[3 * (size_t)i + 2]];
        const double p = (a + b + c) / 2.0;
        S[i] = std::sqrt(p * (p - a) * (p - b) * (p - c));
    }
    std::vector<double> cgp(2 * (size_t)gc * nc), cgw(gc);
    for (int i = 0; i < nc; i++) {
        const int* q = &tri[3 * (size_t)i];
        const double x1 = xy[2 * q[0]], y1 = xy[2 * q[0] + 1], x2 = xy[2 * q[1]], y2 = xy[2 * q[1] + 1];
        const double x3 = xy[2 * q[2]], y3 = xy[2 * q[2] + 1];
        const double a1 = x1 - x3, a2 = y1 - y3, b1 = x2 - x3, b2 = y2 - y3, k1 = x3, k2 = y3;
        double* gp = &cgp[2 * (size_t)gc * i];
        if (gc == 4) {
            const double a = 1.0 / 3.0, b = 1.0 / 5.0, c = 3.0 / 5.0;
            gp[0] = a1 * a + b1 * a + k1; gp[1] = a2 * a + b2 * a + k2;
            gp[2] = a1 * c + b1 * b + k1; gp[3] = a2 * c + b2 * b + k2;
            gp[4] = a1 * b + b1 * c + k1; gp[5] = a2 * b + b2 * c + k2;
            gp[6] = a1 * b + b1 * b + k1; gp[7] = a2 * b + b2 * b + k2;
            cellJ[i] = 0.5 * std::fabs(a1 * b2 - a2 * b1);
        } else {
            const double a = 1.0 / 6.0, b = 2.0 / 3.0;
            gp[0] = a1 * a + b1 * a + k1; gp[1] = a2 * a + b2 * a + k2;
            gp[2] = a1 * a + b1 * b + k1; gp[3] = a2 * a + b2 * b + k2;
            gp[4] = a1 * b + b1 * a + k1; gp[5] = a2 * b + b2 * a + k2;
            cellJ[i] = std::fabs(a1 * b2 - a2 * b1);
        }
    }
    if (gc == 4) { cgw[0] = -27.0 / 48.0; cgw[1] = 25.0 / 48.0; cgw[2] = 25.0 / 48.0; cgw[3] = 25.0 / 48.0; }
    else { cgw[0] = 1.0 / 6.0; cgw[1] = 1.0 / 6.0; cgw[2] = 1.0 / 6.0; }
    // getF at a point (its intent, :1441-1452): (1, (x - xc)/HX, (y - yc)/HY)
    auto basis = [&](int i, double x, double y, double& F1, double& F2) {
        F1 = (x - cx[i]) / HX[i];
        F2 = (y - cy[i]) / HY[i];
    };
    // calcMassMatr (:449-468) and inverseMatr (src/global.cpp:444-470)
    std::vector<double> invA(9 * (size_t)nc);
    for (int i = 0; i < nc; i++) {
        double A[3][3];
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) {
                A[r][q] = 0.0;
                for (int g = 0; g < gc; g++) {
                    double F[3] = {1.0, 0.0, 0.0};
                    basis(i, cgp[2 * ((size_t)gc * i + g)], cgp[2 * ((size_t)gc * i + g) + 1], F[1], F[2]);
                    A[r][q] += cgw[g] * F[r] * F[q];
                }
                A[r][q] *= cellJ[i];
            }
        const double(*a)[3] = A;
        const double det = a[0][0] * a[1][1] * a[2][2] + a[1][0] * a[2][1] * a[0][2] + a[0][1] * a[1][2] * a[2][0] -
                           a[2][0] * a[1][1] * a[0][2] - a[1][0] * a[0][1] * a[2][2] - a[0][0] * a[2][1] * a[1][2];
        double m[3][3];
        m[0][0] = a[1][1] * a[2][2] - a[2][1] * a[1][2];
        m[0][1] = a[2][0] * a[1][2] - a[1][0] * a[2][2];
        m[0][2] = a[1][0] * a[2][1] - a[2][0] * a[1][1];
        m[1][0] = a[2][1] * a[0][2] - a[0][1] * a[2][2];
        m[1][1] = a[0][0] * a[2][2] - a[2][0] * a[0][2];
        m[1][2] = a[2][0] * a[0][1] - a[0][0] * a[2][1];
        m[2][0] = a[0][1] * a[1][2] - a[1][1] * a[0][2];
        m[2][1] = a[1][0] * a[0][2] - a[0][0] * a[1][2];
        m[2][2] = a[0][0] * a[1][1] - a[1][0] * a[0][1];
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) invA[9 * (size_t)i + 3 * r + q] = m[q][r] / det;
    }

    // ---- storage order: RCM of the cell graph; edges by their lower storage cell, boundary last
    {
        Topo tp;
        tp.nc = nc;
        tp.ne = ne;
        tp.c1 = c1;
        tp.c2 = c2;
        perm_ = task_.reorder == 0 ? std::vector<int>() : rcm_order(tp);
        if (perm_.empty()) {
            perm_.resize(nc);
            for (int i = 0; i < nc; i++) perm_[i] = i;
        }
    }
    std::vector<int> iperm(nc);
    for (int s = 0; s < nc; s++) iperm[perm_[s]] = s;
    std::vector<int> eorder(ne);
    for (int e = 0; e < ne; e++) eorder[e] = e;
    std::stable_sort(eorder.begin(), eorder.end(), [&](int x, int y) {
        const bool bx = c2[x] < 0, by = c2[y] < 0;
        if (bx != by) return by;
        const int lx = bx ? iperm[c1[x]] : std::min(iperm[c1[x]], iperm[c2[x]]);
        const int ly = by ? iperm[c1[y]] : std::min(iperm[c1[y]], iperm[c2[y]]);
        return lx < ly;
    });
    std::vector<int> eiperm(ne);
    for (int s = 0; s < ne; s++) eiperm[eorder[s]] = s;
    int n_int = 0;
    while (n_int < ne && c2[eorder[n_int]] >= 0) n_int++;

    // ---- device arrays
    CUDA_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    try {
        DgCase& c = c_;
        c.nc = nc; c.ne = ne; c.n_int = n_int; c.gc = gc; c.ge = ge;
        c.steady = task_.steady;
        c.rk_mode = task_.dg_rk;
        c.newton_cap = task_.newton_cap;
        c.cfl = task_.cfl;
        for (int g = 0; g < 4; g++) c.cgw[g] = g < gc ? cgw[g] : 0.0;
        for (int g = 0; g < 3; g++) c.egw[g] = g < ge ? egw[g] : 0.0;
        // faces of each storage cell in ascending original edge number, with their slot
        std::vector<int> face(3 * (size_t)nc);
        for (int s = 0; s < nc; s++) {
            const int i = perm_[s];
            int k[3] = {0, 1, 2};
            std::sort(k, k + 3, [&](int x, int y) { return cedge[3 * (size_t)i + x] < cedge[3 * (size_t)i + y]; });
            for (int f = 0; f < 3; f++) {
                const int e = cedge[3 * (size_t)i + k[f]];
                const int side = c1[e] == i ? 0 : 1;
                face[(size_t)f * nc + s] = (eiperm[e] << 3) | (k[f] << 1) | side;
            }
        }
        if ((long long)ne >= (1ll << 28)) throw Error(CFD2D_ERR_CAPACITY, "FEM_RKDG: more than 2^28 edges");
        c.face = upload(face);
        std::vector<double> cF(2 * (size_t)gc * nc), ih(2 * (size_t)nc), fc(2 * (size_t)nc), Js(nc), Ss(nc),
            iA(9 * (size_t)nc);
        std::vector<uint8_t> cm(nc), cf(nc);
        const int n_alias = (nc + 1) / 2;  // ro_old shares ro's coefficients (memcpy, :369-372)
        fc_.resize(2 * (size_t)nc);
        iperm_ = iperm;
        for (int s = 0; s < nc; s++) {
            const int i = perm_[s];
            for (int g = 0; g < gc; g++)
                basis(i, cgp[2 * ((size_t)gc * i + g)], cgp[2 * ((size_t)gc * i + g) + 1], cF[2 * ((size_t)gc * s + g)],
                      cF[2 * ((size_t)gc * s + g) + 1]);
            ih[2 * (size_t)s] = 1.0 / HX[i];
            ih[2 * (size_t)s + 1] = 1.0 / HY[i];
            basis(i, cx[i], cy[i], fc[2 * (size_t)s], fc[2 * (size_t)s + 1]);
            fc_[2 * (size_t)i] = fc[2 * (size_t)s];
            fc_[2 * (size_t)i + 1] = fc[2 * (size_t)s + 1];
            Js[s] = cellJ[i];
            Ss[s] = S[i];
            for (int k = 0; k < 9; k++) iA[9 * (size_t)s + k] = invA[9 * (size_t)i + k];
            cm[s] = (uint8_t)cmat_orig_[i];
            cf[s] = i < n_alias ? 1 : 0;
        }
        c.cF = upload(cF); c.ih = upload(ih); c.fc = upload(fc); c.cellJ = upload(Js); c.S = upload(Ss);
        c.invA = upload(iA);
        c.cflag = upload(cf);
        c.iperm = upload(iperm);
        std::vector<int> ec1(ne), ec2(ne), eb(ne);
        std::vector<double> nx(ne), ny(ne), J(ne), eF(4 * (size_t)ge * ne);
        for (int s = 0; s < ne; s++) {
            const int e = eorder[s];
            ec1[s] = iperm[c1[e]];
            ec2[s] = c2[e] >= 0 ? iperm[c2[e]] : -1;
            eb[s] = ebnd[e];
            nx[s] = enx[e]; ny[s] = eny[e]; J[s] = edgeJ[e];
            for (int g = 0; g < ge; g++) {
                const double x = egp[2 * ((size_t)ge * e + g)], y = egp[2 * ((size_t)ge * e + g) + 1];
                double* F = &eF[4 * ((size_t)ge * s + g)];
                basis(c1[e], x, y, F[0], F[1]);
                if (c2[e] >= 0) basis(c2[e], x, y, F[2], F[3]);
                else F[2] = F[3] = 0.0;
            }
        }
        c.ec1 = upload(ec1); c.ec2 = upload(ec2); c.ebnd = upload(eb);
        c.enx = upload(nx); c.eny = upload(ny); c.edgeJ = upload(J); c.eF = upload(eF);
        for (auto& m : task_.mats) {
            DgMat d;
            d.M = m.M;
            d.Cv = m.Cp - kGR / m.M;
            d.gam = m.Cp / d.Cv;  // getGamma, src/global.h:219
            d.gm1 = d.gam - 1;
            d.ig1 = 1.0 / (d.gam - 1.0);
            d.iCv = 1.0 / d.Cv;
            d.rg = rim_gas<double>(d.gam);
            mats_.push_back(d);
        }
        c.mats = upload(mats_);
        c.mat0 = mats_[0];
        if (mats_.size() > 1) c.cmat = upload(cm);
        std::vector<DevBnd> bnds;
        for (auto& b : task_.bnds) {
            DevBnd d{};
            d.kind = b.kind;
            d.u = b.par[0]; d.v = b.par[1]; d.T = b.par[2]; d.p = b.par[3];
            bnds.push_back(d);
        }
        if (bnds.empty()) bnds.push_back(DevBnd{});
        c.bnds = upload(bnds);
        c.A = dalloc<double>(12 * (size_t)nc);
        c.B = dalloc<double>(12 * (size_t)nc);
        c.E1 = dalloc<double>(12 * (size_t)ne);
        c.E2 = dalloc<double>(12 * (size_t)ne);
        c.ctau = dalloc<double>(nc);
        c.tmin = dalloc<unsigned long long>(1);
        c.res = dalloc<unsigned long long>(4);
        c.err = dalloc<unsigned>(1);
        stage_ = dalloc<double>(12 * (size_t)nc);
        CUDA_CHECK(cudaMallocHost(&host_bits_, 5 * sizeof(unsigned long long)));
        CUDA_CHECK(cudaMemsetAsync(c.err, 0, sizeof(unsigned), stream_));
        CUDA_CHECK(cudaMemsetAsync(c.res, 0, 4 * sizeof(unsigned long long), stream_));
        CUDA_CHECK(cudaMemsetAsync(c.E2, 0, 12 * (size_t)ne * sizeof(double), stream_));
        // initial state (:96-168, convertParToCons :1404-1418): URS(2), URS(1) twice
        std::vector<double> U(12 * (size_t)nc, 0.0);
        std::vector<std::array<double, 4>> reg(task_.regions.size());
        for (size_t r = 0; r < reg.size(); r++) {
            const TaskRegion& rg = task_.regions[r];
            const TaskMaterial& mt = task_.mats[rg.matId];
            Par par{};
            par.u = rg.u; par.v = rg.v; par.T = rg.T; par.p = rg.p;
            urs(mt, par, 2); urs(mt, par, 1);
            urs(mt, par, 2); urs(mt, par, 1);
            reg[r] = {par.r, par.r * par.u, par.r * par.v, par.r * (par.e + 0.5 * (par.u * par.u + par.v * par.v))};
        }
        for (int s = 0; s < nc; s++)
            for (int v = 0; v < 4; v++) U[12 * (size_t)s + 3 * v] = reg[creg[perm_[s]]][v];
        CUDA_CHECK(cudaMemcpyAsync(c.A, U.data(), U.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        build_graphs();
        tau_ = task_.tau;
        time_step();
        if (!task_.steady) log_line("\n\nUNSTEADY. Proc = %4d. Time step TAU = %e.\n\n", 0, tau_);
    } catch (...) {
        for (void* p : allocs_) cudaFree(p);
        allocs_.clear();
        if (host_bits_) cudaFreeHost(host_bits_);
        host_bits_ = nullptr;
        if (stream_) cudaStreamDestroy(stream_);
        stream_ = nullptr;
        throw;
    }
}

RkdgSolver::~RkdgSolver() {
    use_device();
    if (stream_) cudaStreamSynchronize(stream_);
    if (g_step_) cudaGraphExecDestroy(g_step_);
    if (g_step_res_) cudaGraphExecDestroy(g_step_res_);
    for (void* p : allocs_) cudaFree(p);
    if (host_bits_) cudaFreeHost(host_bits_);
    if (stream_) cudaStreamDestroy(stream_);
}

// The step's kernels: [time step (steady)], edges + cells of stage 1 from A, edges + cells
// of stage 2 from B (with the residual maxima in the second graph).
void RkdgSolver::build_graphs() {
    auto capture = [&](bool with_res) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ex = nullptr;
        CUDA_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        if (c_.steady) dg_launch_time_step(c_, stream_);
        dg_launch_edges(c_, task_.flux, c_.A, stream_);
        dg_launch_cells(c_, 1, false, stream_);
        dg_launch_edges(c_, task_.flux, c_.B, stream_);
        if (with_res) CUDA_CHECK(cudaMemsetAsync(c_.res, 0, 4 * sizeof(unsigned long long), stream_));
        dg_launch_cells(c_, 2, with_res, stream_);
        CUDA_CHECK(cudaStreamEndCapture(stream_, &g));
        CUDA_CHECK(cudaGraphInstantiate(&ex, g, 0));
        cudaGraphDestroy(g);
        return ex;
    };
    g_step_ = capture(false);
    g_step_res_ = capture(true);
}

// calcTimeStep as init calls it: steady -> cTau per cell (again in every step); unsteady ->
// TAU = min(TAU, CFL min_i S_i / maxU_i), every cell's cTau = TAU.
void RkdgSolver::time_step() {
    if (c_.steady) {
        dg_launch_time_step(c_, stream_);
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        return;
    }
    host_bits_[0] = 0x7ff0000000000000ull;
    CUDA_CHECK(cudaMemcpyAsync(c_.tmin, host_bits_, sizeof(unsigned long long), cudaMemcpyHostToDevice, stream_));
    dg_launch_time_step(c_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(host_bits_, c_.tmin, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    double m;
    std::memcpy(&m, host_bits_, sizeof m);
    double tau = 1.0e+20;
    if (m < tau) tau = m;
    tau *= task_.cfl;
    tau_ = tau_ < tau ? tau_ : tau;  // _min_
    dg_launch_fill(c_.ctau, tau_, c_.nc, stream_);
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void RkdgSolver::one_step(bool with_res) {
    if (!task_.steady) t_ += tau_;
    steps_++;
    CUDA_CHECK(cudaGraphLaunch(with_res ? g_step_res_ : g_step_, stream_));
    res_valid_ = with_res;
}

int RkdgSolver::read_status() {
    unsigned e = 0;
    CUDA_CHECK(cudaMemcpyAsync(&e, c_.err, sizeof e, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaMemsetAsync(c_.err, 0, sizeof(unsigned), stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    if (e & ERRBIT_NONPHYSICAL) return CFD2D_ERR_NONPHYSICAL;
    if (e & ERRBIT_NEWTON_CAP) return CFD2D_ERR_NEWTON_CAP;
    return CFD2D_OK;
}

int RkdgSolver::step(int n) {
    use_device();
    for (int k = 0; k < n; k++) one_step(k == n - 1);
    return read_status();
}

// FEM_RKDG::run, :600-660. A steady run never ends in the reference (t stays 0 while
// t < TMAX); here it ends with CFD2D_ERR_INVALID_ARG before the first step.
int RkdgSolver::run() {
    use_device();
    if (steps_ == 0) save_vtu(0);  // init's save(0), :379
    if (task_.steady && 0.0 < task_.tmax)
        throw Error(CFD2D_ERR_INVALID_ARG, "FEM_RKDG: a steady run has no end (t stays 0 < TMAX); use cfd2d_step");
    while (t_ < task_.tmax) {
        const bool log_now = task_.print_step != 0 && (steps_ + 1) % task_.print_step == 0;
        one_step(log_now && task_.steady);
        if (task_.file_step != 0 && steps_ % task_.file_step == 0) save_vtu(steps_);
        if (log_now) {
            if (!task_.steady) {
                log_line("step: %d\t\ttime step: %.16f\n", steps_, t_);
            } else {
                double r[4];
                residuals(r);
                log_line("step: %6d\tres: ro:%10.5e ru:%10.5e rv:%10.5e re:%10.5e\n", steps_, r[0], r[1], r[2], r[3]);
            }
        }
    }
    return read_status();
}

void RkdgSolver::get_coeffs(double* out) {
    use_device();
    const size_t bytes = 12 * (size_t)c_.nc * sizeof(double);
    if (double* dv = static_cast<double*>(device_view(out))) {
        dg_launch_scatter(c_, c_.A, dv, stream_);
    } else {
        dg_launch_scatter(c_, c_.A, stage_, stream_);
        CUDA_CHECK(cudaMemcpyAsync(out, stage_, bytes, cudaMemcpyDeviceToHost, stream_));
    }
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void RkdgSolver::set_coeffs(const double* in) {
    use_device();
    const size_t bytes = 12 * (size_t)c_.nc * sizeof(double);
    if (const double* dv = static_cast<const double*>(device_view(in))) {
        dg_launch_gather(c_, dv, c_.A, stream_);
    } else {
        CUDA_CHECK(cudaMemcpyAsync(stage_, in, bytes, cudaMemcpyHostToDevice, stream_));
        dg_launch_gather(c_, stage_, c_.A, stream_);
    }
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    tau_ = task_.tau;
    time_step();
}

void RkdgSolver::get_state(double* ro, double* ru, double* rv, double* re) {
    const int nc = c_.nc;
    std::vector<double> U(12 * (size_t)nc);
    get_coeffs(U.data());
    double* dst[4] = {ro, ru, rv, re};
    for (int v = 0; v < 4; v++) {
        if (!dst[v]) continue;
        for (int i = 0; i < nc; i++) dst[v][i] = centre_value(&U[12 * (size_t)i + 3 * v], i);
    }
}

void RkdgSolver::set_state(const double* ro, const double* ru, const double* rv, const double* re) {
    const double* src[4] = {ro, ru, rv, re};
    for (int v = 0; v < 4; v++)
        if (!src[v]) throw Error(CFD2D_ERR_INVALID_ARG, "set_state: all four arrays are required");
    const int nc = c_.nc;
    std::vector<double> U(12 * (size_t)nc, 0.0);
    for (int v = 0; v < 4; v++)
        for (int i = 0; i < nc; i++) U[12 * (size_t)i + 3 * v] = src[v][i];
    set_coeffs(U.data());
}

// SCALAR_PROD at the cell centre, basis (1, (xc - xc)/HX, (yc - yc)/HY)
double RkdgSolver::centre_value(const double* a, int i) const {
    double s = 0;
    s += a[0] * 1.0;
    s += a[1] * fc_[2 * (size_t)i];
    s += a[2] * fc_[2 * (size_t)i + 1];
    return s;
}

void RkdgSolver::get_ctau(double* out) {
    use_device();
    std::vector<double> tmp(c_.nc);
    CUDA_CHECK(cudaMemcpyAsync(tmp.data(), c_.ctau, sizeof(double) * c_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    for (int i = 0; i < c_.nc; i++) out[i] = tmp[iperm_[i]];
}

namespace {
const char kDgStateMagic[8] = {'C', 'F', 'D', '2', 'D', 'D', 'G', '1'};
}

// Restart files (no counterpart in the reference): coefficients (caller order), cTau, the
// step counter, t and TAU; a resumed run continues bit for bit as the uninterrupted one.
void RkdgSolver::save_state(const char* path) {
    use_device();
    const int nc = c_.nc;
    std::vector<double> U(12 * (size_t)nc), ct(nc);
    get_coeffs(U.data());
    get_ctau(ct.data());
    FILE* fp = std::fopen(path, "wb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    const int64_t hdr[2] = {nc, steps_};
    const double hd[2] = {t_, tau_};
    bool ok = std::fwrite(kDgStateMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof hdr, 1, fp) == 1 &&
              std::fwrite(hd, sizeof hd, 1, fp) == 1 &&
              std::fwrite(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fwrite(ct.data(), sizeof(double), ct.size(), fp) == ct.size();
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' write error.");
}

void RkdgSolver::load_state(const char* path) {
    use_device();
    const int nc = c_.nc;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    char magic[8];
    int64_t hdr[2];
    double hd[2];
    std::vector<double> U(12 * (size_t)nc), ct(nc);
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kDgStateMagic, 8) == 0 &&
              std::fread(hdr, sizeof hdr, 1, fp) == 1 && hdr[0] == nc && std::fread(hd, sizeof hd, 1, fp) == 1 &&
              std::fread(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fread(ct.data(), sizeof(double), ct.size(), fp) == ct.size();
    std::fclose(fp);
    if (!ok) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("File '") + path + "' is not a state of this mesh.");
    const size_t bytes = 12 * (size_t)nc * sizeof(double);
    CUDA_CHECK(cudaMemcpyAsync(stage_, U.data(), bytes, cudaMemcpyHostToDevice, stream_));
    dg_launch_gather(c_, stage_, c_.A, stream_);
    std::vector<double> cts(nc);
    for (int i = 0; i < nc; i++) cts[iperm_[i]] = ct[i];
    CUDA_CHECK(cudaMemcpyAsync(c_.ctau, cts.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    steps_ = (int)hdr[1];
    t_ = hd[0];
    tau_ = hd[1];
    res_valid_ = false;
}

void RkdgSolver::set_tau(double tau) {
    use_device();
    tau_ = tau;
    dg_launch_fill(c_.ctau, tau, c_.nc, stream_);
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void RkdgSolver::residuals(double out[4]) {
    use_device();
    if (!res_valid_) {
        for (int v = 0; v < 4; v++) out[v] = 0.0;
        return;
    }
    CUDA_CHECK(cudaMemcpyAsync(host_bits_ + 1, c_.res, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    std::memcpy(out, host_bits_ + 1, 4 * sizeof(double));
}

// save, :662-800: res_%010d.pvtu and vtk_data/res_%010d.0000.vtu (the state at the cell
// centres through convertConsToPar; the vtk_data folder, which the DECOMP method creates in
// the reference's workflow, is created when missing). Formatted in blocks on host threads,
// written in order.
void RkdgSolver::save_vtu(int step) {
    const int nc = mesh_.nc;
    std::vector<double> U(12 * (size_t)nc);
    get_coeffs(U.data());
    char pname[64], vname[64];
    std::snprintf(pname, sizeof pname, "res_%010d.pvtu", step);
    FILE* fp = std::fopen(pname, "w");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + pname + "' opening error.");
    std::fprintf(fp, "<?xml version=\"1.0\"?>\n");
    std::fprintf(fp, "<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
    std::fprintf(fp, "  <PUnstructuredGrid GhostLevel=\"0\">\n");
    std::fprintf(fp, "    <PPoints><PDataArray type=\"Float32\" NumberOfComponents = \"3\" /></PPoints>\n");
    std::fprintf(fp, "    <PCellData Scalars=\"Density, Pressure, Proc\" Vectors=\"Velocity\">\n");
    std::fprintf(fp, "      <PDataArray type=\"Float32\" Name=\"Density\" format=\"ascii\" />\n");
    std::fprintf(fp, "      <PDataArray type=\"Float32\" Name=\"Pressure\" format=\"ascii\" />\n");
    std::fprintf(fp, "      <PDataArray type=\"Float32\" Name=\"Velocity\" format=\"ascii\" NumberOfComponents=\"3\"/>\n");
    std::fprintf(fp, "      <PDataArray type=\"Int32\" Name=\"Proc\" format=\"ascii\" />\n");
    std::fprintf(fp, "      <PDataArray type=\"Int32\" Name=\"Loc_ID\" format=\"ascii\" />\n");
    std::fprintf(fp, "    </PCellData>\n");
    std::fprintf(fp, "    <Piece Source=\"vtk_data/res_%010d.%04d.vtu\"/>\n", step, 0);
    std::fprintf(fp, "  </PUnstructuredGrid>\n");
    std::fprintf(fp, "</VTKFile>\n");
    const bool ok_p = std::ferror(fp) == 0;
    std::fclose(fp);
    if (!ok_p) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + pname + "' write error.");
    log_line("File '%s' saved...\n", pname);

    std::snprintf(vname, sizeof vname, "vtk_data/res_%010d.%04d.vtu", step, 0);
    log_line("File '%s' saved...\n", vname);
    ::mkdir("vtk_data", 0755);
    fp = std::fopen(vname, "w");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + vname + "' opening error.");
    // cell-centre parameters: r, u, v, p (convertConsToPar, :1420-1435)
    std::vector<double> cr(nc), cu(nc), cv(nc), cp(nc);
    for (int i = 0; i < nc; i++) {
        const TaskMaterial& mt = task_.mats[cmat_orig_[i]];
        Par par{};
        par.r = centre_value(&U[12 * (size_t)i], i);
        par.u = centre_value(&U[12 * (size_t)i + 3], i) / par.r;
        par.v = centre_value(&U[12 * (size_t)i + 6], i) / par.r;
        par.E = centre_value(&U[12 * (size_t)i + 9], i) / par.r;
        par.e = par.E - 0.5 * (par.u * par.u + par.v * par.v);
        urs(mt, par, 0);
        cr[i] = par.r; cu[i] = par.u; cv[i] = par.v; cp[i] = par.p;
    }
    const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    constexpr int kBlock = 1 << 15;
    auto section = [&](int n, auto item) {
        std::vector<std::string> buf(nth);
        for (int base = 0; base < n; base += (int)nth * kBlock) {
            auto work = [&](unsigned t) {
                std::string& o = buf[t];
                o.clear();
                const int a = base + (int)t * kBlock, b = std::min(n, a + kBlock);
                for (int i = a; i < b; i++) item(i, o);
            };
            std::vector<std::thread> th;
            for (unsigned t = 1; t < nth; t++) th.emplace_back(work, t);
            work(0);
            for (auto& x : th) x.join();
            for (auto& o : buf) std::fwrite(o.data(), 1, o.size(), fp);
        }
    };
    auto app = [](std::string& o, const char* fmt, auto... v) {
        char tmp[128];
        const int k = std::snprintf(tmp, sizeof tmp, fmt, v...);
        o.append(tmp, (size_t)std::max(0, std::min(k, (int)sizeof tmp - 1)));
    };
    const int nn = mesh_.nn_own;
    std::fprintf(fp, "<?xml version=\"1.0\"?>\n");
    std::fprintf(fp, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
    std::fprintf(fp, "  <UnstructuredGrid GhostLevel=\"0\">\n");
    std::fprintf(fp, "    <Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nn, nc);
    std::fprintf(fp, "      <Points>\n");
    std::fprintf(fp, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    std::fprintf(fp, "          ");
    section(nn, [&](int i, std::string& o) {
        app(o, "%25.15f %25.15f %25.15f ", mesh_.xy[2 * (size_t)i], mesh_.xy[2 * (size_t)i + 1], 0.0);
    });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "        </DataArray>\n");
    std::fprintf(fp, "      </Points>\n");
    std::fprintf(fp, "      <Cells>\n");
    std::fprintf(fp, "        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
    std::fprintf(fp, "          ");
    section(nc, [&](int i, std::string& o) { app(o, "%d ", (i + 1) * 3); });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "        </DataArray>\n");
    std::fprintf(fp, "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
    std::fprintf(fp, "          ");
    section(nc, [&](int i, std::string& o) {
        app(o, "%d %d %d ", mesh_.tri[3 * (size_t)i], mesh_.tri[3 * (size_t)i + 1], mesh_.tri[3 * (size_t)i + 2]);
    });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "        </DataArray>\n");
    std::fprintf(fp, "        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
    std::fprintf(fp, "          ");
    section(nc, [&](int, std::string& o) { o.append("5 "); });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "        </DataArray>\n");
    std::fprintf(fp, "      </Cells>\n");
    std::fprintf(fp, "      <CellData Scalars=\"Density, Pressure, Proc\" Vectors=\"Velocity\">\n");
    // the reference's "i + 1 % 8 == 0" is i + 1 == 0: one newline after the last item
    auto scalars = [&](const char* head, auto item) {
        std::fputs(head, fp);
        std::fprintf(fp, "          ");
        section(nc, [&](int i, std::string& o) {
            item(i, o);
            if (i + 1 == nc) o.append("\n");
        });
        std::fprintf(fp, "        </DataArray>\n");
    };
    scalars("        <DataArray type=\"Float32\" Name=\"Density\" format=\"ascii\">\n",
            [&](int i, std::string& o) { app(o, "%25.16f ", cr[i]); });
    scalars("        <DataArray type=\"Float32\" Name=\"Pressure\" format=\"ascii\">\n",
            [&](int i, std::string& o) { app(o, "%25.16f ", cp[i]); });
    scalars("        <DataArray type=\"Float32\" Name=\"Velocity\" format=\"ascii\" NumberOfComponents=\"3\">\n",
            [&](int i, std::string& o) { app(o, "%25.16f %25.16f %25.16f ", cu[i], cv[i], 0.0); });
    scalars("        <DataArray type=\"Int32\" Name=\"Proc\" format=\"ascii\">\n",
            [&](int, std::string& o) { o.append("0 "); });
    scalars("        <DataArray type=\"Int32\" Name=\"Loc_ID\" format=\"ascii\">\n",
            [&](int i, std::string& o) { app(o, "%d ", i); });
    std::fprintf(fp, "      </CellData>\n");
    std::fprintf(fp, "    </Piece>\n");
    std::fprintf(fp, "  </UnstructuredGrid>\n");
    std::fprintf(fp, "</VTKFile>\n");
    const bool ok = std::ferror(fp) == 0;
    std::fclose(fp);
    if (!ok) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + vname + "' write error.");
}

// n steps between CUDA events on the solver's stream (graph replays); total ms
double RkdgSolver::timed_steps(int n) {
    use_device();
    cudaEvent_t a, b;
    CUDA_CHECK(cudaEventCreate(&a));
    CUDA_CHECK(cudaEventCreate(&b));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    CUDA_CHECK(cudaEventRecord(a, stream_));
    for (int k = 0; k < n; k++) one_step(false);
    CUDA_CHECK(cudaEventRecord(b, stream_));
    CUDA_CHECK(cudaEventSynchronize(b));
    float ms = 0.f;
    CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

void RkdgSolver::profile_steps(int n, double ms[3], int launches[3]) {
    use_device();
    for (int k = 0; k < 3; k++) { ms[k] = 0.0; launches[k] = 0; }
    cudaEvent_t ev[2];
    for (auto& e : ev) CUDA_CHECK(cudaEventCreate(&e));
    auto timed = [&](int slot, auto launch) {
        CUDA_CHECK(cudaEventRecord(ev[0], stream_));
        launch();
        CUDA_CHECK(cudaEventRecord(ev[1], stream_));
        CUDA_CHECK(cudaEventSynchronize(ev[1]));
        float t = 0.f;
        CUDA_CHECK(cudaEventElapsedTime(&t, ev[0], ev[1]));
        ms[slot] += t;
    };
    for (int k = 0; k < n; k++) {
        if (!task_.steady) t_ += tau_;
        steps_++;
        if (c_.steady) timed(2, [&] { dg_launch_time_step(c_, stream_); });
        timed(0, [&] { dg_launch_edges(c_, task_.flux, c_.A, stream_); });
        timed(1, [&] { dg_launch_cells(c_, 1, false, stream_); });
        timed(0, [&] { dg_launch_edges(c_, task_.flux, c_.B, stream_); });
        timed(1, [&] { dg_launch_cells(c_, 2, false, stream_); });
    }
    res_valid_ = false;
    launches[0] = 2;
    launches[1] = 2;
    launches[2] = c_.steady ? 1 : 0;
    for (auto& e : ev) cudaEventDestroy(e);
}

}  // namespace cfd2d
