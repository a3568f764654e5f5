#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>

#include "cfd2d.h"

namespace cfd2d {

namespace {

std::string slurp(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(CFD2D_ERR_FILE_OPENING, "File '" + path + "' opening error.");
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Up to n integers from the start of a line (sscanf("%d %d ...") semantics).
int scan_ints(const char* s, int* out, int n) {
    int k = 0;
    char* end;
    while (k < n) {
        long v = std::strtol(s, &end, 10);
        if (end == s) break;
        out[k++] = (int)v;
        s = end;
    }
    return k;
}

int scan_doubles(const char* s, double* out, int n) {
    int k = 0;
    char* end;
    while (k < n) {
        double v = std::strtod(s, &end);
        if (end == s) break;
        out[k++] = v;
        s = end;
    }
    return k;
}

}  // namespace

// ---------------------------------------------------------------- UNV

RawMesh read_unv(const std::string& path) {
    const std::string text = slurp(path);
    // Lines; a line whose first "-1" ends it is a block delimiter, two of them
    // close a block (read_block, src/mesh/MeshReaderSalomeUnv.cpp:267-286).
    std::vector<std::vector<std::string>> blocks;
    std::vector<std::string> cur;
    int minus = 0;
    size_t p = 0;
    while (p <= text.size()) {
        size_t q = text.find('\n', p);
        if (q == std::string::npos) q = text.size();
        std::string line = text.substr(p, q - p);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        p = q + 1;
        size_t pos = line.find("-1");
        if (pos != std::string::npos && pos + 2 == line.size()) {
            if (++minus == 2) {
                blocks.push_back(std::move(cur));
                cur.clear();
                minus = 0;
            }
            continue;
        }
        cur.push_back(line);
        if (q == text.size()) break;
    }
    if (!cur.empty()) blocks.push_back(std::move(cur));

    RawMesh m;
    struct Elem { int kind = 0; int index = -1; };   // 41 cell, 11 edge element
    std::vector<Elem> elements;
    std::vector<int> edge_label;                    // per UNV edge element: label-1
    std::map<std::string, std::vector<int>> groups; // name -> element labels-1 (sorted by name, like std::map)
    for (auto& b : blocks) {
        if (b.empty()) continue;
        int id = std::atoi(b[0].c_str());
        if (id == 2411) {
            for (size_t k = 1; k + 1 < b.size() + 1 && k < b.size(); k += 2) {
                double c[3] = {0, 0, 0};
                if (k + 1 >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2411: truncated node record");
                scan_doubles(b[k + 1].c_str(), c, 3);
                m.xy.push_back(c[0]);
                m.xy.push_back(c[1]);
            }
        } else if (id == 2412) {
            size_t k = 1;
            while (k < b.size()) {
                int h[6] = {0, 0, 0, 0, 0, 0};
                scan_ints(b[k].c_str(), h, 6);
                int label = h[0] - 1, type = h[1];
                k++;
                if (type == 11) {
                    if (k + 1 >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: truncated edge record");
                    int nd[2] = {0, 0};
                    scan_ints(b[k + 1].c_str(), nd, 2);
                    k += 2;
                    m.bseg.push_back(nd[0] - 1);
                    m.bseg.push_back(nd[1] - 1);
                    edge_label.push_back(label);
                } else if (type == 41) {
                    if (k >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: truncated triangle record");
                    int nd[3] = {0, 0, 0};
                    scan_ints(b[k].c_str(), nd, 3);
                    k += 1;
                    if (label < 0) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: bad element label");
                    if ((int)elements.size() <= label) elements.resize(label + 1);
                    elements[label].kind = 41;
                    elements[label].index = m.nc();
                    for (int j = 0; j < 3; j++) m.tri.push_back(nd[j] - 1);
                } else {
                    throw Error(CFD2D_ERR_MESH_UNV_UNKNOWN_ELEMENT, "Unknown element type '" + std::to_string(type) + "'.");
                }
            }
        } else if (id == 2467) {
            size_t k = 1;
            while (k < b.size()) {
                int h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                scan_ints(b[k].c_str(), h, 8);
                int n = h[7];
                k++;
                if (k >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2467: truncated group");
                char name[256] = {0};
                std::sscanf(b[k].c_str(), "%255s", name);
                k++;
                std::vector<int> ids;
                for (int j = 0; j < n / 2; j++, k++) {
                    if (k >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2467: truncated group entities");
                    int e[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    scan_ints(b[k].c_str(), e, 8);
                    ids.push_back(e[1] - 1);
                    ids.push_back(e[5] - 1);
                }
                if (n % 2 == 1) {
                    if (k >= b.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2467: truncated group entities");
                    int e[4] = {0, 0, 0, 0};
                    scan_ints(b[k].c_str(), e, 4);
                    ids.push_back(e[1] - 1);
                    k++;
                }
                groups[std::string(name)] = ids;
            }
        }
        // blocks 164, 2420 and any other block are skipped
    }
    const int nn = m.nn(), nc = m.nc();
    for (int v : m.tri)
        if (v < 0 || v >= nn) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV: triangle refers to a missing node");
    for (int v : m.bseg)
        if (v < 0 || v >= nn) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV: edge element refers to a missing node");
    // Only the first edge element of a node pair stands for the mesh edge
    // (find_edge, src/mesh/MeshReaderSalomeUnv.cpp:14-22, 204-210).
    std::map<long long, int> first;
    const int nb = (int)edge_label.size();
    std::vector<int> edge_elem_of_label;
    for (int s = 0; s < nb; s++) {
        long long a = m.bseg[2 * s], c = m.bseg[2 * s + 1];
        long long key = std::min(a, c) * (1ll << 32) + std::max(a, c);
        if (!first.count(key)) {
            first[key] = s;
            int label = edge_label[s];
            if (label >= 0) {
                if ((int)elements.size() <= label) elements.resize(label + 1);
                if (elements[label].kind == 0) { elements[label].kind = 11; elements[label].index = s; }
            }
        }
    }
    // Group names, groups visited in name order so the last one wins (:219-248).
    m.cell_name.assign(nc, std::string());
    m.bseg_name.assign(nb, std::string());
    for (auto& g : groups)
        for (int id : g.second) {
            if (id < 0 || id >= (int)elements.size()) continue;
            const Elem& el = elements[id];
            if (el.kind == 41) m.cell_name[el.index] = g.first;
            else if (el.kind == 11) m.bseg_name[el.index] = g.first;
        }
    return m;
}

// ---------------------------------------------------------------- Triangle

RawMesh read_triangle(const std::string& base) {
    RawMesh m;
    m.berkeley = true;
    auto tokens = [](const std::string& s) {
        std::vector<std::string> t;
        std::istringstream is(s);
        std::string w;
        while (is >> w) t.push_back(w);
        return t;
    };
    auto node = tokens(slurp(base + ".node"));
    auto ele = tokens(slurp(base + ".ele"));
    auto nei = tokens(slurp(base + ".neigh"));
    auto poly = tokens(slurp(base + ".poly"));
    auto at = [](const std::vector<std::string>& t, size_t k) -> const std::string& {
        if (k >= t.size()) throw Error(CFD2D_ERR_MESH_FORMAT, "Triangle mesh: truncated file");
        return t[k];
    };
    int nn = std::atoi(at(node, 0).c_str());
    for (int i = 0; i < nn; i++) {  // "%d %lf %lf %d"
        m.xy.push_back(std::strtod(at(node, 4 + 4 * i + 1).c_str(), nullptr));
        m.xy.push_back(std::strtod(at(node, 4 + 4 * i + 2).c_str(), nullptr));
    }
    int nc = std::atoi(at(ele, 0).c_str());
    for (int i = 0; i < nc; i++) {  // "%d %d %d %d %d": index, nodes, attribute
        for (int j = 0; j < 3; j++) m.tri.push_back(std::atoi(at(ele, 3 + 5 * i + 1 + j).c_str()) - 1);
        m.cell_name.push_back(std::to_string(std::atoi(at(ele, 3 + 5 * i + 4).c_str())));
    }
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) m.neigh.push_back(std::atoi(at(nei, 2 + 4 * i + 1 + j).c_str()) - 1);
    int nb = std::atoi(at(poly, 4).c_str());
    for (int i = 0; i < nb; i++) {
        m.bseg.push_back(std::atoi(at(poly, 6 + 4 * i + 1).c_str()) - 1);
        m.bseg.push_back(std::atoi(at(poly, 6 + 4 * i + 2).c_str()) - 1);
        m.bseg_marker.push_back(std::atoi(at(poly, 6 + 4 * i + 3).c_str()));
    }
    for (int v : m.tri)
        if (v < 0 || v >= nn) throw Error(CFD2D_ERR_MESH_FORMAT, "Triangle mesh: element refers to a missing node");
    for (int v : m.neigh)
        if (v < -2 || v >= nc) throw Error(CFD2D_ERR_MESH_FORMAT, "Triangle mesh: bad neighbour");
    return m;
}

// ---------------------------------------------------------------- topology

Topo build_topology(int nn, const double* xy, int nc, const int* tri, const int* neigh_berkeley,
                    int nb, const int* bseg, bool require_segment, int gauss_points) {
    Topo t;
    t.nn = nn; t.nc = nc;
    t.xy.assign(xy, xy + 2 * (size_t)nn);
    t.tri.assign(tri, tri + 3 * (size_t)nc);
    const bool berk = neigh_berkeley != nullptr;
    for (int k = 0; k < 3 * nc; k++)
        if (tri[k] < 0 || tri[k] >= nn) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: triangle refers to a missing node");
    t.cx.resize(nc); t.cy.resize(nc);
    for (int i = 0; i < nc; i++) {  // src/mesh/MeshReaderSalomeUnv.cpp:89-90
        const int* v = tri + 3 * i;
        t.cx[i] = (xy[2 * v[0]] + xy[2 * v[1]] + xy[2 * v[2]]) / 3.0;
        t.cy[i] = (xy[2 * v[0] + 1] + xy[2 * v[1] + 1] + xy[2 * v[2] + 1]) / 3.0;
    }
    std::vector<int> neigh(3 * (size_t)nc);
    if (berk) {
        std::copy(neigh_berkeley, neigh_berkeley + 3 * (size_t)nc, neigh.begin());
    } else {
        // node -> cells (ascending); neighbour across (k, k+1) = the last other
        // cell holding both nodes (src/mesh/MeshReaderSalomeUnv.cpp:64-116)
        std::vector<int> off(nn + 1, 0);
        for (int k = 0; k < 3 * nc; k++) off[tri[k] + 1]++;
        for (int i = 0; i < nn; i++) off[i + 1] += off[i];
        std::vector<int> fill(off.begin(), off.end() - 1), lst(3 * (size_t)nc);
        for (int i = 0; i < nc; i++)
            for (int k = 0; k < 3; k++) lst[fill[tri[3 * i + k]]++] = i;
        for (int i = 0; i < nc; i++)
            for (int k = 0; k < 3; k++) {
                int a = tri[3 * i + k], b = tri[3 * i + (k + 1) % 3];
                int ia = off[a], ib = off[b], nbh = -2;
                while (ia < off[a + 1] && ib < off[b + 1]) {
                    if (lst[ia] < lst[ib]) ia++;
                    else if (lst[ia] > lst[ib]) ib++;
                    else { if (lst[ia] != i) nbh = lst[ia]; ia++; ib++; }
                }
                neigh[3 * i + k] = nbh;
            }
    }
    int ne = 0;  // count, clearing each neighbour's back reference (:118-135)
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            int p = neigh[3 * i + j];
            if (p > -1) {
                for (int k = 0; k < 3; k++)
                    if (neigh[3 * p + k] == i) neigh[3 * p + k] = -1;
                ne++;
            }
            if (p == -2) ne++;
        }
    t.ne = ne;
    t.cedges.assign(3 * (size_t)nc, -1);
    t.n1.resize(ne); t.n2.resize(ne); t.c1.resize(ne); t.c2.resize(ne); t.npts.resize(ne);
    t.bseg_of_edge.assign(ne, -1);
    t.nx.resize(ne); t.ny.resize(ne); t.l.resize(ne);
    t.pts.assign(6 * (size_t)ne, 0.0);
    t.S.resize(nc);
    std::vector<int> cfi(nc, 0);
    std::vector<std::pair<long long, int>> keys(nb);
    for (int s = 0; s < nb; s++) {
        long long a = bseg[2 * s], b = bseg[2 * s + 1];
        keys[s] = {std::min(a, b) * (1ll << 32) + std::max(a, b), s};
    }
    std::sort(keys.begin(), keys.end());
    const double sq3 = 1.0 / std::sqrt(3.0);
    const int npts = berk ? (gauss_points == 2 ? 3 : 1) : 3;
    int e = 0;
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            int p = neigh[3 * i + j];
            if (p == -1) continue;
            if (p < -2 || p >= nc) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: bad neighbour index");
            const int* v = tri + 3 * i;
            int a = berk ? v[(j + 1) % 3] : v[j];
            int b = berk ? v[(j + 2) % 3] : v[(j + 1) % 3];
            t.n1[e] = a; t.n2[e] = b;
            double x1 = xy[2 * a], y1 = xy[2 * a + 1], x2 = xy[2 * b], y2 = xy[2 * b + 1];
            double* P = &t.pts[6 * (size_t)e];
            P[0] = (x1 + x2) / 2.0;  // midpoint, then Gauss points at -+1/sqrt(3) of the half length
            P[1] = (y1 + y2) / 2.0;
            if (npts == 3) {
                P[2] = (x1 + x2) / 2.0 - sq3 * (x2 - x1) / 2.0;
                P[3] = (y1 + y2) / 2.0 - sq3 * (y2 - y1) / 2.0;
                P[4] = (x1 + x2) / 2.0 + sq3 * (x2 - x1) / 2.0;
                P[5] = (y1 + y2) / 2.0 + sq3 * (y2 - y1) / 2.0;
            }
            t.npts[e] = npts;
            double nx = y2 - y1, ny = x1 - x2;
            double l = std::sqrt(nx * nx + ny * ny);
            nx /= l; ny /= l;
            t.l[e] = l;
            t.c1[e] = i;
            t.cedges[3 * i + cfi[i]++] = e;
            if (!berk) {  // turn the normal outward from c1 (:181-187)
                double vx = t.cx[i] - P[0], vy = t.cy[i] - P[1];
                if (vx * nx + vy * ny > 0) { nx *= -1; ny *= -1; }
            }
            t.nx[e] = nx; t.ny[e] = ny;
            if (p > -1) {
                t.c2[e] = p;
                if (cfi[p] >= 3) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: a cell has more than three edges");
                t.cedges[3 * p + cfi[p]++] = e;
            } else {
                t.c2[e] = -1;
                long long key = std::min<long long>(a, b) * (1ll << 32) + std::max<long long>(a, b);
                auto it = std::lower_bound(keys.begin(), keys.end(), std::make_pair(key, -1));
                if (it != keys.end() && it->first == key) t.bseg_of_edge[e] = it->second;
                else if (require_segment)
                    throw Error(CFD2D_ERR_MESH_UNV_NOT_DEFINED_BND_EDGE,
                                "Boundary edge #" + std::to_string(e) + " not defined in UNV file.");
            }
            e++;
        }
    for (int i = 0; i < nc; i++) {  // Heron, :250-255
        if (cfi[i] != 3) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: cell " + std::to_string(i) + " is not a closed triangle");
        double a = t.l[t.cedges[3 * i]], b = t.l[t.cedges[3 * i + 1]], c = t.l[t.cedges[3 * i + 2]];
        double p = (a + b + c) / 2.0;
        t.S[i] = std::sqrt(p * (p - a) * (p - b) * (p - c));
    }
    return t;
}

// ---------------------------------------------------------------- layout

std::vector<int> rcm_order(const Topo& t) {
    const int nc = t.nc;
    std::vector<int> deg(nc, 0), adj(3 * (size_t)nc, -1);
    for (int e = 0; e < t.ne; e++) {
        int a = t.c1[e], b = t.c2[e];
        if (b < 0) continue;
        adj[3 * a + deg[a]++] = b;
        adj[3 * b + deg[b]++] = a;
    }
    std::vector<int> order;
    order.reserve(nc);
    std::vector<char> seen(nc, 0);
    std::vector<int> level(nc, -1);
    auto bfs_last = [&](int s) {  // farthest cell of s's component (for a pseudo-peripheral start)
        std::vector<int> q{s};
        level[s] = 0;
        size_t h = 0;
        int last = s;
        while (h < q.size()) {
            int u = q[h++];
            last = u;
            for (int k = 0; k < deg[u]; k++) {
                int w = adj[3 * u + k];
                if (level[w] < 0) { level[w] = level[u] + 1; q.push_back(w); }
            }
        }
        for (int u : q) level[u] = -1;
        return last;
    };
    for (int s0 = 0; s0 < nc; s0++) {
        if (seen[s0]) continue;
        int s = bfs_last(bfs_last(s0));
        size_t start = order.size();
        order.push_back(s);
        seen[s] = 1;
        for (size_t h = start; h < order.size(); h++) {
            int u = order[h];
            int nb[3], m = 0;
            for (int k = 0; k < deg[u]; k++) {
                int w = adj[3 * u + k];
                if (!seen[w]) { seen[w] = 1; nb[m++] = w; }
            }
            std::sort(nb, nb + m, [&](int x, int y) { return deg[x] != deg[y] ? deg[x] < deg[y] : x < y; });
            for (int k = 0; k < m; k++) order.push_back(nb[k]);
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

Layout make_layout(const Topo& t, const std::vector<int>& cell_mat, const std::vector<int>& edge_bnd, bool rcm) {
    Layout L;
    const int nc = t.nc, ne = t.ne;
    L.nc = nc; L.ne = ne;
    if (rcm) L.perm = rcm_order(t);
    else { L.perm.resize(nc); std::iota(L.perm.begin(), L.perm.end(), 0); }
    L.iperm.resize(nc);
    for (int i = 0; i < nc; i++) L.iperm[L.perm[i]] = i;
    // edges: interior ones by (lower, upper) storage cell, then boundary ones by cell
    std::vector<std::pair<long long, int>> key(ne);
    int n_int = 0;
    for (int e = 0; e < ne; e++) {
        long long a = L.iperm[t.c1[e]];
        if (t.c2[e] >= 0) {
            long long b = L.iperm[t.c2[e]];
            key[e] = {std::min(a, b) * (1ll << 32) + std::max(a, b), e};
            n_int++;
        } else {
            key[e] = {(1ll << 62) + a * 4, e};
        }
    }
    std::sort(key.begin(), key.end());
    L.n_int = n_int;
    L.eorig.resize(ne);
    std::vector<int> enew(ne);
    for (int k = 0; k < ne; k++) { L.eorig[k] = key[k].second; enew[key[k].second] = k; }
    L.ec1.resize(ne); L.ec2.resize(ne); L.ebnd.resize(ne);
    L.nx.resize(ne); L.ny.resize(ne); L.l.resize(ne); L.dl.assign(8 * (size_t)ne, 0.0);
    for (int k = 0; k < ne; k++) {
        int e = L.eorig[k];
        int a = t.c1[e], b = t.c2[e];
        L.ec1[k] = L.iperm[a];
        L.ec2[k] = b >= 0 ? L.iperm[b] : -1;
        L.ebnd[k] = b >= 0 ? -1 : edge_bnd[e];
        L.nx[k] = t.nx[e]; L.ny[k] = t.ny[e]; L.l[k] = t.l[e];
        for (int gp = 0; gp < 2; gp++) {  // the reference's points c[1], c[2] minus each centroid
            double px = t.pts[6 * (size_t)e + 2 + 2 * gp], py = t.pts[6 * (size_t)e + 3 + 2 * gp];
            L.dl[(size_t)(4 * gp) * ne + k] = px - t.cx[a];
            L.dl[(size_t)(4 * gp + 1) * ne + k] = py - t.cy[a];
            if (b >= 0) {
                L.dl[(size_t)(4 * gp + 2) * ne + k] = px - t.cx[b];
                L.dl[(size_t)(4 * gp + 3) * ne + k] = py - t.cy[b];
            }
        }
    }
    L.face.resize(3 * (size_t)nc);
    L.rem_nb.resize(3 * (size_t)nc);
    L.S.resize(nc);
    L.cmat.resize(nc);
    for (int i = 0; i < nc; i++) {
        int o = L.perm[i];
        L.S[i] = t.S[o];
        L.cmat[i] = (uint8_t)cell_mat[o];
        for (int k = 0; k < 3; k++) {
            int e = t.cedges[3 * o + k];
            int side = t.c1[e] == o ? 0 : 1;
            L.face[(size_t)k * nc + i] = (enew[e] << 1) | side;
            int j = t.c2[e];
            L.rem_nb[(size_t)k * nc + i] = j >= 0 ? L.iperm[j] : -1;
        }
    }
    return L;
}

}  // namespace cfd2d
