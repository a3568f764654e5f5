#include "mesh.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>
#include <thread>

#include "cfd2d.h"

namespace cfd2d {

namespace {

std::string slurp(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(CFD2D_ERR_FILE_OPENING, "File '" + path + "' opening error.");
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0, std::ios::beg);
    std::string s(n > 0 ? (size_t)n : 0, '\0');
    if (n > 0) f.read(&s[0], n);
    return s;
}

// f(begin, end) over [0, n) split into contiguous ranges, one per host thread (up to 16);
// the first exception (in range order) is rethrown after all threads joined.
template <typename F>
void parallel_ranges(size_t n, size_t min_per_thread, F&& f) {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    nt = (unsigned)std::max<size_t>(1, std::min<size_t>(nt, n / std::max<size_t>(1, min_per_thread)));
    if (nt <= 1) { f(size_t(0), n); return; }
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err(nt);
    const size_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        const size_t a = std::min(n, t * chunk), b = std::min(n, a + chunk);
        th.emplace_back([&, t, a, b] {
            try { f(a, b); } catch (...) { err[t] = std::current_exception(); }
        });
    }
    for (auto& x : th) x.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f' || c == '\n'; }

// Up to n integers from the start of the line [s, e) (sscanf("%d %d ...") / strtol
// semantics: optional sign, decimal digits, stop at the first non-number).
int scan_ints(const char* s, const char* e, int* out, int n) {
    int k = 0;
    while (k < n) {
        while (s < e && is_space(*s)) s++;
        const char* p = s;
        bool neg = false;
        if (p < e && (*p == '+' || *p == '-')) { neg = *p == '-'; p++; }
        if (p >= e || *p < '0' || *p > '9') break;
        long v = 0;
        while (p < e && *p >= '0' && *p <= '9') { v = v * 10 + (*p - '0'); p++; }
        out[k++] = (int)(neg ? -v : v);
        s = p;
    }
    return k;
}

// Up to n doubles from the line [s, e), each read by strtod.
int scan_doubles(const char* s, const char* e, double* out, int n) {
    int k = 0;
    while (k < n) {
        while (s < e && is_space(*s)) s++;
        if (s >= e) break;
        char* end;
        const double v = std::strtod(s, &end);
        if (end == s) break;
        out[k++] = v;
        s = end;
    }
    return k;
}

// The first whitespace-delimited token of [s, e), at most 255 characters (sscanf "%255s").
std::string first_token(const char* s, const char* e) {
    while (s < e && is_space(*s)) s++;
    const char* p = s;
    while (p < e && !is_space(*p) && p - s < 255) p++;
    return std::string(s, p);
}

// The UNV text cut into lines with the block delimiters removed: content line k is
// [text + start[k], text + start[k] + len[k]) (a trailing '\r' dropped), and block
// b is content lines [block[b], block[b + 1]).
struct UnvLines {
    const char* text = nullptr;
    std::vector<uint64_t> start;
    std::vector<uint32_t> len;
    std::vector<size_t> block;
    const char* s(size_t k) const { return text + start[k]; }
    const char* e(size_t k) const { return text + start[k] + len[k]; }
};

// A line whose first "-1" ends it is a block delimiter; every second one closes a
// block (read_block, src/mesh/MeshReaderSalomeUnv.cpp:267-286). The text is split into
// chunks at line starts, scanned in parallel and stitched in order.
UnvLines split_unv(const std::string& text) {
    UnvLines L;
    L.text = text.data();
    const char* T = text.data();
    const size_t N = text.size();
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (N < (1u << 20)) nt = 1;
    std::vector<size_t> cut(nt + 1, N);
    cut[0] = 0;
    for (unsigned t = 1; t < nt; t++) {
        size_t p = std::max(cut[t - 1], t * (N / nt));
        const void* q = p < N ? std::memchr(T + p, '\n', N - p) : nullptr;
        cut[t] = q ? (size_t)((const char*)q - T) + 1 : N;
    }
    cut[nt] = N + 1;  // the (possibly empty) line after the last newline belongs to the last chunk
    struct Part { std::vector<uint64_t> start; std::vector<uint32_t> len; std::vector<size_t> delim; };
    std::vector<Part> parts(nt);
    auto scan = [&](unsigned t) {
        Part& P = parts[t];
        size_t p = cut[t];
        const size_t stop = cut[t + 1];
        while (p < stop && p <= N) {
            const void* q = p < N ? std::memchr(T + p, '\n', N - p) : nullptr;
            const size_t nl = q ? (size_t)((const char*)q - T) : N;
            size_t e = nl;
            if (e > p && T[e - 1] == '\r') e--;
            size_t m = e;  // first "-1"
            for (size_t i = p; i + 1 < e; i++)
                if (T[i] == '-' && T[i + 1] == '1') { m = i; break; }
            if (m != e && m + 2 == e) {
                P.delim.push_back(P.start.size());
            } else {
                P.start.push_back(p);
                P.len.push_back((uint32_t)(e - p));
            }
            if (nl >= N) break;
            p = nl + 1;
        }
    };
    if (nt == 1) scan(0);
    else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; t++) th.emplace_back(scan, t);
        for (auto& x : th) x.join();
    }
    size_t total = 0;
    for (auto& P : parts) total += P.start.size();
    L.start.reserve(total);
    L.len.reserve(total);
    std::vector<size_t> delim;
    for (auto& P : parts) {
        const size_t base = L.start.size();
        for (size_t d : P.delim) delim.push_back(base + d);
        L.start.insert(L.start.end(), P.start.begin(), P.start.end());
        L.len.insert(L.len.end(), P.len.begin(), P.len.end());
        std::vector<uint64_t>().swap(P.start);
        std::vector<uint32_t>().swap(P.len);
    }
    L.block.push_back(0);
    for (size_t d = 1; d < delim.size(); d += 2) L.block.push_back(delim[d]);
    if (L.block.back() < L.start.size()) L.block.push_back(L.start.size());
    return L;
}

}  // namespace

// ---------------------------------------------------------------- UNV

RawMesh read_unv(const std::string& path) {
    const std::string text = slurp(path);
    const UnvLines L = split_unv(text);

    RawMesh m;
    m.names.push_back(std::string());
    struct Elem { int kind = 0; int index = -1; };   // 41 cell, 11 edge element
    std::vector<Elem> elements;
    std::vector<int> edge_label;                    // per UNV edge element: label-1
    std::map<std::string, std::vector<int>> groups; // name -> element labels-1 (sorted by name, like std::map)
    for (size_t bi = 0; bi + 1 < L.block.size(); bi++) {
        const size_t b0 = L.block[bi], b1 = L.block[bi + 1], size = b1 - b0;
        if (size == 0) continue;
        int id = 0;
        scan_ints(L.s(b0), L.e(b0), &id, 1);
        if (id == 2411) {
            if ((size - 1) % 2 != 0) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2411: truncated node record");
            const size_t nrec = (size - 1) / 2, base = m.xy.size();
            m.xy.resize(base + 2 * nrec);
            parallel_ranges(nrec, 1 << 16, [&](size_t a, size_t b) {
                for (size_t r = a; r < b; r++) {
                    double c[3] = {0, 0, 0};
                    const size_t k = b0 + 2 + 2 * r;
                    scan_doubles(L.s(k), L.e(k), c, 3);
                    m.xy[base + 2 * r] = c[0];
                    m.xy[base + 2 * r + 1] = c[1];
                }
            });
        } else if (id == 2412) {
            // record starts and kinds in order (header line: label, type, ...), then the
            // records parsed in parallel into their places
            std::vector<size_t> rec;
            std::vector<char> is_tri;
            size_t k = b0 + 1;
            while (k < b1) {
                int h[2] = {0, 0};
                scan_ints(L.s(k), L.e(k), h, 2);
                const int type = h[1];
                rec.push_back(k);
                k++;
                if (type == 11) {
                    if (k + 1 >= b1) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: truncated edge record");
                    is_tri.push_back(0);
                    k += 2;
                } else if (type == 41) {
                    if (k >= b1) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: truncated triangle record");
                    is_tri.push_back(1);
                    k += 1;
                } else {
                    throw Error(CFD2D_ERR_MESH_UNV_UNKNOWN_ELEMENT, "Unknown element type '" + std::to_string(type) + "'.");
                }
            }
            const size_t nrec = rec.size();
            std::vector<int> slot(nrec);  // index among the block's triangles / edge elements
            size_t ntri = 0, nedge = 0;
            for (size_t r = 0; r < nrec; r++) slot[r] = is_tri[r] ? (int)ntri++ : (int)nedge++;
            const size_t tri0 = m.tri.size() / 3, seg0 = m.bseg.size() / 2, lab0 = edge_label.size();
            m.tri.resize(3 * (tri0 + ntri));
            m.bseg.resize(2 * (seg0 + nedge));
            edge_label.resize(lab0 + nedge);
            std::vector<int> tri_label(ntri);
            parallel_ranges(nrec, 1 << 15, [&](size_t a, size_t b) {
                for (size_t r = a; r < b; r++) {
                    int h[6] = {0, 0, 0, 0, 0, 0};
                    const size_t q = rec[r];
                    scan_ints(L.s(q), L.e(q), h, 6);
                    const int label = h[0] - 1;
                    if (is_tri[r]) {
                        int nd[3] = {0, 0, 0};
                        scan_ints(L.s(q + 1), L.e(q + 1), nd, 3);
                        const size_t t = tri0 + slot[r];
                        for (int j = 0; j < 3; j++) m.tri[3 * t + j] = nd[j] - 1;
                        tri_label[slot[r]] = label;
                    } else {
                        int nd[2] = {0, 0};
                        scan_ints(L.s(q + 2), L.e(q + 2), nd, 2);
                        const size_t s2 = seg0 + slot[r];
                        m.bseg[2 * s2] = nd[0] - 1;
                        m.bseg[2 * s2 + 1] = nd[1] - 1;
                        edge_label[lab0 + slot[r]] = label;
                    }
                }
            });
            for (size_t t = 0; t < ntri; t++) {
                const int label = tri_label[t];
                if (label < 0) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2412: bad element label");
                if ((int)elements.size() <= label) elements.resize(label + 1);
                elements[label].kind = 41;
                elements[label].index = (int)(tri0 + t);
            }
        } else if (id == 2467) {
            size_t k = b0 + 1;
            while (k < b1) {
                int h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                scan_ints(L.s(k), L.e(k), h, 8);
                const int n = h[7];
                k++;
                if (k >= b1) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2467: truncated group");
                const std::string name = first_token(L.s(k), L.e(k));
                k++;
                const size_t pairs = n > 0 ? (size_t)(n / 2) : 0, odd = n > 0 ? (size_t)(n % 2) : 0;
                if (k + pairs + odd > b1) throw Error(CFD2D_ERR_MESH_FORMAT, "UNV block 2467: truncated group entities");
                std::vector<int> ids(2 * pairs + odd);
                parallel_ranges(pairs, 1 << 15, [&](size_t a, size_t b) {
                    for (size_t j = a; j < b; j++) {
                        int e[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                        scan_ints(L.s(k + j), L.e(k + j), e, 8);
                        ids[2 * j] = e[1] - 1;
                        ids[2 * j + 1] = e[5] - 1;
                    }
                });
                k += pairs;
                if (odd) {
                    int e[4] = {0, 0, 0, 0};
                    scan_ints(L.s(k), L.e(k), e, 4);
                    ids[2 * pairs] = e[1] - 1;
                    k++;
                }
                groups[name] = std::move(ids);
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
    m.cell_name.assign(nc, 0);
    m.bseg_name.assign(nb, 0);
    for (auto& g : groups) {
        const int gi = (int)m.names.size();
        m.names.push_back(g.first);
        for (int id : g.second) {
            if (id < 0 || id >= (int)elements.size()) continue;
            const Elem& el = elements[id];
            if (el.kind == 41) m.cell_name[el.index] = gi;
            else if (el.kind == 11) m.bseg_name[el.index] = gi;
        }
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
    m.names.push_back(std::string());
    std::map<std::string, int> name_id;
    for (int i = 0; i < nc; i++) {  // "%d %d %d %d %d": index, nodes, attribute
        for (int j = 0; j < 3; j++) m.tri.push_back(std::atoi(at(ele, 3 + 5 * i + 1 + j).c_str()) - 1);
        const std::string nm = std::to_string(std::atoi(at(ele, 3 + 5 * i + 4).c_str()));
        auto it = name_id.find(nm);
        if (it == name_id.end()) {
            it = name_id.emplace(nm, (int)m.names.size()).first;
            m.names.push_back(nm);
        }
        m.cell_name.push_back(it->second);
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
        parallel_ranges((size_t)nc, 1 << 15, [&](size_t i0, size_t i1) {
            for (int i = (int)i0; i < (int)i1; i++)
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
        });
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
    // edge numbers, cells and nodes in the reference's order (sequential) ...
    int e = 0;
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            int p = neigh[3 * i + j];
            if (p == -1) continue;
            if (p < -2 || p >= nc) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: bad neighbour index");
            const int* v = tri + 3 * i;
            t.n1[e] = berk ? v[(j + 1) % 3] : v[j];
            t.n2[e] = berk ? v[(j + 2) % 3] : v[(j + 1) % 3];
            t.c1[e] = i;
            t.cedges[3 * i + cfi[i]++] = e;
            if (p > -1) {
                t.c2[e] = p;
                if (cfi[p] >= 3) throw Error(CFD2D_ERR_MESH_FORMAT, "mesh: a cell has more than three edges");
                t.cedges[3 * p + cfi[p]++] = e;
            } else {
                t.c2[e] = -1;
            }
            e++;
        }
    // ... then each edge's points, normal, length and boundary segment (independent, threaded)
    std::vector<int> missing(std::max(1u, std::min(16u, std::thread::hardware_concurrency())) + 1, ne);
    std::atomic<int> slot{0};
    parallel_ranges((size_t)ne, 1 << 15, [&](size_t e0, size_t e1) {
        int first_missing = ne;
        for (int q = (int)e0; q < (int)e1; q++) {
            const int a = t.n1[q], b = t.n2[q], i = t.c1[q];
            double x1 = xy[2 * a], y1 = xy[2 * a + 1], x2 = xy[2 * b], y2 = xy[2 * b + 1];
            double* P = &t.pts[6 * (size_t)q];
            P[0] = (x1 + x2) / 2.0;  // midpoint, then Gauss points at -+1/sqrt(3) of the half length
            P[1] = (y1 + y2) / 2.0;
            if (npts == 3) {
                P[2] = (x1 + x2) / 2.0 - sq3 * (x2 - x1) / 2.0;
                P[3] = (y1 + y2) / 2.0 - sq3 * (y2 - y1) / 2.0;
                P[4] = (x1 + x2) / 2.0 + sq3 * (x2 - x1) / 2.0;
                P[5] = (y1 + y2) / 2.0 + sq3 * (y2 - y1) / 2.0;
            }
            t.npts[q] = npts;
            double nx = y2 - y1, ny = x1 - x2;
            double l = std::sqrt(nx * nx + ny * ny);
            nx /= l; ny /= l;
            t.l[q] = l;
            if (!berk) {  // turn the normal outward from c1 (:181-187)
                double vx = t.cx[i] - P[0], vy = t.cy[i] - P[1];
                if (vx * nx + vy * ny > 0) { nx *= -1; ny *= -1; }
            }
            t.nx[q] = nx; t.ny[q] = ny;
            if (t.c2[q] < 0) {
                long long key = std::min<long long>(a, b) * (1ll << 32) + std::max<long long>(a, b);
                auto it = std::lower_bound(keys.begin(), keys.end(), std::make_pair(key, -1));
                if (it != keys.end() && it->first == key) t.bseg_of_edge[q] = it->second;
                else if (first_missing == ne) first_missing = q;
            }
        }
        missing[slot++ % missing.size()] = first_missing;  // one slot per thread
    });
    const int first_missing = *std::min_element(missing.begin(), missing.end());
    if (require_segment && first_missing < ne)
        throw Error(CFD2D_ERR_MESH_UNV_NOT_DEFINED_BND_EDGE,
                    "Boundary edge #" + std::to_string(first_missing) + " not defined in UNV file.");
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
            auto before = [&](int x, int y) { return deg[x] != deg[y] ? deg[x] < deg[y] : x < y; };
            for (int a = 1; a < m; a++)  // at most three: insertion sort
                for (int b = a; b > 0 && before(nb[b], nb[b - 1]); b--) std::swap(nb[b], nb[b - 1]);
            for (int k = 0; k < m; k++) order.push_back(nb[k]);
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// Cells along a Hilbert curve through their centroids (quantised to a 2^16 x 2^16
// grid over the bounding box; ties by cell number): consecutive cells form compact
// patches, which the tiled kernels need. The curve index follows the standard
// quadrant-rotation construction (Hilbert 1891; e.g. Butz 1971).
std::vector<int> hilbert_order(const Topo& t) {
    const int nc = t.nc;
    double x0 = 0, x1 = 0, y0 = 0, y1 = 0;
    for (int i = 0; i < nc; i++) {
        if (i == 0 || t.cx[i] < x0) x0 = t.cx[i];
        if (i == 0 || t.cx[i] > x1) x1 = t.cx[i];
        if (i == 0 || t.cy[i] < y0) y0 = t.cy[i];
        if (i == 0 || t.cy[i] > y1) y1 = t.cy[i];
    }
    const double span = std::max(std::max(x1 - x0, y1 - y0), 1e-300);
    const uint32_t n = 1u << 16;
    std::vector<std::pair<uint64_t, int>> key(nc);
    parallel_ranges((size_t)nc, 1 << 16, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; i++) {
            uint32_t x = (uint32_t)std::min<double>(n - 1, std::floor((t.cx[i] - x0) / span * n));
            uint32_t y = (uint32_t)std::min<double>(n - 1, std::floor((t.cy[i] - y0) / span * n));
            uint64_t d = 0;
            for (uint32_t q = n / 2; q > 0; q /= 2) {
                const uint32_t rx = (x & q) ? 1u : 0u, ry = (y & q) ? 1u : 0u;
                d += (uint64_t)q * q * ((3u * rx) ^ ry);
                if (ry == 0) {  // rotate the quadrant so the sub-curve joins its neighbours
                    if (rx == 1) { x = n - 1 - x; y = n - 1 - y; }
                    std::swap(x, y);
                }
            }
            key[i] = {d, (int)i};
        }
    });
    std::sort(key.begin(), key.end());
    std::vector<int> order(nc);
    for (int i = 0; i < nc; i++) order[i] = key[i].second;
    return order;
}

Layout make_layout(const Topo& t, const std::vector<int>& cell_mat, const std::vector<int>& edge_bnd, int order) {
    Layout L;
    const int nc = t.nc, ne = t.ne;
    L.nc = nc; L.ne = ne;
    if (order == ORDER_RCM) L.perm = rcm_order(t);
    else if (order == ORDER_HILBERT) L.perm = hilbert_order(t);
    else { L.perm.resize(nc); std::iota(L.perm.begin(), L.perm.end(), 0); }
    L.iperm.resize(nc);
    for (int i = 0; i < nc; i++) L.iperm[L.perm[i]] = i;
    // edges: interior ones by (lower, upper) storage cell, then boundary ones by cell
    // (ties between a cell's boundary edges by edge number): a counting sort by the
    // lower / boundary cell, each cell's few interior edges then ordered by the upper one
    std::vector<int> cnt(nc + 1, 0), bcnt(nc + 1, 0);
    int n_int = 0;
    for (int e = 0; e < ne; e++) {
        const int a = L.iperm[t.c1[e]];
        if (t.c2[e] >= 0) { cnt[std::min(a, L.iperm[t.c2[e]]) + 1]++; n_int++; }
        else bcnt[a + 1]++;
    }
    for (int i = 0; i < nc; i++) { cnt[i + 1] += cnt[i]; bcnt[i + 1] += bcnt[i]; }
    L.n_int = n_int;
    L.eorig.resize(ne);
    {
        std::vector<int> fill(cnt.begin(), cnt.end() - 1), bfill(bcnt.begin(), bcnt.end() - 1);
        for (int e = 0; e < ne; e++) {  // ascending e: stable within a bucket
            const int a = L.iperm[t.c1[e]];
            if (t.c2[e] >= 0) L.eorig[fill[std::min(a, L.iperm[t.c2[e]])]++] = e;
            else L.eorig[n_int + bfill[a]++] = e;
        }
        parallel_ranges((size_t)nc, 1 << 16, [&](size_t i0, size_t i1) {
            for (size_t i = i0; i < i1; i++) {  // order a bucket's interior edges by the upper cell
                int* b = L.eorig.data() + cnt[i];
                const int m = cnt[i + 1] - cnt[i];
                auto hi = [&](int e) { return std::max(L.iperm[t.c1[e]], L.iperm[t.c2[e]]); };
                for (int x = 1; x < m; x++)
                    for (int y = x; y > 0 && hi(b[y - 1]) > hi(b[y]); y--) std::swap(b[y - 1], b[y]);
            }
        });
    }
    std::vector<int> enew(ne);
    for (int k = 0; k < ne; k++) enew[L.eorig[k]] = k;
    L.ec1.resize(ne); L.ec2.resize(ne); L.ebnd.resize(ne);
    L.nx.resize(ne); L.ny.resize(ne); L.l.resize(ne); L.dl.assign(8 * (size_t)ne, 0.0);
    parallel_ranges((size_t)ne, 1 << 16, [&](size_t k0, size_t k1) {
        for (size_t k = k0; k < k1; k++) {
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
    });
    L.face.resize(3 * (size_t)nc);
    L.rem_nb.resize(3 * (size_t)nc);
    L.S.resize(nc);
    L.cmat.resize(nc);
    parallel_ranges((size_t)nc, 1 << 16, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; i++) {
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
    });
    return L;
}

}  // namespace cfd2d
