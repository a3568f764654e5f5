// Mesh input (the reference's mesh plugins), edge topology and device layout.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace cfd2d {

// Error carrying one of the reference's Exception/EXIT codes (src/global.h:241-248)
// or a library code (include/cfd2d.h).
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A mesh as read from its files, before it is bound to a task.
struct RawMesh {
    std::vector<double> xy;               // 2*nn
    std::vector<int> tri;                 // 3*nc, 0-based node numbers
    std::vector<std::string> names;       // distinct group / region names; names[0] == ""
    std::vector<int> cell_name;           // region name of each cell, an index into names (0: in no group)
    bool berkeley = false;
    std::vector<int> neigh;               // Berkeley-Triangle .neigh, 0-based, -2 = none
    std::vector<int> bseg;                // 2*nb boundary segments (UNV edge elements / .poly segments)
    std::vector<int> bseg_name;           // UNV: group name of the segment, an index into names (0: none)
    std::vector<int> bseg_marker;         // Berkeley: .poly boundary marker
    int nn() const { return (int)xy.size() / 2; }
    int nc() const { return (int)tri.size() / 3; }
};

// Salome UNV reader, blocks 2411/2412/2467 (src/mesh/MeshReaderSalomeUnv.cpp:25-447).
RawMesh read_unv(const std::string& path);
// Berkeley Triangle reader, .node/.ele/.neigh/.poly (src/mesh/MeshReaderBerkleyTriangle.cpp:3-170).
RawMesh read_triangle(const std::string& base);

// Edge structure in the reference's numbering (src/mesh/grid.h:18-100).
struct Topo {
    int nn = 0, nc = 0, ne = 0;
    std::vector<double> xy;
    std::vector<int> tri;
    std::vector<int> cedges;              // 3*nc, ascending edge numbers (Cell::edgesInd)
    std::vector<double> S, cx, cy;
    std::vector<int> n1, n2, c1, c2, npts;
    std::vector<int> bseg_of_edge;        // boundary edges: the first matching segment, or -1
    std::vector<double> nx, ny, l;
    std::vector<double> pts;              // 6*ne: midpoint and the two Gauss points
};

// Neighbours and edges by the UNV reader's rules (node-pair intersection, normals
// turned outward from c1, 3 points per edge) or, with neigh_berkeley, by the
// Triangle reader's rules (neighbour j opposite node j, 1 point per edge unless
// gauss_points == 2). Throws Error(222) for a boundary edge with no segment when
// require_segment is set.
Topo build_topology(int nn, const double* xy, int nc, const int* tri, const int* neigh_berkeley,
                    int nb, const int* bseg, bool require_segment, int gauss_points);

// Storage layout for the device (see kernels.hpp for the array meanings).
struct Layout {
    int nc = 0, ne = 0, n_int = 0;
    std::vector<int> perm, iperm;         // storage cell -> original, original -> storage
    std::vector<int> eorig;               // storage edge -> original edge
    std::vector<int> face;                // 3*nc
    std::vector<int> ec1, ec2, ebnd;      // ne
    std::vector<double> nx, ny, l, dl;    // ne, dl 8*ne
    std::vector<double> S;                // nc
    std::vector<int> rem_nb;              // 3*nc
    std::vector<uint8_t> cmat;            // nc
};

// Reverse Cuthill-McKee order of the cell graph (storage -> original).
std::vector<int> rcm_order(const Topo& t);
// Hilbert-curve order of the cell centroids (storage -> original).
std::vector<int> hilbert_order(const Topo& t);
enum CellOrder { ORDER_NONE = 0, ORDER_RCM = 1, ORDER_HILBERT = 2 };
Layout make_layout(const Topo& t, const std::vector<int>& cell_mat, const std::vector<int>& edge_bnd, int order);

}  // namespace cfd2d
