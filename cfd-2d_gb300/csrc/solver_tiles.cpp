// Tiles for the mixed form's fused stage kernel (<FUSED_STAGE value="1"/>): each tile
// owns a run of storage cells (compact when the cells are in Hilbert order) and lists
// its two-ring halo, the edges of its own cells and, per gradient cell, its faces in
// local numbering. Measured on the 2,097,152-triangle four-quadrant case the fused
// stage runs at 0.645 ms/step against 0.61 ms for the per-kernel path (its gradient,
// flux and update phases serialise on barriers and wait on geometry and state
// loads with only a few resident tiles per SM; fetching the next tile's primitives
// during the current tile did not change that), so it is opt-in.
#include <algorithm>
#include <thread>
#include <vector>

#include "cfd2d.h"
#include "solver.hpp"

namespace cfd2d {

namespace {
constexpr int kTile = 256;                       // own cells per tile (= threads per CTA)
constexpr size_t kMaxSmem = 200 * 1024;          // shared-memory bytes a tile may use
constexpr int kNone = 0xffff;

struct TileLists {
    std::vector<int> halo;      // H1 then H2
    int nh1 = 0;
    std::vector<int2> tedge, gface;
};
}  // namespace

void Solver::build_tiles() {
    fused_ = 0;
    // the mixed form's default (FUSED_STAGE absent) for a single instance: gradients formed in
    // the flux kernel (0.554 against 0.574 ms per step of the 2.1M-triangle four-quadrant case);
    // a batch keeps the per-kernel path, whose launch shapes the autotuner sets (256 uneven
    // instances, Roe: 6.8 against 8.5 ms per step)
    const int want = task_.fused < 0 ? (inst_.empty() ? 3 : 0) : task_.fused;
    if (task_.precision == PREC_MIXED && want == 3 && gauss_points_ != 0 && task_.recon != RECON_NONE) {
        fused_ = 3;  // gradients formed in the flux kernel: no tiles
        return;
    }
    const bool applies = task_.precision == PREC_MIXED && (task_.fused == 1 || task_.fused == 2) && gauss_points_ != 0 &&
                         (task_.scheme == TIME_SSPRK3 || task_.scheme == TIME_HEUN);
    if (!applies) return;
    const int mode = task_.fused;
    const int nc = dc_.nc;
    const int nt = (nc + kTile - 1) / kTile;
    const Layout& L = lay_;
    auto nbr = [&](int i, int k) {
        const int f = L.face[(size_t)k * nc + i], e = f >> 1;
        return (f & 1) ? L.ec1[e] : L.ec2[e];
    };
    std::vector<TileLists> tl(nt);
    std::vector<char> ok(nt, 1);
    auto build = [&](int t) {
        TileLists& T = tl[t];
        const int o0 = t * kTile, o1 = std::min(nc, o0 + kTile), n_own = o1 - o0;
        auto own = [&](int j) { return j >= o0 && j < o1; };
        std::vector<int> h1, h2, edges;
        for (int i = o0; i < o1; i++)
            for (int k = 0; k < 3; k++) {
                const int j = nbr(i, k);
                if (j >= 0 && !own(j)) h1.push_back(j);
                edges.push_back(L.face[(size_t)k * nc + i] >> 1);
            }
        std::sort(h1.begin(), h1.end());
        h1.erase(std::unique(h1.begin(), h1.end()), h1.end());
        auto in = [](const std::vector<int>& v, int j) { return std::binary_search(v.begin(), v.end(), j); };
        for (int i : h1)
            for (int k = 0; k < 3; k++) {
                const int j = nbr(i, k);
                if (j >= 0 && !own(j) && !in(h1, j)) h2.push_back(j);
            }
        std::sort(h2.begin(), h2.end());
        h2.erase(std::unique(h2.begin(), h2.end()), h2.end());
        std::sort(edges.begin(), edges.end());
        edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
        const int nh1 = (int)h1.size(), nL = n_own + nh1 + (int)h2.size();
        if (nL >= kNone || (int)edges.size() >= kNone) { ok[t] = 0; return; }
        auto local = [&](int j) -> int {
            if (j < 0) return kNone;
            if (own(j)) return j - o0;
            auto a = std::lower_bound(h1.begin(), h1.end(), j);
            if (a != h1.end() && *a == j) return n_own + (int)(a - h1.begin());
            auto b = std::lower_bound(h2.begin(), h2.end(), j);
            if (b != h2.end() && *b == j) return n_own + nh1 + (int)(b - h2.begin());
            return -1;
        };
        auto ledge = [&](int e) { return (int)(std::lower_bound(edges.begin(), edges.end(), e) - edges.begin()); };
        T.nh1 = nh1;
        T.halo = h1;
        T.halo.insert(T.halo.end(), h2.begin(), h2.end());
        for (int e : edges) {
            const int a = local(L.ec1[e]), b = local(L.ec2[e]);
            if (a < 0 || b < 0 || a == kNone) { ok[t] = 0; return; }
            T.tedge.push_back(make_int2(e, a | (b << 16)));
        }
        for (int q = 0; q < n_own + nh1; q++) {
            const int i = q < n_own ? o0 + q : h1[q - n_own];
            for (int k = 0; k < 3; k++) {
                const int f = L.face[(size_t)k * nc + i];
                const int nb = local(nbr(i, k));
                if (nb < 0) { ok[t] = 0; return; }
                const int le = q < n_own ? ledge(f >> 1) : kNone;
                T.gface.push_back(make_int2(f, nb | (le << 16)));
            }
        }
    };
    {
        const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (unsigned w = 0; w < nth; w++)
            th.emplace_back([&, w] {
                for (int t = (int)w; t < nt; t += (int)nth) build(t);
            });
        for (auto& x : th) x.join();
    }
    for (char c : ok)
        if (!c) return;  // a tile too large for 16-bit local numbers: stay with the per-kernel path
    std::vector<int> halo_off(nt + 1, 0), edge_off(nt + 1, 0), gface_off(nt + 1, 0), n_h1(nt);
    int max_cells = 0, max_grad = 0, max_edges = 0;
    for (int t = 0; t < nt; t++) {
        const int n_own = std::min(nc, (t + 1) * kTile) - t * kTile;
        halo_off[t + 1] = halo_off[t] + (int)tl[t].halo.size();
        edge_off[t + 1] = edge_off[t] + (int)tl[t].tedge.size();
        gface_off[t + 1] = gface_off[t] + n_own + tl[t].nh1;
        n_h1[t] = tl[t].nh1;
        max_cells = std::max(max_cells, n_own + (int)tl[t].halo.size());
        max_grad = std::max(max_grad, n_own + tl[t].nh1);
        max_edges = std::max(max_edges, (int)tl[t].tedge.size());
    }
    const size_t smem = mode == 1 ? 16 * (2 * (size_t)max_cells + 2 * (size_t)max_grad + (size_t)max_edges)
                                  : 16 * (size_t)max_edges;  // flux-and-update: the tile's edge fluxes only
    if (smem > kMaxSmem) return;
    std::vector<int> halo;
    std::vector<int2> tedge, gface;
    halo.reserve(halo_off[nt]);
    tedge.reserve(edge_off[nt]);
    gface.reserve(3 * (size_t)gface_off[nt]);
    for (auto& T : tl) {
        halo.insert(halo.end(), T.halo.begin(), T.halo.end());
        tedge.insert(tedge.end(), T.tedge.begin(), T.tedge.end());
        gface.insert(gface.end(), T.gface.begin(), T.gface.end());
        std::vector<int>().swap(T.halo);
        std::vector<int2>().swap(T.tedge);
        std::vector<int2>().swap(T.gface);
    }
    DevTiles d;
    d.n_tiles = nt;
    d.tile = kTile;
    d.max_cells = max_cells;
    d.max_grad = max_grad;
    d.max_edges = max_edges;
    d.halo_off = upload(halo_off);
    d.halo = upload(halo.empty() ? std::vector<int>{0} : halo);
    d.n_h1 = upload(n_h1);
    d.edge_off = upload(edge_off);
    d.tedge = upload(tedge);
    d.gface_off = upload(gface_off);
    d.gface = upload(gface);
    tiles_ = d;
    const int nst = task_.scheme == TIME_SSPRK3 ? 3 : 2;
    wrot_[0] = dc_.W32;
    for (int k = 1; k < nst; k++) wrot_[k] = dalloc<float>(4 * (size_t)nc);
    fused_ = mode;
}

}  // namespace cfd2d
