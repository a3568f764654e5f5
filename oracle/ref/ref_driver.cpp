/*
 * Oracle harness around the reference's own FVM_TVD (test infrastructure only;
 * nothing in the product links or runs this).
 *
 * It drives the unmodified reference sources exactly as src/main.cpp:10-39 does
 * (Parallel::init, hLog, FVM_TVD::init(xml), FVM_TVD::run), and adds three
 * harness-only things the reference has no interface for:
 *   - zero the Cell::flag words after init (src/mesh/grid.h:35 leaves them
 *     uninitialised for the UNV reader, which makes the limiter flag test in
 *     src/methods/fvm_tvd.cpp:368 read indeterminate memory);
 *   - optionally overwrite the initial conserved state with a per-cell binary
 *     field (the reference XML can only express uniform regions,
 *     src/methods/fvm_tvd.cpp:71-95,199-204) and redo calcTimeStep() from the
 *     XML TAU, as FVM_TVD::init does (src/methods/fvm_tvd.cpp:211);
 *   - dump the Grid and the final state as flat binary arrays.
 *
 * Usage: ref_fvm_tvd <task.xml> <out_prefix> [init_state.bin]
 * Run it with the working directory holding the mesh file (the reference opens
 * the mesh by the relative name in <mesh><name>).
 *
 * Compiled with -Dprivate=public -Dprotected=public for this translation unit
 * only, so the harness can read FVM_TVD's state arrays without editing the
 * reference headers.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <chrono>
#include "fvm_tvd.h"
#include "tinyxml.h"

static void wr(FILE* f, const void* p, size_t bytes) {
    if (bytes && fwrite(p, 1, bytes, f) != bytes) { fprintf(stderr, "write failed\n"); exit(3); }
}

static void dump_grid(FVM_TVD& m, const char* path) {
    Grid& g = m.grid;
    FILE* f = fopen(path, "wb");
    if (!f) { perror(path); exit(3); }
    int hdr[4] = { g.cCount, g.eCount, g.nCount, 0 };
    wr(f, hdr, sizeof hdr);
    std::vector<double> d; std::vector<int> iv;
    for (int i = 0; i < g.nCount; i++) { d.push_back(g.nodes[i].x); d.push_back(g.nodes[i].y); }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int i = 0; i < g.cCount; i++) for (int k = 0; k < 3; k++) iv.push_back(g.cells[i].nodesInd[k]);
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int i = 0; i < g.cCount; i++) for (int k = 0; k < 3; k++) iv.push_back(g.cells[i].edgesInd[k]);
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int i = 0; i < g.cCount; i++) d.push_back(g.cells[i].S);
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int i = 0; i < g.cCount; i++) { d.push_back(g.cells[i].c.x); d.push_back(g.cells[i].c.y); }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int e = 0; e < g.eCount; e++) { iv.push_back(g.edges[e].n1); iv.push_back(g.edges[e].n2); }
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) { iv.push_back(g.edges[e].c1); iv.push_back(g.edges[e].c2); }
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) iv.push_back(g.edges[e].type);
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) {
        int b = -1;
        for (size_t k = 0; k < m.boundaries.size(); k++) if (m.boundaries[k] == g.edges[e].bnd) b = (int)k;
        iv.push_back(b);
    }
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) iv.push_back(g.edges[e].cCount);
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) { d.push_back(g.edges[e].n.x); d.push_back(g.edges[e].n.y); }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int e = 0; e < g.eCount; e++) d.push_back(g.edges[e].l);
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int e = 0; e < g.eCount; e++)
        for (int k = 0; k < 3; k++) {
            if (k < g.edges[e].cCount) { d.push_back(g.edges[e].c[k].x); d.push_back(g.edges[e].c[k].y); }
            else { d.push_back(0.0); d.push_back(0.0); }
        }
    wr(f, d.data(), d.size() * 8); d.clear();
    fclose(f);
}

static void dump_state(FVM_TVD& m, const char* path, double run_seconds) {
    int nc = m.grid.cCount;
    FILE* f = fopen(path, "wb");
    if (!f) { perror(path); exit(3); }
    int hdr[4] = { nc, 0, 0, 0 };
    wr(f, hdr, sizeof hdr);
    double scal[2] = { m.TAU, run_seconds };
    wr(f, scal, sizeof scal);
    wr(f, m.ro, nc * 8); wr(f, m.ru, nc * 8); wr(f, m.rv, nc * 8); wr(f, m.re, nc * 8);
    wr(f, m.cTau, nc * 8);
    std::vector<unsigned> fl(nc);
    for (int i = 0; i < nc; i++) fl[i] = m.grid.cells[i].flag;
    wr(f, fl.data(), nc * 4);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s task.xml out_prefix [init_state.bin]\n", argv[0]); return 2; }
    Parallel::init(&argc, &argv);
    hLog = fopen("task.log", "w");
    FVM_TVD m;
    m.init(argv[1]);
    for (int i = 0; i < m.grid.cCount; i++) m.grid.cells[i].flag = 0;
    if (argc > 3) {
        int nc = m.grid.cCount;
        FILE* f = fopen(argv[3], "rb");
        if (!f) { perror(argv[3]); return 3; }
        std::vector<double> u(4 * (size_t)nc);
        if (fread(u.data(), 8, u.size(), f) != u.size()) { fprintf(stderr, "short init file\n"); return 3; }
        fclose(f);
        for (int i = 0; i < nc; i++) {
            m.ro[i] = m.ro_old[i] = u[i];
            m.ru[i] = m.ru_old[i] = u[nc + i];
            m.rv[i] = m.rv_old[i] = u[2 * nc + i];
            m.re[i] = m.re_old[i] = u[3 * nc + i];
        }
        // TAU back to the XML value, then the reference's own CFL pass.
        TiXmlDocument doc(argv[1]);
        doc.LoadFile(TIXML_ENCODING_UTF8);
        doc.FirstChild("task")->FirstChild("control")->FirstChild("TAU")->ToElement()->Attribute("value", &m.TAU);
        m.calcTimeStep();
    }
    std::string p(argv[2]);
    dump_grid(m, (p + ".grid.bin").c_str());
    dump_state(m, (p + ".init.bin").c_str(), 0.0);
    auto t0 = std::chrono::steady_clock::now();
    m.run();
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    dump_state(m, (p + ".state.bin").c_str(), secs);
    fprintf(stderr, "ref_fvm_tvd: cells=%d steps_max=%d run_seconds=%.6f\n", m.grid.cCount, m.STEP_MAX, secs);
    fclose(hLog);
    Parallel::done();
    return 0;
}
