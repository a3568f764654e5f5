/*
 * Oracle harness around the reference's own FEM_RKDG (test infrastructure only;
 * nothing in the product links or runs this).
 *
 * The reference method cannot run as written: FEM_RKDG::getF(int, Point)
 * (src/methods/fem_rkdg.cpp:1441-1465) returns a reference to a local VECTOR, a
 * dangling reference that GCC compiles as a null one. The recipe compiles
 * fem_rkdg.cpp at -O0 (so every call goes through the symbol, none is inlined)
 * and weakens that one symbol; this file defines the function with the same body
 * returning a reference that stays valid until the caller has used it (every
 * caller reads or copies the vector at once). Everything else is the reference's
 * code, unmodified, apart from the log() every harness here replaces (below).
 *
 * It drives the method as src/main.cpp:10-39 does (Parallel::init, hLog,
 * FEM_RKDG::init, which reads mesh/mesh.0000.proc from the working directory and
 * writes the step-0 VTU files), then
 *   - optionally overwrites the coefficients with a per-cell binary field
 *     (ro[3] ru[3] rv[3] re[3] per cell; the XML can only express uniform regions)
 *     and redoes calcTimeStep() from the XML TAU, as init does;
 *   - optionally overrides the time step (the reference's calcTimeStep reads past
 *     the edge Gauss-point array with two points per edge, :397-403);
 *   - unsteady: sets TMAX to the time of the requested step and calls run();
 *     steady (run() never ends: t stays 0): calls the members in run()'s order
 *     (:609-647) for the requested number of steps;
 *   - dumps geometry, quadrature, mass-matrix inverses, the initial and final
 *     coefficients, cTau and the residuals as flat binary arrays.
 *
 * Usage: ref_fem_rkdg <task.xml> <out_prefix> <steps> [init_coeffs.bin|-] [tau]
 * Compiled with -Dprivate=public -Dprotected=public for this translation unit only.
 */
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <sys/stat.h>
#include "fem_rkdg.h"
#include "tinyxml.h"

VECTOR& FEM_RKDG::getF(int iCell, Point pt) {
    static VECTOR ring[16];
    static int k = 0;
    k = (k + 1) & 15;
    VECTOR& v = ring[k];
    if (FUNC_COUNT != 3) {
        fprintf(stderr, "ref_fem_rkdg: BASE_FUNC_COUNT %d: inverseMatr (src/global.cpp:444-470) inverts 3x3 only\n",
                FUNC_COUNT);
        exit(4);
    }
    if (v.n != 3) v.init(3);
    v[0] = 1.0;
    v[1] = (pt.x - grid.cells[iCell].c.x) / grid.cells[iCell].HX;
    v[2] = (pt.y - grid.cells[iCell].c.y) / grid.cells[iCell].HY;
    return v;
}

// The reference's log() (src/global.cpp:32-46) reads its va_list twice, which crashes
// on the first "%s" argument (save() logs its file names); the recipe links a copy of
// global.o whose log is weak, and this one copies the va_list.
void log(char* format, ...) {
    if (!Parallel::isRoot()) return;
    va_list a, b;
    va_start(a, format);
    va_copy(b, a);
    vprintf(format, a);
    if (hLog) vfprintf(hLog, format, b);
    va_end(b);
    va_end(a);
    fflush(stdout);
    if (hLog) fflush(hLog);
}

static void wr(FILE* f, const void* p, size_t bytes) {
    if (bytes && fwrite(p, 1, bytes, f) != bytes) { fprintf(stderr, "write failed\n"); exit(3); }
}

static void dump_geom(FEM_RKDG& m, const char* path) {
    Grid& g = m.grid;
    FILE* f = fopen(path, "wb");
    if (!f) { perror(path); exit(3); }
    int hdr[8] = { g.cCount, g.eCount, g.nCount, m.GP_CELL_COUNT, m.GP_EDGE_COUNT, m.FUNC_COUNT, 0, 0 };
    wr(f, hdr, sizeof hdr);
    std::vector<double> d; std::vector<int> iv;
    for (int i = 0; i < g.cCount; i++) for (int k = 0; k < 3; k++) iv.push_back(g.cells[i].edgesInd[k]);
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int e = 0; e < g.eCount; e++) { iv.push_back(g.edges[e].c1); iv.push_back(g.edges[e].c2); }
    wr(f, iv.data(), iv.size() * 4); iv.clear();
    for (int i = 0; i < g.cCount; i++) {
        d.push_back(g.cells[i].c.x); d.push_back(g.cells[i].c.y);
        d.push_back(g.cells[i].HX); d.push_back(g.cells[i].HY); d.push_back(g.cells[i].S);
        d.push_back(m.cellJ[i]);
    }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int i = 0; i < g.cCount; i++)
        for (int k = 0; k < m.GP_CELL_COUNT; k++) {
            d.push_back(m.cellGP[i][k].x); d.push_back(m.cellGP[i][k].y); d.push_back(m.cellGW[i][k]);
        }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int i = 0; i < g.cCount; i++)
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) d.push_back(m.matrInvA[i][r][c]);
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int e = 0; e < g.eCount; e++) {
        d.push_back(g.edges[e].n.x); d.push_back(g.edges[e].n.y); d.push_back(g.edges[e].l); d.push_back(m.edgeJ[e]);
    }
    wr(f, d.data(), d.size() * 8); d.clear();
    for (int e = 0; e < g.eCount; e++)
        for (int k = 0; k < m.GP_EDGE_COUNT; k++) {
            d.push_back(m.edgeGP[e][k].x); d.push_back(m.edgeGP[e][k].y); d.push_back(m.edgeGW[e][k]);
        }
    wr(f, d.data(), d.size() * 8); d.clear();
    fclose(f);
}

static void dump_state(FEM_RKDG& m, const char* path) {
    int nc = m.grid.cCount;
    FILE* f = fopen(path, "wb");
    if (!f) { perror(path); exit(3); }
    int hdr[4] = { nc, 0, 0, 0 };
    wr(f, hdr, sizeof hdr);
    double scal[6] = { m.TAU, m.TMAX, m.ro_res, m.ru_res, m.rv_res, m.re_res };
    wr(f, scal, sizeof scal);
    VECTOR* fld[4] = { m.ro, m.ru, m.rv, m.re };
    std::vector<double> d;
    for (int i = 0; i < nc; i++)
        for (int v = 0; v < 4; v++) for (int k = 0; k < 3; k++) d.push_back(fld[v][i][k]);
    wr(f, d.data(), d.size() * 8);
    wr(f, m.cTau, nc * 8);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s task.xml out_prefix steps [init_coeffs.bin|-] [tau]\n", argv[0]);
        return 2;
    }
    Parallel::init(&argc, &argv);
    hLog = fopen("task.log", "w");
    mkdir("vtk_data", 0755);
    const int steps = atoi(argv[3]);
    FEM_RKDG m;
    m.init(argv[1]);
    const int nc = m.grid.cCount;
    if (argc > 4 && strcmp(argv[4], "-") != 0) {
        FILE* f = fopen(argv[4], "rb");
        if (!f) { perror(argv[4]); return 3; }
        std::vector<double> u(12 * (size_t)nc);
        if (fread(u.data(), 8, u.size(), f) != u.size()) { fprintf(stderr, "short init file\n"); return 3; }
        fclose(f);
        VECTOR* fld[4] = { m.ro, m.ru, m.rv, m.re };
        for (int i = 0; i < nc; i++)
            for (int v = 0; v < 4; v++) for (int k = 0; k < 3; k++) fld[v][i][k] = u[12 * (size_t)i + 3 * v + k];
        TiXmlDocument doc(argv[1]);
        doc.LoadFile(TIXML_ENCODING_UTF8);
        doc.FirstChild("task")->FirstChild("control")->FirstChild("TAU")->ToElement()->Attribute("value", &m.TAU);
        m.calcTimeStep();
    }
    if (argc > 5) {
        m.TAU = atof(argv[5]);
        for (int i = 0; i < nc; i++) m.cTau[i] = m.TAU;
    }
    std::string p(argv[2]);
    dump_geom(m, (p + ".geom.bin").c_str());
    dump_state(m, (p + ".init.bin").c_str());
    if (!m.STEADY) {
        double t = 0.0;
        for (int s = 0; s < steps; s++) t += m.TAU;
        m.TMAX = t;
        if (steps > 0) m.run();
    } else {
        for (int s = 0; s < steps; s++) {
            m.calcTimeStep();
            m.copyToOld();
            m.zeroIntegrals(); m.calcLimiters(); m.procExchangeData();
            m.calcConvectionVol(); m.calcConvectionSurf(); m.calcNewFields(); m.procExchangeData();
            m.zeroIntegrals(); m.calcLimiters(); m.procExchangeData();
            m.calcConvectionVol(); m.calcConvectionSurf(); m.calcNewFields2(); m.procExchangeData();
            m.calcResiduals();
        }
    }
    dump_state(m, (p + ".state.bin").c_str());
    fprintf(stderr, "ref_fem_rkdg: cells=%d steps=%d TAU=%.17g\n", nc, steps, m.TAU);
    fclose(hLog);
    Parallel::done();
    return 0;
}
