/*
 * Oracle harness around the reference's own FVM_TVD_IMPLICIT (test infrastructure
 * only; nothing in the product links or runs this).
 *
 * It drives the unmodified src/methods/fvm_tvd_implicit.cpp the way src/main.cpp
 * does (Parallel::init, hLog, init(xml), run). The reference solves its block
 * system with HYPRE's GMRES (src/methods/solvers/SolverHypreGmres.cpp), and HYPRE
 * is not part of the reference tree, so this harness supplies the matrix solver:
 *   - MatrixSolver's base methods (declared in src/methods/solvers/MatrixSolver.h,
 *     defined by the reference in MatrixSolver.cpp together with the HYPRE
 *     solvers) and MatrixSolver::create, which returns a solver that stores the
 *     4x4 blocks the reference adds (diagonal per cell, one block per face) and
 *     solves with the oracle's GMRES (orc_gmres_block in ../cfd2d_oracle.c);
 *   - optionally a per-cell initial state (the reference's XML can only express
 *     uniform regions) and a dump of the final state, cTau, flags and CFL.
 * Everything else (gradients, Roe averages, eigen-decompositions, A+/A-, fluxes,
 * smoothing, update, limits, remediation, CFL control) is the reference's code.
 *
 * Usage: ref_fvm_tvd_implicit <task.xml> <out_prefix> [init_state.bin]
 * Run it with the working directory holding the mesh files.
 *
 * Compiled with -Dprivate=public -Dprotected=public for this translation unit
 * only, so the harness can read the method's arrays without editing its headers.
 */
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fvm_tvd_implicit.h"
#include "tinyxml.h"

extern "C" {
#include "cfd2d_oracle.h"
}

static Grid* g_grid = nullptr;  // the grid whose cells are the block rows
static int g_iters = 0;         // the last solve's iterations and relative residual
static double g_rel = 0.0;

// ---- MatrixSolver's own methods (src/methods/solvers/MatrixSolver.h:24-45); the
// harness solver below overrides the ones the implicit method calls.
void MatrixSolver::init(int cellsCount, int blockDimension) {
    blockDim = blockDimension;
    a = nullptr;
    b = new double[(size_t)cellsCount * blockDim]();
    x = new double[(size_t)cellsCount * blockDim]();
}
void MatrixSolver::zero() {}
MatrixSolver::~MatrixSolver() {
    delete[] b;
    delete[] x;
}
void MatrixSolver::setMatrElement(int, int, double**) { fprintf(stderr, "setMatrElement unused\n"); exit(4); }
void MatrixSolver::setRightElement(int, double*) {}
void MatrixSolver::addMatrElement(int, int, double**) {}
void MatrixSolver::addRightElement(int, double*) { fprintf(stderr, "addRightElement unused\n"); exit(4); }
void MatrixSolver::createMatrElement(int, int) {}
void MatrixSolver::initCSR() {}
void MatrixSolver::printToFile(const char*) {}

class HarnessSolver : public MatrixSolver {
public:
    int nc = 0;
    std::vector<double> diag, off;
    std::vector<int> nbr;
    void init(int cellsCount, int blockDimension) override {
        MatrixSolver::init(cellsCount, blockDimension);
        nc = cellsCount;
        diag.assign(16 * (size_t)nc, 0.0);
        off.assign(48 * (size_t)nc, 0.0);
        nbr.assign(3 * (size_t)nc, -1);
        for (int c = 0; c < nc; c++)
            for (int k = 0; k < 3; k++) {
                const Edge& e = g_grid->edges[g_grid->cells[c].edgesInd[k]];
                nbr[3 * c + k] = e.c1 == c ? e.c2 : e.c1;
            }
    }
    void zero() override {
        std::fill(diag.begin(), diag.end(), 0.0);
        std::fill(off.begin(), off.end(), 0.0);
        memset(b, 0, sizeof(double) * 4 * (size_t)nc);
        memset(x, 0, sizeof(double) * 4 * (size_t)nc);
    }
    double* block(int i, int j) {
        if (i == j) return &diag[16 * (size_t)i];
        for (int k = 0; k < 3; k++)
            if (nbr[3 * i + k] == j) return &off[48 * (size_t)i + 16 * k];
        fprintf(stderr, "block (%d, %d) outside the face structure\n", i, j);
        exit(4);
    }
    void addMatrElement(int i, int j, double** m) override {
        double* p = block(i, j);
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) p[4 * r + c] += m[r][c];
    }
    void setRightElement(int i, double* v) override {
        for (int k = 0; k < 4; k++) b[4 * (size_t)i + k] = v[k];
    }
    void createMatrElement(int, int) override {}
    int solve(double eps, int& maxIter) override {
        int st = orc_gmres_block(nc, nbr.data(), diag.data(), off.data(), b, x, eps, maxIter, 30, &g_iters, &g_rel);
        maxIter = g_iters;
        return st;
    }
    char* getName() override { return (char*)"HARNESS_GMRES"; }
};

MatrixSolver* MatrixSolver::create(const char*) { return new HarnessSolver(); }

// The reference's log (src/global.cpp:32-46) passes one va_list to vprintf and then
// to vfprintf; the second read of a "%s" argument crashes. The same output, with
// the list copied for the second print (the build makes the reference's copy weak).
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

static void dump_state(FVM_TVD_IMPLICIT& m, const char* path, double run_seconds) {
    int nc = m.grid.cCount;
    FILE* f = fopen(path, "wb");
    if (!f) { perror(path); exit(3); }
    int hdr[4] = { nc, g_iters, 0, 0 };
    wr(f, hdr, sizeof hdr);
    double scal[4] = { m.TAU, run_seconds, m.CFL, g_rel };
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
    FVM_TVD_IMPLICIT m;
    m.init(argv[1]);
    g_grid = &m.grid;
    for (int i = 0; i < m.grid.cCount; i++) m.grid.cells[i].flag = 0;
    if (argc > 3) {
        int nc = m.grid.cCount;
        FILE* f = fopen(argv[3], "rb");
        if (!f) { perror(argv[3]); return 3; }
        std::vector<double> u(4 * (size_t)nc);
        if (fread(u.data(), 8, u.size(), f) != u.size()) { fprintf(stderr, "short init file\n"); return 3; }
        fclose(f);
        for (int i = 0; i < nc; i++) {
            m.ro[i] = u[i];
            m.ru[i] = u[nc + i];
            m.rv[i] = u[2 * nc + i];
            m.re[i] = u[3 * nc + i];
        }
    }
    std::string p(argv[2]);
    dump_state(m, (p + ".init.bin").c_str(), 0.0);
    auto t0 = std::chrono::steady_clock::now();
    m.run();
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    dump_state(m, (p + ".state.bin").c_str(), secs);
    fprintf(stderr, "ref_fvm_tvd_implicit: cells=%d steps_max=%d run_seconds=%.6f\n", m.grid.cCount, m.STEP_MAX,
            secs);
    fclose(hLog);
    Parallel::done();
    return 0;
}
