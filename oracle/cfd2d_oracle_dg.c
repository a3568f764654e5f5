/*
 * CPU restatement of the reference's explicit discontinuous Galerkin method FEM_RKDG
 * (src/methods/fem_rkdg.cpp) -- TEST INFRASTRUCTURE ONLY. The GPU library never links,
 * loads or calls this file; the tests, the smoke check and the CPU baseline of the
 * benchmark use it to check the GPU results against. Compiled with -ffp-contract=off so every product
 * and sum rounds on its own, as in the reference's build.
 *
 * Scope: P1 basis (BASE_FUNC_COUNT 3: 1, (x-xc)/HX, (y-yc)/HY, :1441-1452), cell
 * quadrature of 3 or 4 points and edge quadrature of 2 or 3 points (calcGaussPar,
 * :470-598), mass matrices and their 3x3 cofactor inverses (calcMassMatr :449-468,
 * inverseMatr src/global.cpp:444-470), the volume and surface integrals (:1124-1210,
 * :995-1122), GODUNOV and LAX fluxes (:918-960), the boundary ghost states
 * (:1324-1343, src/bnd_cond.cpp:75-110), the two Runge-Kutta stages (:609-627,
 * :1216-1284), residuals (:1286-1319) and the time step (:382-447).
 *
 * Two things of the reference are undefined and are restated by their evident intent:
 * getF returns a dangling reference (:1441-1465): here the basis vector itself; and
 * calcTimeStep reads edgeGP[edge][slot] with the edge's slot in the cell (0..2) as the
 * Gauss-point index (:397-403), past the array when an edge has two points: such a
 * slot is skipped here (ORC_DG_RK_REFERENCE) -- the harness pins those runs with a
 * given time step.
 *
 * ORC_DG_RK_REFERENCE (the reference as written, defined behaviour kept):
 *  - init copies cCountEx doubles' worth of VECTOR objects from ro into ro_old
 *    (memcpy, :369-372), so ro_old[i] shares ro[i]'s coefficients for the first
 *    ceil(nc/2) cells (a VECTOR is a pointer and an int, 16 bytes) for the whole run;
 *  - the second stage's zeroIntegrals copies the first stage's result into ro_old
 *    (:962-979), so calcNewFields2 averages with that result, not with U^n: U^{n+1} =
 *    ((U1 + dU(U1)) + U1) / 2, and for the shared cells ((U1 + dU) + (U1 + dU)) / 2;
 *  - residuals compare with ro_old after the step (0 for the shared cells).
 * ORC_DG_RK_HEUN (the evident intent): U^{n+1} = ((U1 + dU(U1)) + U^n) / 2, residuals
 * against U^n, every Gauss point of every edge in the time step.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cfd2d_oracle.h"

#define DG_GR 8.314472 /* Material::gR, src/global.cpp:6 */

struct orc_dg {
    orc_dg_params p;
    int nn, nc, ne, nreg, nbnd, gc, ge;
    double* xy;
    int *tri, *creg, *en, *ebnd, *cedge, *c1, *c2;
    double *cx, *cy, *HX, *HY, *S, *cellJ;
    double *cgp, *cgw;     /* 2*gc per cell, gc per cell */
    double *enx, *eny, *el, *edgeJ;
    double *egp, *egw;     /* 2*ge per edge, ge per edge */
    double* invA;          /* 9 per cell */
    double* reg;           /* 6 per region: M Cp u v T p */
    int* bkind;
    double* bpar;          /* 4 per boundary: u v T p */
    double *U, *Uold, *Uint; /* 12 per cell: ro[3] ru[3] rv[3] re[3] */
    int n_alias;           /* cells whose ro_old is ro (reference mode) */
    double* ctau;
    double TAU, t, res[4];
    int step;
    unsigned err;
};

typedef struct { double r, u, v, E, e, p, cz, T; } dg_par;

static double mat_M(const orc_dg* d, int cell) { return d->reg[6 * d->creg[cell] + 0]; }
static double mat_Cp(const orc_dg* d, int cell) { return d->reg[6 * d->creg[cell] + 1]; }

/* Material::URS, src/global.cpp:9-30 */
static void urs(double M, double Cp, dg_par* par, int flag) {
    double Cv = Cp - DG_GR / M;
    double gam = Cp / Cv;
    switch (flag) {
    case 0: par->p = par->r * par->e * (gam - 1); par->cz = sqrt(gam * par->p / par->r); break;
    case 1: par->e = par->p / (par->r * (gam - 1)); par->T = par->e / Cv; break;
    case 2: par->r = par->p * M / (par->T * DG_GR); par->cz = sqrt(gam * par->p / par->r); break;
    }
}

/* getF (:1441-1452, its intent): the P1 basis of a cell at a point */
static void basis(const orc_dg* d, int cell, double x, double y, double F[3]) {
    F[0] = 1.0;
    F[1] = (x - d->cx[cell]) / d->HX[cell];
    F[2] = (y - d->cy[cell]) / d->HY[cell];
}

/* VECTOR::SCALAR_PROD, src/global.h:128-135 */
static double sprod(const double* a, const double F[3]) {
    double s = 0;
    for (int i = 0; i < 3; i++) s += a[i] * F[i];
    return s;
}

/* convertConsToPar (:1420-1430) at a point */
static void cons2par(const orc_dg* d, const double* Uc, int cell, double x, double y, dg_par* par) {
    double F[3];
    basis(d, cell, x, y, F);
    par->r = sprod(Uc, F);
    par->u = sprod(Uc + 3, F) / par->r;
    par->v = sprod(Uc + 6, F) / par->r;
    par->E = sprod(Uc + 9, F) / par->r;
    par->e = par->E - 0.5 * (par->u * par->u + par->v * par->v);
    urs(mat_M(d, cell), mat_Cp(d, cell), par, 0);
    urs(mat_M(d, cell), mat_Cp(d, cell), par, 1);
}

/* calcTimeStep, :382-447 */
static void dg_time_step(orc_dg* d) {
    const double* U = d->U;
    double tau = 1.0e+20;
    for (int i = 0; i < d->nc; i++) {
        dg_par p;
        double Uv, maxU = 0.0;
        for (int g = 0; g < d->gc; g++) {
            cons2par(d, U + 12 * (size_t)i, i, d->cgp[2 * (d->gc * (size_t)i + g)], d->cgp[2 * (d->gc * (size_t)i + g) + 1], &p);
            Uv = sqrt(p.u * p.u + p.v * p.v) + p.cz;
            if (maxU < Uv) maxU = Uv;
        }
        for (int k = 0; k < 3; k++) {
            int e = d->cedge[3 * i + k];
            for (int g = 0; g < d->ge; g++) {
                int gp = g;
                if (d->p.rk_mode == ORC_DG_RK_REFERENCE) {
                    if (k >= d->ge) break; /* past the edge's points in the reference */
                    gp = k;
                }
                cons2par(d, U + 12 * (size_t)i, i, d->egp[2 * (d->ge * (size_t)e + gp)],
                         d->egp[2 * (d->ge * (size_t)e + gp) + 1], &p);
                Uv = sqrt(p.u * p.u + p.v * p.v) + p.cz;
                if (maxU < Uv) maxU = Uv;
            }
        }
        cons2par(d, U + 12 * (size_t)i, i, d->cx[i], d->cy[i], &p);
        Uv = sqrt(p.u * p.u + p.v * p.v) + p.cz;
        if (maxU < Uv) maxU = Uv;
        if (!d->p.steady) {
            double tmp = d->S[i] / maxU;
            if (tmp < tau) tau = tmp;
        } else {
            d->ctau[i] = d->p.cfl * d->S[i] / maxU;
        }
    }
    if (!d->p.steady) {
        tau *= d->p.cfl;
        d->TAU = d->TAU < tau ? d->TAU : tau; /* _min_, src/mesh/grid.h:107 */
        for (int i = 0; i < d->nc; i++) d->ctau[i] = d->TAU;
    }
}

/* calcFlux, :918-960 */
static int dg_flux(const orc_dg* d, double f[4], const dg_par* L, const dg_par* R, double nx, double ny, double GAM) {
    int hit = 0;
    if (d->p.flux == ORC_FLUX_GODUNOV) {
        double RI, EI, PI, UN, UT;
        double unl = L->u * nx + L->v * ny;
        double unr = R->u * nx + R->v * ny;
        double utl = L->u * ny - L->v * nx;
        double utr = R->u * ny - R->v * nx;
        hit = orc_riemann_exact(&RI, &EI, &PI, &UN, &UT, L->r, L->p, unl, utl, R->r, R->p, unr, utr, GAM,
                                d->p.newton_cap);
        double UI = UN * nx + UT * ny;
        double VI = UN * ny - UT * nx;
        f[0] = RI * UN;
        f[1] = f[0] * UI + PI * nx;
        f[2] = f[0] * VI + PI * ny;
        f[3] = (RI * (EI + 0.5 * (UI * UI + VI * VI)) + PI) * UN;
    } else {
        double unl = L->u * nx + L->v * ny;
        double unr = R->u * nx + R->v * ny;
        double al = fabs(unl) + sqrt(GAM * L->p / L->r), ar = fabs(unr) + sqrt(GAM * R->p / R->r);
        double alpha = al > ar ? al : ar; /* _max_, src/mesh/grid.h:102 */
        double rol = L->r, rul = L->r * L->u, rvl = L->r * L->v;
        double rel = L->p / (GAM - 1.0) + 0.5 * L->r * (L->u * L->u + L->v * L->v);
        double ror = R->r, rur = R->r * R->u, rvr = R->r * R->v;
        double rer = R->p / (GAM - 1.0) + 0.5 * R->r * (R->u * R->u + R->v * R->v);
        double frl = rol * unl, frr = ror * unr;
        f[0] = 0.5 * (frr + frl - alpha * (ror - rol));
        f[1] = 0.5 * (frr * R->u + frl * L->u + (R->p + L->p) * nx - alpha * (rur - rul));
        f[2] = 0.5 * (frr * R->v + frl * L->v + (R->p + L->p) * ny - alpha * (rvr - rvl));
        f[3] = 0.5 * ((rer + R->p) * unr + (rel + L->p) * unl - alpha * (rer - rel));
    }
    return hit;
}

/* boundaryCond (:1324-1343): CFDBnd*::run, then URS(2), URS(1) for the ghost */
static void dg_ghost(const orc_dg* d, int e, const dg_par* L, dg_par* R) {
    int b = d->ebnd[e], c1 = d->c1[e];
    const double* bp = d->bpar + 4 * b;
    if (d->bkind[b] == ORC_BND_INLET) {
        memset(R, 0, sizeof *R);
        R->u = bp[0]; R->v = bp[1]; R->T = bp[2]; R->p = bp[3];
    } else if (d->bkind[b] == ORC_BND_OUTLET) {
        *R = *L;
    } else { /* BOUND_WALL_SLIP; BOUND_WALL_NO_SLIP constructs the slip class (src/bnd_cond.cpp:50-55) */
        *R = *L;
        double Un = L->u * d->enx[e] + L->v * d->eny[e];
        double Vx = d->enx[e] * Un * 2.0, Vy = d->eny[e] * Un * 2.0;
        R->u = L->u - Vx;
        R->v = L->v - Vy;
    }
    urs(mat_M(d, c1), mat_Cp(d, c1), R, 2);
    urs(mat_M(d, c1), mat_Cp(d, c1), R, 1);
    R->E = R->e + 0.5 * (R->u * R->u + R->v * R->v);
}

/* zeroIntegrals + calcConvectionVol + calcConvectionSurf: Uint from the coefficients Ucur */
static void dg_integrals(orc_dg* d, const double* Ucur) {
    const int gc = d->gc, ge = d->ge;
    memset(d->Uint, 0, sizeof(double) * 12 * (size_t)d->nc);
    for (int i = 0; i < d->nc; i++) { /* calcConvectionVol, :1124-1210 */
        double in[4][3] = {{0}};
        const double* Uc = Ucur + 12 * (size_t)i;
        for (int g = 0; g < gc; g++) {
            double x = d->cgp[2 * (gc * (size_t)i + g)], y = d->cgp[2 * (gc * (size_t)i + g) + 1];
            dg_par par;
            cons2par(d, Uc, i, x, y, &par);
            double fr = par.r * par.u;
            double fu = fr * par.u + par.p;
            double fv = fr * par.v;
            double fe = par.u * (par.r * par.E + par.p);
            double gr = par.r * par.v;
            double gu = gr * par.u;
            double gv = gr * par.v + par.p;
            double ge_ = par.v * (par.r * par.E + par.p);
            const double fx[4] = {fr, fu, fv, fe}, gy[4] = {gr, gu, gv, ge_};
            const double dfdx[3] = {0.0, 1.0 / d->HX[i], 0.0}, dfdy[3] = {0.0, 0.0, 1.0 / d->HY[i]};
            for (int v = 0; v < 4; v++) {
                double tmp[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < 3; k++) tmp[k] += dfdx[k] * fx[v];
                for (int k = 0; k < 3; k++) tmp[k] += dfdy[k] * gy[v];
                for (int k = 0; k < 3; k++) tmp[k] *= d->cgw[gc * (size_t)i + g];
                for (int k = 0; k < 3; k++) in[v][k] += tmp[k];
            }
        }
        for (int v = 0; v < 4; v++)
            for (int k = 0; k < 3; k++) {
                in[v][k] *= d->cellJ[i];
                d->Uint[12 * (size_t)i + 3 * v + k] += in[v][k];
            }
    }
    for (int e = 0; e < d->ne; e++) { /* calcConvectionSurf, :995-1122 */
        int c1 = d->c1[e], c2 = d->c2[e];
        double i1[4][3] = {{0}}, i2[4][3] = {{0}};
        double GAM = mat_Cp(d, c1) / (mat_Cp(d, c1) - DG_GR / mat_M(d, c1)); /* getGamma, src/global.h:219 */
        for (int g = 0; g < ge; g++) {
            double x = d->egp[2 * (ge * (size_t)e + g)], y = d->egp[2 * (ge * (size_t)e + g) + 1];
            double w = d->egw[ge * (size_t)e + g];
            dg_par L, R;
            double f[4], F1[3], F2[3];
            cons2par(d, Ucur + 12 * (size_t)c1, c1, x, y, &L);
            if (c2 >= 0) cons2par(d, Ucur + 12 * (size_t)c2, c2, x, y, &R);
            else dg_ghost(d, e, &L, &R);
            if (dg_flux(d, f, &L, &R, d->enx[e], d->eny[e], GAM)) d->err |= ORC_ERR_NEWTON_CAP;
            basis(d, c1, x, y, F1);
            for (int k = 0; k < 3; k++) F1[k] *= w;
            for (int v = 0; v < 4; v++)
                for (int k = 0; k < 3; k++) i1[v][k] += F1[k] * f[v];
            if (c2 >= 0) {
                basis(d, c2, x, y, F2);
                for (int k = 0; k < 3; k++) F2[k] *= w;
                for (int v = 0; v < 4; v++)
                    for (int k = 0; k < 3; k++) i2[v][k] += F2[k] * f[v];
            }
        }
        for (int v = 0; v < 4; v++)
            for (int k = 0; k < 3; k++) {
                i1[v][k] *= d->edgeJ[e];
                d->Uint[12 * (size_t)c1 + 3 * v + k] -= i1[v][k];
                if (c2 >= 0) {
                    i2[v][k] *= d->edgeJ[e];
                    d->Uint[12 * (size_t)c2 + 3 * v + k] += i2[v][k];
                }
            }
    }
}

/* calcNewFields (:1216-1242): U += cTau * invA * Uint, per variable */
static void dg_new_fields(orc_dg* d, double* U) {
    for (int i = 0; i < d->nc; i++) {
        const double* A = d->invA + 9 * (size_t)i;
        for (int v = 0; v < 4; v++) {
            const double* t = d->Uint + 12 * (size_t)i + 3 * v;
            double tmp[3];
            for (int r = 0; r < 3; r++) {
                tmp[r] = 0.0;
                for (int c = 0; c < 3; c++) tmp[r] += A[3 * r + c] * t[c];
            }
            for (int r = 0; r < 3; r++) tmp[r] *= d->ctau[i];
            for (int r = 0; r < 3; r++) U[12 * (size_t)i + 3 * v + r] += tmp[r];
        }
    }
}

static void dg_one_step(orc_dg* d) {
    const size_t n12 = 12 * (size_t)d->nc;
    if (!d->p.steady) d->t += d->TAU;
    else dg_time_step(d);
    d->step++;
    memcpy(d->Uold, d->U, n12 * sizeof(double)); /* copyToOld */
    dg_integrals(d, d->U);                        /* stage 1 */
    dg_new_fields(d, d->U);
    if (d->p.rk_mode == ORC_DG_RK_REFERENCE) memcpy(d->Uold, d->U, n12 * sizeof(double)); /* zeroIntegrals */
    dg_integrals(d, d->U);                        /* stage 2 */
    dg_new_fields(d, d->U);
    for (int i = 0; i < d->nc; i++) {             /* calcNewFields2's average */
        const int shared = d->p.rk_mode == ORC_DG_RK_REFERENCE && i < d->n_alias;
        for (int k = 0; k < 12; k++) {
            double* u = d->U + 12 * (size_t)i + k;
            const double o = shared ? *u : d->Uold[12 * (size_t)i + k];
            *u += o;
            *u *= 0.5;
        }
    }
    for (int v = 0; v < 4; v++) d->res[v] = 0.0;  /* calcResiduals, :1286-1319 */
    for (int i = 0; i < d->nc; i++) {
        const int shared = d->p.rk_mode == ORC_DG_RK_REFERENCE && i < d->n_alias;
        for (int v = 0; v < 4; v++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) {
                const double u = d->U[12 * (size_t)i + 3 * v + k];
                const double x = fabs(u - (shared ? u : d->Uold[12 * (size_t)i + 3 * v + k]));
                s += x * x;
            }
            const double res = sqrt(s);
            if (res > d->res[v]) d->res[v] = res;
        }
    }
    if (d->p.rk_mode == ORC_DG_RK_REFERENCE) /* ro_old of the shared cells is ro */
        for (int i = 0; i < d->n_alias; i++) memcpy(d->Uold + 12 * (size_t)i, d->U + 12 * (size_t)i, 12 * sizeof(double));
}

orc_dg* orc_dg_create(const orc_dg_params* p, int nn, const double* xy, int nc, const int* tri,
                      const int* cell_region, int ne, const int* en, const int* ebnd, int nreg, const double* reg,
                      int nbnd, const int* bkind, const double* bpar) {
    if (p->gp_cell != 3 && p->gp_cell != 4) return NULL;
    if (p->gp_edge != 2 && p->gp_edge != 3) return NULL;
    orc_dg* d = (orc_dg*)calloc(1, sizeof *d);
    d->p = *p;
    d->nn = nn; d->nc = nc; d->ne = ne; d->nreg = nreg; d->nbnd = nbnd;
    d->gc = p->gp_cell; d->ge = p->gp_edge;
#define DUP(dst, src, n, T) do { dst = (T*)malloc(sizeof(T) * (size_t)(n) + 1); memcpy(dst, src, sizeof(T) * (size_t)(n)); } while (0)
#define NEW(dst, n, T) dst = (T*)calloc((size_t)(n) + 1, sizeof(T))
    DUP(d->xy, xy, 2 * nn, double);
    DUP(d->tri, tri, 3 * nc, int);
    DUP(d->creg, cell_region, nc, int);
    DUP(d->en, en, 2 * ne, int);
    DUP(d->ebnd, ebnd, ne, int);
    DUP(d->reg, reg, 6 * nreg, double);
    DUP(d->bkind, bkind, nbnd, int);
    DUP(d->bpar, bpar, 4 * nbnd, double);
    NEW(d->cedge, 3 * nc, int); NEW(d->c1, ne, int); NEW(d->c2, ne, int);
    NEW(d->cx, nc, double); NEW(d->cy, nc, double); NEW(d->HX, nc, double); NEW(d->HY, nc, double);
    NEW(d->S, nc, double); NEW(d->cellJ, nc, double);
    NEW(d->cgp, 2 * d->gc * nc, double); NEW(d->cgw, d->gc * nc, double);
    NEW(d->enx, ne, double); NEW(d->eny, ne, double); NEW(d->el, ne, double); NEW(d->edgeJ, ne, double);
    NEW(d->egp, 2 * d->ge * ne, double); NEW(d->egw, d->ge * ne, double);
    NEW(d->invA, 9 * nc, double);
    NEW(d->U, 12 * nc, double); NEW(d->Uold, 12 * nc, double); NEW(d->Uint, 12 * nc, double);
    NEW(d->ctau, nc, double);
#undef DUP
#undef NEW
    /* Grid::readMeshFiles (src/mesh/grid.cpp:275-420): centres, HX/HY, edges of each
       cell by node pair, c1/c2 in cell order, normals turned away from c1, Heron areas */
    for (int i = 0; i < nc; i++) {
        const int* t = tri + 3 * i;
        double x0 = xy[2 * t[0]], x1 = xy[2 * t[1]], x2 = xy[2 * t[2]];
        double y0 = xy[2 * t[0] + 1], y1 = xy[2 * t[1] + 1], y2 = xy[2 * t[2] + 1];
        d->cx[i] = (x0 + x1 + x2) / 3.0;
        d->cy[i] = (y0 + y1 + y2) / 3.0;
        double a = fabs(x0 - x1), b = fabs(x1 - x2), c = fabs(x0 - x2);
        double bc = b > c ? b : c;
        d->HX[i] = a > bc ? a : bc;
        a = fabs(y0 - y1); b = fabs(y1 - y2); c = fabs(y0 - y2);
        bc = b > c ? b : c;
        d->HY[i] = a > bc ? a : bc;
    }
    /* edge lookup by node pair: sort (min, max, edge) keys */
    long long* key = (long long*)malloc(sizeof(long long) * (size_t)ne + 8);
    int* ord = (int*)malloc(sizeof(int) * (size_t)ne + 4);
    for (int e = 0; e < ne; e++) {
        long long a = en[2 * e], b = en[2 * e + 1];
        key[e] = (a < b ? a : b) * (1ll << 31) + (a < b ? b : a);
        ord[e] = e;
    }
    /* simple heap sort of ord by key (test sizes) */
    for (int start = ne / 2 - 1; start >= -0 && ne > 1; start--) {
        int r = start;
        for (;;) {
            int ch = 2 * r + 1;
            if (ch >= ne) break;
            if (ch + 1 < ne && key[ord[ch + 1]] > key[ord[ch]]) ch++;
            if (key[ord[r]] >= key[ord[ch]]) break;
            int tmp = ord[r]; ord[r] = ord[ch]; ord[ch] = tmp; r = ch;
        }
        if (start == 0) break;
    }
    for (int end = ne - 1; end > 0; end--) {
        int tmp = ord[0]; ord[0] = ord[end]; ord[end] = tmp;
        int r = 0;
        for (;;) {
            int ch = 2 * r + 1;
            if (ch >= end) break;
            if (ch + 1 < end && key[ord[ch + 1]] > key[ord[ch]]) ch++;
            if (key[ord[r]] >= key[ord[ch]]) break;
            tmp = ord[r]; ord[r] = ord[ch]; ord[ch] = tmp; r = ch;
        }
    }
    int* ncell = (int*)calloc((size_t)ne + 1, sizeof(int));
    for (int e = 0; e < ne; e++) { d->c1[e] = -1; d->c2[e] = -1; }
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            long long a = tri[3 * i + j], b = tri[3 * i + (j + 1) % 3];
            long long k = (a < b ? a : b) * (1ll << 31) + (a < b ? b : a);
            int lo = 0, hi = ne - 1, found = -1;
            while (lo <= hi) {
                int mid = (lo + hi) / 2;
                if (key[ord[mid]] < k) lo = mid + 1;
                else if (key[ord[mid]] > k) hi = mid - 1;
                else { found = ord[mid]; break; }
            }
            if (found < 0) { free(key); free(ord); free(ncell); orc_dg_free(d); return NULL; }
            d->cedge[3 * i + j] = found;
            if (ncell[found] == 0) d->c1[found] = i;
            else if (ncell[found] == 1) d->c2[found] = i;
            ncell[found]++;
        }
    for (int e = 0; e < ne; e++)
        if (ncell[e] < 1 || ncell[e] > 2) { free(key); free(ord); free(ncell); orc_dg_free(d); return NULL; }
    free(key); free(ord); free(ncell);
    for (int e = 0; e < ne; e++) {
        double xa = xy[2 * en[2 * e]], ya = xy[2 * en[2 * e] + 1];
        double xb = xy[2 * en[2 * e + 1]], yb = xy[2 * en[2 * e + 1] + 1];
        double mx = (xa + xb) / 2.0, my = (ya + yb) / 2.0;
        double nx = yb - ya, ny = xa - xb;
        double l = sqrt(nx * nx + ny * ny);
        nx /= l; ny /= l;
        double vx = d->cx[d->c1[e]] - mx, vy = d->cy[d->c1[e]] - my;
        if (vx * nx + vy * ny > 0) { nx *= -1; ny *= -1; }
        d->enx[e] = nx; d->eny[e] = ny; d->el[e] = l;
    }
    for (int i = 0; i < nc; i++) {
        double a = d->el[d->cedge[3 * i]], b = d->el[d->cedge[3 * i + 1]], c = d->el[d->cedge[3 * i + 2]];
        double pp = (a + b + c) / 2.0;
        d->S[i] = sqrt(pp * (pp - a) * (pp - b) * (pp - c));
    }
    /* calcGaussPar, :470-598 */
    for (int i = 0; i < nc; i++) {
        const int* t = tri + 3 * i;
        double x1 = xy[2 * t[0]], y1 = xy[2 * t[0] + 1], x2 = xy[2 * t[1]], y2 = xy[2 * t[1] + 1];
        double x3 = xy[2 * t[2]], y3 = xy[2 * t[2] + 1];
        double a1 = x1 - x3, a2 = y1 - y3, b1 = x2 - x3, b2 = y2 - y3, c1 = x3, c2 = y3;
        double* gp = d->cgp + 2 * d->gc * (size_t)i;
        double* gw = d->cgw + d->gc * (size_t)i;
        if (d->gc == 4) {
            double a = 1.0 / 3.0, b = 1.0 / 5.0, c = 3.0 / 5.0;
            gw[0] = -27.0 / 48.0; gp[0] = a1 * a + b1 * a + c1; gp[1] = a2 * a + b2 * a + c2;
            gw[1] = 25.0 / 48.0;  gp[2] = a1 * c + b1 * b + c1; gp[3] = a2 * c + b2 * b + c2;
            gw[2] = 25.0 / 48.0;  gp[4] = a1 * b + b1 * c + c1; gp[5] = a2 * b + b2 * c + c2;
            gw[3] = 25.0 / 48.0;  gp[6] = a1 * b + b1 * b + c1; gp[7] = a2 * b + b2 * b + c2;
            d->cellJ[i] = 0.5 * fabs(a1 * b2 - a2 * b1);
        } else {
            double a = 1.0 / 6.0, b = 2.0 / 3.0;
            gw[0] = 1.0 / 6.0; gp[0] = a1 * a + b1 * a + c1; gp[1] = a2 * a + b2 * a + c2;
            gw[1] = 1.0 / 6.0; gp[2] = a1 * a + b1 * b + c1; gp[3] = a2 * a + b2 * b + c2;
            gw[2] = 1.0 / 6.0; gp[4] = a1 * b + b1 * a + c1; gp[5] = a2 * b + b2 * a + c2;
            d->cellJ[i] = fabs(a1 * b2 - a2 * b1);
        }
    }
    for (int e = 0; e < ne; e++) {
        double x1 = xy[2 * en[2 * e]], y1 = xy[2 * en[2 * e] + 1];
        double x2 = xy[2 * en[2 * e + 1]], y2 = xy[2 * en[2 * e + 1] + 1];
        double* gp = d->egp + 2 * d->ge * (size_t)e;
        double* gw = d->egw + d->ge * (size_t)e;
        if (d->ge == 3) {
            double g1 = -3.0 / 5.0, g3 = 3.0 / 5.0;
            gw[0] = 5.0 / 9.0; gp[0] = ((x1 + x2) + g1 * (x2 - x1)) / 2.0; gp[1] = ((y1 + y2) + g1 * (y2 - y1)) / 2.0;
            gw[1] = 8.0 / 9.0; gp[2] = (x1 + x2) / 2.0; gp[3] = (y1 + y2) / 2.0;
            gw[2] = 5.0 / 9.0; gp[4] = ((x1 + x2) + g3 * (x2 - x1)) / 2.0; gp[5] = ((y1 + y2) + g3 * (y2 - y1)) / 2.0;
        } else {
            double s3 = 1.0 / sqrt(3.0);
            gw[0] = 1.0; gp[0] = ((x1 + x2) - s3 * (x2 - x1)) * 0.5; gp[1] = ((y1 + y2) - s3 * (y2 - y1)) * 0.5;
            gw[1] = 1.0; gp[2] = ((x1 + x2) + s3 * (x2 - x1)) * 0.5; gp[3] = ((y1 + y2) + s3 * (y2 - y1)) * 0.5;
        }
        d->edgeJ[e] = sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)) * 0.5;
    }
    /* calcMassMatr + inverseMatr */
    for (int i = 0; i < nc; i++) {
        double A[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                A[r][c] = 0.0;
                for (int g = 0; g < d->gc; g++) {
                    double F[3];
                    basis(d, i, d->cgp[2 * (d->gc * (size_t)i + g)], d->cgp[2 * (d->gc * (size_t)i + g) + 1], F);
                    A[r][c] += d->cgw[d->gc * (size_t)i + g] * F[r] * F[c];
                }
                A[r][c] *= d->cellJ[i];
            }
        double (*a)[3] = A;
        double detA = a[0][0] * a[1][1] * a[2][2] + a[1][0] * a[2][1] * a[0][2] + a[0][1] * a[1][2] * a[2][0]
                    - a[2][0] * a[1][1] * a[0][2] - a[1][0] * a[0][1] * a[2][2] - a[0][0] * a[2][1] * a[1][2];
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
        double* am = d->invA + 9 * (size_t)i;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) am[3 * r + c] = m[c][r] / detA;
    }
    /* initial state: the region parameters through URS(2), URS(1) twice (init, :96-168),
       convertParToCons (:1404-1418) */
    for (int i = 0; i < nc; i++) {
        const double* rg = reg + 6 * cell_region[i];
        dg_par par;
        memset(&par, 0, sizeof par);
        par.u = rg[2]; par.v = rg[3]; par.T = rg[4]; par.p = rg[5];
        urs(rg[0], rg[1], &par, 2); urs(rg[0], rg[1], &par, 1);
        urs(rg[0], rg[1], &par, 2); urs(rg[0], rg[1], &par, 1);
        double* Uc = d->U + 12 * (size_t)i;
        Uc[0] = par.r;
        Uc[3] = par.r * par.u;
        Uc[6] = par.r * par.v;
        Uc[9] = par.r * (par.e + 0.5 * (par.u * par.u + par.v * par.v));
    }
    d->n_alias = (nc + 1) / 2;
    memcpy(d->Uold, d->U, sizeof(double) * 12 * (size_t)nc);
    d->TAU = p->tau;
    dg_time_step(d);
    return d;
}

void orc_dg_set(orc_dg* d, const double* coeffs) {
    memcpy(d->U, coeffs, sizeof(double) * 12 * (size_t)d->nc);
    if (d->p.rk_mode == ORC_DG_RK_REFERENCE)
        for (int i = 0; i < d->n_alias; i++) memcpy(d->Uold + 12 * (size_t)i, d->U + 12 * (size_t)i, 12 * sizeof(double));
    d->TAU = d->p.tau;
    dg_time_step(d);
}

void orc_dg_set_tau(orc_dg* d, double tau) {
    d->TAU = tau;
    for (int i = 0; i < d->nc; i++) d->ctau[i] = tau;
}

unsigned orc_dg_step(orc_dg* d, int n) {
    for (int s = 0; s < n; s++) dg_one_step(d);
    return d->err;
}

void orc_dg_get(const orc_dg* d, double* coeffs, double* ctau, double* scal) {
    if (coeffs) memcpy(coeffs, d->U, sizeof(double) * 12 * (size_t)d->nc);
    if (ctau) memcpy(ctau, d->ctau, sizeof(double) * (size_t)d->nc);
    if (scal) {
        scal[0] = d->TAU; scal[1] = d->t;
        for (int v = 0; v < 4; v++) scal[2 + v] = d->res[v];
        scal[6] = d->step;
    }
}

void orc_dg_geom(const orc_dg* d, int* cedge, int* c1c2, double* cell6, double* invA, double* edge4) {
    for (int i = 0; i < d->nc; i++) {
        if (cedge) for (int k = 0; k < 3; k++) cedge[3 * i + k] = d->cedge[3 * i + k];
        if (cell6) {
            double* c = cell6 + 6 * (size_t)i;
            c[0] = d->cx[i]; c[1] = d->cy[i]; c[2] = d->HX[i]; c[3] = d->HY[i]; c[4] = d->S[i]; c[5] = d->cellJ[i];
        }
        if (invA) memcpy(invA + 9 * (size_t)i, d->invA + 9 * (size_t)i, 9 * sizeof(double));
    }
    for (int e = 0; e < d->ne; e++) {
        if (c1c2) { c1c2[2 * e] = d->c1[e]; c1c2[2 * e + 1] = d->c2[e]; }
        if (edge4) { edge4[4 * e] = d->enx[e]; edge4[4 * e + 1] = d->eny[e]; edge4[4 * e + 2] = d->el[e]; edge4[4 * e + 3] = d->edgeJ[e]; }
    }
}

/* cell-centre values for the VTU file (save, :662-800: convertConsToPar at the centre) */
void orc_dg_centre(const orc_dg* d, double* rpuv) {
    for (int i = 0; i < d->nc; i++) {
        dg_par p;
        cons2par(d, d->U + 12 * (size_t)i, i, d->cx[i], d->cy[i], &p);
        rpuv[4 * i] = p.r; rpuv[4 * i + 1] = p.p; rpuv[4 * i + 2] = p.u; rpuv[4 * i + 3] = p.v;
    }
}

void orc_dg_free(orc_dg* d) {
    if (!d) return;
    void* ptrs[] = {d->xy, d->tri, d->creg, d->en, d->ebnd, d->cedge, d->c1, d->c2, d->cx, d->cy, d->HX, d->HY,
                    d->S, d->cellJ, d->cgp, d->cgw, d->enx, d->eny, d->el, d->edgeJ, d->egp, d->egw, d->invA,
                    d->reg, d->bkind, d->bpar, d->U, d->Uold, d->Uint, d->ctau};
    for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; k++) free(ptrs[k]);
    free(d);
}
