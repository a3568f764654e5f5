/*
 * cfd2d oracle: plain-C restatement of the reference FVM_TVD explicit solver.
 * TEST INFRASTRUCTURE ONLY (see cfd2d_oracle.h): a reference to check against, never the product.
 *
 * Structure mirrors the reference on purpose: array-of-edges loops that scatter
 * into cells (src/methods/fvm_tvd.cpp:242-301, 329-365), the same conversions,
 * the same ghost recipe and the same operation order, so that in reference mode
 * the result equals the reference bit for bit.
 */
#include "cfd2d_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GAS_R 8.314472 /* Material::gR, src/global.cpp:6 */

/* Param, src/global.h:180-194 (viscosity unused on this path). */
typedef struct { double r, p, e, E, u, v, cz, T; } Par;

struct orc_mesh {
    int nn, nc, ne;
    int* cnodes;   /* nc x 3 */
    int* cedges;   /* nc x 3, Cell::edgesInd: ascending edge numbers */
    double *S, *cx, *cy;
    int *n1, *n2, *c1, *c2, *bnd, *npts;
    double *nx, *ny, *l;
    double* pts;   /* ne x 3 x 2 */
};

struct orc_solver {
    const orc_mesh* m;
    orc_params p;
    int nm;
    double *matM, *matCp;
    int* cell_mat;
    int nbnd;
    int* bkind;
    double* bpar;
    double *ro, *ru, *rv, *re;
    double *ro_old, *ru_old, *rv_old, *re_old;
    double *ro_int, *ru_int, *rv_int, *re_int;
    double* grad; /* nc x 8: r.x r.y p.x p.y u.x u.y v.x v.y */
    double* cTau;
    unsigned* flag;
    double TAU, t;
    int newton_hit;
};

static double dmax(double a, double b) { return a > b ? a : b; } /* _max_, src/mesh/grid.h:102 */
static double dmin(double a, double b) { return a < b ? a : b; }

/* ------------------------------------------------------------------ mesh */

static int* node_cells(int nn, int nc, const int* tri, int** off_out) {
    int* off = (int*)calloc((size_t)nn + 1, sizeof(int));
    for (int i = 0; i < 3 * nc; i++) off[tri[i] + 1]++;
    for (int i = 0; i < nn; i++) off[i + 1] += off[i];
    int* fill = (int*)malloc(sizeof(int) * (size_t)nn);
    memcpy(fill, off, sizeof(int) * (size_t)nn);
    int* lst = (int*)malloc(sizeof(int) * (size_t)(3 * nc > 0 ? 3 * nc : 1));
    for (int i = 0; i < nc; i++)
        for (int k = 0; k < 3; k++) lst[fill[tri[3 * i + k]]++] = i; /* ascending cell order */
    free(fill);
    *off_out = off;
    return lst;
}

static long long pair_key(int a, int b) {
    if (a > b) { int t = a; a = b; b = t; }
    return ((long long)a << 32) | (unsigned)b;
}

typedef struct { long long key; int idx; } KeyIdx;
static int cmp_keyidx(const void* x, const void* y) {
    const KeyIdx* a = (const KeyIdx*)x; const KeyIdx* b = (const KeyIdx*)y;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return a->idx - b->idx;
}

int orc_mesh_build(int nn, const double* xy, int nc, const int* tri, const int* neigh_berkeley,
                   int nb, const int* bseg, const int* bseg_bnd, int berkeley, orc_mesh** out) {
    *out = NULL;
    int* neigh = (int*)malloc(sizeof(int) * 3 * (size_t)nc);
    orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
    m->nn = nn; m->nc = nc;
    m->cnodes = (int*)malloc(sizeof(int) * 3 * (size_t)nc);
    memcpy(m->cnodes, tri, sizeof(int) * 3 * (size_t)nc);
    m->cx = (double*)malloc(sizeof(double) * nc);
    m->cy = (double*)malloc(sizeof(double) * nc);
    for (int i = 0; i < nc; i++) { /* src/mesh/MeshReaderSalomeUnv.cpp:89-90 */
        const int* t = tri + 3 * i;
        m->cx[i] = (xy[2 * t[0]] + xy[2 * t[1]] + xy[2 * t[2]]) / 3.0;
        m->cy[i] = (xy[2 * t[0] + 1] + xy[2 * t[1] + 1] + xy[2 * t[2] + 1]) / 3.0;
    }
    if (berkeley) {
        memcpy(neigh, neigh_berkeley, sizeof(int) * 3 * (size_t)nc);
    } else { /* neighbour across nodes (k, k+1): src/mesh/MeshReaderSalomeUnv.cpp:100-115 */
        int* off; int* lst = node_cells(nn, nc, tri, &off);
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
        free(off); free(lst);
    }
    /* edge count, clearing the neighbour's back reference (:118-135) */
    int ne = 0;
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < 3; j++) {
            int p = neigh[3 * i + j];
            if (p > -1) {
                for (int k = 0; k < 3; k++) if (neigh[3 * p + k] == i) neigh[3 * p + k] = -1;
                ne++;
            }
            if (p == -2) ne++;
        }
    m->ne = ne;
    m->cedges = (int*)malloc(sizeof(int) * 3 * (size_t)nc);
    m->n1 = (int*)malloc(sizeof(int) * ne); m->n2 = (int*)malloc(sizeof(int) * ne);
    m->c1 = (int*)malloc(sizeof(int) * ne); m->c2 = (int*)malloc(sizeof(int) * ne);
    m->bnd = (int*)malloc(sizeof(int) * ne); m->npts = (int*)malloc(sizeof(int) * ne);
    m->nx = (double*)malloc(sizeof(double) * ne); m->ny = (double*)malloc(sizeof(double) * ne);
    m->l = (double*)malloc(sizeof(double) * ne);
    m->pts = (double*)calloc((size_t)ne * 6, sizeof(double));
    m->S = (double*)malloc(sizeof(double) * nc);
    int* cfi = (int*)calloc((size_t)nc, sizeof(int));

    KeyIdx* bk = (KeyIdx*)malloc(sizeof(KeyIdx) * (size_t)(nb > 0 ? nb : 1));
    for (int s = 0; s < nb; s++) { bk[s].key = pair_key(bseg[2 * s], bseg[2 * s + 1]); bk[s].idx = s; }
    qsort(bk, (size_t)nb, sizeof(KeyIdx), cmp_keyidx);

    const double sq3 = 1.0 / sqrt(3.0);
    int e = 0, err = 0;
    for (int i = 0; i < nc && !err; i++)
        for (int j = 0; j < 3; j++) {
            int p = neigh[3 * i + j];
            if (p == -1) continue;
            const int* t = tri + 3 * i;
            int a = berkeley ? t[(j + 1) % 3] : t[j];
            int b = berkeley ? t[(j + 2) % 3] : t[(j + 1) % 3];
            m->n1[e] = a; m->n2[e] = b;
            double x1 = xy[2 * a], y1 = xy[2 * a + 1], x2 = xy[2 * b], y2 = xy[2 * b + 1];
            double* P = m->pts + 6 * (size_t)e;
            P[0] = (x1 + x2) / 2.0;
            P[1] = (y1 + y2) / 2.0;
            if (berkeley == 1) {
                m->npts[e] = 1; /* src/mesh/MeshReaderBerkleyTriangle.cpp:102-105 */
            } else {            /* src/mesh/MeshReaderSalomeUnv.cpp:158-169, src/mesh/grid.cpp:153-162 */
                m->npts[e] = 3;
                P[2] = (x1 + x2) / 2.0 - sq3 * (x2 - x1) / 2.0;
                P[3] = (y1 + y2) / 2.0 - sq3 * (y2 - y1) / 2.0;
                P[4] = (x1 + x2) / 2.0 + sq3 * (x2 - x1) / 2.0;
                P[5] = (y1 + y2) / 2.0 + sq3 * (y2 - y1) / 2.0;
            }
            double nx = y2 - y1, ny = x1 - x2;
            double l = sqrt(nx * nx + ny * ny);
            nx /= l; ny /= l;
            m->l[e] = l;
            m->c1[e] = i;
            m->cedges[3 * i + cfi[i]++] = e;
            if (!berkeley) { /* outward from c1 (:181-187) */
                double vx = m->cx[i] - P[0], vy = m->cy[i] - P[1];
                if (vx * nx + vy * ny > 0) { nx *= -1; ny *= -1; }
            }
            m->nx[e] = nx; m->ny[e] = ny;
            m->bnd[e] = -1;
            if (p > -1) {
                m->c2[e] = p;
                m->cedges[3 * p + cfi[p]++] = e;
            } else {
                m->c2[e] = -1;
                KeyIdx q; q.key = pair_key(a, b); q.idx = -1;
                int lo = 0, hi = nb; /* first segment with this node pair */
                while (lo < hi) { int mid = (lo + hi) / 2; if (bk[mid].key < q.key) lo = mid + 1; else hi = mid; }
                if (lo < nb && bk[lo].key == q.key) m->bnd[e] = bseg_bnd[bk[lo].idx];
                else { err = -222; break; } /* Exception TYPE_MESH_UNV_NOT_DEFINED_BND_EDGE */
            }
            e++;
        }
    free(bk); free(neigh);
    if (!err)
        for (int i = 0; i < nc; i++) {
            if (cfi[i] != 3) { err = -221; break; }
            double a = m->l[m->cedges[3 * i]], b = m->l[m->cedges[3 * i + 1]], c = m->l[m->cedges[3 * i + 2]];
            double p = (a + b + c) / 2.0; /* Heron, src/mesh/MeshReaderSalomeUnv.cpp:250-255 */
            m->S[i] = sqrt(p * (p - a) * (p - b) * (p - c));
        }
    free(cfi);
    if (err) { orc_mesh_free(m); return err; }
    *out = m;
    return 0;
}

void orc_mesh_sizes(const orc_mesh* m, int* nc, int* ne) { *nc = m->nc; *ne = m->ne; }

void orc_mesh_export(const orc_mesh* m, int* cell_edges, double* cell_S, double* cell_c,
                     int* edge_n12, int* edge_c12, int* edge_bnd, int* edge_npts,
                     double* edge_n, double* edge_l, double* edge_pts) {
    for (int i = 0; i < m->nc; i++) {
        for (int k = 0; k < 3; k++) cell_edges[3 * i + k] = m->cedges[3 * i + k];
        cell_S[i] = m->S[i];
        cell_c[2 * i] = m->cx[i]; cell_c[2 * i + 1] = m->cy[i];
    }
    for (int e = 0; e < m->ne; e++) {
        edge_n12[2 * e] = m->n1[e]; edge_n12[2 * e + 1] = m->n2[e];
        edge_c12[2 * e] = m->c1[e]; edge_c12[2 * e + 1] = m->c2[e];
        edge_bnd[e] = m->bnd[e]; edge_npts[e] = m->npts[e];
        edge_n[2 * e] = m->nx[e]; edge_n[2 * e + 1] = m->ny[e];
        edge_l[e] = m->l[e];
        for (int k = 0; k < 6; k++) edge_pts[6 * e + k] = m->pts[6 * e + k];
    }
}

void orc_mesh_free(orc_mesh* m) {
    if (!m) return;
    free(m->cnodes); free(m->cedges); free(m->S); free(m->cx); free(m->cy);
    free(m->n1); free(m->n2); free(m->c1); free(m->c2); free(m->bnd); free(m->npts);
    free(m->nx); free(m->ny); free(m->l); free(m->pts);
    free(m);
}

/* ------------------------------------------------------------------ physics */

/* Material::URS, src/global.cpp:9-30 */
static void urs(double M, double Cp, Par* par, int flag) {
    double Cv = Cp - GAS_R / M;
    double gam = Cp / Cv;
    switch (flag) {
    case 0: par->p = par->r * par->e * (gam - 1); par->cz = sqrt(gam * par->p / par->r); break;
    case 1: par->e = par->p / (par->r * (gam - 1)); par->T = par->e / Cv; break;
    case 2: par->r = par->p * M / (par->T * GAS_R); par->cz = sqrt(gam * par->p / par->r); break;
    }
}

void orc_region_state(double M, double Cp, double u, double v, double T, double p, double* U4) {
    Par par; memset(&par, 0, sizeof par);
    par.u = u; par.v = v; par.T = T; par.p = p;
    urs(M, Cp, &par, 2); /* src/methods/fvm_tvd.cpp:91-92 */
    urs(M, Cp, &par, 1);
    U4[0] = par.r;       /* convertParToCons, :795-801 */
    U4[1] = par.r * par.u;
    U4[2] = par.r * par.v;
    U4[3] = par.r * (par.e + 0.5 * (par.u * par.u + par.v * par.v));
}

/* convertConsToPar, src/methods/fvm_tvd.cpp:803-813 */
static void cons2par(const orc_solver* s, int i, Par* par) {
    int mt = s->cell_mat[i];
    par->r = s->ro[i];
    par->u = s->ru[i] / s->ro[i];
    par->v = s->rv[i] / s->ro[i];
    par->E = s->re[i] / s->ro[i];
    par->e = par->E - 0.5 * (par->u * par->u + par->v * par->v);
    urs(s->matM[mt], s->matCp[mt], par, 0);
    urs(s->matM[mt], s->matCp[mt], par, 1);
}

/* boundaryCond + CFDBnd*::run, src/methods/fvm_tvd.cpp:694-705, src/bnd_cond.cpp:75-110 */
static void boundary_cond(const orc_solver* s, int e, const Par* pL, Par* pR) {
    const orc_mesh* m = s->m;
    int b = m->bnd[e];
    int kind = s->bkind[b];
    const double* bp = s->bpar + 4 * b;
    if (kind == ORC_BND_INLET) {
        pR->u = bp[0]; pR->v = bp[1]; pR->T = bp[2]; pR->p = bp[3];
    } else if (kind == ORC_BND_OUTLET) {
        *pR = *pL;
    } else { /* BOUND_WALL_SLIP, and BOUND_WALL_NO_SLIP which the reference maps to the slip class */
        *pR = *pL;
        double Un = pL->u * m->nx[e] + pL->v * m->ny[e];
        double Vx = m->nx[e] * Un * 2.0, Vy = m->ny[e] * Un * 2.0;
        pR->u = pL->u - Vx;
        pR->v = pL->v - Vy;
    }
    int mt = s->cell_mat[m->c1[e]];
    urs(s->matM[mt], s->matCp[mt], pR, 2);
    urs(s->matM[mt], s->matCp[mt], pR, 1);
    pR->E = pR->e + 0.5 * (pR->u * pR->u + pR->v * pR->v);
}

/* Exact Riemann solver rim_orig, src/global.cpp:232-405, restated with structured
 * control flow and an optional cap on its Newton loop. VB/VE are the tangential
 * velocities carried through; the third component the reference passes is 0. */
static int riemann_exact(double* RI_, double* EI_, double* PI_, double* UI_, double* VI_,
                         double RB, double PB, double UB, double VB,
                         double RE, double PE, double UE, double VE, double GAM, int cap) {
    double AGAM = (GAM - 1.0);
    double DGAM = (2.0 / AGAM);
    double GGAM = (sqrt(GAM * AGAM));
    double HGAM = (AGAM / 2.0);
    double FGAM = (3.0 * GAM - 1.0);
    double OGAM = (AGAM / (2.0 * GAM));
    double QGAM = (GAM + 1.0);
    double PGAM = (QGAM / (2.0 * GAM));
    double RGAM = (4.0 * GAM);
    double SGAM = (GAM * AGAM);
    double TGAM = (QGAM / 2.0);
    double US = 0.0, UF = 0.0;
    double RF, RS, EF, ES, SBL, SFL, SSL, SEL, D, P;
    double eps = 1.0e-5;
    double CB = sqrt(GAM * PB / RB);
    double CE = sqrt(GAM * PE / RE);
    double EB = CB * CB / SGAM;
    double EE = CE * CE / SGAM;
    double RCB = RB * CB;
    double RCE = RE * CE;
    double DU = UB - UE;
    double RI, EI, UI, VI;
    int hit = 0;
    if (DU < -2.0 * (CB + CE) / AGAM) { /* vacuum */
        RF = 0.0; RS = 0.0; EF = 0.0; ES = 0.0;
        SBL = UB - CB;
        SFL = UB + 2.0 * CB / AGAM;
        SSL = UE - 2.0 * CE / AGAM;
        SEL = UE + CE;
    } else {
        P = (PB * RCE + PE * RCB + DU * RCB * RCE) / (RCB + RCE);
        int it = 0;
        for (;;) {
            double PPB, PPE, F1, FS1, F2, FS2;
            if (P < eps) P = eps;
            PPB = P / PB;
            if (PB > P) {
                double ZFB = CB * exp(log(PPB) * OGAM);
                F1 = DGAM * (ZFB - CB);
                FS1 = ZFB / (GAM * P);
            } else {
                double PKB = PGAM * PPB + OGAM;
                double ZNB = RCB * sqrt(PKB);
                F1 = (P - PB) / ZNB;
                FS1 = (QGAM * PPB + FGAM) / (RGAM * ZNB * PKB);
            }
            PPE = P / PE;
            if (PE > P) {
                double ZFE = CE * exp(log(PPE) * OGAM);
                F2 = DGAM * (ZFE - CE);
                FS2 = ZFE / (GAM * P);
            } else {
                double PKE = PGAM * PPE + OGAM;
                double ZNE = RCE * sqrt(PKE);
                F2 = (P - PE) / ZNE;
                FS2 = (QGAM * PPE + FGAM) / (RGAM * ZNE * PKE);
            }
            double DP = (DU - F1 - F2) / (FS1 + FS2);
            P = P + DP;
            if (!(fabs(DU - F1 - F2) > eps)) break;
            if (cap > 0 && ++it >= cap) { hit = 1; break; }
        }
        double PPB = P / PB, PPE = P / PE;
        double ZFB = CB * exp(log(PPB) * OGAM);
        double ZFE = CE * exp(log(PPE) * OGAM);
        if (!(PB > P)) { /* left shock */
            D = UB - sqrt((TGAM * P + HGAM * PB) / RB);
            double UBD = UB - D, RUBD = RB * UBD;
            RF = RUBD * RUBD / (PB - P + RUBD * UBD);
            UF = D + RUBD / RF;
            EF = P / (AGAM * RF);
            SBL = D; SFL = D;
        } else {         /* left rarefaction */
            EF = ZFB * ZFB / SGAM;
            UF = UB + DGAM * (CB - ZFB);
            RF = P / (AGAM * EF);
            SBL = UB - CB;
            SFL = UF - ZFB;
        }
        if (!(PE > P)) { /* right shock */
            D = UE + sqrt((TGAM * P + HGAM * PE) / RE);
            double UED = UE - D, RUED = RE * UED;
            RS = RUED * RUED / (PE - P + RUED * UED);
            US = D + RUED / RS;
            ES = P / (AGAM * RS);
            SEL = D; SSL = D;
        } else {         /* right rarefaction */
            ES = ZFE * ZFE / SGAM;
            US = UE - DGAM * (CE - ZFE);
            RS = P / (AGAM * ES);
            SSL = US + ZFE;
            SEL = UE + CE;
        }
    }
    /* sample at x/t = 0 */
    if (SEL <= 0.0) { RI = RE; EI = EE; UI = UE; VI = VE; }
    else if (SBL >= 0.0) { RI = RB; EI = EB; UI = UB; VI = VB; }
    else if ((SSL >= 0.0) && (SFL <= 0.0)) {
        if (US >= 0.0) { RI = RF; EI = EF; UI = UF; VI = VB; }
        else { RI = RS; EI = ES; UI = US; VI = VE; }
    } else if (SFL > 0.0) {
        UI = (UB + DGAM * GGAM * sqrt(EB)) / (1 + DGAM);
        VI = VB;
        EI = (UI * UI) / SGAM;
        RI = RB * exp(log(EI / EB) * (1 / AGAM));
    } else {
        UI = (UE - DGAM * GGAM * sqrt(EE)) / (1 + DGAM);
        VI = VE;
        EI = (UI * UI) / SGAM;
        RI = RE * exp(log(EI / EE) * (1 / AGAM));
    }
    *RI_ = RI; *EI_ = EI; *UI_ = UI; *VI_ = VI;
    *PI_ = AGAM * EI * RI;
    return hit;
}

/* Godunov flux, FVM_TVD::calcFlux, src/methods/fvm_tvd.cpp:602-622 */
/* the exact Riemann solver for the discontinuous Galerkin restatement (cfd2d_oracle_dg.c) */
int orc_riemann_exact(double* RI, double* EI, double* PI, double* UI, double* VI, double RB, double PB, double UB,
                      double VB, double RE, double PE, double UE, double VE, double GAM, int cap) {
    return riemann_exact(RI, EI, PI, UI, VI, RB, PB, UB, VB, RE, PE, UE, VE, GAM, cap);
}

static int flux_godunov(double* f, const Par* pL, const Par* pR, double nx, double ny, double GAM, int cap) {
    double RI, EI, PI, UN, UT;
    double unl = pL->u * nx + pL->v * ny;
    double unr = pR->u * nx + pR->v * ny;
    double utl = pL->u * ny - pL->v * nx;
    double utr = pR->u * ny - pR->v * nx;
    int hit = riemann_exact(&RI, &EI, &PI, &UN, &UT, pL->r, pL->p, unl, utl, pR->r, pR->p, unr, utr, GAM, cap);
    double UI = UN * nx + UT * ny;
    double VI = UN * ny - UT * nx;
    f[0] = RI * UN;
    f[1] = f[0] * UI + PI * nx;
    f[2] = f[0] * VI + PI * ny;
    f[3] = (RI * (EI + 0.5 * (UI * UI + VI * VI)) + PI) * UN;
    return hit;
}

/* Lax-Friedrichs (Rusanov) flux, the reference's template in
 * src/methods/fvm_tvd_implicit.cpp:939-960 (energy from p). */
static void flux_lax(double* f, const Par* pL, const Par* pR, double nx, double ny, double GAM) {
    double unl = pL->u * nx + pL->v * ny;
    double unr = pR->u * nx + pR->v * ny;
    double alpha = dmax(fabs(unl) + sqrt(GAM * pL->p / pL->r), fabs(unr) + sqrt(GAM * pR->p / pR->r));
    double rol = pL->r, rul = pL->r * pL->u, rvl = pL->r * pL->v;
    double rel = pL->p / (GAM - 1.0) + 0.5 * pL->r * (pL->u * pL->u + pL->v * pL->v);
    double ror = pR->r, rur = pR->r * pR->u, rvr = pR->r * pR->v;
    double rer = pR->p / (GAM - 1.0) + 0.5 * pR->r * (pR->u * pR->u + pR->v * pR->v);
    double frl = rol * unl, frr = ror * unr;
    f[0] = 0.5 * (frr + frl - alpha * (ror - rol));
    f[1] = 0.5 * (frr * pR->u + frl * pL->u + (pR->p + pL->p) * nx - alpha * (rur - rul));
    f[2] = 0.5 * (frr * pR->v + frl * pL->v + (pR->p + pL->p) * ny - alpha * (rvr - rvl));
    f[3] = 0.5 * ((rer + pR->p) * unr + (rel + pL->p) * unl - alpha * (rer - rel));
}

/* Physical flux through the unit normal n for a primitive state; E is the total
 * energy per unit volume. The fluxes defined here (HLLC, Roe, the minmod
 * increment) have no counterpart in the reference; their multiply-adds are
 * fused (C99 fma), exactly as the GPU evaluates them. */
static void phys_flux(double* f, double r, double u, double v, double p, double E, double un, double nx, double ny) {
    double m = r * un;
    f[0] = m;
    f[1] = fma(m, u, p * nx);
    f[2] = fma(m, v, p * ny);
    f[3] = (E + p) * un;
}

/* a x + b y with one rounding less */
static double dot2(double a, double x, double b, double y) { return fma(a, x, b * y); }
/* kinetic part p*IG1 + (0.5 r)(u^2 + v^2) of the total energy */
static double energy(double r, double u, double v, double p, double IG1) {
    return fma(p, IG1, (0.5 * r) * fma(u, u, v * v));
}

/* Newton-refined quotient, reciprocal and sound speed of the FP64 HLLC flux: this
 * project's definition of that flux's arithmetic, the same operations as the GPU
 * (hllc_quot / hllc_recip / hllc_sound in the library's kernels). A binary32 seed
 * (x truncated: sign, rebiased exponent, top 23 fraction bits), correctly rounded
 * binary32 operations, then FP64 Newton steps with fma (Newton-Raphson for 1/b and
 * sqrt(a/r); the quotient corrected as in Markstein, "IA-64 and Elementary
 * Functions", 2000). Within |x| in [2^-60, 2^60) every binary32 value is normal;
 * other operands take the IEEE expression. */
static int hllc_in_range(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    int e = (int)((b >> 52) & 0x7ff);
    return e >= 1023 - 60 && e < 1023 + 60;
}
static float hllc_seed(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
    uint32_t ex = (uint32_t)((b >> 52) & 0x7ff) - (1023u - 127u);
    uint32_t f = sgn | (ex << 23) | ((uint32_t)(b >> 29) & 0x7fffffu);
    float r;
    memcpy(&r, &f, 4);
    return r;
}
static double hllc_rcp1(double b) {
    double y0 = (double)(1.0f / hllc_seed(b));  /* a correctly rounded binary32 division */
    return fma(y0, fma(-b, y0, 1.0), y0);
}
static double hllc_quot(double a, double b) {
    if (hllc_in_range(b)) {
        if (hllc_in_range(a)) {
            double y = hllc_rcp1(b), q = a * y;
            return fma(fma(-q, b, a), y, q);
        }
        if (a == 0.0) return copysign(0.0, a) * copysign(1.0, b);
    }
    return a / b;
}
static double hllc_recip(double b) {
    if (!hllc_in_range(b)) return 1.0 / b;
    double y = hllc_rcp1(b);
    return fma(y, fma(-b, y, 1.0), y);
}
static double hllc_sound(double a, double r) {
    if (!(a > 0.0) || !(r > 0.0) || !hllc_in_range(a) || !hllc_in_range(r)) return sqrt(a / r);
    float af = hllc_seed(a), rf = hllc_seed(r);
    float qf = af / rf;
    float sf = sqrtf(qf);
    float tf = rf * sf;
    float hf = 0.5f / tf;
    double h = (double)hf, s = (double)sf;
    s = fma(fma(-(r * s), s, a), h, s);
    s = fma(fma(-(r * s), s, a), h, s);
    return s;
}

/* HLLC flux (Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics,
 * 3rd ed., sec. 10.4-10.6) with Davis wave-speed estimates
 * S_L = min(un_L - c_L, un_R - c_R), S_R = max(un_L + c_L, un_R + c_R), and the
 * star flux in the form with a single division,
 *   F*_K = [S*(S_K U_K - F_K) + S_K p* D*] / (S_K - S*),  D* = (0, nx, ny, S*),
 *   p* = p_K + rho_K (S_K - un_K)(S* - un_K),
 * which equals F_K + S_K (U*_K - U_K) for Toro's star state U*_K, with
 *   S_K U_K - F_K = (m_K, m_K u - p nx, m_K v - p ny, E_K (S_K - un_K) - p un_K),
 *   m_K = rho_K (S_K - un_K); only the side used forms its energy. Energies use
 * p/(gamma-1) as p * (1/(gamma-1)). c = hllc_sound(GAMMA p, rho), S* = hllc_quot,
 * 1/(S_K - S*) = hllc_recip. */
static void flux_hllc(double* f, const Par* pL, const Par* pR, double nx, double ny, double GAM) {
    double IG1 = 1.0 / (GAM - 1.0);
    double cL = hllc_sound(GAM * pL->p, pL->r), cR = hllc_sound(GAM * pR->p, pR->r);
    double unL = dot2(pL->u, nx, pL->v, ny), unR = dot2(pR->u, nx, pR->v, ny);
    double SL = dmin(unL - cL, unR - cR), SR = dmax(unL + cL, unR + cR);
    if (SL >= 0.0) {
        phys_flux(f, pL->r, pL->u, pL->v, pL->p, energy(pL->r, pL->u, pL->v, pL->p, IG1), unL, nx, ny);
        return;
    }
    if (SR <= 0.0) {
        phys_flux(f, pR->r, pR->u, pR->v, pR->p, energy(pR->r, pR->u, pR->v, pR->p, IG1), unR, nx, ny);
        return;
    }
    double dL = SL - unL, dR = SR - unR;
    double mL = pL->r * dL, mR = pR->r * dR;
    double Ss = hllc_quot(fma(-mR, unR, fma(mL, unL, pR->p - pL->p)), mL - mR);
    const Par* K; double SK, unK, dK, mK;
    if (Ss >= 0.0) { K = pL; SK = SL; unK = unL; dK = dL; mK = mL; }
    else { K = pR; SK = SR; unK = unR; dK = dR; mK = mR; }
    double EK = energy(K->r, K->u, K->v, K->p, IG1);
    /* S_K U_K - F_K = (m_K, m_K u - p nx, m_K v - p ny, E_K (S_K - un_K) - p un_K) */
    double A1 = fma(mK, K->u, -(K->p * nx)), A2 = fma(mK, K->v, -(K->p * ny)), A3 = fma(EK, dK, -(K->p * unK));
    double ps = fma(mK, Ss - unK, K->p);
    double inv = hllc_recip(SK - Ss);
    double sp = SK * ps;
    f[0] = (Ss * mK) * inv;
    f[1] = fma(Ss, A1, sp * nx) * inv;
    f[2] = fma(Ss, A2, sp * ny) * inv;
    f[3] = fma(Ss, A3, sp * Ss) * inv;
}

/* 1/sqrt(x) for x > 0 in [2^-60, 2^60): t = RN32(1 / RN32(sqrt(x truncated to binary32))),
 * then two Newton steps t <- t + (t/2)(1 - x t t); other operands: IEEE. */
static double roe_rsqrt(double x) {
    if (!(x > 0.0) || !hllc_in_range(x)) return 1.0 / sqrt(x);
    float sf = sqrtf(hllc_seed(x));
    float tf = 1.0f / sf;
    double t = (double)tf;
    t = fma(0.5 * t, fma(-(x * t), t, 1.0), t);
    t = fma(0.5 * t, fma(-(x * t), t, 1.0), t);
    return t;
}

/* Roe flux (Roe, J. Comput. Phys. 43, 1981) in the face-normal frame with the
 * Harten-Hyman entropy fix on the acoustic waves (Harten & Hyman, J. Comput.
 * Phys. 50, 1983): delta = max(0, lam~ - lam_L, lam_R - lam~), |lam~| -> delta
 * where |lam~| < delta. Roe averages as in the reference's roe_orig
 * (src/global.cpp:407-441). This project's arithmetic: the averages from
 * t = 1/sqrt(rho) (sqrt(rho) = rho t, sqrt(rho) H = (E + p) t), c~ = c~^2 t~ and
 * 1/c~^2 = t~^2 with t~ = 1/sqrt(c~^2), the side sound speeds as HLLC's,
 * 1/(sqrt(rho_L) + sqrt(rho_R)) Newton-refined, the wave sums fused. */
static void flux_roe(double* f, const Par* pL, const Par* pR, double nx, double ny, double GAM) {
    double G1 = GAM - 1.0, IG1 = 1.0 / (GAM - 1.0);
    double unL = dot2(pL->u, nx, pL->v, ny), unR = dot2(pR->u, nx, pR->v, ny);
    double EL = energy(pL->r, pL->u, pL->v, pL->p, IG1);
    double ER = energy(pR->r, pR->u, pR->v, pR->p, IG1);
    double tL = roe_rsqrt(pL->r), tR = roe_rsqrt(pR->r);
    double sL = pL->r * tL, sR = pR->r * tR;
    double w = hllc_recip(sL + sR);
    double ut = fma(sL, pL->u, sR * pR->u) * w, vt = fma(sL, pL->v, sR * pR->v) * w;
    double Ht = fma(EL + pL->p, tL, (ER + pR->p) * tR) * w;
    double q2 = fma(ut, ut, vt * vt);
    double c2 = G1 * fma(-0.5, q2, Ht);
    double c, ic2;
    if (c2 > 0.0 && hllc_in_range(c2)) {
        double t = roe_rsqrt(c2);
        c = c2 * t;
        ic2 = t * t;
    } else {
        c = sqrt(c2);
        ic2 = 1.0 / c2;
    }
    double unt = dot2(ut, nx, vt, ny);
    double rt = sL * sR;
    double dr = pR->r - pL->r, dp = pR->p - pL->p, dun = unR - unL;
    double dtx = fma(-dun, nx, pR->u - pL->u), dty = fma(-dun, ny, pR->v - pL->v);
    double h = 0.5 * ic2, x = (rt * c) * dun;
    double a1 = (dp - x) * h, a2 = fma(-dp, ic2, dr), a4 = (dp + x) * h;
    double l1 = unt - c, l4 = unt + c;
    double cL = hllc_sound(GAM * pL->p, pL->r), cR = hllc_sound(GAM * pR->p, pR->r);
    double d1 = dmax(0.0, dmax(l1 - (unL - cL), (unR - cR) - l1));
    double d4 = dmax(0.0, dmax(l4 - (unL + cL), (unR + cR) - l4));
    double al1 = fabs(l1); if (al1 < d1) al1 = d1;
    double al4 = fabs(l4); if (al4 < d4) al4 = d4;
    double al2 = fabs(unt);
    double w1 = al1 * a1, w2 = al2 * a2, w4 = al4 * a4, ws = al2 * rt;
    double cx = c * nx, cy = c * ny, cu = unt * c;
    double D0 = (w1 + w2) + w4;
    double D1 = fma(w4, ut + cx, fma(w1, ut - cx, fma(w2, ut, ws * dtx)));
    double D2 = fma(w4, vt + cy, fma(w1, vt - cy, fma(w2, vt, ws * dty)));
    double D3 = fma(w4, Ht + cu, fma(w1, Ht - cu, fma(0.5 * w2, q2, ws * dot2(ut, dtx, vt, dty))));
    double FL[4], FR[4];
    phys_flux(FL, pL->r, pL->u, pL->v, pL->p, EL, unL, nx, ny);
    phys_flux(FR, pR->r, pR->u, pR->v, pR->p, ER, unR, nx, ny);
    f[0] = 0.5 * ((FL[0] + FR[0]) - D0);
    f[1] = 0.5 * ((FL[1] + FR[1]) - D1);
    f[2] = 0.5 * ((FL[2] + FR[2]) - D2);
    f[3] = 0.5 * ((FL[3] + FR[3]) - D3);
}

/* MINMOD, src/methods/LimiterDGCockburn.cpp:110-123 */
static double minmod(double a, double b) {
    if (a * b > 0.0) return fabs(a) < fabs(b) ? a : b;
    return 0;
}

/* ------------------------------------------------------------------ solver */

static double* dalloc(int n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

/* calcTimeStep, src/methods/fvm_tvd.cpp:216-240 */
static void calc_time_step(orc_solver* s) {
    const orc_mesh* m = s->m;
    if (s->p.steady) {
        for (int i = 0; i < m->nc; i++) {
            Par p; cons2par(s, i, &p);
            s->cTau[i] = s->p.cfl * m->S[i] / dmax(fabs(p.u) + p.cz, fabs(p.v) + p.cz);
        }
    } else {
        for (int i = 0; i < m->nc; i++) {
            Par p; cons2par(s, i, &p);
            double t = s->p.cfl * m->S[i] / dmax(fabs(p.u) + p.cz, fabs(p.v) + p.cz);
            if (s->TAU > t) s->TAU = t;
        }
        for (int i = 0; i < m->nc; i++) s->cTau[i] = s->TAU;
    }
}

int orc_solver_create(const orc_mesh* m, const orc_params* prm, int nm, const double* mat,
                      const int* cell_mat, int nbnd, const int* bnd_kind, const double* bnd_par,
                      const double* U0, orc_solver** out) {
    orc_solver* s = (orc_solver*)calloc(1, sizeof(orc_solver));
    int nc = m->nc;
    s->m = m; s->p = *prm; s->nm = nm; s->nbnd = nbnd;
    s->matM = dalloc(nm); s->matCp = dalloc(nm);
    for (int k = 0; k < nm; k++) { s->matM[k] = mat[2 * k]; s->matCp[k] = mat[2 * k + 1]; }
    s->cell_mat = (int*)malloc(sizeof(int) * (size_t)nc);
    memcpy(s->cell_mat, cell_mat, sizeof(int) * (size_t)nc);
    s->bkind = (int*)malloc(sizeof(int) * (size_t)(nbnd > 0 ? nbnd : 1));
    s->bpar = dalloc(4 * nbnd);
    if (nbnd) { memcpy(s->bkind, bnd_kind, sizeof(int) * nbnd); memcpy(s->bpar, bnd_par, sizeof(double) * 4 * nbnd); }
    s->ro = dalloc(nc); s->ru = dalloc(nc); s->rv = dalloc(nc); s->re = dalloc(nc);
    s->ro_old = dalloc(nc); s->ru_old = dalloc(nc); s->rv_old = dalloc(nc); s->re_old = dalloc(nc);
    s->ro_int = dalloc(nc); s->ru_int = dalloc(nc); s->rv_int = dalloc(nc); s->re_int = dalloc(nc);
    s->grad = dalloc(8 * nc);
    s->cTau = dalloc(nc);
    s->flag = (unsigned*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(unsigned));
    orc_set_state(s, U0);
    s->TAU = prm->tau_xml;
    calc_time_step(s); /* FVM_TVD::init, :211 */
    *out = s;
    return 0;
}

double orc_tau(const orc_solver* s) { return s->TAU; }

void orc_set_state(orc_solver* s, const double* U) {
    int nc = s->m->nc;
    memcpy(s->ro, U, sizeof(double) * nc);
    memcpy(s->ru, U + nc, sizeof(double) * nc);
    memcpy(s->rv, U + 2 * (size_t)nc, sizeof(double) * nc);
    memcpy(s->re, U + 3 * (size_t)nc, sizeof(double) * nc);
}

void orc_get_state(const orc_solver* s, double* U, double* ctau, unsigned* flags) {
    int nc = s->m->nc;
    if (U) {
        memcpy(U, s->ro, sizeof(double) * nc);
        memcpy(U + nc, s->ru, sizeof(double) * nc);
        memcpy(U + 2 * (size_t)nc, s->rv, sizeof(double) * nc);
        memcpy(U + 3 * (size_t)nc, s->re, sizeof(double) * nc);
    }
    if (ctau) memcpy(ctau, s->cTau, sizeof(double) * nc);
    if (flags) memcpy(flags, s->flag, sizeof(unsigned) * nc);
}

/* The gradients minmod reconstructs from, in this project's arithmetic (the GPU's
 * grad_one_mm): per edge s = phi_1 + phi_2 and the weights a = RN(RN(n l) / 2); per cell
 * g = (sum over its edges in ascending order of +-s a, the first term taken as it is,
 * c2 subtracting) * RN(1/S). The same Green-Gauss formula as calcGrad's, rounded
 * differently. */
static void calc_grad_minmod(orc_solver* s) {
    const orc_mesh* m = s->m;
    double* g = s->grad;
    unsigned char* seen = (unsigned char*)calloc((size_t)m->nc, 1);
    if (!seen) abort();
    for (int e = 0; e < m->ne; e++) {
        int c1 = m->c1[e], c2 = m->c2[e];
        Par pL, pR;
        cons2par(s, c1, &pL);
        if (c2 > -1) cons2par(s, c2, &pR);
        else boundary_cond(s, e, &pL, &pR);
        double ax = m->nx[e] * m->l[e] * 0.5, ay = m->ny[e] * m->l[e] * 0.5;
        double sr = pL.r + pR.r, sp = pL.p + pR.p, su = pL.u + pR.u, sv = pL.v + pR.v;
        double v[8] = {sr * ax, sr * ay, sp * ax, sp * ay, su * ax, su * ay, sv * ax, sv * ay};
        double* g1 = g + 8 * (size_t)c1;
        for (int k = 0; k < 8; k++) g1[k] = seen[c1] ? g1[k] + v[k] : v[k];
        seen[c1] = 1;
        if (c2 > -1) {
            double* g2 = g + 8 * (size_t)c2;
            for (int k = 0; k < 8; k++) g2[k] = seen[c2] ? g2[k] + (-v[k]) : -v[k];
            seen[c2] = 1;
        }
    }
    for (int i = 0; i < m->nc; i++) {
        double y = 1.0 / m->S[i];
        for (int k = 0; k < 8; k++) g[8 * (size_t)i + k] *= y;
    }
    free(seen);
}

/* calcGrad, src/methods/fvm_tvd.cpp:242-301 */
static void calc_grad(orc_solver* s) {
    const orc_mesh* m = s->m;
    double* g = s->grad;
    if (s->p.recon == ORC_RECON_MINMOD) {
        calc_grad_minmod(s);
        return;
    }
    memset(g, 0, sizeof(double) * 8 * (size_t)m->nc);
    for (int e = 0; e < m->ne; e++) {
        int c1 = m->c1[e], c2 = m->c2[e];
        Par pL, pR;
        cons2par(s, c1, &pL);
        if (c2 > -1) cons2par(s, c2, &pR);
        else boundary_cond(s, e, &pL, &pR);
        double nx = m->nx[e], ny = m->ny[e], l = m->l[e];
        double v[8];
        v[0] = (pL.r + pR.r) / 2 * nx * l; v[1] = (pL.r + pR.r) / 2 * ny * l;
        v[2] = (pL.p + pR.p) / 2 * nx * l; v[3] = (pL.p + pR.p) / 2 * ny * l;
        v[4] = (pL.u + pR.u) / 2 * nx * l; v[5] = (pL.u + pR.u) / 2 * ny * l;
        v[6] = (pL.v + pR.v) / 2 * nx * l; v[7] = (pL.v + pR.v) / 2 * ny * l;
        for (int k = 0; k < 8; k++) g[8 * (size_t)c1 + k] += v[k];
        if (c2 > -1) for (int k = 0; k < 8; k++) g[8 * (size_t)c2 + k] -= v[k];
    }
    for (int i = 0; i < m->nc; i++) {
        double si = m->S[i];
        for (int k = 0; k < 8; k++) g[8 * (size_t)i + k] /= si;
    }
}

/* One side's reconstruction at point (px, py): phi += grad(phi) . (P - C),
 * src/methods/fvm_tvd.cpp:646-691; with MINMOD the increment is
 * minmod(grad(phi) . (P - C), phi_neighbour - phi). */
static void recon_side(const orc_solver* s, int c, double px, double py, Par* q, const Par* nb) {
    const orc_mesh* m = s->m;
    const double* g = s->grad + 8 * (size_t)c;
    double dx = px - m->cx[c], dy = py - m->cy[c];
    double dr, dp, du, dv;
    if (s->p.recon == ORC_RECON_MINMOD) { /* this project's limiter: fused projections */
        dr = dot2(g[0], dx, g[1], dy); dp = dot2(g[2], dx, g[3], dy);
        du = dot2(g[4], dx, g[5], dy); dv = dot2(g[6], dx, g[7], dy);
    } else {                              /* the reference's reconstruction, unfused */
        dr = g[0] * dx + g[1] * dy; dp = g[2] * dx + g[3] * dy;
        du = g[4] * dx + g[5] * dy; dv = g[6] * dx + g[7] * dy;
    }
    if (s->p.recon == ORC_RECON_MINMOD) {
        dr = minmod(dr, nb->r - q->r);
        dp = minmod(dp, nb->p - q->p);
        du = minmod(du, nb->u - q->u);
        dv = minmod(dv, nb->v - q->v);
    }
    q->r += dr; q->p += dp; q->u += du; q->v += dv;
}

static void face_states(const orc_solver* s, int e, int gp, Par* pL, Par* pR) {
    const orc_mesh* m = s->m;
    int c1 = m->c1[e], c2 = m->c2[e];
    double px = m->pts[6 * (size_t)e + 2 * gp], py = m->pts[6 * (size_t)e + 2 * gp + 1];
    cons2par(s, c1, pL);
    if (c2 > -1) {
        cons2par(s, c2, pR);
        if (s->p.recon != ORC_RECON_NONE) {
            Par cL = *pL, cR = *pR;
            recon_side(s, c1, px, py, pL, &cR);
            recon_side(s, c2, px, py, pR, &cL);
        }
    } else {
        if (s->p.recon != ORC_RECON_NONE) {
            Par ghost;
            if (s->p.recon == ORC_RECON_MINMOD) boundary_cond(s, e, pL, &ghost);
            recon_side(s, c1, px, py, pL, &ghost);
        }
        boundary_cond(s, e, pL, pR);
    }
}

static int calc_flux(const orc_solver* s, double* f, const Par* pL, const Par* pR, double nx, double ny) {
    double GAM = s->p.gam_flux;
    switch (s->p.flux) {
    case ORC_FLUX_LAX: flux_lax(f, pL, pR, nx, ny, GAM); return 0;
    case ORC_FLUX_ROE: flux_roe(f, pL, pR, nx, ny, GAM); return 0;
    case ORC_FLUX_HLLC: flux_hllc(f, pL, pR, nx, ny, GAM); return 0;
    default: return flux_godunov(f, pL, pR, nx, ny, GAM, s->p.newton_cap);
    }
}

/* Edge loop of one Runge-Kutta stage, src/methods/fvm_tvd.cpp:324-365 */
static void stage_residual(orc_solver* s) {
    const orc_mesh* m = s->m;
    int nc = m->nc;
    memset(s->ro_int, 0, sizeof(double) * nc); memset(s->ru_int, 0, sizeof(double) * nc);
    memset(s->rv_int, 0, sizeof(double) * nc); memset(s->re_int, 0, sizeof(double) * nc);
    if (s->p.recon != ORC_RECON_NONE) calc_grad(s);
    for (int e = 0; e < m->ne; e++) {
        int c1 = m->c1[e], c2 = m->c2[e];
        double nx = m->nx[e], ny = m->ny[e];
        double l = m->l[e] * 0.5;
        double fr = 0.0, fu = 0.0, fv = 0.0, fe = 0.0;
        for (int gp = 1; gp < m->npts[e]; gp++) {
            Par pL, pR; double f[4];
            face_states(s, e, gp, &pL, &pR);
            s->newton_hit |= calc_flux(s, f, &pL, &pR, nx, ny);
            if (gp == 1 && (s->p.flux == ORC_FLUX_HLLC || s->p.flux == ORC_FLUX_ROE)) {
                /* this project's fluxes start from the first point's flux */
                fr = f[0]; fu = f[1]; fv = f[2]; fe = f[3];
            } else {
                fr += f[0]; fu += f[1]; fv += f[2]; fe += f[3];
            }
        }
        s->ro_int[c1] -= fr * l; s->ru_int[c1] -= fu * l;
        s->rv_int[c1] -= fv * l; s->re_int[c1] -= fe * l;
        if (c2 > -1) {
            s->ro_int[c2] += fr * l; s->ru_int[c2] += fu * l;
            s->rv_int[c2] += fv * l; s->re_int[c2] += fe * l;
        }
    }
}

void orc_residual(orc_solver* s, double* R) {
    int nc = s->m->nc;
    stage_residual(s);
    memcpy(R, s->ro_int, sizeof(double) * nc);
    memcpy(R + nc, s->ru_int, sizeof(double) * nc);
    memcpy(R + 2 * (size_t)nc, s->rv_int, sizeof(double) * nc);
    memcpy(R + 3 * (size_t)nc, s->re_int, sizeof(double) * nc);
}

static int is_lim(const orc_solver* s, int i) { return (s->flag[i] & 0x2u) > 0; }

static void stage_update(orc_solver* s) { /* :366-374 */
    const orc_mesh* m = s->m;
    for (int i = 0; i < m->nc; i++) {
        if (is_lim(s, i)) continue;
        double cfl = s->cTau[i] / m->S[i];
        if (s->p.scheme == ORC_TIME_SSPRK3) { /* this project's scheme: fused */
            s->ro[i] = fma(cfl, s->ro_int[i], s->ro[i]); s->ru[i] = fma(cfl, s->ru_int[i], s->ru[i]);
            s->rv[i] = fma(cfl, s->rv_int[i], s->rv[i]); s->re[i] = fma(cfl, s->re_int[i], s->re[i]);
        } else {
            s->ro[i] += cfl * s->ro_int[i]; s->ru[i] += cfl * s->ru_int[i];
            s->rv[i] += cfl * s->rv_int[i]; s->re[i] += cfl * s->re_int[i];
        }
    }
}

static void check_limits(orc_solver* s, int i) { /* :439-446 */
    Par par; cons2par(s, i, &par);
    if (par.r < s->p.lim_rmin) s->flag[i] |= 0x2u;
    if (par.r > s->p.lim_rmax) s->flag[i] |= 0x2u;
    if (par.p < s->p.lim_pmin) s->flag[i] |= 0x2u;
    if (par.p > s->p.lim_pmax) s->flag[i] |= 0x2u;
    if (fabs(par.u) > s->p.lim_umax) s->flag[i] |= 0x2u;
    if (fabs(par.v) > s->p.lim_umax) s->flag[i] |= 0x2u;
}

static void remediate(orc_solver* s) { /* remediateLimCells, :464-499 */
    const orc_mesh* m = s->m;
    for (int i = 0; i < m->nc; i++) {
        if (!is_lim(s, i)) continue;
        double sRO = 0.0, sRU = 0.0, sRV = 0.0, sRE = 0.0, S = 0.0;
        for (int k = 0; k < 3; k++) {
            int j = m->c2[m->cedges[3 * i + k]];
            if (j >= 0) {
                double sj = m->S[j];
                S += sj;
                sRO += s->ro[j] * sj; sRU += s->ru[j] * sj; sRV += s->rv[j] * sj; sRE += s->re[j] * sj;
            }
        }
        s->ro[i] = sRO / S; s->ru[i] = sRU / S; s->rv[i] = sRV / S; s->re[i] = sRE / S;
        s->flag[i] += 0x010000u;
        if (s->flag[i] & 0x200000u) s->flag[i] &= 0x001110u;
    }
}

int orc_step(orc_solver* s, int nsteps) {
    const orc_mesh* m = s->m;
    int nc = m->nc;
    int nst = s->p.scheme == ORC_TIME_EULER ? 1 : (s->p.scheme == ORC_TIME_HEUN ? 2 : 3);
    const double c13 = 1.0 / 3.0, c23 = 2.0 / 3.0;
    s->newton_hit = 0;
    for (int step = 0; step < nsteps; step++) {
        if (!s->p.steady) s->t += s->TAU;
        else calc_time_step(s);
        memcpy(s->ro_old, s->ro, sizeof(double) * nc); memcpy(s->ru_old, s->ru, sizeof(double) * nc);
        memcpy(s->rv_old, s->rv, sizeof(double) * nc); memcpy(s->re_old, s->re, sizeof(double) * nc);
        for (int st = 0; st < nst; st++) {
            stage_residual(s);
            stage_update(s);
            if (s->p.scheme == ORC_TIME_SSPRK3 && st == 1)
                for (int i = 0; i < nc; i++) {
                    if (is_lim(s, i)) continue;
                    s->ro[i] = fma(0.25, s->ro[i], 0.75 * s->ro_old[i]);
                    s->ru[i] = fma(0.25, s->ru[i], 0.75 * s->ru_old[i]);
                    s->rv[i] = fma(0.25, s->rv[i], 0.75 * s->rv_old[i]);
                    s->re[i] = fma(0.25, s->re[i], 0.75 * s->re_old[i]);
                }
        }
        for (int i = 0; i < nc; i++) {
            if (is_lim(s, i)) continue;
            if (s->p.scheme == ORC_TIME_HEUN) { /* ICASE 97-65 eq. (4.10), :429-437 */
                s->ro[i] = 0.5 * (s->ro_old[i] + s->ro[i]); s->ru[i] = 0.5 * (s->ru_old[i] + s->ru[i]);
                s->rv[i] = 0.5 * (s->rv_old[i] + s->rv[i]); s->re[i] = 0.5 * (s->re_old[i] + s->re[i]);
            } else if (s->p.scheme == ORC_TIME_SSPRK3) { /* Shu-Osher third stage, fused */
                s->ro[i] = fma(c23, s->ro[i], c13 * s->ro_old[i]); s->ru[i] = fma(c23, s->ru[i], c13 * s->ru_old[i]);
                s->rv[i] = fma(c23, s->rv[i], c13 * s->rv_old[i]); s->re[i] = fma(c23, s->re[i], c13 * s->re_old[i]);
            }
            check_limits(s, i);
        }
        remediate(s);
    }
    return s->newton_hit;
}

void orc_solver_free(orc_solver* s) {
    if (!s) return;
    free(s->matM); free(s->matCp); free(s->cell_mat); free(s->bkind); free(s->bpar);
    free(s->ro); free(s->ru); free(s->rv); free(s->re);
    free(s->ro_old); free(s->ru_old); free(s->rv_old); free(s->re_old);
    free(s->ro_int); free(s->ru_int); free(s->rv_int); free(s->re_int);
    free(s->grad); free(s->cTau); free(s->flag);
    free(s);
}

/* ================================================================ FVM_TVD_IMPLICIT
 *
 * Restatement of the reference's implicit method (src/methods/fvm_tvd_implicit.cpp):
 * per step a Roe-linearised block system (S/cTau I + sum_faces l A+-) dU = -sum F l,
 * assembled by the reference's edge loop, solved by restarted GMRES, then the
 * reference's smoothing, update with limits, remediation and CFL control. The
 * reference solves with HYPRE's GMRES (src/methods/solvers/SolverHypreGmres.cpp),
 * which is not part of the reference tree; orc_gmres_block restates the published
 * GMRES (Saad and Schultz 1986, Givens rotations, modified Gram-Schmidt) with the
 * reference's parameters and HYPRE's stopping rule |r| <= eps |b|. */

struct orc_imp {
    const orc_mesh* m;
    orc_imp_params p;
    int nm;
    double *matM, *matCp;
    int* cell_mat;
    int nbnd;
    int* bkind;
    double* bpar;               /* nbnd x (T, P, Vx, Vy), the order of Boundary::par */
    double *ro, *ru, *rv, *re;
    double* grad;               /* nc x 8 */
    double* cTau;
    double* tmpArr;
    int* tmpArrInt;
    unsigned* flag;
    double *diag, *off, *rhs;   /* nc x 16, nc x 3 x 16 (faces in Cell::edgesInd order), nc x 4 */
    int* nbr;                   /* nc x 3: the cell across each face, -1 on the boundary */
    double* x;                  /* 4 nc, x[4 c + k] like MatrixSolver::x */
    double t, CFL;
    int step, solverErr;
    int last_iters, last_status;
    double last_rel;
    int newton_hit;
};

/* FVM_TVD_IMPLICIT::convertConsToPar, :1058-1068 (URS(0) then URS(1)) */
static void imp_cons2par(const orc_imp* s, int i, Par* par) {
    int mt = s->cell_mat[i];
    par->r = s->ro[i];
    par->u = s->ru[i] / s->ro[i];
    par->v = s->rv[i] / s->ro[i];
    par->E = s->re[i] / s->ro[i];
    par->e = par->E - 0.5 * (par->u * par->u + par->v * par->v);
    urs(s->matM[mt], s->matCp[mt], par, 0);
    urs(s->matM[mt], s->matCp[mt], par, 1);
}

/* FVM_TVD_IMPLICIT::convertParToCons, :1050-1056 */
static void imp_par2cons(orc_imp* s, int i, const Par* par) {
    s->ro[i] = par->r;
    s->ru[i] = par->r * par->u;
    s->rv[i] = par->r * par->v;
    s->re[i] = par->r * (par->e + 0.5 * (par->u * par->u + par->v * par->v));
}

/* FVM_TVD_IMPLICIT::boundaryCond, :963-1008 */
static void imp_boundary(const orc_imp* s, int e, const Par* pL, Par* pR) {
    const orc_mesh* m = s->m;
    int b = m->bnd[e];
    const double* bp = s->bpar + 4 * b;
    int mt = s->cell_mat[m->c1[e]];
    switch (s->bkind[b]) {
    case ORC_IBND_INLET:
        pR->T = bp[0]; pR->p = bp[1]; pR->u = bp[2]; pR->v = bp[3];
        urs(s->matM[mt], s->matCp[mt], pR, 2);
        urs(s->matM[mt], s->matCp[mt], pR, 1);
        break;
    case ORC_IBND_OUTLET:
        *pR = *pL;
        break;
    default: { /* BOUND_WALL */
        *pR = *pL;
        double Un = pL->u * m->nx[e] + pL->v * m->ny[e];
        double Vx = m->nx[e] * Un * 2.0, Vy = m->ny[e] * Un * 2.0;
        pR->u = pL->u - Vx;
        pR->v = pL->v - Vy;
    }
    }
}

/* reconstruct(iFace, pL, pR), :431-442: the cell-centre states */
static void imp_centre_states(const orc_imp* s, int e, Par* pL, Par* pR) {
    const orc_mesh* m = s->m;
    imp_cons2par(s, m->c1[e], pL);
    if (m->c2[e] > -1) imp_cons2par(s, m->c2[e], pR);
    else imp_boundary(s, e, pL, pR);
}

/* reconstruct(iFace, pL, pR, p), :444-476: linear on interior faces, centre + ghost on the boundary */
static void imp_point_states(const orc_imp* s, int e, int gp, Par* pL, Par* pR) {
    const orc_mesh* m = s->m;
    int c1 = m->c1[e], c2 = m->c2[e];
    double px = m->pts[6 * (size_t)e + 2 * gp], py = m->pts[6 * (size_t)e + 2 * gp + 1];
    if (c2 > -1) {
        imp_cons2par(s, c1, pL);
        imp_cons2par(s, c2, pR);
        const double* g1 = s->grad + 8 * (size_t)c1;
        const double* g2 = s->grad + 8 * (size_t)c2;
        double d1x = px - m->cx[c1], d1y = py - m->cy[c1];
        double d2x = px - m->cx[c2], d2y = py - m->cy[c2];
        pL->r += g1[0] * d1x + g1[1] * d1y;
        pL->p += g1[2] * d1x + g1[3] * d1y;
        pL->u += g1[4] * d1x + g1[5] * d1y;
        pL->v += g1[6] * d1x + g1[7] * d1y;
        pR->r += g2[0] * d2x + g2[1] * d2y;
        pR->p += g2[2] * d2x + g2[3] * d2y;
        pR->u += g2[4] * d2x + g2[5] * d2y;
        pR->v += g2[6] * d2x + g2[7] * d2y;
    } else {
        imp_cons2par(s, c1, pL);
        imp_boundary(s, e, pL, pR);
    }
}

/* FVM_TVD_IMPLICIT::calcGrad, :186-252 */
static void imp_calc_grad(orc_imp* s) {
    const orc_mesh* m = s->m;
    double* g = s->grad;
    memset(g, 0, sizeof(double) * 8 * (size_t)m->nc);
    for (int e = 0; e < m->ne; e++) {
        int c1 = m->c1[e], c2 = m->c2[e];
        Par pL, pR;
        imp_centre_states(s, e, &pL, &pR);
        double nx = m->nx[e], ny = m->ny[e], l = m->l[e];
        double v[8];
        v[0] = (pL.r + pR.r) / 2 * nx * l; v[1] = (pL.r + pR.r) / 2 * ny * l;
        v[2] = (pL.p + pR.p) / 2 * nx * l; v[3] = (pL.p + pR.p) / 2 * ny * l;
        v[4] = (pL.u + pR.u) / 2 * nx * l; v[5] = (pL.u + pR.u) / 2 * ny * l;
        v[6] = (pL.v + pR.v) / 2 * nx * l; v[7] = (pL.v + pR.v) / 2 * ny * l;
        for (int k = 0; k < 8; k++) g[8 * (size_t)c1 + k] += v[k];
        if (c2 > -1) for (int k = 0; k < 8; k++) g[8 * (size_t)c2 + k] -= v[k];
    }
    for (int i = 0; i < m->nc; i++) {
        double si = m->S[i];
        for (int k = 0; k < 8; k++) g[8 * (size_t)i + k] /= si;
    }
}

/* roe_orig, src/global.cpp:407-441 (W components 0) */
static void roe_average(Par* a, const Par* pL, const Par* pR, double GAM) {
    double AGAM = (GAM - 1.0);
    double fG = GAM;
    double fSB = sqrt(pL->r), fSE = sqrt(pR->r);
    double fS_ = 1.0 / (fSB + fSE);
    double RI = fSB * fSE;
    double UI = (fSB * pL->u + fSE * pR->u) * fS_;
    double VI = (fSB * pL->v + fSE * pR->v) * fS_;
    double WI = (fSB * 0.0 + fSE * 0.0) * fS_;
    double EB = pL->p / (pL->r * AGAM), EE = pR->p / (pR->r * AGAM);
    double HB = EB + (pL->u * pL->u + pL->v * pL->v + 0.0 * 0.0) * 0.5 + pL->p / pL->r;
    double HE = EE + (pR->u * pR->u + pR->v * pR->v + 0.0 * 0.0) * 0.5 + pR->p / pR->r;
    double HI = (fSB * HB + fSE * HE) * fS_;
    double PI = (HI - (UI * UI + VI * VI + WI * WI) * 0.5) * RI * (fG - 1.0) / fG;
    double EI = PI / (RI * AGAM);
    /* calcRoeAverage, :408-429 */
    a->r = RI; a->e = EI; a->p = PI; a->u = UI; a->v = VI;
    a->cz = sqrt(GAM * a->p / a->r);
    a->E = a->e + 0.5 * (a->u * a->u + a->v * a->v);
}

typedef double M4[4][4];

static void mult4(M4 d, M4 a, M4 b) { /* multMtx4, :264-277 */
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double sum = 0;
            for (int k = 0; k < 4; ++k) sum += a[i][k] * b[k][j];
            d[i][j] = sum;
        }
}

/* eigenValues / rightEigenVector / leftEigenVector, :335-370 */
static void eigen_values(M4 d, double c, double u, double nx, double v, double ny) {
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) d[i][j] = 0;
    double qn = u * nx + v * ny;
    d[0][0] = qn - c; d[1][1] = qn; d[2][2] = qn + c; d[3][3] = qn;
}
static void right_eigen(M4 d, double c, double u, double nx, double v, double ny, double H) {
    double qn = u * nx + v * ny, q2 = u * u + v * v;
    double lx = -ny, ly = nx;
    double ql = u * lx + v * ly;
    d[0][0] = 1.0;         d[0][1] = 1.0;    d[0][2] = 1.0;         d[0][3] = 0.0;
    d[1][0] = u - c * nx;  d[1][1] = u;      d[1][2] = u + c * nx;  d[1][3] = lx;
    d[2][0] = v - c * ny;  d[2][1] = v;      d[2][2] = v + c * ny;  d[2][3] = ly;
    d[3][0] = H - qn * c;  d[3][1] = q2 / 2; d[3][2] = H + qn * c;  d[3][3] = ql;
}
static void left_eigen(M4 d, double c, double GAM, double u, double nx, double v, double ny) {
    double qn = u * nx + v * ny, q2 = u * u + v * v;
    double lx = -ny, ly = nx;
    double ql = u * lx + v * ly;
    double g1 = GAM - 1.0, c2 = c * c;
    d[0][0] = 0.5 * (0.5 * q2 * g1 / c2 + qn / c); d[0][1] = -0.5 * (g1 * u / c2 + nx / c);
    d[0][2] = -0.5 * (g1 * v / c2 + ny / c);      d[0][3] = 0.5 * g1 / c2;
    d[1][0] = 1 - 0.5 * q2 * g1 / c2;             d[1][1] = g1 * u / c2;
    d[1][2] = g1 * v / c2;                        d[1][3] = -g1 / c2;
    d[2][0] = 0.5 * (0.5 * q2 * g1 / c2 - qn / c); d[2][1] = -0.5 * (g1 * u / c2 - nx / c);
    d[2][2] = -0.5 * (g1 * v / c2 - ny / c);      d[2][3] = 0.5 * g1 / c2;
    d[3][0] = -ql;                                d[3][1] = lx;
    d[3][2] = ly;                                 d[3][3] = 0;
}
/* calcAP / calcAM, :371-406: 0.5 R diag(max(lam,0)) L, 0.5 R diag(min(lam,0)) L */
static void calc_apm(M4 d, M4 R, M4 E, M4 L, int plus) {
    M4 t;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            d[i][j] = plus ? (E[i][j] > 0 ? E[i][j] : 0) : (E[i][j] < 0 ? E[i][j] : 0);
    mult4(t, R, d);
    mult4(d, t, L);
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) d[i][j] *= 0.5;
}

/* A+ and A- of face normal (nx, ny), times l */
static void jacobians(const Par* a, double GAM, double nx, double ny, double l, M4 AP, M4 AM) {
    M4 E, R, L;
    double H = a->E + a->p / a->r;
    eigen_values(E, a->cz, a->u, nx, a->v, ny);
    right_eigen(R, a->cz, a->u, nx, a->v, ny, H);
    left_eigen(L, a->cz, GAM, a->u, nx, a->v, ny);
    calc_apm(AP, R, E, L, 1);
    calc_apm(AM, R, E, L, 0);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) { AM[i][j] *= l; AP[i][j] *= l; }
}

static void blk_add(double* b, M4 a) { for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) b[4 * i + j] += a[i][j]; }
static int face_slot(const orc_mesh* m, int c, int e) {
    for (int k = 0; k < 3; k++) if (m->cedges[3 * c + k] == e) return k;
    return -1;
}

/* calcFlux, :917-961 */
static int imp_flux(const orc_imp* s, double* f, const Par* pL, const Par* pR, double nx, double ny, double GAM) {
    if (s->p.flux == ORC_FLUX_LAX) { flux_lax(f, pL, pR, nx, ny, GAM); return 0; }
    return flux_godunov(f, pL, pR, nx, ny, GAM, s->p.newton_cap);
}

/* The edge loop of FVM_TVD_IMPLICIT::run, :541-634, and the diagonal of :640-664. */
static void imp_assemble(orc_imp* s) {
    const orc_mesh* m = s->m;
    int nc = m->nc;
    const double GAM = 1.4; /* __GAM, :536 */
    memset(s->diag, 0, sizeof(double) * 16 * (size_t)nc);
    memset(s->off, 0, sizeof(double) * 48 * (size_t)nc);
    memset(s->rhs, 0, sizeof(double) * 4 * (size_t)nc);
    memset(s->tmpArr, 0, sizeof(double) * (size_t)nc);
    imp_calc_grad(s);
    for (int e = 0; e < m->ne; e++) {
        int c1 = m->c1[e], c2 = m->c2[e];
        double l = m->l[e], nx = m->nx[e], ny = m->ny[e];
        Par cellL, cellR, avg;
        imp_centre_states(s, e, &cellL, &cellR);
        roe_average(&avg, &cellL, &cellR, GAM);
        if (s->p.steady) {
            double lambda = sqrt(avg.u * avg.u + avg.v * avg.v) + avg.cz;
            lambda *= l;
            s->tmpArr[c1] += lambda;
            if (c2 >= 0) s->tmpArr[c2] += lambda;
        }
        M4 AP, AM;
        jacobians(&avg, GAM, nx, ny, l, AP, AM);
        blk_add(s->diag + 16 * (size_t)c1, AP);
        if (c2 >= 0) {
            blk_add(s->off + 48 * (size_t)c1 + 16 * face_slot(m, c1, e), AM);
            jacobians(&avg, GAM, -nx, -ny, l, AP, AM);
            blk_add(s->diag + 16 * (size_t)c2, AP);
            blk_add(s->off + 48 * (size_t)c2 + 16 * face_slot(m, c2, e), AM);
        }
        /* the flux of the centre states (:608) is computed by the reference and unused */
        double fr = 0.0, fu = 0.0, fv = 0.0, fe = 0.0;
        for (int gp = 1; gp < m->npts[e]; ++gp) {
            double f[4];
            imp_point_states(s, e, gp, &cellL, &cellR);
            s->newton_hit |= imp_flux(s, f, &cellL, &cellR, nx, ny, GAM);
            fr += f[0]; fu += f[1]; fv += f[2]; fe += f[3];
        }
        double* b1 = s->rhs + 4 * (size_t)c1;
        b1[0] -= 0.5 * l * fr; b1[1] -= 0.5 * l * fu; b1[2] -= 0.5 * l * fv; b1[3] -= 0.5 * l * fe;
        if (c2 >= 0) {
            double* b2 = s->rhs + 4 * (size_t)c2;
            b2[0] += 0.5 * l * fr; b2[1] += 0.5 * l * fu; b2[2] += 0.5 * l * fv; b2[3] += 0.5 * l * fe;
        }
    }
    if (s->p.steady)
        for (int i = 0; i < nc; i++) s->cTau[i] = 2.0 * s->CFL * m->S[i] / (s->tmpArr[i] + 1.0e-100);
    for (int i = 0; i < nc; i++) {
        M4 d;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) d[a][b] = a == b ? m->S[i] / s->cTau[i] : 0.0;
        blk_add(s->diag + 16 * (size_t)i, d);
    }
}

/* y = A x of the block system: per cell its diagonal block, then its faces' blocks in order */
static void block_matvec(int nc, const int* nbr, const double* diag, const double* off, const double* x, double* y) {
    for (int c = 0; c < nc; c++)
        for (int i = 0; i < 4; i++) {
            double sum = 0.0;
            const double* d = diag + 16 * (size_t)c + 4 * i;
            for (int j = 0; j < 4; j++) sum += d[j] * x[4 * (size_t)c + j];
            for (int k = 0; k < 3; k++) {
                int nb = nbr[3 * (size_t)c + k];
                if (nb < 0) continue;
                const double* o = off + 48 * (size_t)c + 16 * k + 4 * i;
                for (int j = 0; j < 4; j++) sum += o[j] * x[4 * (size_t)nb + j];
            }
            y[4 * (size_t)c + i] = sum;
        }
}

static double vdot(size_t n, const double* a, const double* b) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

int orc_gmres_block(int nc, const int* nbr, const double* diag, const double* off, const double* b, double* x,
                    double eps, int maxit, int kdim, int* iters, double* final_rel) {
    size_t n = 4 * (size_t)nc;
    int m = kdim < 1 ? 1 : kdim;
    double* V = (double*)calloc(n * (size_t)(m + 1), sizeof(double));
    double* w = (double*)malloc(sizeof(double) * (n ? n : 1));
    double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double)); /* H[i*m + j] */
    double* cs = (double*)calloc((size_t)m, sizeof(double));
    double* sn = (double*)calloc((size_t)m, sizeof(double));
    double* g = (double*)calloc((size_t)m + 1, sizeof(double));
    double* y = (double*)calloc((size_t)m, sizeof(double));
    memset(x, 0, sizeof(double) * n);
    double bnorm = sqrt(vdot(n, b, b));
    double epsilon = eps * bnorm;
    int it = 0, status = 0;
    double rnorm = bnorm;
    memcpy(w, b, sizeof(double) * n); /* r0 = b - A 0 */
    if (bnorm > 0.0) {
        for (;;) { /* restart cycles */
            double beta = sqrt(vdot(n, w, w));
            rnorm = beta;
            if (beta <= epsilon || it >= maxit) break;
            for (size_t q = 0; q < n; q++) V[q] = w[q] / beta;
            memset(g, 0, sizeof(double) * (size_t)(m + 1));
            g[0] = beta;
            int j = 0;
            for (; j < m && it < maxit; j++) {
                it++;
                double* vj1 = V + n * (size_t)(j + 1);
                block_matvec(nc, nbr, diag, off, V + n * (size_t)j, vj1);
                for (int i = 0; i <= j; i++) { /* modified Gram-Schmidt */
                    double h = vdot(n, vj1, V + n * (size_t)i);
                    H[i * m + j] = h;
                    for (size_t q = 0; q < n; q++) vj1[q] -= h * V[n * (size_t)i + q];
                }
                double hn = sqrt(vdot(n, vj1, vj1));
                H[(j + 1) * m + j] = hn;
                if (hn != 0.0) for (size_t q = 0; q < n; q++) vj1[q] /= hn;
                for (int i = 0; i < j; i++) { /* previous rotations */
                    double a = H[i * m + j], c = H[(i + 1) * m + j];
                    H[i * m + j] = cs[i] * a + sn[i] * c;
                    H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
                }
                double a = H[j * m + j], c = H[(j + 1) * m + j];
                double r = sqrt(a * a + c * c);
                if (r == 0.0) { cs[j] = 1.0; sn[j] = 0.0; }
                else { cs[j] = a / r; sn[j] = c / r; }
                H[j * m + j] = cs[j] * a + sn[j] * c;
                H[(j + 1) * m + j] = 0.0;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                rnorm = fabs(g[j + 1]);
                if (rnorm <= epsilon) { j++; break; }
            }
            for (int i = j - 1; i >= 0; i--) { /* back substitution */
                double sum = g[i];
                for (int k = i + 1; k < j; k++) sum -= H[i * m + k] * y[k];
                y[i] = sum / H[i * m + i];
            }
            for (int i = 0; i < j; i++)
                for (size_t q = 0; q < n; q++) x[q] += y[i] * V[n * (size_t)i + q];
            block_matvec(nc, nbr, diag, off, x, w); /* the true residual */
            for (size_t q = 0; q < n; q++) w[q] = b[q] - w[q];
            rnorm = sqrt(vdot(n, w, w));
            if (rnorm <= epsilon || it >= maxit) break;
        }
    }
    double rel = bnorm > 0.0 ? rnorm / bnorm : 0.0;
    if (it >= maxit) status |= ORC_SOLVE_MAX_ITER;
    if (rel >= eps || !isfinite(rel)) status |= ORC_SOLVE_CONVERG;
    if (iters) *iters = it;
    if (final_rel) *final_rel = rel;
    free(V); free(w); free(H); free(cs); free(sn); free(g); free(y);
    return status;
}

/* smoothingDelta, :790-808 */
static void imp_smoothing(orc_imp* s, double* p) {
    const orc_mesh* m = s->m;
    for (int shift = 0; shift < 4; shift++) {
        memset(s->tmpArr, 0, sizeof(double) * (size_t)m->nc);
        memset(s->tmpArrInt, 0, sizeof(int) * (size_t)m->nc);
        for (int e = 0; e < m->ne; e++) {
            if (m->c2[e] >= 0) {
                int c1 = m->c1[e], c2 = m->c2[e];
                if (!(s->flag[c2] & 0x2u)) { s->tmpArr[c1] += p[c2 * 4 + shift]; s->tmpArrInt[c1]++; }
                if (!(s->flag[c1] & 0x2u)) { s->tmpArr[c2] += p[c1 * 4 + shift]; s->tmpArrInt[c2]++; }
            }
        }
        for (int i = 0; i < m->nc; i++) {
            int q = i * 4 + shift;
            p[q] = (p[q] + s->p.smoothing_par * s->tmpArr[i]) / (1.0 + s->p.smoothing_par * s->tmpArrInt[i]);
        }
    }
}

/* FVM_TVD_IMPLICIT::remediateLimCells, :740-780 */
static void imp_remediate(orc_imp* s) {
    const orc_mesh* m = s->m;
    for (int i = 0; i < m->nc; i++) {
        if (!(s->flag[i] & 0x2u)) continue;
        double sRO = 0.0, sRU = 0.0, sRV = 0.0, sRE = 0.0, S = 0.0;
        for (int k = 0; k < 3; k++) {
            int e = m->cedges[3 * i + k];
            int j = m->c2[e];
            if (j == i) j = m->c1[e];
            if (j >= 0) {
                double sj = m->S[j];
                S += sj;
                sRO += s->ro[j] * sj; sRU += s->ru[j] * sj; sRV += s->rv[j] * sj; sRE += s->re[j] * sj;
            }
        }
        if (S >= s->p.tau_xml * s->p.tau_xml) {
            s->ro[i] = sRO / S; s->ru[i] = sRU / S; s->rv[i] = sRV / S; s->re[i] = sRE / S;
        }
        s->flag[i] += 0x010000u;
        if (s->flag[i] & 0x200000u) s->flag[i] &= 0x001110u;
    }
}

static void imp_dec_cfl(orc_imp* s) { /* :1070-1077 */
    if (s->CFL > 0.1) { s->CFL *= 0.75; if (s->CFL < 0.1) s->CFL = 0.1; }
}
static void imp_inc_cfl(orc_imp* s) { /* :1079-1086 */
    if (s->CFL < s->p.cfl_max) { s->CFL *= s->p.cfl_scale; if (s->CFL > s->p.cfl_max) s->CFL = s->p.cfl_max; }
}

int orc_imp_create(const orc_mesh* m, const orc_imp_params* prm, int nm, const double* mat, const int* cell_mat,
                   int nbnd, const int* bnd_kind, const double* bnd_par, const double* U0, orc_imp** out) {
    orc_imp* s = (orc_imp*)calloc(1, sizeof(orc_imp));
    int nc = m->nc;
    s->m = m; s->p = *prm; s->nm = nm; s->nbnd = nbnd;
    s->matM = dalloc(nm); s->matCp = dalloc(nm);
    for (int k = 0; k < nm; k++) { s->matM[k] = mat[2 * k]; s->matCp[k] = mat[2 * k + 1]; }
    s->cell_mat = (int*)malloc(sizeof(int) * (size_t)(nc > 0 ? nc : 1));
    memcpy(s->cell_mat, cell_mat, sizeof(int) * (size_t)nc);
    s->bkind = (int*)malloc(sizeof(int) * (size_t)(nbnd > 0 ? nbnd : 1));
    s->bpar = dalloc(4 * nbnd);
    if (nbnd) { memcpy(s->bkind, bnd_kind, sizeof(int) * nbnd); memcpy(s->bpar, bnd_par, sizeof(double) * 4 * nbnd); }
    s->ro = dalloc(nc); s->ru = dalloc(nc); s->rv = dalloc(nc); s->re = dalloc(nc);
    s->grad = dalloc(8 * nc);
    s->cTau = dalloc(nc);
    s->tmpArr = dalloc(nc);
    s->tmpArrInt = (int*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(int));
    s->flag = (unsigned*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(unsigned));
    s->diag = dalloc(16 * nc); s->off = dalloc(48 * nc); s->rhs = dalloc(4 * nc); s->x = dalloc(4 * nc);
    s->nbr = (int*)malloc(sizeof(int) * 3 * (size_t)(nc > 0 ? nc : 1));
    for (int c = 0; c < nc; c++)
        for (int k = 0; k < 3; k++) {
            int e = m->cedges[3 * c + k];
            int j = m->c1[e] == c ? m->c2[e] : m->c1[e];
            s->nbr[3 * c + k] = j;
        }
    for (int e = 0; e < m->ne; e++)
        if (m->c2[e] < 0 && (m->bnd[e] < 0 || m->bnd[e] >= nbnd)) { orc_imp_free(s); return -1; }
    orc_imp_set_state(s, U0);
    s->CFL = prm->cfl;
    if (!prm->steady) for (int i = 0; i < nc; i++) s->cTau[i] = prm->tau_xml; /* calcTimeStep, :296-333 */
    *out = s;
    return 0;
}

void orc_imp_set_state(orc_imp* s, const double* U) {
    int nc = s->m->nc;
    memcpy(s->ro, U, sizeof(double) * nc);
    memcpy(s->ru, U + nc, sizeof(double) * nc);
    memcpy(s->rv, U + 2 * (size_t)nc, sizeof(double) * nc);
    memcpy(s->re, U + 3 * (size_t)nc, sizeof(double) * nc);
}

void orc_imp_get_state(const orc_imp* s, double* U, double* ctau, unsigned* flags) {
    int nc = s->m->nc;
    if (U) {
        memcpy(U, s->ro, sizeof(double) * nc);
        memcpy(U + nc, s->ru, sizeof(double) * nc);
        memcpy(U + 2 * (size_t)nc, s->rv, sizeof(double) * nc);
        memcpy(U + 3 * (size_t)nc, s->re, sizeof(double) * nc);
    }
    if (ctau) memcpy(ctau, s->cTau, sizeof(double) * nc);
    if (flags) memcpy(flags, s->flag, sizeof(unsigned) * nc);
}

void orc_imp_system(orc_imp* s, double* diag, double* off, double* rhs, double* ctau) {
    int nc = s->m->nc;
    imp_assemble(s);
    if (diag) memcpy(diag, s->diag, sizeof(double) * 16 * (size_t)nc);
    if (off) memcpy(off, s->off, sizeof(double) * 48 * (size_t)nc);
    if (rhs) memcpy(rhs, s->rhs, sizeof(double) * 4 * (size_t)nc);
    if (ctau) memcpy(ctau, s->cTau, sizeof(double) * nc);
}

/* Apply the update of a solved system: :675-692, then remediation and the CFL rules. */
static void imp_apply(orc_imp* s, const double* dx) {
    const orc_mesh* m = s->m;
    const double GAM = 1.4;
    for (int c = 0, ind = 0; c < m->nc; c++, ind += 4) {
        if (s->flag[c] & 0x2u) continue;
        s->ro[c] += dx[ind + 0]; s->ru[c] += dx[ind + 1];
        s->rv[c] += dx[ind + 2]; s->re[c] += dx[ind + 3];
        Par par; imp_cons2par(s, c, &par);
        if (par.r > s->p.lim_rmax) { par.r = s->p.lim_rmax; s->flag[c] |= 0x2u; }
        if (par.r < s->p.lim_rmin) { par.r = s->p.lim_rmin; s->flag[c] |= 0x2u; }
        if (fabs(par.u) > s->p.lim_umax) { par.u = s->p.lim_umax * par.u / fabs(par.u); s->flag[c] |= 0x2u; }
        if (fabs(par.v) > s->p.lim_umax) { par.v = s->p.lim_umax * par.v / fabs(par.v); s->flag[c] |= 0x2u; }
        if (par.p > s->p.lim_pmax) { par.p = s->p.lim_pmax; s->flag[c] |= 0x2u; }
        if (par.p < s->p.lim_pmin) { par.p = s->p.lim_pmin; s->flag[c] |= 0x2u; }
        if (s->flag[c] & 0x2u) { par.e = par.p / ((GAM - 1) * par.r); imp_par2cons(s, c, &par); }
    }
    imp_remediate(s);
}

int orc_imp_lim_count(const orc_imp* s) {
    int n = 0;
    for (int i = 0; i < s->m->nc; i++) if (s->flag[i] & 0x2u) n++;
    return n;
}

/* nsteps passes of the loop body of FVM_TVD_IMPLICIT::run, :527-735 */
int orc_imp_step(orc_imp* s, int nsteps) {
    s->newton_hit = 0;
    for (int k = 0; k < nsteps; k++) {
        if (!s->p.steady) s->t += s->p.tau_xml;
        if (!s->solverErr) s->step++;
        imp_assemble(s);
        int iters = 0; double rel = 0.0;
        s->solverErr = orc_gmres_block(s->m->nc, s->nbr, s->diag, s->off, s->rhs, s->x, s->p.gmres_eps,
                                       s->p.gmres_maxit, s->p.gmres_kdim, &iters, &rel);
        s->last_iters = iters; s->last_rel = rel; s->last_status = s->solverErr;
        if (s->solverErr == 0) {
            if (s->p.smoothing) imp_smoothing(s, s->x);
            imp_apply(s, s->x);
            int lim = orc_imp_lim_count(s);
            if (s->p.steady && lim >= s->p.max_lim_cells) imp_dec_cfl(s);
            if (s->p.steady && s->p.cfl_step > 0 && s->step % s->p.cfl_step == 0) imp_inc_cfl(s);
        } else {
            if (s->p.steady) imp_dec_cfl(s);
            else s->solverErr = 0;
        }
    }
    return s->newton_hit;
}

void orc_imp_info(const orc_imp* s, double* t, double* cfl, int* step, int* iters, double* rel, int* status) {
    if (t) *t = s->t;
    if (cfl) *cfl = s->CFL;
    if (step) *step = s->step;
    if (iters) *iters = s->last_iters;
    if (rel) *rel = s->last_rel;
    if (status) *status = s->last_status;
}

void orc_imp_free(orc_imp* s) {
    if (!s) return;
    free(s->matM); free(s->matCp); free(s->cell_mat); free(s->bkind); free(s->bpar);
    free(s->ro); free(s->ru); free(s->rv); free(s->re);
    free(s->grad); free(s->cTau); free(s->tmpArr); free(s->tmpArrInt); free(s->flag);
    free(s->diag); free(s->off); free(s->rhs); free(s->x); free(s->nbr);
    free(s);
}
