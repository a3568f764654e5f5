/*
 * cfd2d oracle: a plain-C restatement of the reference's explicit finite-volume
 * solver FVM_TVD (src/methods/fvm_tvd.cpp) and of the pieces it calls.
 *
 * TEST INFRASTRUCTURE ONLY. The product (libcfd2d_gpu.so) never links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, to check the GPU results against.
 *
 * Parity: pinned against the reference's own FVM_TVD compiled from its sources
 * (oracle/Makefile, target "reference") on the fixtures in tests/golden/: in the
 * reference's only mode (exact Godunov flux, unlimited linear reconstruction,
 * Heun) this restatement reproduces the reference's state bit for bit.
 * Options the reference does not have (Lax-Friedrichs, Roe, HLLC, minmod,
 * explicit Euler, SSP-RK3) reuse the same structure, conventions and ghost
 * states; their formulas are the published ones named at each function.
 *
 * The implicit method (orc_imp_*) is pinned the same way against the reference's
 * FVM_TVD_IMPLICIT compiled from its sources (oracle/ref/ref_implicit.cpp), which
 * needs a matrix solver in place of HYPRE (absent from the reference tree): both
 * sides then use orc_gmres_block, and the assembled systems, updates, limits,
 * remediation and CFL control agree bit for bit. The GMRES itself follows the
 * published algorithm (parity unpinned against HYPRE's own code).
 *
 * Arithmetic order follows the reference expression by expression; build with
 * -ffp-contract=off so no multiply-add is fused.
 */
#ifndef CFD2D_ORACLE_H
#define CFD2D_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FLUX_GODUNOV = 0, ORC_FLUX_LAX = 1, ORC_FLUX_ROE = 2, ORC_FLUX_HLLC = 3 };
enum { ORC_RECON_NONE = 0, ORC_RECON_LINEAR = 1, ORC_RECON_MINMOD = 2 };
enum { ORC_TIME_EULER = 0, ORC_TIME_HEUN = 1, ORC_TIME_SSPRK3 = 2 };
enum { ORC_BND_INLET = 1, ORC_BND_OUTLET = 2, ORC_BND_WALL_SLIP = 3, ORC_BND_WALL_NO_SLIP = 4 };

typedef struct orc_mesh orc_mesh;
typedef struct orc_solver orc_solver;

typedef struct {
    int flux, recon, scheme, steady;
    int newton_cap;          /* Godunov Newton iteration cap; 0 = none (the reference has none) */
    int pad;
    double tau_xml, cfl;
    double lim_rmin, lim_rmax, lim_pmin, lim_pmax, lim_umax;
    double gam_flux;         /* the reference hard-codes 1.4 in FVM_TVD::run */
} orc_params;

/* Edge structure by the Salome-UNV reader's rules (3 points per edge: midpoint +
 * 2 Gauss points; normals flipped outward from c1), or by the Berkeley-Triangle
 * reader's rules when berkeley == 1 (1 point per edge, neighbour j opposite node j
 * taken from neigh[], no flip), or by Grid::initFromFiles (src/mesh/grid.cpp:51-252,
 * the loader of FVM_TVD_IMPLICIT) when berkeley == 2: the Triangle topology with
 * the midpoint and 2 Gauss points per edge. bseg: nb node pairs, bseg_bnd: their
 * boundary index. Returns 0 or a negative error. */
int orc_mesh_build(int nn, const double* xy, int nc, const int* tri, const int* neigh_berkeley,
                   int nb, const int* bseg, const int* bseg_bnd, int berkeley, orc_mesh** out);
void orc_mesh_sizes(const orc_mesh* m, int* nc, int* ne);
void orc_mesh_export(const orc_mesh* m, int* cell_edges, double* cell_S, double* cell_c,
                     int* edge_n12, int* edge_c12, int* edge_bnd, int* edge_npts,
                     double* edge_n, double* edge_l, double* edge_pts);
void orc_mesh_free(orc_mesh* m);

/* Region state the way FVM_TVD::init forms it: URS(2), URS(1), convertParToCons. */
void orc_region_state(double M, double Cp, double u, double v, double T, double p, double* U4);

/* mat: nm x (M, Cp); cell_mat[nc]; bnd_kind[nbnd]; bnd_par: nbnd x (Vx, Vy, T, P);
 * U0: 4 x nc (rho | rho u | rho v | rho E). Computes TAU as FVM_TVD::init does. */
int orc_solver_create(const orc_mesh* m, const orc_params* prm, int nm, const double* mat,
                      const int* cell_mat, int nbnd, const int* bnd_kind, const double* bnd_par,
                      const double* U0, orc_solver** out);
double orc_tau(const orc_solver* s);
/* Advance nsteps steps of FVM_TVD::run's loop body. Returns 0, or 1 if the
 * Newton cap was hit at least once. */
int orc_step(orc_solver* s, int nsteps);
void orc_get_state(const orc_solver* s, double* U4, double* ctau, unsigned* flags);
void orc_set_state(orc_solver* s, const double* U4);
/* R = residual of the current state (one stage's right-hand side, the
 * reference's ro_int..re_int after the edge loop), 4 x nc. */
void orc_residual(orc_solver* s, double* R4);
void orc_solver_free(orc_solver* s);

/* ---------------------------------------------------------------- FVM_TVD_IMPLICIT
 * Restatement of src/methods/fvm_tvd_implicit.cpp: Roe-linearised block system per
 * step, GMRES, smoothing, update with limits, remediation, CFL control. Boundary
 * kinds are the implicit method's own (Boundary::BOUND_*, par = T, P, Vx, Vy). */
enum { ORC_IBND_INLET = 1, ORC_IBND_OUTLET = 2, ORC_IBND_WALL = 3 };
/* MatrixSolver::RESULT_*, src/methods/solvers/MatrixSolver.h:13-16 */
enum { ORC_SOLVE_MAX_ITER = 0x2, ORC_SOLVE_CONVERG = 0x4 };

typedef struct orc_imp orc_imp;
typedef struct {
    int flux;                /* ORC_FLUX_GODUNOV or ORC_FLUX_LAX */
    int steady;
    int smoothing;
    int cfl_step;            /* <CFL><step> */
    int gmres_maxit, gmres_kdim;
    int newton_cap;
    int pad;
    double tau_xml;
    double cfl, cfl_scale, cfl_max, max_lim_cells;  /* <CFL> start, scale, max, max_limited_cells */
    double smoothing_par;
    double lim_rmin, lim_rmax, lim_pmin, lim_pmax, lim_umax;
    double gmres_eps;
} orc_imp_params;

/* The mesh must come from orc_mesh_build(..., berkeley = 2) for the reference's
 * loader; every boundary edge needs a boundary index < nbnd (else -1). */
int orc_imp_create(const orc_mesh* m, const orc_imp_params* prm, int nm, const double* mat, const int* cell_mat,
                   int nbnd, const int* bnd_kind, const double* bnd_par, const double* U0, orc_imp** out);
/* nsteps passes of run()'s loop body; returns 1 if the Newton cap was hit */
int orc_imp_step(orc_imp* s, int nsteps);
void orc_imp_get_state(const orc_imp* s, double* U4, double* ctau, unsigned* flags);
void orc_imp_set_state(orc_imp* s, const double* U4);
/* The block system of the current state: per cell its diagonal block (16, row
 * major), its three faces' off-diagonal blocks in Cell::edgesInd order (48; zero
 * on boundary faces) and right-hand side (4); cTau as used for the diagonal. */
void orc_imp_system(orc_imp* s, double* diag, double* off, double* rhs, double* ctau);
int orc_imp_lim_count(const orc_imp* s);
void orc_imp_info(const orc_imp* s, double* t, double* cfl, int* step, int* iters, double* rel, int* status);
void orc_imp_free(orc_imp* s);
/* GMRES(kdim) on the block system (nbr: nc x 3, -1 on boundary faces), x0 = 0;
 * returns ORC_SOLVE_* bits like MatrixSolver::solve. */
int orc_gmres_block(int nc, const int* nbr, const double* diag, const double* off, const double* b, double* x,
                    double eps, int maxit, int kdim, int* iters, double* final_rel);

/* ---------------------------------------------------------------- FEM_RKDG
 * Restatement of src/methods/fem_rkdg.cpp (cfd2d_oracle_dg.c): P1 discontinuous
 * Galerkin, two Runge-Kutta stages. The mesh is a .proc part in file order: nodes,
 * triangles with their region, edges (node pairs) with their boundary index (-1
 * inside). reg: nreg x (M, Cp, Vx, Vy, T, P) -- the region's material and initial
 * state; bpar: nbnd x (Vx, Vy, T, P). Coefficients: 12 per cell, ro[3] ru[3] rv[3]
 * re[3] (the reference's VECTOR ro[i] etc.). */
enum { ORC_DG_RK_REFERENCE = 0, ORC_DG_RK_HEUN = 1 };
enum { ORC_ERR_NEWTON_CAP = 1 };
typedef struct orc_dg orc_dg;
typedef struct {
    int steady, flux, gp_cell, gp_edge, rk_mode, newton_cap;
    double tau, tmax, cfl;
} orc_dg_params;
orc_dg* orc_dg_create(const orc_dg_params* p, int nn, const double* xy, int nc, const int* tri,
                      const int* cell_region, int ne, const int* en, const int* ebnd, int nreg, const double* reg,
                      int nbnd, const int* bkind, const double* bpar);
/* coefficients, then the time step as init forms it from the XML TAU */
void orc_dg_set(orc_dg* d, const double* coeffs);
void orc_dg_set_tau(orc_dg* d, double tau);
/* n passes of run()'s loop body; returns ORC_ERR_* bits */
unsigned orc_dg_step(orc_dg* d, int n);
/* scal: TAU, t, residuals ro ru rv re, step */
void orc_dg_get(const orc_dg* d, double* coeffs, double* ctau, double* scal);
/* cell6: cx cy HX HY S cellJ; invA: 9 per cell (row major); edge4: nx ny l edgeJ */
void orc_dg_geom(const orc_dg* d, int* cedge, int* c1c2, double* cell6, double* invA, double* edge4);
/* density, pressure, u, v at each cell centre (the VTU fields) */
void orc_dg_centre(const orc_dg* d, double* rpuv);
void orc_dg_free(orc_dg* d);
int orc_riemann_exact(double* RI, double* EI, double* PI, double* UI, double* VI, double RB, double PB, double UB,
                      double VB, double RE, double PE, double UE, double VE, double GAM, int cap);

#ifdef __cplusplus
}
#endif
#endif
