/*
 * cfd2d_gb300 — C ABI of the GB300 drop-in for the reference's explicit
 * finite-volume method FVM_TVD (zhrv/cfd-2d).
 *
 * The reference selects the method through its C++ plugin interface
 *   class Method { virtual void init(char* xml); virtual void run(); virtual void done(); }
 *   (src/methods/method.h:6-11), instantiated by name in Solver::initMethod
 *   (src/methods/solver.cpp:13-61) from <task method="FVM_TVD">.
 * These entry points replace FVM_TVD::init / run / done
 * (src/methods/fvm_tvd.cpp:7-213, 303-462, 731-752) one for one, and add the
 * state access a caller outside the reference's process needs. Plain C types
 * only; every entry point returns 0 or an error code and never exits the
 * process (the reference calls exit()/EXIT() on errors, src/global.cpp:48-53).
 *
 * State arrays are in the reference's cell order (the order of the triangles in
 * the mesh file); the library reorders cells internally for locality.
 */
#ifndef CFD2D_H
#define CFD2D_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CFD2D_OK 0
/* the reference's Exception / EXIT codes (src/global.h:241-248) */
#define CFD2D_ERR_BOUND_NOPAR 101                   /* BOUND_INLET without Vx/Vy/T/P */
#define CFD2D_ERR_BOUND_UNKNOWN 102                 /* unknown <boundCond><type> */
#define CFD2D_ERR_MESH_WRONG_NAME 201               /* unknown <mesh><filesType> */
#define CFD2D_ERR_MESH_UNV_UNKNOWN_ELEMENT 221      /* UNV element type other than 11/41 */
#define CFD2D_ERR_MESH_UNV_NOT_DEFINED_BND_EDGE 222 /* boundary edge without a UNV edge element */
#define CFD2D_ERR_FILE_OPENING 301
/* conditions the reference ends with EXIT(1) or undefined behaviour */
#define CFD2D_ERR_XML 1              /* task file cannot be read or parsed (reference: exit(ErrorId)) */
#define CFD2D_ERR_TASK 2             /* a required task element/attribute is missing */
#define CFD2D_ERR_REGION_UNKNOWN 3   /* a cell's region name is not in <regions> (fvm_tvd.cpp:773-781) */
#define CFD2D_ERR_EDGE_UNKNOWN 4     /* a boundary edge matches no <boundCond> (fvm_tvd.cpp:148-170) */
#define CFD2D_ERR_MESH_FORMAT 5      /* malformed mesh file or arrays */
#define CFD2D_ERR_INVALID_ARG 6
/* GPU-side conditions */
#define CFD2D_ERR_CUDA 501           /* a CUDA call failed; see cfd2d_last_error */
#define CFD2D_ERR_NO_DEVICE 502
#define CFD2D_ERR_NEWTON_CAP 503     /* the exact Riemann solver hit its iteration cap (state still advanced) */
#define CFD2D_ERR_NONPHYSICAL 504    /* non-positive or NaN density/pressure appeared (state still advanced) */
#define CFD2D_ERR_CAPACITY 505       /* a size exceeds a fixed capacity of the entry point */
#define CFD2D_ERR_SOLVER 506         /* FVM_TVD_IMPLICIT: a steady run's linear solves kept failing (run stops) */

/* ---- method selections (task.xml <control> extensions) ------------------ */
enum { CFD2D_FLUX_GODUNOV = 0, CFD2D_FLUX_LAX = 1, CFD2D_FLUX_ROE = 2, CFD2D_FLUX_HLLC = 3 };
enum { CFD2D_RECON_NONE = 0, CFD2D_RECON_LINEAR = 1, CFD2D_RECON_MINMOD = 2 };
enum { CFD2D_TIME_EULER = 0, CFD2D_TIME_HEUN = 1, CFD2D_TIME_SSPRK3 = 2 };
enum { CFD2D_PREC_FP64 = 0, CFD2D_PREC_MIXED = 1 };

typedef struct cfd2d_solver cfd2d_t;
typedef struct cfd2d_mesh cfd2d_mesh_t;

/* A mesh handed over as arrays instead of a mesh file. Regions and boundary
 * conditions are referred to by position in the task's <regions> and
 * <boundaries> lists (document order). */
typedef struct {
    int n_nodes;
    const double* xy;        /* 2*n_nodes */
    int n_cells;
    const int* tri;          /* 3*n_cells, 0-based node numbers */
    const int* cell_region;  /* n_cells */
    int n_bsegs;
    const int* bseg;         /* 2*n_bsegs boundary node pairs */
    const int* bseg_bnd;     /* n_bsegs */
} cfd2d_mesh_desc;

typedef struct {
    int n_cells, n_edges, n_boundary_edges, n_nodes;
    int step;                /* steps taken */
    int flux, recon, scheme, precision, steady;  /* recon, scheme: -1 on a FEM_RKDG handle */
    double time;             /* t as the reference accumulates it (t += TAU per unsteady step) */
    double tau;              /* global time step TAU (unsteady) */
    size_t device_bytes;     /* device memory held by the handle */
    int n_instances;         /* 1, or the number of instances of a batch */
} cfd2d_info_t;

/* FVM_TVD::init (src/methods/fvm_tvd.cpp:7-213): read task.xml and its mesh,
 * set the initial state from the regions and compute TAU. A relative mesh name
 * is opened relative to the working directory, else to task.xml's directory. */
int cfd2d_create(const char* task_xml_path, cfd2d_t** out);

/* FVM_TVD::init with the mesh given as arrays (the task's <mesh> is ignored). */
int cfd2d_create_with_mesh(const char* task_xml_path, const cfd2d_mesh_desc* mesh, cfd2d_t** out);

/* nsteps iterations of FVM_TVD::run's loop body (src/methods/fvm_tvd.cpp:310-460)
 * without file output; blocks until done. */
int cfd2d_step(cfd2d_t* h, int nsteps);

/* FVM_TVD::run: the whole loop while t < TMAX and step < STEP_MAX, writing
 * res_%010d.vtk every FILE_OUTPUT_STEP (and res_0000000000.vtk first when
 * starting from step 0, which the reference writes at the end of init) and the
 * log line every LOG_OUTPUT_STEP. */
int cfd2d_run(cfd2d_t* h);

/* FVM_TVD::done: free everything the handle owns. */
int cfd2d_destroy(cfd2d_t* h);

int cfd2d_get_info(const cfd2d_t* h, cfd2d_info_t* info);

/* Conserved state ro, ru, rv, re (FVM_TVD's arrays, src/methods/fvm_tvd.h:86-89).
 * The arrays of get_state / set_state are host memory (pinned or pageable) or device
 * memory of the handle's GPU; kernels read and write them in place where the GPU can
 * address them (pinned, managed, device, or pageable on systems with coherent host
 * access such as Grace), else through a staging copy. Device data must be complete
 * when the call is made (the library works on its own stream); both calls return
 * with the transfer done. */
int cfd2d_get_state(cfd2d_t* h, double* ro, double* ru, double* rv, double* re);
/* Replace the conserved state. reset_time_step != 0 redoes init's time step
 * (TAU = min(TAU from task.xml, CFL pass), src/methods/fvm_tvd.cpp:211). */
int cfd2d_set_state(cfd2d_t* h, const double* ro, const double* ru, const double* rv, const double* re,
                    int reset_time_step);
/* Per-cell time step cTau and cell flag words (CELL_FLAG_LIM = 2, src/mesh/grid.h:12-14). */
int cfd2d_get_time_step(cfd2d_t* h, double* ctau);
int cfd2d_get_flags(cfd2d_t* h, unsigned* flags);
/* One stage's right-hand side for the current state: the reference's
 * ro_int..re_int after the edge loop (src/methods/fvm_tvd.cpp:324-365), 4 x n_cells. */
int cfd2d_residual(cfd2d_t* h, double* R);
/* Sums over cells of S*(ro, ru, rv, re) in FP64, summed in a fixed order. */
int cfd2d_conservation(cfd2d_t* h, double sums[4]);
/* FVM_TVD::save (src/methods/fvm_tvd.cpp:501-600): res_%010d.vtk in the working directory. */
int cfd2d_save_vtk(cfd2d_t* h, int step);
/* Restart files (no counterpart in the reference, which cannot restart): the
 * conserved state, cTau, the cell flags, the step count and the time, in the
 * mesh files' cell order (an FVM_TVD_IMPLICIT handle also keeps its CFL number and
 * last solve status). cfd2d_load_state into a handle made from the same task and
 * mesh continues the run exactly as if it had not stopped. */
int cfd2d_save_state(cfd2d_t* h, const char* path);
int cfd2d_load_state(cfd2d_t* h, const char* path);

/* ---- batches -------------------------------------------------------------- */
/* No counterpart in the reference (one FVM_TVD per process there): n
 * independent instances, each a task file and (meshes != NULL) its mesh as
 * arrays, else the task's own mesh file, solved together by one set of kernels
 * per stage over the union of their meshes. Instances share FLUX,
 * RECONSTRUCTION, TIME_SCHEME, PRECISION, STEADY and the limits of the first
 * task; each keeps its own mesh, regions, materials, boundary conditions, CFL
 * and time step, and its results equal its single-instance solve bit for bit.
 * The handle works with every entry point above; the state arrays hold the
 * instances one after another (see cfd2d_batch_instance). */
int cfd2d_batch_create(int n, const char* const* task_xml_paths, const cfd2d_mesh_desc* meshes, cfd2d_t** out);
/* Instance k of a batch: first cell in the state arrays, cell count, its TAU and time. */
int cfd2d_batch_instance(const cfd2d_t* h, int k, int* cell_offset, int* n_cells, double* tau, double* time);
/* Time each kernel kind over block sizes {64,128,256} x grids {one thread per
 * item, 1/2/4/8 persistent blocks per SM} on this handle's mesh, keep the
 * fastest, re-capture the step graph, and write the choice as JSON to
 * json_path (NULL: do not write). Results do not depend on the shapes. */
int cfd2d_autotune(cfd2d_t* h, const char* json_path);
/* Apply launch shapes saved by cfd2d_autotune. */
int cfd2d_load_tuning(cfd2d_t* h, const char* json_path);

/* ---- discrete adjoint (forward/backward pair) ---------------------------- */
/* Objective of the final state: J = sum_i w_i (p_i - p_ref)^2 (kind 0) or
 * J = sum_i w_i rho_i^2 (kind 1); weights per cell in the reference's order. */
int cfd2d_set_objective(cfd2d_t* h, int kind, const double* weights, double p_ref);
/* nsteps steps from the current state keeping a checkpoint of the state every
 * checkpoint_every steps; *J receives the objective of the final state. The
 * state ends at step nsteps as with cfd2d_step. Needs STEADY=0 (TAU held
 * fixed), the HLLC or LAX flux and no active limiter. */
int cfd2d_forward(cfd2d_t* h, int nsteps, int checkpoint_every, double* J);
/* Gradient of that J by the hand-written discrete adjoint of the forward's
 * steps (recomputed segment by segment from the checkpoints): dJdU0 (4 x
 * n_cells, ro|ru|rv|re) with respect to the state cfd2d_forward started from,
 * and dJdbnd (4 per <boundCond>: Vx, Vy, T, P) with respect to the boundary
 * parameters; either pointer may be NULL. */
int cfd2d_backward(cfd2d_t* h, double* dJdU0, double* dJdbnd);
/* Replace the parameters (Vx, Vy, T, P) of the b-th <boundCond>. */
int cfd2d_set_boundary(cfd2d_t* h, int b, const double par[4]);

/* Device time in milliseconds of nsteps steps, from CUDA events recorded on the
 * handle's stream around the step graph launches (the steps are taken). */
int cfd2d_timed_steps(cfd2d_t* h, int nsteps, double* device_ms);
/* nsteps steps launched kernel by kernel with CUDA events around each launch:
 * per kernel kind (0 gradients, 1 edge fluxes, 2 stage updates, 3 remediation)
 * the total device ms and the number of launches (the steps are taken). On an
 * FVM_TVD_IMPLICIT handle the kinds are phases of the step: 0 primitives and
 * gradients, 1 Gauss-point fluxes and Roe states, 2 block-row assembly, 3 GMRES and
 * the update. */
int cfd2d_profile_steps(cfd2d_t* h, int nsteps, double kernel_ms[4], int kernel_launches[4]);

/* Built-in check of the device arithmetic helpers on n seeded random operands,
 * against the hardware operation on the current device: which = 0 FP64 division
 * through a precomputed reciprocal (must equal '/' bit for bit), 1 FP32->FP64
 * widening on the integer pipe (must equal the conversion), 2 FP64->FP32
 * narrowing on the integer pipe (within 1 ulp), 3 FP64 minmod with its
 * integer-pipe sign test (must equal a*b > 0 ? (|a| < |b| ? a : b) : 0 bit for
 * bit). *mismatches receives the count. */
int cfd2d_selftest(int which, long long n, unsigned long long seed, long long* mismatches);

/* ---- FVM_TVD_IMPLICIT ---------------------------------------------------- */
/* A task.xml with <task method="FVM_TVD_IMPLICIT"> (src/methods/fvm_tvd_implicit.cpp,
 * selected by name in Solver::initMethod, src/methods/solver.cpp:41-44) creates an
 * implicit handle through cfd2d_create / cfd2d_create_with_mesh: the mesh is read as
 * Grid::initFromFiles does (Triangle files <name>.node/.ele/.neigh/.poly, midpoint and
 * two Gauss points per edge), regions bind by cell type and boundaries by edge type.
 * cfd2d_step / run / get_info / get_state / set_state / get_time_step / get_flags /
 * save_vtk / timed_steps / destroy serve it (one step = one pass of
 * FVM_TVD_IMPLICIT::run's loop: assembly, GMRES, smoothing, update, remediation, CFL
 * rules); the explicit-only entry points return CFD2D_ERR_INVALID_ARG on it. */
typedef struct {
    int iterations;       /* GMRES iterations of the last solve */
    int status;           /* MatrixSolver result bits (src/methods/solvers/MatrixSolver.h:13-16):
                             0 solved, 2 iteration limit reached, 4 not converged */
    int n_limited;        /* cells flagged CELL_FLAG_LIM after the last update (getLimitedCellsCount) */
    int pad;
    double rel_residual;  /* |b - A x| / |b| of the last solve */
    double cfl;           /* the CFL number of the steady rules (incCFL / decCFL) */
} cfd2d_implicit_stats_t;
/* The block system of the current state as the next step assembles it (the state is
 * not advanced): per cell, in the reference's cell order, the diagonal 4x4 block
 * (16, row major; S/cTau I + sum of l A+), the three faces' 4x4 blocks (48; l A- of
 * the face, in Cell::edgesInd order, zero on boundary faces) and the right-hand side
 * (4; -sum F l/2), and cTau. Unknowns are x[4 c + k] as in MatrixSolver. Any pointer
 * may be NULL. */
int cfd2d_implicit_system(cfd2d_t* h, double* diag, double* off, double* rhs, double* ctau);
int cfd2d_implicit_stats(const cfd2d_t* h, cfd2d_implicit_stats_t* stats);

/* ---- FEM_RKDG -------------------------------------------------------------- */
/* A task.xml with <task method="FEM_RKDG"> (src/methods/fem_rkdg.cpp, the reference's
 * explicit P1 discontinuous Galerkin method; Solver::initMethod, src/methods/solver.cpp:
 * 49-51) gives a handle of that method: cfd2d_create = FEM_RKDG::init (it reads the mesh
 * part mesh/mesh.0000.proc that the DECOMP method writes, from the working directory or
 * the task's folder, Grid::readMeshFiles src/mesh/grid.cpp:275-420; cfd2d_create_with_mesh
 * takes mesh arrays instead, cell_region and bseg_bnd indexing <regions> and
 * <boundaries>), cfd2d_run = FEM_RKDG::run (:600-660; a steady task has no end there and
 * returns CFD2D_ERR_INVALID_ARG), cfd2d_step advances whole steps (both Runge-Kutta
 * stages), cfd2d_save_vtk writes save()'s res_%010d.pvtu and vtk_data/res_%010d.0000.vtu
 * (:662-800). cfd2d_get_state gives the polynomials at the cell centres, cfd2d_set_state
 * sets piecewise constant coefficients (value, 0, 0) as init does from the regions, and
 * cfd2d_get_time_step cTau. The control element <RK_MODE value="HEUN"/> (no counterpart
 * in the reference) averages the second stage with U^n instead of the reference's
 * first-stage result. */

/* The P1 coefficients, 12 per cell in the reference's cell order: ro[3] ru[3] rv[3] re[3]
 * (FEM_RKDG's VECTOR ro[i], ru[i], rv[i], re[i], basis 1, (x-xc)/HX, (y-yc)/HY). Any host
 * or device pointer. cfd2d_dg_set_coeffs then recomputes the time step from the task's
 * TAU as init does (calcTimeStep, :382-447). */
int cfd2d_dg_get_coeffs(cfd2d_t* h, double* coeffs);
int cfd2d_dg_set_coeffs(cfd2d_t* h, const double* coeffs);
/* Impose a time step (every cell's cTau = TAU = tau). */
int cfd2d_dg_set_time_step(cfd2d_t* h, double tau);
/* calcResiduals (:1286-1319) of the last step taken by cfd2d_step or cfd2d_run: the
 * largest |U - ro_old| norm per variable (ro, ru, rv, re). */
int cfd2d_dg_residuals(cfd2d_t* h, double res[4]);

/* Select the CUDA device that cfd2d_create* places new solvers on (default: the
 * calling thread's current device). A solver keeps its device for life. */
int cfd2d_set_device(int device);

/* ---- fixed-scratch residual (allocates nothing) ------------------------- */
/* No counterpart in the reference. For callers that cannot allocate device
 * memory when they call in (recording a CUDA graph, where cudaMalloc is not
 * allowed during capture; a host framework whose memory pool owns the device;
 * a real-time loop that forbids allocation after start-up): the first-order
 * residual R (the reference's ro_int..re_int with the cell-centre states, as
 * cfd2d_residual returns for RECONSTRUCTION NONE) of the state U, computed with
 * no cudaMalloc/cudaFree and no allocating library call. Its only scratch, one
 * FP64 flux per edge, is a fixed device array of CFD2D_STATIC_MAX_EDGES x 4
 * doubles (8 MiB) in the library, held by every GPU that loads the library
 * until exit. All pointers except bnd_kind/bnd_par (host, n_bnd <= 16 entries)
 * are device memory, in the reference's numbering as cfd2d_mesh_export writes
 * it: cell_edges 3*n_cells (ascending), edge_c12 2*n_edges, edge_n 2*n_edges,
 * edge_l and edge_bnd n_edges, U and R 4*n_cells. One material (M, Cp); flux
 * is CFD2D_FLUX_*. Runs asynchronously on stream (a cudaStream_t, NULL = the
 * default stream). The first call on a device looks up the array's device
 * address (make it before any stream capture). All calls share the array:
 * calls that overlap on the GPU race, so order them on one stream. Returns
 * CFD2D_ERR_CAPACITY when n_edges > CFD2D_STATIC_MAX_EDGES or n_bnd > 16,
 * CFD2D_ERR_INVALID_ARG for a null pointer, a non-positive size, an unknown
 * flux or a bnd_kind outside 1..4 (1 INLET, 2 OUTLET, 3 WALL_SLIP,
 * 4 WALL_NO_SLIP), CFD2D_ERR_CUDA when the array lookup or a launch fails, or,
 * before anything runs, when a CUDA error of earlier work is pending on the
 * thread (it is left pending for its owner); it leaves the cfd2d_last_error
 * message untouched (setting it could allocate). n_bnd may be 0 when no edge
 * is a boundary edge. An index outside the mesh, or a boundary edge whose
 * edge_bnd is not in 0..n_bnd-1, gives NaN in R, never an out-of-bounds
 * access. The device address of the array is cached per device; after
 * cudaDeviceReset call cfd2d_static_reset before the next call on that
 * device. */
#define CFD2D_STATIC_MAX_EDGES 262144
int cfd2d_residual_first_order_static(int n_cells, int n_edges, const int* cell_edges, const int* edge_c12,
                                      const double* edge_n, const double* edge_l, const int* edge_bnd, int n_bnd,
                                      const int* bnd_kind, const double* bnd_par, double M, double Cp, int flux,
                                      const double* U, double* R, void* stream);
/* Forget the device addresses cfd2d_residual_first_order_static cached (needed after
 * a cudaDeviceReset, which ends the context they belong to). No counterpart in the
 * reference. */
int cfd2d_static_reset(void);

/* Message of the last failed call on this thread. */
int cfd2d_last_error(char* buf, size_t n);
/* Log lines (the reference's log(), src/global.cpp:32-46) go to stdout unless
 * verbosity is 0, and are appended to path when a log file is set (NULL closes). */
int cfd2d_set_verbosity(int level);
int cfd2d_set_log_file(const char* path);

/* ---- host-only mesh inspection (no GPU needed) -------------------------- */
/* Read the mesh a task names and build its edges exactly as the reference's
 * reader does (MeshReader::create, src/mesh/MeshReader.cpp:7-23). */
int cfd2d_mesh_load(const char* task_xml_path, cfd2d_mesh_t** out);
/* Same from arrays (berkeley_neigh != NULL selects the Triangle reader's rules). */
int cfd2d_mesh_build(const cfd2d_mesh_desc* mesh, const int* berkeley_neigh, cfd2d_mesh_t** out);
int cfd2d_mesh_sizes(const cfd2d_mesh_t* m, int* n_cells, int* n_edges);
/* Cell::edgesInd/S/c and Edge n1,n2/c1,c2/boundary index/point count/n/l/points
 * (src/mesh/grid.h:18-67); any pointer may be NULL. */
int cfd2d_mesh_export(const cfd2d_mesh_t* m, int* cell_edges, double* cell_S, double* cell_c,
                      int* edge_n12, int* edge_c12, int* edge_bnd, int* edge_npts,
                      double* edge_n, double* edge_l, double* edge_pts);
/* The locality order the solver would use: storage cell -> reference cell. */
int cfd2d_mesh_order(const cfd2d_mesh_t* m, int rcm, int* perm);
int cfd2d_mesh_free(cfd2d_mesh_t* m);

#ifdef __cplusplus
}
#endif
#endif
