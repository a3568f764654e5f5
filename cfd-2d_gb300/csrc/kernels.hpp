// Device data layout and kernel launchers of the GB300 FVM_TVD path.
//
// Layout in HBM (all structure-of-arrays, cells and edges in the locality order
// chosen on the host; "original" numbers are the reference's cell and edge
// numbers, src/mesh/MeshReaderSalomeUnv.cpp:118-217):
//   cells (nc):  conserved state A[4][nc] and stage state B[4][nc] (FP64),
//                primitives W[nc][4] (r, u, v, p) and Green-Gauss gradients
//                G[nc][8] in the face precision (records, gathered by index), cfl[nc] = cTau/S, cTau[nc],
//                flags[nc], faces face[3][nc] = (edge << 1) | side ordered by
//                ascending original edge number, S[nc], rem_nb[3][nc].
//   edges (ne):  c1/c2[ne] (c2 = -1 for boundary edges, which are stored last),
//                nx, ny, l[ne], Gauss-point offsets dl[8][ne] from each side's
//                centroid (gp0: dxL dyL dxR dyR, gp1: ...), edge flux F[ne][4]
//                (already multiplied by l/2), boundary index bnd[ne].
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace cfd2d {

enum FluxKind { FLUX_GODUNOV = 0, FLUX_LAX = 1, FLUX_ROE = 2, FLUX_HLLC = 3 };
enum ReconKind { RECON_NONE = 0, RECON_LINEAR = 1, RECON_MINMOD = 2 };
enum SchemeKind { TIME_EULER = 0, TIME_HEUN = 1, TIME_SSPRK3 = 2 };
enum PrecisionKind { PREC_FP64 = 0, PREC_MIXED = 1 };
enum BndKind { BND_INLET = 1, BND_OUTLET = 2, BND_WALL_SLIP = 3, BND_WALL_NO_SLIP = 4 };

// error word bits (device -> host)
enum : unsigned { ERRBIT_NEWTON_CAP = 1u, ERRBIT_NONPHYSICAL = 2u };

constexpr double GAS_R = 8.314472;  // Material::gR, src/global.cpp:6

struct DevMat {     // Material (src/global.h:208-222) with its derived constants
    double M, Cp, Cv, gam, gm1;
};

struct DevBnd {     // one <boundCond>: kind and (Vx, Vy, T, P)
    int kind, pad;
    double u, v, T, p;
};

// The constants rim_orig derives from GAM (src/global.cpp:240-250), formed as it forms
// them; a caller with a fixed gas forms them once. iAGAM, iSGAM, i1DGAM are RN(1/AGAM),
// RN(1/SGAM), RN(1/(1 + DGAM)) for the quotients by them (div_x), eAGAM is 1/AGAM as the
// reference writes it in the sonic-rarefaction exponent.
template <typename T> struct RimGas {
    T GAM, AGAM, DGAM, GGAM, HGAM, FGAM, OGAM, QGAM, PGAM, RGAM, SGAM, TGAM, iAGAM, iSGAM, i1DGAM, eAGAM;
};
template <typename T>
__host__ __device__ __forceinline__ RimGas<T> rim_gas(T GAM) {
    RimGas<T> g;
    g.GAM = GAM;
    g.AGAM = (GAM - T(1.0));
    g.DGAM = (T(2.0) / g.AGAM);
#ifdef __CUDA_ARCH__
    g.GGAM = (::sqrt(GAM * g.AGAM));
#else
    g.GGAM = (std::sqrt(GAM * g.AGAM));
#endif
    g.HGAM = (g.AGAM / T(2.0));
    g.FGAM = (T(3.0) * GAM - T(1.0));
    g.OGAM = (g.AGAM / (T(2.0) * GAM));
    g.QGAM = (GAM + T(1.0));
    g.PGAM = (g.QGAM / (T(2.0) * GAM));
    g.RGAM = (T(4.0) * GAM);
    g.SGAM = (GAM * g.AGAM);
    g.TGAM = (g.QGAM / T(2.0));
    g.iAGAM = T(1) / g.AGAM;
    g.iSGAM = T(1) / g.SGAM;
    g.i1DGAM = T(1) / (T(1) + g.DGAM);
    g.eAGAM = T(1) / g.AGAM;
    return g;
}
// Launch shape of one kernel kind: threads per block and blocks (0 = one
// thread per item; otherwise a persistent grid that strides over the items).
// Default: 64-thread blocks, one thread per item (measured best for the single
// four-quadrant workload in both precisions; the autotuner can override it).
// What a forward HLLC flux evaluation leaves for the adjoint's recorded path, per edge (SoA,
// face precision): v[(10 g + j) ne + e] for Gauss point g, j 0-3 the left face state (r, u,
// v, p), 4-7 the right one, 8-9 the left and right sound speeds; bits[e] minmod's branches
// (2 bits per variable r, p, u, v; 8 bits per side, left then right; 16 per Gauss point).
struct FluxRec {
    void* v = nullptr;
    unsigned* bits = nullptr;
};

struct LaunchShape { int block = 64, grid = 0; };
enum { KIND_GRAD = 0, KIND_FLUX = 1, KIND_UPDATE = 2, N_TUNED_KINDS = 3 };

// Everything a kernel needs; passed by value.
struct DevCase {
    int nc, ne, n_int;
    LaunchShape shape[N_TUNED_KINDS];
    // geometry
    const int* face;       // 3*nc
    // the same faces seen from the cell, for the gradient gather (one level of
    // indirection instead of three): cf_nb = (neighbour << 1) | side, or -(edge + 1)
    // on the boundary; the edge's normal (outward from c1) and length per face
    const int* cf_nb;      // 3*nc
    const double* cf_nx;   // 3*nc (FP64 form)
    const double* cf_ny;
    const double* cf_l;
    // 3*nc (FP64 form with minmod, else nullptr): RN(RN(nx l) / 2), RN(RN(ny l) / 2) per
    // face, the weights of this project's Green-Gauss arithmetic (grad_one_mm)
    const double* cf_ax;
    const double* cf_ay;
    // 3*nc (mixed form): RN32(nx l / 2), RN32(ny l / 2) per face, the weights of the mixed
    // form's Green-Gauss arithmetic (grad_one_w)
    const float* cf_ax32;
    const float* cf_ay32;
    const int* ec1;        // ne
    const int* ec2;        // ne
    const int* ebnd;       // ne (boundary index, -1 inside)
    const double* nx;      // ne
    const double* ny;
    const double* l;
    const double* dl;      // 8*ne
    const float* nx32;
    const float* ny32;
    const float* l32;
    const float* ax32;     // ne (mixed form): the per-edge gradient weights, as cf_ax32
    const float* ay32;
    // 3*ne (mixed form): per edge {nx, ny, l, 0} and the two Gauss points' offsets
    // {dxL, dyL, dxR, dyR}: the flux kernels' geometry in three vector loads
    const float4* geo32;
    const float* dl32;
    const double* S;       // nc
    const double* invS;    // nc, RN(1/S) (FP64 form)
    const int* rem_nb;     // 3*nc
    const int* iperm;      // original cell -> storage cell
    const uint8_t* cmat;   // nc, nullptr when one material
    // tables
    const DevMat* mats;
    const DevBnd* bnds;
    DevMat mat0;
    float mat0_f[3];       // M, Cv, gam-1 of material 0 in FP32 (mixed form)
    float gam_flux_f;
    float ig1_flux_f;      // 1/(gam_flux - 1) in FP32
    float lim_f[5];        // limits in FP32 (mixed form)
    const float* invS32;   // nc, 1/S in FP32 (mixed form)
    const float4* cfrec32; // 3*nc (mixed form): per cell and face {cf_nb bits, a_x, a_y, 0} in one 16-byte record
    double gam_flux;
    double ig1_flux;       // RN(1/(gam_flux - 1)), computed on the host
    RimGas<double> rg_flux;  // the exact Riemann solver's constants of gam_flux
    double cfl_number;
    double lim_rmin, lim_rmax, lim_pmin, lim_pmax, lim_umax;
    int steady;
    int newton_cap;
    int flux_pipe;         // mixed form: the software-pipelined flux kernel (k_flux_pipe)
    // state
    double* A;             // 4*nc conserved state U^n (and result)
    double* B;             // 4*nc stage state
    double* cfl;           // nc   cTau/S of the step about to run
    double* ctau;          // nc   cTau of the last step (the reference's cTau array)
    double* ctau_next;     // nc   cTau of the next step (local time step)
    unsigned* flags;       // nc
    int* n_lim;            // 1
    unsigned* err;         // 1
    double* W64;           // 4*nc
    double* G64;           // 8*nc
    double* F64;           // 4*ne
    float* W32;
    float* G32;
    float* F32;
};

// ---- launchers (kern_fp64.cu / kern_mixed.cu / kern_common.cu)
void launch_grad(const DevCase& c, int precision, cudaStream_t s);
void launch_flux(const DevCase& c, int precision, int flux, int recon, cudaStream_t s);
// the mixed form's pipelined flux kernels' launch attributes, set once before any capture
void launch_flux_prepare_mixed();
// stage update; reads A (and B for later stages), writes B or A and the next primitives
void launch_update(const DevCase& c, int precision, int scheme, int stage, cudaStream_t s);
void launch_remediate(const DevCase& c, int precision, cudaStream_t s);
// primitives (+ local time step when steady) from A, for every cell
void launch_prims(const DevCase& c, int precision, cudaStream_t s);
// min over cells of CFL*S/max(|u|+c,|v|+c) into *out (as ordered bits of a positive double)
void launch_dt_min(const DevCase& c, unsigned long long* out, cudaStream_t s);
// cfl[i] = tau / S[i]
void launch_fill_cfl(const DevCase& c, double tau, cudaStream_t s);
// state permutation between caller order (original cells) and storage order
void launch_gather_state(const DevCase& c, const double* src_orig, double* dst_store, cudaStream_t s);
void launch_scatter_state(const DevCase& c, const double* src_store, double* dst_orig, cudaStream_t s);
// the same from / to four device-addressable host arrays (see device_view in solver.cpp)
struct HostArrays4 { double* p[4]; };
void launch_gather_state_host(const DevCase& c, const HostArrays4& src_orig, double* dst_store, cudaStream_t s);
void launch_scatter_state_host(const DevCase& c, const double* src_store, const HostArrays4& dst_orig,
                               cudaStream_t s);
void launch_permute_scalar(const DevCase& c, const double* src_store, double* dst_orig, cudaStream_t s);
void launch_permute_flags(const DevCase& c, const unsigned* src_store, unsigned* dst_orig, cudaStream_t s);
// residual of one stage (the reference's ro_int..re_int) in storage order
void launch_residual(const DevCase& c, int precision, double* R, cudaStream_t s);
// ---- discrete adjoint (adjoint.cu)
// Adjoint work arrays of one backward stage.
// Tiles of the mixed form's fused stage kernel (one CTA per tile): tile t owns the
// storage cells [t*tile, (t+1)*tile) and reads a halo of two cell rings around them.
// Local cell numbers: own cells first, then the first ring (H1), then the second
// (H2). Gradients are formed for own + H1 cells, fluxes for the edges of own cells.
struct DevTiles {
    int n_tiles = 0, tile = 0;
    int max_cells = 0, max_grad = 0, max_edges = 0;  // shared-memory capacities (max over tiles)
    const int* halo_off = nullptr;   // n_tiles + 1, into halo
    const int* halo = nullptr;       // H1 then H2 storage cells of each tile
    const int* n_h1 = nullptr;       // n_tiles
    const int* edge_off = nullptr;   // n_tiles + 1, into tedge
    const int2* tedge = nullptr;     // flux edges: x = storage edge, y = local c1 | local c2 << 16 (0xffff: boundary)
    const int* gface_off = nullptr;  // n_tiles + 1, into gface (in cells; 3 entries per cell)
    const int2* gface = nullptr;     // per gradient cell and face: x = (edge << 1) | side,
                                     // y = local neighbour (0xffff: boundary) | local flux edge << 16 (own cells)
};
// the mixed form's flux kernel that forms its two cells' gradients itself (no G array)
void launch_flux_grad_mixed(const DevCase& c, int flux, int recon, cudaStream_t s);
void launch_flux_update_mixed(const DevCase& c, const DevTiles& t, int flux, int recon, int scheme, int stage,
                              float* w_out, cudaStream_t s);
void launch_stage_fused_mixed(const DevCase& c, const DevTiles& t, int flux, int recon, int scheme, int stage,
                              const float* w_in, float* w_out, cudaStream_t s);

struct AdjCase {
    const double* mu;  // nc x 4 (AoS) cfl * t_bar
    void* eq;          // ne x 24 in the face precision: q1_bar(4) g1_bar(8) q2_bar(4) g2_bar(8)
    double* eb;        // (ne - n_int) x 4 boundary-parameter adjoints, flux path
    double* eb2;       // (ne - n_int) x 4 boundary-parameter adjoints, gradient path
    double* qbar;      // nc x 4: r, u, v, p
    void* gbar;        // nc x 8 in the face precision
    double* tb;        // 4*nc (SoA) t_bar of the current stage
    double* acc;       // 4*nc adjoint accumulated for the step's input U^n
    double* lam;       // 4*nc adjoint of the step's output / input
    double* mu_out;    // nc x 4
    double* dbnd;      // n_bnd x 4 accumulated boundary-parameter adjoints
    int n_bnd;
};

// precision: PREC_FP64 (FP64 faces) or PREC_MIXED (FP32 faces, FP64 per-cell sums)
void launch_adj_flux(const DevCase& c, const AdjCase& a, int flux, int recon, int precision, cudaStream_t s);
// HLLC only: the forward flux of a recomputed stage with its record, and the flux VJP reading it
void launch_flux_rec(const DevCase& c, int recon, const FluxRec& r, int precision, cudaStream_t s);
void launch_adj_flux_rec(const DevCase& c, const AdjCase& a, int recon, const FluxRec& r, int precision,
                         cudaStream_t s);
void launch_adj_gather(const DevCase& c, const AdjCase& a, int precision, cudaStream_t s);
void launch_adj_cell(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, int first, int precision,
                     cudaStream_t s);
void launch_adj_step_start(const DevCase& c, const AdjCase& a, double coef_t, double coef_acc, cudaStream_t s);
void launch_adj_bnd_reduce(const DevCase& c, const AdjCase& a, cudaStream_t s);
void launch_objective(const DevCase& c, const double* w, int kind, double p_ref, double* partial, int nblocks,
                      cudaStream_t s);
void launch_objective_grad(const DevCase& c, const AdjCase& a, const double* w, int kind, double p_ref,
                           cudaStream_t s);

// built-in checks of the arithmetic helpers against the hardware operations
// (which: 0 div_rn vs '/', 1 widen vs (double), 2 narrow vs (float) within 1 ulp)
long long selftest_arith(int which, long long n, unsigned long long seed);
// deterministic FP64 sums of S*U over cells (mass, x/y momentum, energy)
void launch_conservation(const DevCase& c, double* partial, int nblocks, cudaStream_t s);

}  // namespace cfd2d
