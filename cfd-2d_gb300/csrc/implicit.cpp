// Host driver of FVM_TVD_IMPLICIT on the GPU (src/methods/fvm_tvd_implicit.cpp).
#include "implicit.hpp"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "cfd2d.h"
#include "solver.hpp"

namespace cfd2d {

template <typename T>
T* ImplicitSolver::dalloc(size_t n) {
    void* p = nullptr;
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    CUDA_CHECK(cudaMalloc(&p, b));
    allocs_.push_back(p);
    bytes_ += b;
    return static_cast<T*>(p);
}

template <typename T>
T* ImplicitSolver::upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) CUDA_CHECK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
    return p;
}

namespace {
// the permutation kernels of the explicit path read only nc and iperm
DevCase perm_case(const ImpCase& c) {
    DevCase d{};
    d.nc = c.nc;
    d.iperm = c.iperm;
    return d;
}
}  // namespace

ImplicitSolver::ImplicitSolver(const TaskConfig& t, Topo&& topo, const std::vector<int>& cell_region,
                               const std::vector<int>& edge_bnd)
    : task_(t), topo_(std::move(topo)) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(CFD2D_ERR_NO_DEVICE, "no CUDA device");
    CUDA_CHECK(cudaGetDevice(&dev_));
    if (task_.gmres_kdim < 1 || task_.gmres_kdim > kGmresMaxKdim)
        throw Error(CFD2D_ERR_INVALID_ARG, "Krylov dimension out of range");
    const int nc = topo_.nc;
    std::vector<int> cell_mat(nc);
    for (int i = 0; i < nc; i++) cell_mat[i] = task_.regions[cell_region[i]].matId;
    lay_ = make_layout(topo_, cell_mat, edge_bnd, task_.reorder >= 0 ? task_.reorder : ORDER_RCM);
    const int ne = lay_.ne;
    CUDA_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    try {
        ImpCase& c = ic_;
        c.nc = nc; c.ne = ne; c.n_int = lay_.n_int;
        c.flux = task_.flux;
        c.steady = task_.steady;
        c.smoothing = task_.smoothing;
        c.newton_cap = task_.newton_cap;
        c.kdim = task_.gmres_kdim;
        c.maxit = task_.gmres_maxit;
        c.eps = task_.gmres_eps;
        c.smoothing_par = task_.smoothing_par;
        c.tau_xml = task_.tau;
        c.gam_flux = 1.4;  // __GAM, src/methods/fvm_tvd_implicit.cpp:536
        c.ig1_flux = 1.0 / (c.gam_flux - 1.0);
        c.rg_flux = rim_gas<double>(c.gam_flux);
        c.lim_rmin = task_.lim_rmin; c.lim_rmax = task_.lim_rmax;
        c.lim_pmin = task_.lim_pmin; c.lim_pmax = task_.lim_pmax; c.lim_umax = task_.lim_umax;
        c.face = upload(lay_.face);
        c.ec1 = upload(lay_.ec1);
        c.ec2 = upload(lay_.ec2);
        c.ebnd = upload(lay_.ebnd);
        c.nx = upload(lay_.nx);
        c.ny = upload(lay_.ny);
        c.l = upload(lay_.l);
        c.dl = upload(lay_.dl);
        c.S = upload(lay_.S);
        std::vector<double> is(nc);
        for (int i = 0; i < nc; i++) is[i] = 1.0 / lay_.S[i];
        c.invS = upload(is);
        {  // the matrix-vector product's neighbours; a boundary face's block is zero, so it reads the cell itself
            std::vector<int> nb(3 * (size_t)nc);
            for (int k = 0; k < 3; k++)
                for (int i = 0; i < nc; i++) {
                    const int f = lay_.face[(size_t)k * nc + i], e = f >> 1;
                    nb[(size_t)k * nc + i] = e < lay_.n_int ? ((f & 1) ? lay_.ec1[e] : lay_.ec2[e]) : i;
                }
            c.nbr = upload(nb);
        }
        c.iperm = upload(lay_.iperm);
        std::vector<DevMat> mats;
        for (auto& m : task_.mats) {
            DevMat d;
            d.M = m.M; d.Cp = m.Cp;
            d.Cv = m.Cp - GAS_R / m.M;  // Material::URS, src/global.cpp:11-12
            d.gam = m.Cp / d.Cv;
            d.gm1 = d.gam - 1;
            mats.push_back(d);
        }
        c.mats = upload(mats);
        c.mat0 = mats[0];
        if (mats.size() > 1) c.cmat = upload(lay_.cmat);
        std::vector<DevBnd> bnds;
        for (auto& b : task_.bnds) {
            DevBnd d{};
            d.kind = b.kind;
            d.u = b.par[0]; d.v = b.par[1]; d.T = b.par[2]; d.p = b.par[3];
            bnds.push_back(d);
        }
        if (bnds.empty()) bnds.push_back(DevBnd{});
        c.bnds = upload(bnds);
        const size_t n4 = 4 * (size_t)nc;
        c.A = dalloc<double>(n4);
        c.W = dalloc<double>(n4);
        c.G = dalloc<double>(8 * (size_t)nc);
        c.F = dalloc<double>(4 * (size_t)ne);
        c.R = dalloc<double>(4 * (size_t)ne);
        c.ctau = dalloc<double>(nc);
        c.cfl = dalloc<double>(1);
        c.flags = dalloc<unsigned>(nc);
        c.err = dalloc<unsigned>(1);
        c.D = dalloc<double>(16 * (size_t)nc);
        c.O = dalloc<double>(48 * (size_t)nc);
        c.b = dalloc<double>(n4);
        c.x = dalloc<double>(n4);
        c.x2 = task_.smoothing ? dalloc<double>(n4) : c.x;
        c.V = dalloc<double>((size_t)(c.kdim + 1) * n4);
        c.r = dalloc<double>(n4);
        c.part = dalloc<double>((size_t)(kGmresMaxKdim + 1) * kRedBlocks);
        c.ctl = dalloc<GmresCtl>(1);
        c.n_lim = dalloc<int>(1);
        stage_ = dalloc<double>(48 * (size_t)nc);
        CUDA_CHECK(cudaMallocHost(&ctl_host_, sizeof(GmresCtl)));
        std::memset(ctl_host_, 0, sizeof(GmresCtl));
        CUDA_CHECK(cudaMemsetAsync(c.flags, 0, sizeof(unsigned) * nc, stream_));
        CUDA_CHECK(cudaMemsetAsync(c.err, 0, sizeof(unsigned), stream_));
        CUDA_CHECK(cudaMemsetAsync(c.ctl, 0, sizeof(GmresCtl), stream_));
        // initial state from the regions (:176-180), storage order
        std::vector<double> U(n4);
        std::vector<std::array<double, 4>> reg(task_.regions.size());
        for (size_t r = 0; r < reg.size(); r++)
            region_state(task_.mats[task_.regions[r].matId], task_.regions[r], reg[r].data());
        for (int i = 0; i < nc; i++) {
            const auto& u = reg[cell_region[lay_.perm[i]]];
            for (int k = 0; k < 4; k++) U[(size_t)k * nc + i] = u[k];
        }
        CUDA_CHECK(cudaMemcpyAsync(c.A, U.data(), U.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
        // calcTimeStep, :296-333: STEADY=0 gives every cell TAU; STEADY=1 forms cTau in each
        // step's assembly and leaves the array unset before the first (new double[], read by
        // save(0)): zero here, which is what a fresh allocation reads as
        std::vector<double> ct(nc, task_.steady ? 0.0 : task_.tau);
        CUDA_CHECK(cudaMemcpyAsync(c.ctau, ct.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
        cfl_ = task_.cfl;
        CUDA_CHECK(cudaMemcpyAsync(c.cfl, &cfl_, sizeof(double), cudaMemcpyHostToDevice, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        build_graphs();
    } catch (...) {
        for (void* p : allocs_) cudaFree(p);
        allocs_.clear();
        if (ctl_host_) cudaFreeHost(ctl_host_);
        ctl_host_ = nullptr;
        if (stream_) cudaStreamDestroy(stream_);
        stream_ = nullptr;
        throw;
    }
}

ImplicitSolver::~ImplicitSolver() {
    use_device();
    if (stream_) cudaStreamSynchronize(stream_);
    if (g_step_) cudaGraphExecDestroy(g_step_);
    if (g_restart_) cudaGraphExecDestroy(g_restart_);
    for (void* p : allocs_) cudaFree(p);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    if (stream_) cudaStreamDestroy(stream_);
}

// The step as two graphs: assembly + first GMRES cycle + post-solve update, and a
// further cycle + update for the rare case where the true residual asks for a restart.
// Each ends with a copy of the control block into pinned host memory.
void ImplicitSolver::build_graphs() {
    auto capture = [&](bool first) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ex = nullptr;
        CUDA_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        if (first) {
            imp_launch_prims(ic_, stream_);
            imp_launch_grad(ic_, stream_);
            imp_launch_flux(ic_, stream_);
            imp_launch_assemble(ic_, stream_);
        }
        imp_launch_gmres_cycle(ic_, first, stream_);
        imp_launch_post(ic_, stream_);
        CUDA_CHECK(cudaMemcpyAsync(ctl_host_, ic_.ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, stream_));
        CUDA_CHECK(cudaStreamEndCapture(stream_, &g));
        CUDA_CHECK(cudaGraphInstantiate(&ex, g, 0));
        cudaGraphDestroy(g);
        return ex;
    };
    g_step_ = capture(true);
    g_restart_ = capture(false);
}

// One pass of run()'s loop body, :527-735. The host keeps t, the step counter and the
// CFL rules; the solve status, iteration count and limited-cell count come back in
// the control block.
void ImplicitSolver::one_step() {
    if (!task_.steady) t_ += task_.tau;
    if (!solver_err_) steps_++;
    CUDA_CHECK(cudaGraphLaunch(g_step_, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    for (int guard = 0; ctl_host_->restart && guard <= task_.gmres_maxit; guard++) {
        CUDA_CHECK(cudaGraphLaunch(g_restart_, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
    }
    last_ = *ctl_host_;
    solver_err_ = last_.status;
    const double cfl0 = cfl_;
    auto dec_cfl = [&] {  // decCFL, :1070-1077
        if (cfl_ > 0.1) {
            cfl_ *= 0.75;
            if (cfl_ < 0.1) cfl_ = 0.1;
            log_line(" CFL Number has been decreased : %f \n", cfl_);
        }
    };
    if (solver_err_ == SOLVE_OK) {
        failed_in_row_ = 0;
        if (task_.steady && last_.n_lim >= task_.max_lim_cells) dec_cfl();
    } else {
        failed_in_row_++;
        if (task_.steady) dec_cfl();
        else solver_err_ = 0;
    }
    if (cfl_ != cfl0) CUDA_CHECK(cudaMemcpyAsync(ic_.cfl, &cfl_, sizeof(double), cudaMemcpyHostToDevice, stream_));
}

// incCFL, :1079-1086, at the end of a successful step
static bool inc_cfl(double& cfl, const TaskConfig& t) {
    if (cfl < t.cfl_max) {
        cfl *= t.cfl_scale;
        if (cfl > t.cfl_max) cfl = t.cfl_max;
        log_line(" CFL Number has been increased : %f \n", cfl);
        return true;
    }
    return false;
}

int ImplicitSolver::step(int n) {
    use_device();
    for (int k = 0; k < n; k++) {
        one_step();
        if (solver_err_ == SOLVE_OK && task_.steady && task_.cfl_step > 0 && steps_ % task_.cfl_step == 0)
            if (inc_cfl(cfl_, task_))
                CUDA_CHECK(cudaMemcpyAsync(ic_.cfl, &cfl_, sizeof(double), cudaMemcpyHostToDevice, stream_));
    }
    return read_status();
}

// The device error word since the last read (cleared): the Newton cap of the exact Riemann
// solver, or a non-positive / NaN density or pressure seen by the step.
int ImplicitSolver::read_status() {
    unsigned e = 0;
    CUDA_CHECK(cudaMemcpyAsync(&e, ic_.err, sizeof e, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaMemsetAsync(ic_.err, 0, sizeof(unsigned), stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    if (e & ERRBIT_NONPHYSICAL) return CFD2D_ERR_NONPHYSICAL;
    if (e & ERRBIT_NEWTON_CAP) return CFD2D_ERR_NEWTON_CAP;
    return CFD2D_OK;
}

int ImplicitSolver::run() {  // FVM_TVD_IMPLICIT::run, :478-738
    use_device();
    if (steps_ == 0) save_vtk(0);  // init's save(0), :183
    const int ne = topo_.ne;
    log_line(task_.steady ? "Steady-State Flow\n" : "Unsteady-State Flow\n");
    log_line("TMAX = %e STEP_MAX = %d\n", task_.tmax, task_.step_max);
    log_line("Flux calculation method: %s\n", task_.flux == FLUX_LAX ? "LAX" : "GODUNOV");
    log_line("Matrix structure initialization:\n");
    for (int e = 0; e < ne; e += 100) log_line("\tfor edge: %d\n", e);
    log_line("\tcomplete...\n");
    int status = CFD2D_OK;
    const unsigned smax = (unsigned)task_.step_max;
    while (t_ < task_.tmax && (unsigned)steps_ < smax) {
        auto t0 = std::chrono::steady_clock::now();
        one_step();
        // a steady run whose solves keep failing never advances its step counter (the
        // reference loops forever there); stop after kMaxFailedSolves passes in a row
        if (task_.steady && failed_in_row_ >= kMaxFailedSolves)
            throw Error(CFD2D_ERR_SOLVER, "the linear solver failed " + std::to_string(failed_in_row_) +
                                              " times in a row at the smallest CFL number");
        if (solver_err_ == SOLVE_OK) {
            auto t1 = std::chrono::steady_clock::now();
            const long ms = (long)std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
            if (task_.file_step != 0 && steps_ % task_.file_step == 0) save_vtk(steps_);
            if (task_.print_step != 0 && steps_ % task_.print_step == 0) {
                if (!task_.steady)
                    log_line("step: %d\ttime step: %.16f\tmax iter: %d\tlim: %d\ttime: %ld ms\n", steps_, t_, last_.it,
                             last_.n_lim, ms);
                else
                    log_line("step: %d\tmax iter: %d\tlim: %d\ttime: %ld ms\n", steps_, last_.it, last_.n_lim, ms);
            }
            if (task_.steady && task_.cfl_step > 0 && steps_ % task_.cfl_step == 0)
                if (inc_cfl(cfl_, task_))
                    CUDA_CHECK(cudaMemcpyAsync(ic_.cfl, &cfl_, sizeof(double), cudaMemcpyHostToDevice, stream_));
        }
    }
    const int s = read_status();
    return s != CFD2D_OK ? s : status;
}

void ImplicitSolver::get_state(double* ro, double* ru, double* rv, double* re) {
    use_device();
    const int nc = ic_.nc;
    HostArrays4 hv;
    bool direct = true;
    double* dst4[4] = {ro, ru, rv, re};
    for (int k = 0; k < 4; k++) {
        hv.p[k] = dst4[k] ? static_cast<double*>(device_view(dst4[k])) : nullptr;
        if (dst4[k] && !hv.p[k]) direct = false;
    }
    if (direct) {  // one pass: permute and write over the host link
        launch_scatter_state_host(perm_case(ic_), ic_.A, hv, stream_);
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        return;
    }
    launch_scatter_state(perm_case(ic_), ic_.A, stage_, stream_);
    double* dst[4] = {ro, ru, rv, re};
    for (int k = 0; k < 4; k++)
        if (dst[k])
            CUDA_CHECK(cudaMemcpyAsync(dst[k], stage_ + (size_t)k * nc, sizeof(double) * nc, cudaMemcpyDeviceToHost,
                                       stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void ImplicitSolver::set_state(const double* ro, const double* ru, const double* rv, const double* re) {
    use_device();
    const int nc = ic_.nc;
    const double* src[4] = {ro, ru, rv, re};
    HostArrays4 hv;
    bool direct = true;
    for (int k = 0; k < 4; k++) {
        if (!src[k]) throw Error(CFD2D_ERR_INVALID_ARG, "set_state: all four arrays are required");
        hv.p[k] = static_cast<double*>(device_view(src[k]));
        if (!hv.p[k]) direct = false;
    }
    if (direct) {
        launch_gather_state_host(perm_case(ic_), hv, ic_.A, stream_);
    } else {
        for (int k = 0; k < 4; k++)
            CUDA_CHECK(cudaMemcpyAsync(stage_ + (size_t)k * nc, src[k], sizeof(double) * nc, cudaMemcpyHostToDevice,
                                       stream_));
        launch_gather_state(perm_case(ic_), stage_, ic_.A, stream_);
    }
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void ImplicitSolver::get_ctau(double* out) {
    use_device();
    launch_permute_scalar(perm_case(ic_), ic_.ctau, stage_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(out, stage_, sizeof(double) * ic_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void ImplicitSolver::get_flags(unsigned* out) {
    use_device();
    unsigned* tmp = reinterpret_cast<unsigned*>(stage_);
    launch_permute_flags(perm_case(ic_), ic_.flags, tmp, stream_);
    CUDA_CHECK(cudaMemcpyAsync(out, tmp, sizeof(unsigned) * ic_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void ImplicitSolver::assemble_only() {
    imp_launch_prims(ic_, stream_);
    imp_launch_grad(ic_, stream_);
    imp_launch_flux(ic_, stream_);
    imp_launch_assemble(ic_, stream_);
}

void ImplicitSolver::system(double* diag, double* off, double* rhs, double* ctau) {
    use_device();
    const size_t nc = (size_t)ic_.nc;
    assemble_only();
    struct Part { double* dst; int which; size_t per; };
    const Part parts[3] = {{diag, 0, 16}, {off, 1, 48}, {rhs, 2, 4}};
    for (const Part& p : parts) {
        if (!p.dst) continue;
        imp_launch_permute_blocks(ic_, stage_, p.which, stream_);
        CUDA_CHECK(cudaMemcpyAsync(p.dst, stage_, sizeof(double) * p.per * nc, cudaMemcpyDeviceToHost, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
    }
    if (ctau) get_ctau(ctau);
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void ImplicitSolver::save_vtk(int step) {
    const int nc = topo_.nc;
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    get_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc);
    get_ctau(ct.data());
    std::vector<int> cell_mat(nc);
    for (int i = 0; i < nc; i++) cell_mat[i] = lay_.cmat.empty() ? 0 : lay_.cmat[lay_.iperm[i]];
    char name[64];
    std::snprintf(name, sizeof name, "res_%010d.vtk", step);
    write_vtk_file(name, topo_, task_.mats, cell_mat, U.data(), ct.data(), true);
    announce_vtk(name);
}

void ImplicitSolver::profile_steps(int n, double ms[4], int launches[4]) {
    use_device();
    for (int k = 0; k < 4; k++) { ms[k] = 0.0; launches[k] = 0; }
    cudaEvent_t ev[5];
    for (auto& e : ev) CUDA_CHECK(cudaEventCreate(&e));
    // kernels of one GMRES cycle and the update: reset, |src|, v0; per column spmv, the
    // inner-product passes (12 vectors each), hcol, orth, givens; solve, x, residual,
    // finish; post_begin, [smoothing], update, remediation, count
    const int jmax = std::min(ic_.kdim, ic_.maxit);
    int gm_launches = 3 + 4 + 4 + (task_.smoothing ? 1 : 0);
    for (int j = 0; j < jmax; j++) gm_launches += 4 + (j + 12) / 12;
    for (int s = 0; s < n; s++) {
        if (!task_.steady) t_ += task_.tau;
        if (!solver_err_) steps_++;
        CUDA_CHECK(cudaEventRecord(ev[0], stream_));
        imp_launch_prims(ic_, stream_);
        imp_launch_grad(ic_, stream_);
        CUDA_CHECK(cudaEventRecord(ev[1], stream_));
        imp_launch_flux(ic_, stream_);
        CUDA_CHECK(cudaEventRecord(ev[2], stream_));
        imp_launch_assemble(ic_, stream_);
        CUDA_CHECK(cudaEventRecord(ev[3], stream_));
        imp_launch_gmres_cycle(ic_, true, stream_);
        imp_launch_post(ic_, stream_);
        CUDA_CHECK(cudaEventRecord(ev[4], stream_));
        CUDA_CHECK(cudaMemcpyAsync(ctl_host_, ic_.ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        for (int k = 0; k < 4; k++) {
            float t = 0;
            CUDA_CHECK(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            ms[k] += t;
        }
        launches[0] += 2; launches[1] += 1; launches[2] += 1; launches[3] += gm_launches;
        for (int guard = 0; ctl_host_->restart && guard <= task_.gmres_maxit; guard++) {
            CUDA_CHECK(cudaGraphLaunch(g_restart_, stream_));
            CUDA_CHECK(cudaStreamSynchronize(stream_));
        }
        last_ = *ctl_host_;
        solver_err_ = last_.status;
        if (solver_err_ != SOLVE_OK && !task_.steady) solver_err_ = 0;
    }
    for (auto& e : ev) cudaEventDestroy(e);
}

// Binary restart file of an implicit handle: "CFD2DIM1", cell count, step counter and the
// last solve's status (int64), time and CFL number, then the conserved state (4 x nc,
// cell order of the mesh files), cTau (nc) and the flag words (nc).
namespace {
constexpr char kImpStateMagic[8] = {'C', 'F', 'D', '2', 'D', 'I', 'M', '1'};
}

void ImplicitSolver::save_state(const char* path) {
    use_device();
    const int nc = ic_.nc;
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    std::vector<unsigned> fl(nc);
    get_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc);
    get_ctau(ct.data());
    get_flags(fl.data());
    FILE* fp = std::fopen(path, "wb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    const int64_t hdr[3] = {nc, steps_, solver_err_};
    const double hd[2] = {t_, cfl_};
    bool ok = std::fwrite(kImpStateMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof hdr, 1, fp) == 1 &&
              std::fwrite(hd, sizeof hd, 1, fp) == 1 &&
              std::fwrite(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fwrite(ct.data(), sizeof(double), ct.size(), fp) == ct.size() &&
              std::fwrite(fl.data(), sizeof(unsigned), fl.size(), fp) == fl.size();
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' write error.");
}

void ImplicitSolver::load_state(const char* path) {
    use_device();
    const int nc = ic_.nc;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    char magic[8];
    int64_t hdr[3];
    double hd[2];
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    std::vector<unsigned> fl(nc);
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kImpStateMagic, 8) == 0 &&
              std::fread(hdr, sizeof hdr, 1, fp) == 1 && hdr[0] == nc && std::fread(hd, sizeof hd, 1, fp) == 1 &&
              std::fread(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fread(ct.data(), sizeof(double), ct.size(), fp) == ct.size() &&
              std::fread(fl.data(), sizeof(unsigned), fl.size(), fp) == fl.size();
    std::fclose(fp);
    if (!ok) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("File '") + path + "' is not a state of this mesh.");
    set_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc);
    steps_ = (int)hdr[1];
    solver_err_ = (int)hdr[2];
    t_ = hd[0];
    cfl_ = hd[1];
    std::vector<double> cts(nc);
    std::vector<unsigned> fls(nc);
    for (int i = 0; i < nc; i++) {  // storage cell i holds file cell perm[i]
        cts[i] = ct[lay_.perm[i]];
        fls[i] = fl[lay_.perm[i]];
    }
    CUDA_CHECK(cudaMemcpyAsync(ic_.ctau, cts.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaMemcpyAsync(ic_.flags, fls.data(), sizeof(unsigned) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaMemcpyAsync(ic_.cfl, &cfl_, sizeof(double), cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

double ImplicitSolver::timed_steps(int n) {
    use_device();
    cudaEvent_t a, b;
    CUDA_CHECK(cudaEventCreate(&a));
    CUDA_CHECK(cudaEventCreate(&b));
    CUDA_CHECK(cudaEventRecord(a, stream_));
    step(n);
    CUDA_CHECK(cudaEventRecord(b, stream_));
    CUDA_CHECK(cudaEventSynchronize(b));
    float ms = 0;
    CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

}  // namespace cfd2d
