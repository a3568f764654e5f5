#include "solver.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>

#include "cfd2d.h"

namespace cfd2d {

// ------------------------------------------------------------------ logging

namespace {
std::mutex g_log_mu;
int g_verbosity = 1;
FILE* g_log_file = nullptr;
constexpr int kConservationBlocks = 512;
}  // namespace

void log_line(const char* fmt, ...) {  // log(), src/global.cpp:32-46
    std::lock_guard<std::mutex> lk(g_log_mu);
    if (g_verbosity > 0) {
        va_list a;
        va_start(a, fmt);
        std::vprintf(fmt, a);
        va_end(a);
        std::fflush(stdout);
    }
    if (g_log_file) {
        va_list a;
        va_start(a, fmt);
        std::vfprintf(g_log_file, fmt, a);
        va_end(a);
        std::fflush(g_log_file);
    }
}

void set_verbosity(int v) {
    std::lock_guard<std::mutex> lk(g_log_mu);
    g_verbosity = v;
}

void set_log_file(const char* path) {
    std::lock_guard<std::mutex> lk(g_log_mu);
    if (g_log_file) std::fclose(g_log_file);
    g_log_file = path ? std::fopen(path, "a") : nullptr;
    if (path && !g_log_file) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
}

// ------------------------------------------------------------------ solver

template <typename T>
static std::vector<float> to_f32(const std::vector<T>& v) {
    return std::vector<float>(v.begin(), v.end());
}

Solver::Solver(const TaskConfig& t, Topo&& topo, const std::vector<int>& cell_region,
               const std::vector<int>& edge_bnd, int gauss_points, std::vector<Instance> instances)
    : task_(t), topo_(std::move(topo)), gauss_points_(gauss_points), inst_(std::move(instances)) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(CFD2D_ERR_NO_DEVICE, "no CUDA device");
    CUDA_CHECK(cudaGetDevice(&dev_));
    const int nc = topo_.nc;
    cell_mat_.resize(nc);
    for (int i = 0; i < nc; i++) cell_mat_[i] = task_.regions[cell_region[i]].matId;
    const int order = task_.reorder >= 0 ? task_.reorder
                                         : (task_.fused == 1 || task_.fused == 2 ? ORDER_HILBERT : ORDER_RCM);
    lay_ = make_layout(topo_, cell_mat_, edge_bnd, order);
    const int ne = lay_.ne;
    CUDA_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    try {
        DevCase& c = dc_;
        c.nc = nc; c.ne = ne; c.n_int = lay_.n_int;
        c.face = upload(lay_.face);
        c.ec1 = upload(lay_.ec1);
        c.ec2 = upload(lay_.ec2);
        c.ebnd = upload(lay_.ebnd);
        c.S = upload(lay_.S);
        c.rem_nb = upload(lay_.rem_nb);
        c.iperm = upload(lay_.iperm);
        const bool mixed = task_.precision == PREC_MIXED;
        {
            std::vector<int> nb(3 * (size_t)nc);
            std::vector<double> fx(3 * (size_t)nc), fy(3 * (size_t)nc), fl(3 * (size_t)nc);
            for (size_t q = 0; q < 3 * (size_t)nc; q++) {
                const int f = lay_.face[q], e = f >> 1, side = f & 1;
                const int j = side ? lay_.ec1[e] : lay_.ec2[e];
                nb[q] = j >= 0 ? ((j << 1) | side) : -(e + 1);
                fx[q] = lay_.nx[e]; fy[q] = lay_.ny[e]; fl[q] = lay_.l[e];
            }
            c.cf_nb = upload(nb);
            if (mixed) {
                // the mixed form's gradient weights RN32(n l / 2), from the FP64 product
                std::vector<float> ax(3 * (size_t)nc), ay(3 * (size_t)nc);
                for (size_t q = 0; q < 3 * (size_t)nc; q++) {
                    ax[q] = (float)(fx[q] * fl[q] * 0.5);
                    ay[q] = (float)(fy[q] * fl[q] * 0.5);
                }
                c.cf_ax32 = upload(ax); c.cf_ay32 = upload(ay);
                std::vector<float4> rec(3 * (size_t)nc);
                for (int i = 0; i < nc; i++)
                    for (int k = 0; k < 3; k++) {
                        const size_t q = (size_t)k * nc + i;
                        float nbf;
                        std::memcpy(&nbf, &nb[q], sizeof nbf);
                        rec[3 * (size_t)i + k] = make_float4(nbf, ax[q], ay[q], 0.f);
                    }
                c.cfrec32 = upload(rec);
            } else {
                c.cf_nx = upload(fx); c.cf_ny = upload(fy); c.cf_l = upload(fl);
                if (task_.recon == RECON_MINMOD) {
                    std::vector<double> ax(3 * (size_t)nc), ay(3 * (size_t)nc);
                    for (size_t q = 0; q < 3 * (size_t)nc; q++) {
                        ax[q] = fx[q] * fl[q] * 0.5;
                        ay[q] = fy[q] * fl[q] * 0.5;
                    }
                    c.cf_ax = upload(ax); c.cf_ay = upload(ay);
                }
            }
        }
        if (mixed) {
            c.nx32 = upload(to_f32(lay_.nx));
            c.ny32 = upload(to_f32(lay_.ny));
            c.l32 = upload(to_f32(lay_.l));
            std::vector<float> ex(ne), ey(ne);
            for (int e = 0; e < ne; e++) {
                ex[e] = (float)(lay_.nx[e] * lay_.l[e] * 0.5);
                ey[e] = (float)(lay_.ny[e] * lay_.l[e] * 0.5);
            }
            c.ax32 = upload(ex); c.ay32 = upload(ey);
            std::vector<float4> geo(3 * (size_t)ne);
            for (int e = 0; e < ne; e++) {
                const double* d = lay_.dl.data() + e;
                auto dl = [&](int k) { return (float)d[(size_t)k * ne]; };
                geo[3 * (size_t)e] = make_float4((float)lay_.nx[e], (float)lay_.ny[e], (float)lay_.l[e], 0.f);
                geo[3 * (size_t)e + 1] = make_float4(dl(0), dl(1), dl(2), dl(3));
                geo[3 * (size_t)e + 2] = make_float4(dl(4), dl(5), dl(6), dl(7));
            }
            c.geo32 = upload(geo);
            c.dl32 = upload(to_f32(lay_.dl));
            std::vector<float> is(nc);
            for (int i = 0; i < nc; i++) is[i] = (float)(1.0 / lay_.S[i]);
            c.invS32 = upload(is);
        } else {
            std::vector<double> is(nc);
            for (int i = 0; i < nc; i++) is[i] = 1.0 / lay_.S[i];
            c.invS = upload(is);
            c.nx = upload(lay_.nx);
            c.ny = upload(lay_.ny);
            c.l = upload(lay_.l);
            c.dl = upload(lay_.dl);
        }
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
        c.mat0_f[0] = (float)mats[0].M; c.mat0_f[1] = (float)mats[0].Cv; c.mat0_f[2] = (float)mats[0].gm1;
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
        c.gam_flux = 1.4;  // hard-coded in FVM_TVD::run, src/methods/fvm_tvd.cpp:345,398
        c.gam_flux_f = 1.4f;
        c.ig1_flux = 1.0 / (c.gam_flux - 1.0);
        c.rg_flux = rim_gas<double>(c.gam_flux);
        c.ig1_flux_f = 1.0f / (c.gam_flux_f - 1.0f);
        c.lim_f[0] = (float)task_.lim_rmin; c.lim_f[1] = (float)task_.lim_rmax;
        c.lim_f[2] = (float)task_.lim_pmin; c.lim_f[3] = (float)task_.lim_pmax; c.lim_f[4] = (float)task_.lim_umax;
        c.cfl_number = task_.cfl;
        c.lim_rmin = task_.lim_rmin; c.lim_rmax = task_.lim_rmax;
        c.lim_pmin = task_.lim_pmin; c.lim_pmax = task_.lim_pmax; c.lim_umax = task_.lim_umax;
        c.steady = task_.steady;
        c.newton_cap = task_.newton_cap;
        c.flux_pipe = mixed && task_.flux_pipe != 0 ? 1 : 0;
        if (c.flux_pipe) launch_flux_prepare_mixed();
        c.A = dalloc<double>(4 * (size_t)nc);
        c.B = dalloc<double>(4 * (size_t)nc);
        c.cfl = dalloc<double>(nc);
        c.ctau = dalloc<double>(nc);
        c.ctau_next = task_.steady ? dalloc<double>(nc) : c.ctau;
        c.flags = dalloc<unsigned>(nc);
        c.n_lim = dalloc<int>(1);
        c.err = dalloc<unsigned>(1);
        if (mixed) {
            c.W32 = dalloc<float>(4 * (size_t)nc);
            c.G32 = dalloc<float>(8 * (size_t)nc);
            c.F32 = dalloc<float>(4 * (size_t)ne);
        } else {
            c.W64 = dalloc<double>(4 * (size_t)nc);
            c.G64 = dalloc<double>(8 * (size_t)nc);
            c.F64 = dalloc<double>(4 * (size_t)ne);
        }
        stage_ = dalloc<double>(4 * (size_t)nc);
        dtmin_ = dalloc<unsigned long long>(1);
        partial_ = dalloc<double>(4 * kConservationBlocks);
        CUDA_CHECK(cudaMemsetAsync(c.flags, 0, sizeof(unsigned) * nc, stream_));
        CUDA_CHECK(cudaMemsetAsync(c.n_lim, 0, sizeof(int), stream_));
        CUDA_CHECK(cudaMemsetAsync(c.err, 0, sizeof(unsigned), stream_));
        // initial state from the regions (src/methods/fvm_tvd.cpp:199-204), storage order
        std::vector<double> U(4 * (size_t)nc);
        std::vector<std::array<double, 4>> reg(task_.regions.size());
        for (size_t r = 0; r < reg.size(); r++)
            region_state(task_.mats[task_.regions[r].matId], task_.regions[r], reg[r].data());
        for (int i = 0; i < nc; i++) {
            const auto& u = reg[cell_region[lay_.perm[i]]];
            for (int k = 0; k < 4; k++) U[(size_t)k * nc + i] = u[k];
        }
        CUDA_CHECK(cudaMemcpyAsync(c.A, U.data(), U.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
        tau_ = task_.tau;
        launch_prims(c, task_.precision, stream_);
        compute_tau();
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        if (!task_.steady && inst_.empty()) log_line("time step: %25.16E\n", tau_);  // calcTimeStep, :238
        build_tiles();
        build_graph();
    } catch (...) {
        for (void* p : allocs_) cudaFree(p);
        allocs_.clear();
        if (stream_) cudaStreamDestroy(stream_);
        stream_ = nullptr;
        throw;
    }
}

void Solver::release(void* p, size_t bytes) {
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    auto it = std::find(allocs_.begin(), allocs_.end(), p);
    if (it == allocs_.end()) return;
    allocs_.erase(it);
    cudaFree(p);
    bytes_ -= std::min(bytes_, bytes);
}

Solver::~Solver() {
    use_device();
    if (vtk_thread_.joinable()) {
        {
            std::lock_guard<std::mutex> lk(vtk_mu_);
            vtk_stop_ = true;
        }
        vtk_cv_.notify_all();
        vtk_thread_.join();
    }
    for (int k = 0; k < 2; k++) {
        if (snap_host_[k]) cudaFreeHost(snap_host_[k]);
        if (snap_ev_[k]) cudaEventDestroy(snap_ev_[k]);
    }
    drop_record_graphs();
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (stream_) cudaStreamSynchronize(stream_);
    for (void* p : allocs_) cudaFree(p);
    if (stream_) cudaStreamDestroy(stream_);
}

// calcTimeStep at init (src/methods/fvm_tvd.cpp:216-240): STEADY=1 leaves the
// per-cell cTau from launch_prims; STEADY=0 takes TAU = min(TAU, min_i ...).
void Solver::compute_tau() {
    if (task_.steady) return;
    if (!inst_.empty()) {
        compute_tau_batch();
        return;
    }
    unsigned long long init;
    double t0 = tau_;
    std::memcpy(&init, &t0, sizeof init);
    if (!(t0 > 0)) init = 0x7ff0000000000000ull;
    CUDA_CHECK(cudaMemcpyAsync(dtmin_, &init, sizeof init, cudaMemcpyHostToDevice, stream_));
    launch_dt_min(dc_, dtmin_, stream_);
    unsigned long long bits;
    CUDA_CHECK(cudaMemcpyAsync(&bits, dtmin_, sizeof bits, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    double m;
    std::memcpy(&m, &bits, sizeof m);
    if (!(t0 > m)) m = t0;
    tau_ = m;
    launch_fill_cfl(dc_, tau_, stream_);
}

// One time step. With ev/kinds/nev, an event pair brackets each kernel launch
// (profiling); the captured graph has no events.
void Solver::enqueue_step(cudaEvent_t* ev, int* kinds, int* nev) {
    const int nst = task_.scheme == TIME_EULER ? 1 : (task_.scheme == TIME_HEUN ? 2 : 3);
    const int p = task_.precision;
    auto mark = [&](int kind, bool begin) {
        if (!ev) return;
        if (begin) kinds[*nev / 2] = kind;
        CUDA_CHECK(cudaEventRecord(ev[(*nev)++], stream_));
    };
    if (fused_ == 2 && gauss_points_ != 0) {  // gradients, then one tiled flux-and-update kernel per stage
        for (int st = 0; st < nst; st++) {
            DevCase cs = dc_;  // the stage's primitives, rotated through wrot_
            cs.W32 = wrot_[st];
            if (task_.recon != RECON_NONE) {
                mark(0, true);
                launch_grad(cs, p, stream_);
                mark(0, false);
            }
            mark(1, true);
            launch_flux_update_mixed(cs, tiles_, task_.flux, task_.recon, task_.scheme, st, wrot_[(st + 1) % nst],
                                     stream_);
            mark(1, false);
        }
        mark(3, true);
        launch_remediate(dc_, p, stream_);
        mark(3, false);
        return;
    }
    if (fused_ == 1 && gauss_points_ != 0) {  // one tiled kernel per stage, primitives rotated through wrot_
        for (int st = 0; st < nst; st++) {
            mark(1, true);
            launch_stage_fused_mixed(dc_, tiles_, task_.flux, task_.recon, task_.scheme, st, wrot_[st],
                                     wrot_[(st + 1) % nst], stream_);
            mark(1, false);
        }
        mark(3, true);
        launch_remediate(dc_, p, stream_);
        mark(3, false);
        return;
    }
    for (int st = 0; st < nst; st++) {
        if (fused_ == 3) {  // the flux kernel forms the gradients it needs
            mark(1, true);
            launch_flux_grad_mixed(dc_, task_.flux, task_.recon, stream_);
            mark(1, false);
        } else if (gauss_points_ == 0) {  // 1-point edges: the Gauss-point loop is empty, no flux
            size_t b = 4 * (size_t)dc_.ne * (p == PREC_MIXED ? sizeof(float) : sizeof(double));
            CUDA_CHECK(cudaMemsetAsync(p == PREC_MIXED ? (void*)dc_.F32 : (void*)dc_.F64, 0, b, stream_));
        } else {
            if (task_.recon != RECON_NONE) {
                mark(0, true);
                launch_grad(dc_, p, stream_);
                mark(0, false);
            }
            mark(1, true);
            launch_flux(dc_, p, task_.flux, task_.recon, stream_);
            mark(1, false);
        }
        mark(2, true);
        launch_update(dc_, p, task_.scheme, st, stream_);
        mark(2, false);
    }
    mark(3, true);
    launch_remediate(dc_, p, stream_);
    mark(3, false);
}

double Solver::timed_steps(int n) {
    use_device();
    cudaEvent_t a, b;
    CUDA_CHECK(cudaEventCreate(&a));
    CUDA_CHECK(cudaEventCreate(&b));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    CUDA_CHECK(cudaEventRecord(a, stream_));
    for (int k = 0; k < n; k++) {
        if (!task_.steady) t_ += tau_;
        CUDA_CHECK(cudaGraphLaunch(gexec_, stream_));
        steps_++;
    }
    CUDA_CHECK(cudaEventRecord(b, stream_));
    CUDA_CHECK(cudaEventSynchronize(b));
    float ms = 0;
    CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

void Solver::profile_steps(int n, double ms[4], int launches[4]) {
    use_device();
    for (int k = 0; k < 4; k++) { ms[k] = 0; launches[k] = 0; }
    std::vector<cudaEvent_t> ev(32);
    for (auto& e : ev) CUDA_CHECK(cudaEventCreate(&e));
    int kinds[16];
    for (int s = 0; s < n; s++) {
        int nev = 0;
        if (!task_.steady) t_ += tau_;
        enqueue_step(ev.data(), kinds, &nev);
        steps_++;
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        for (int j = 0; j + 1 < nev; j += 2) {
            float t = 0;
            CUDA_CHECK(cudaEventElapsedTime(&t, ev[j], ev[j + 1]));
            ms[kinds[j / 2]] += t;
            launches[kinds[j / 2]]++;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
}

void Solver::build_graph() {
    CUDA_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue_step();
    } catch (...) {
        cudaGraph_t g;
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    CUDA_CHECK(cudaStreamEndCapture(stream_, &graph_));
    CUDA_CHECK(cudaGraphInstantiate(&gexec_, graph_, 0));
}

int Solver::read_status() {
    unsigned e = 0;
    CUDA_CHECK(cudaMemcpyAsync(&e, dc_.err, sizeof e, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaMemsetAsync(dc_.err, 0, sizeof(unsigned), stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    if (e & ERRBIT_NEWTON_CAP) return CFD2D_ERR_NEWTON_CAP;
    if (e & ERRBIT_NONPHYSICAL) return CFD2D_ERR_NONPHYSICAL;
    return CFD2D_OK;
}

int Solver::step(int n) {
    use_device();
    for (int k = 0; k < n; k++) {
        if (!task_.steady) t_ += tau_;  // src/methods/fvm_tvd.cpp:312-316
        if (!task_.steady)
            for (auto& in : inst_) in.t += in.tau;
        CUDA_CHECK(cudaGraphLaunch(gexec_, stream_));
        steps_++;
    }
    return read_status();
}

int Solver::run() {  // FVM_TVD::run, src/methods/fvm_tvd.cpp:303-462
    use_device();
    if (steps_ == 0) save_vtk_async(0);
    int status = CFD2D_OK;
    const unsigned smax = (unsigned)task_.step_max;
    while (t_ < task_.tmax && (unsigned)steps_ < smax) {
        if (!task_.steady) t_ += tau_;
        CUDA_CHECK(cudaGraphLaunch(gexec_, stream_));
        steps_++;
        const bool save = task_.file_step != 0 && steps_ % task_.file_step == 0;
        const bool print = task_.print_step != 0 && steps_ % task_.print_step == 0;
        if (save || print) {
            int s = read_status();
            if (s != CFD2D_OK) status = s;
            if (save) save_vtk_async(steps_);
            if (print) log_line("step: %d\t\ttime step: %.16f\n", steps_, t_);
        }
    }
    int s = read_status();
    vtk_flush();
    return s != CFD2D_OK ? s : status;
}

void* device_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if ((a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged) && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice) {  // device memory of the current GPU: used in place
        int dev = -1;
        return cudaGetDevice(&dev) == cudaSuccess && dev == a.device ? const_cast<void*>(p) : nullptr;
    }
    if (a.type == cudaMemoryTypeUnregistered) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v)
            return const_cast<void*>(p);
    }
    return nullptr;
}

// all four arrays as device views, or false (any array missing or not addressable)
static bool host_views(const double* const a[4], HostArrays4& v, bool all_required) {
    for (int k = 0; k < 4; k++) {
        if (!a[k]) {
            if (all_required) return false;
            v.p[k] = nullptr;
            continue;
        }
        v.p[k] = static_cast<double*>(device_view(a[k]));
        if (!v.p[k]) return false;
    }
    return true;
}

void Solver::get_state(double* ro, double* ru, double* rv, double* re) {
    use_device();
    const int nc = dc_.nc;
    const double* dst4[4] = {ro, ru, rv, re};
    HostArrays4 hv;
    if (host_views(dst4, hv, false)) {  // one pass: permute and write over the host link
        launch_scatter_state_host(dc_, dc_.A, hv, stream_);
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        return;
    }
    launch_scatter_state(dc_, dc_.A, stage_, stream_);
    double* dst[4] = {ro, ru, rv, re};
    for (int k = 0; k < 4; k++)
        if (dst[k])
            CUDA_CHECK(cudaMemcpyAsync(dst[k], stage_ + (size_t)k * nc, sizeof(double) * nc, cudaMemcpyDeviceToHost,
                                       stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::set_state(const double* ro, const double* ru, const double* rv, const double* re, bool reset_tau) {
    use_device();
    const int nc = dc_.nc;
    const double* src[4] = {ro, ru, rv, re};
    for (int k = 0; k < 4; k++)
        if (!src[k]) throw Error(CFD2D_ERR_INVALID_ARG, "set_state: all four arrays are required");
    HostArrays4 hv;
    if (host_views(src, hv, true)) {  // one pass: read over the host link and permute
        launch_gather_state_host(dc_, hv, dc_.A, stream_);
    } else {
        for (int k = 0; k < 4; k++)
            CUDA_CHECK(cudaMemcpyAsync(stage_ + (size_t)k * nc, src[k], sizeof(double) * nc, cudaMemcpyHostToDevice,
                                       stream_));
        launch_gather_state(dc_, stage_, dc_.A, stream_);
    }
    launch_prims(dc_, task_.precision, stream_);
    if (reset_tau) {
        tau_ = task_.tau;
        compute_tau();
    }
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::get_ctau(double* out) {
    use_device();
    launch_permute_scalar(dc_, dc_.ctau, stage_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(out, stage_, sizeof(double) * dc_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::get_flags(unsigned* out) {
    use_device();
    unsigned* tmp = reinterpret_cast<unsigned*>(stage_);
    launch_permute_flags(dc_, dc_.flags, tmp, stream_);
    CUDA_CHECK(cudaMemcpyAsync(out, tmp, sizeof(unsigned) * dc_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

// Binary restart file: "CFD2DST1", cell count, steps, time, global time step, then the
// conserved state (4 x nc, cell order of the mesh files), cTau (nc) and the flag words
// (nc), all little-endian as the host writes them.
namespace {
constexpr char kStateMagic[8] = {'C', 'F', 'D', '2', 'D', 'S', 'T', '1'};
}

void Solver::save_state(const char* path) {
    use_device();
    const int nc = dc_.nc;
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    std::vector<unsigned> fl(nc);
    get_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc);
    get_ctau(ct.data());
    get_flags(fl.data());
    FILE* fp = std::fopen(path, "wb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    const int64_t hdr[2] = {nc, steps_};
    const double hd[2] = {t_, tau_};
    bool ok = std::fwrite(kStateMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof hdr, 1, fp) == 1 &&
              std::fwrite(hd, sizeof hd, 1, fp) == 1 &&
              std::fwrite(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fwrite(ct.data(), sizeof(double), ct.size(), fp) == ct.size() &&
              std::fwrite(fl.data(), sizeof(unsigned), fl.size(), fp) == fl.size();
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' write error.");
}

void Solver::load_state(const char* path) {
    use_device();
    const int nc = dc_.nc;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + path + "' opening error.");
    char magic[8];
    int64_t hdr[2];
    double hd[2];
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    std::vector<unsigned> fl(nc);
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kStateMagic, 8) == 0 &&
              std::fread(hdr, sizeof hdr, 1, fp) == 1 && hdr[0] == nc && std::fread(hd, sizeof hd, 1, fp) == 1 &&
              std::fread(U.data(), sizeof(double), U.size(), fp) == U.size() &&
              std::fread(ct.data(), sizeof(double), ct.size(), fp) == ct.size() &&
              std::fread(fl.data(), sizeof(unsigned), fl.size(), fp) == fl.size();
    std::fclose(fp);
    if (!ok) throw Error(CFD2D_ERR_MESH_FORMAT, std::string("File '") + path + "' is not a state of this mesh.");
    set_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc, false);
    steps_ = (int)hdr[1];
    t_ = hd[0];
    tau_ = hd[1];
    // storage order: cell i holds file cell perm[i]
    std::vector<double> cts(nc);
    std::vector<unsigned> fls(nc);
    for (int i = 0; i < nc; i++) {
        cts[i] = ct[lay_.perm[i]];
        fls[i] = fl[lay_.perm[i]];
    }
    CUDA_CHECK(cudaMemcpyAsync(dc_.flags, fls.data(), sizeof(unsigned) * nc, cudaMemcpyHostToDevice, stream_));
    // STEADY=0: the saved global step; STEADY=1: the next step runs on ctau_next, which
    // set_state derived from the state, and cTau reads as saved
    if (!task_.steady) launch_fill_cfl(dc_, tau_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(dc_.ctau, cts.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::residual(double* R) {
    use_device();
    const int p = task_.precision;
    if (gauss_points_ == 0) {
        size_t b = 4 * (size_t)dc_.ne * (p == PREC_MIXED ? sizeof(float) : sizeof(double));
        CUDA_CHECK(cudaMemsetAsync(p == PREC_MIXED ? (void*)dc_.F32 : (void*)dc_.F64, 0, b, stream_));
    } else {
        if (task_.recon != RECON_NONE) launch_grad(dc_, p, stream_);
        launch_flux(dc_, p, task_.flux, task_.recon, stream_);
    }
    launch_residual(dc_, p, dc_.B, stream_);  // B is scratch between steps
    launch_scatter_state(dc_, dc_.B, stage_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(R, stage_, sizeof(double) * 4 * dc_.nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

void Solver::conservation(double sums[4]) {
    use_device();
    launch_conservation(dc_, partial_, kConservationBlocks, stream_);
    std::vector<double> h(4 * kConservationBlocks);
    CUDA_CHECK(cudaMemcpyAsync(h.data(), partial_, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    for (int k = 0; k < 4; k++) {
        double s = 0.0;
        for (int b = 0; b < kConservationBlocks; b++) s += h[4 * b + k];
        sums[k] = s;
    }
}

// FVM_TVD::save, src/methods/fvm_tvd.cpp:501-600 (same fields, formats and quirks).

// The VTK file of one state, exactly as FVM_TVD::save writes it (file name, fields,
// number formats, the single newline at the end of each field, the 8-per-line
// total pressure, the "Velosity" spelling; src/methods/fvm_tvd.cpp:501-600). The
// numbers are formatted on host threads, a block of items per thread, and written
// in order, so the bytes are those of a sequential fprintf loop.
// With implicit_format, FVM_TVD_IMPLICIT::save's variant (src/methods/fvm_tvd_implicit.cpp:
// 840-903): Mach number |u|/c, a Total_energy field, total pressure in %25.16e.
void write_vtk_file(const char* name, const Topo& topo, const std::vector<TaskMaterial>& mats,
                    const std::vector<int>& cell_mat, const double* U, const double* ct, bool implicit_format) {
    const int nc = topo.nc, nn = topo.nn;
    FILE* fp = std::fopen(name, "w");
    if (!fp) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + name + "' opening error.");
    struct P { double r, u, v, p, cz, T, gam, E; };
    auto par = [&](int i) {
        const TaskMaterial& m = mats[cell_mat[i]];
        double Cv = m.Cp - GAS_R / m.M, gam = m.Cp / Cv;
        P q;
        q.r = U[i];
        q.u = U[nc + i] / U[i];
        q.v = U[2 * (size_t)nc + i] / U[i];
        double E = U[3 * (size_t)nc + i] / U[i];
        q.E = E;
        double e = E - 0.5 * (q.u * q.u + q.v * q.v);
        q.p = q.r * e * (gam - 1);
        q.cz = std::sqrt(gam * q.p / q.r);
        double e2 = q.p / (q.r * (gam - 1));
        q.T = e2 / Cv;
        q.gam = gam;
        return q;
    };
    const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    constexpr int kBlock = 1 << 15;
    // items [0, n): item(i, out) appends item i's text; blocks formatted in parallel, written in order
    auto section = [&](int n, auto item) {
        std::vector<std::string> buf(nth);
        for (int base = 0; base < n; base += (int)nth * kBlock) {
            auto work = [&](unsigned t) {
                std::string& o = buf[t];
                o.clear();
                const int a = base + (int)t * kBlock, b = std::min(n, a + kBlock);
                for (int i = a; i < b; i++) item(i, o);
            };
            std::vector<std::thread> th;
            for (unsigned t = 1; t < nth; t++) th.emplace_back(work, t);
            work(0);
            for (auto& x : th) x.join();
            for (auto& o : buf) std::fwrite(o.data(), 1, o.size(), fp);
        }
    };
    auto app = [](std::string& o, const char* fmt, auto... v) {
        char tmp[128];
        const int k = std::snprintf(tmp, sizeof tmp, fmt, v...);
        o.append(tmp, (size_t)std::max(0, std::min(k, (int)sizeof tmp - 1)));
    };
    std::fprintf(fp, "# vtk DataFile Version 2.0\nGASDIN data file\nASCII\nDATASET UNSTRUCTURED_GRID\n");
    std::fprintf(fp, "POINTS %d float\n", nn);
    section(nn, [&](int i, std::string& o) { app(o, "%f %f %f  ", topo.xy[2 * i], topo.xy[2 * i + 1], 0.0); });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "CELLS %d %d\n", nc, 4 * nc);
    section(nc, [&](int i, std::string& o) {
        app(o, "3 %d %d %d\n", topo.tri[3 * i], topo.tri[3 * i + 1], topo.tri[3 * i + 2]);
    });
    std::fprintf(fp, "\n");
    std::fprintf(fp, "CELL_TYPES %d\n", nc);
    section(nc, [&](int, std::string& o) { o.append("5\n"); });
    std::fprintf(fp, "\n");
    // the reference's "i+1 % 8 == 0" is i+1 == 0: one newline at the end of each field
    auto field = [&](const char* head, auto val) {
        std::fputs(head, fp);
        section(nc, [&](int i, std::string& o) {
            app(o, "%25.16f ", val(i));
            if (i + 1 == nc) o.append("\n");
        });
    };
    std::fprintf(fp, "CELL_DATA %d\n", nc);
    field("SCALARS Density float 1\nLOOKUP_TABLE default\n", [&](int i) { return par(i).r; });
    field("SCALARS Pressure float 1\nLOOKUP_TABLE default\n", [&](int i) { return par(i).p; });
    field("SCALARS Temperature float 1\nLOOKUP_TABLE default\n", [&](int i) { return par(i).T; });
    field("SCALARS MachNumber float 1\nLOOKUP_TABLE default\n", [&](int i) {
        P q = par(i);
        return implicit_format ? std::sqrt(q.u * q.u + q.v * q.v) / q.cz : (q.u * q.u + q.v * q.v) / q.cz;
    });
    std::fprintf(fp, "VECTORS Velosity float\n");
    section(nc, [&](int i, std::string& o) {
        P q = par(i);
        app(o, "%25.16f %25.16f %25.16f ", q.u, q.v, 0.0);
        if (i + 1 == nc) o.append("\n");
    });
    if (implicit_format) field("SCALARS Total_energy float 1\nLOOKUP_TABLE default\n", [&](int i) { return par(i).E; });
    std::fprintf(fp, "SCALARS Total_pressure float 1\nLOOKUP_TABLE default\n");
    section(nc, [&](int i, std::string& o) {
        P q = par(i);
        double agam = q.gam - 1.0;
        if (implicit_format) {
            double M2 = (q.u * q.u + q.v * q.v) / (q.cz * q.cz);
            app(o, "%25.16e ", q.p * std::pow(1.0 + 0.5 * M2 * agam, q.gam / agam));
        } else {
            double M2 = (q.u * q.u + q.v * q.v) / (q.gam * q.p / q.r);
            app(o, "%f ", q.p * std::pow(1.0 + 0.5 * M2 * agam, q.gam / (q.gam - 1.0)));
        }
        if ((i + 1) % 8 == 0 || i + 1 == nc) o.append("\n");
    });
    field("SCALARS TAU float 1\nLOOKUP_TABLE default\n", [&](int i) { return ct[i]; });
    const bool bad = std::ferror(fp) != 0;
    std::fclose(fp);
    if (bad) throw Error(CFD2D_ERR_FILE_OPENING, std::string("File '") + name + "' write error.");
}

void announce_vtk(const char* name) {
    if (g_verbosity > 0) {
        std::printf("File '%s' saved...\n", name);
        std::fflush(stdout);
    }
}

void Solver::save_vtk(int step) {
    const int nc = topo_.nc;
    std::vector<double> U(4 * (size_t)nc), ct(nc);
    get_state(U.data(), U.data() + nc, U.data() + 2 * (size_t)nc, U.data() + 3 * (size_t)nc);
    get_ctau(ct.data());
    char name[64];
    std::snprintf(name, sizeof name, "res_%010d.vtk", step);
    write_vtk_file(name, topo_, task_.mats, cell_mat_, U.data(), ct.data());
    announce_vtk(name);
}

// run()'s output: the state (and cTau) are copied on the solver's stream into one of
// two pinned host buffers, and a writer thread formats and writes the file while the
// GPU keeps stepping; a buffer is reused once its file is written.
void Solver::save_vtk_async(int step) {
    const int nc = topo_.nc;
    if (!snap_host_[0]) {
        for (int k = 0; k < 2; k++) {
            CUDA_CHECK(cudaMallocHost(&snap_host_[k], sizeof(double) * 5 * (size_t)nc));
            CUDA_CHECK(cudaEventCreateWithFlags(&snap_ev_[k], cudaEventDisableTiming));
        }
        vtk_stop_ = false;
        vtk_thread_ = std::thread([this] { vtk_writer(); });
    }
    int k = -1;
    {
        std::unique_lock<std::mutex> lk(vtk_mu_);
        vtk_cv_.wait(lk, [&] { return !snap_busy_[0] || !snap_busy_[1] || vtk_err_; });
        if (vtk_err_) {
            auto e = vtk_err_;
            vtk_err_ = nullptr;
            std::rethrow_exception(e);
        }
        k = snap_busy_[0] ? 1 : 0;
        snap_busy_[k] = true;
    }
    double* h = snap_host_[k];
    launch_scatter_state(dc_, dc_.A, stage_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(h, stage_, sizeof(double) * 4 * nc, cudaMemcpyDeviceToHost, stream_));
    launch_permute_scalar(dc_, dc_.ctau, stage_, stream_);
    CUDA_CHECK(cudaMemcpyAsync(h + 4 * (size_t)nc, stage_, sizeof(double) * nc, cudaMemcpyDeviceToHost, stream_));
    CUDA_CHECK(cudaEventRecord(snap_ev_[k], stream_));
    char name[64];
    std::snprintf(name, sizeof name, "res_%010d.vtk", step);
    {
        std::lock_guard<std::mutex> lk(vtk_mu_);
        vtk_jobs_.push_back({step, k});
    }
    vtk_cv_.notify_all();
    announce_vtk(name);  // in run()'s order of log lines
}

void Solver::vtk_writer() {
    cudaSetDevice(dev_);
    for (;;) {
        VtkJob job;
        {
            std::unique_lock<std::mutex> lk(vtk_mu_);
            vtk_cv_.wait(lk, [&] { return vtk_stop_ || !vtk_jobs_.empty(); });
            if (vtk_jobs_.empty()) return;
            job = vtk_jobs_.front();
            vtk_jobs_.pop_front();
        }
        try {
            const cudaError_t e = cudaEventSynchronize(snap_ev_[job.buf]);
            if (e != cudaSuccess) throw Error(CFD2D_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
            char name[64];
            std::snprintf(name, sizeof name, "res_%010d.vtk", job.step);
            const double* h = snap_host_[job.buf];
            write_vtk_file(name, topo_, task_.mats, cell_mat_, h, h + 4 * (size_t)topo_.nc);
        } catch (...) {
            std::lock_guard<std::mutex> lk(vtk_mu_);
            if (!vtk_err_) vtk_err_ = std::current_exception();
        }
        {
            std::lock_guard<std::mutex> lk(vtk_mu_);
            snap_busy_[job.buf] = false;
        }
        vtk_cv_.notify_all();
    }
}

// Wait for every file run() has issued; rethrow the first write error.
void Solver::vtk_flush() {
    if (!vtk_thread_.joinable()) return;
    std::unique_lock<std::mutex> lk(vtk_mu_);
    vtk_cv_.wait(lk, [&] { return vtk_jobs_.empty() && !snap_busy_[0] && !snap_busy_[1]; });
    if (vtk_err_) {
        auto e = vtk_err_;
        vtk_err_ = nullptr;
        std::rethrow_exception(e);
    }
}

}  // namespace cfd2d
