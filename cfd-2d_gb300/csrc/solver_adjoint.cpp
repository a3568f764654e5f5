// Discrete adjoint driver: checkpointed forward, backward sweep with segment
// recompute (the forward's own kernels re-run from each checkpoint, so the
// recomputed stage states are the forward's bit for bit), objective and its
// gradient, boundary-parameter sensitivities.
#include <algorithm>
#include <cstring>
#include <vector>

#include "cfd2d.h"
#include "solver.hpp"

namespace cfd2d {

namespace {
constexpr int kObjBlocks = 512;

int n_stages(int scheme) { return scheme == TIME_EULER ? 1 : (scheme == TIME_HEUN ? 2 : 3); }

// (coef_t, coef_acc) of the step's last combination, U^{n+1} = coef_acc U^n + coef_t t_last
void final_coefs(int scheme, double& ct, double& ca) {
    if (scheme == TIME_SSPRK3) { ct = 2.0 / 3.0; ca = 1.0 / 3.0; }
    else if (scheme == TIME_HEUN) { ct = 0.5; ca = 0.5; }
    else { ct = 1.0; ca = 0.0; }
}

// the input X_s of stage s > 0 as a combination of the previous stage's output and U^n
void stage_coefs(int scheme, int s, double& ct, double& ca) {
    if (scheme == TIME_SSPRK3 && s == 2) { ct = 0.25; ca = 0.75; }
    else { ct = 1.0; ca = 0.0; }
}
}  // namespace

void Solver::adjoint_setup() {
    if (adj_ready_) return;
    const int nc = dc_.nc, ne = dc_.ne, nb = dc_.ne - dc_.n_int;
    if (task_.steady) throw Error(CFD2D_ERR_INVALID_ARG, "the adjoint needs a global time step (STEADY=0)");
    if (task_.flux != FLUX_HLLC && task_.flux != FLUX_LAX)
        throw Error(CFD2D_ERR_INVALID_ARG, "the adjoint differentiates the HLLC and LAX fluxes");
    if (gauss_points_ == 0) throw Error(CFD2D_ERR_INVALID_ARG, "the adjoint needs two-point edges");
    adj_dc_ = dc_;  // the adjoint runs in the forward's face precision on the forward's geometry
    adj_eq_ = dalloc<double>(24 * (size_t)ne);  // sized for FP64 faces; FP32 faces use half
    adj_eb_ = dalloc<double>(4 * (size_t)std::max(nb, 1));
    adj_eb2_ = dalloc<double>(4 * (size_t)std::max(nb, 1));
    adj_qbar_ = dalloc<double>(4 * (size_t)nc);
    adj_gbar_ = dalloc<double>(8 * (size_t)nc);
    adj_tb_ = dalloc<double>(4 * (size_t)nc);
    adj_acc_ = dalloc<double>(4 * (size_t)nc);
    adj_lam_ = dalloc<double>(4 * (size_t)nc);
    adj_mu_ = dalloc<double>(4 * (size_t)nc);
    adj_dbnd_ = dalloc<double>(4 * std::max<size_t>(task_.bnds.size(), 1));
    adj_final_ = dalloc<double>(4 * (size_t)nc);
    obj_partial_ = dalloc<double>(kObjBlocks);
    CUDA_CHECK(cudaMemsetAsync(adj_eb_, 0, sizeof(double) * 4 * std::max(nb, 1), stream_));
    CUDA_CHECK(cudaMemsetAsync(adj_eb2_, 0, sizeof(double) * 4 * std::max(nb, 1), stream_));
    adj_ready_ = true;
}

void Solver::set_objective(int kind, const double* w, double p_ref) {
    use_device();
    if (kind != 0 && kind != 1) throw Error(CFD2D_ERR_INVALID_ARG, "objective kind is 0 (pressure) or 1 (density)");
    adjoint_setup();
    const int nc = dc_.nc;
    std::vector<double> ws(nc);
    for (int i = 0; i < nc; i++) ws[i] = w[lay_.perm[i]];
    if (!obj_w_) obj_w_ = dalloc<double>(nc);
    CUDA_CHECK(cudaMemcpyAsync(obj_w_, ws.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    obj_kind_ = kind;
    obj_pref_ = p_ref;
}

void Solver::set_boundary_params(int b, const double par[4]) {
    use_device();
    if (b < 0 || b >= (int)task_.bnds.size()) throw Error(CFD2D_ERR_INVALID_ARG, "boundary index out of range");
    for (int k = 0; k < 4; k++) task_.bnds[b].par[k] = par[k];
    DevBnd d{};
    d.kind = task_.bnds[b].kind;
    d.u = par[0]; d.v = par[1]; d.T = par[2]; d.p = par[3];
    CUDA_CHECK(cudaMemcpyAsync(const_cast<DevBnd*>(dc_.bnds) + b, &d, sizeof d, cudaMemcpyHostToDevice, stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
}

double Solver::forward(int nsteps, int k, int* status) {
    use_device();
    if (obj_kind_ < 0) throw Error(CFD2D_ERR_INVALID_ARG, "set an objective first");
    if (nsteps < 1 || k < 1) throw Error(CFD2D_ERR_INVALID_ARG, "nsteps and the checkpoint interval must be >= 1");
    adjoint_setup();
    const size_t nc = dc_.nc;
    const size_t nseg = (nsteps + k - 1) / k;
    if (nseg > ckpt_slots_) {
        ckpt_ = dalloc<double>(nseg * 4 * nc);
        ckpt_slots_ = nseg;
    }
    const int nst = n_stages(task_.scheme);
    // What the backward sweep keeps of each recorded stage. The reverse kernels read
    // only the stage's primitives W and gradients G (face precision), so the first
    // choice is W and G, then W alone (G re-derived per stage); the FP64 stage states
    // (from which both are re-derived) only when W does not fit either. "Fits": within
    // 80% of the free device memory beyond what is allocated already and, with an
    // ADJOINT_MEMORY budget, with the handle's device bytes (solver, adjoint arrays,
    // checkpoints and this store) at most the budget.
    store_wg_ = false;
    store_g_ = false;
    store_rec_ = false;
    {
        const size_t fsize = task_.precision == PREC_MIXED ? sizeof(float) : sizeof(double);
        const size_t dbl = sizeof(double);
        const size_t need = ((size_t)k * nst * 12 * nc * fsize + dbl - 1) / dbl;   // W and G, in doubles
        const size_t need_w = ((size_t)k * nst * 4 * nc * fsize + dbl - 1) / dbl;  // W
        const size_t need_x = (size_t)k * nst * 4 * nc;                            // FP64 states
        const size_t need_rec = (size_t)k * nst * rec_stage_bytes();              // HLLC flux records, bytes
        size_t free_b = 0, total_b = 0;
        CUDA_CHECK(cudaMemGetInfo(&free_b, &total_b));
        const size_t have = wg_slots_ * dbl + seg_slots_ * 4 * nc * dbl + rec_bytes_;  // reusable if released
        const size_t base = bytes_ - std::min(bytes_, have);                        // everything but the store
        const double budget = task_.adj_memory;
        auto in_budget = [&](size_t bytes) { return budget <= 0.0 || (double)(base + bytes) <= budget; };
        auto fits_bytes = [&](size_t bytes) { return bytes <= (free_b + have) / 10 * 8 && in_budget(bytes); };
        auto fits = [&](size_t doubles) {
            return (doubles <= wg_slots_ || doubles * dbl <= (free_b + have) / 10 * 8) && in_budget(doubles * dbl);
        };
        if (!in_budget(std::min(need_w, need_x) * dbl))
            throw Error(CFD2D_ERR_CAPACITY, "the adjoint's smallest segment store exceeds ADJOINT_MEMORY");
        const int mode = task_.adj_store;
        // flux records with FP64 faces only: FP32 faces are compiled with contraction, which
        // the compiler may apply differently in the recording kernel than in the forward's
        const bool rec_ok = task_.flux == FLUX_HLLC && task_.precision != PREC_MIXED;
        if (rec_ok && (mode == 3 || (mode < 0 && fits_bytes(need * dbl + need_rec)))) {
            store_wg_ = store_g_ = store_rec_ = true;
        } else if (mode >= 2 || (mode < 0 && fits(need))) {
            store_wg_ = store_g_ = true;
        } else if (mode == 1 || (mode < 0 && fits(need_w))) {
            store_wg_ = true;
        }
        const size_t want = store_g_ ? need : (store_wg_ ? need_w : 0);
        const size_t want_rec = store_rec_ ? need_rec : 0;
        if ((store_wg_ && segstore_) || want > wg_slots_ || (!store_wg_ && (size_t)k * nst > seg_slots_) ||
            want_rec > rec_bytes_ || (!store_rec_ && recstore_))
            drop_record_graphs();  // the store moves: graphs captured on it are stale
        if (recstore_ && (!store_rec_ || want_rec > rec_bytes_)) {
            release(recstore_, rec_bytes_);
            recstore_ = nullptr;
            rec_bytes_ = 0;
        }
        if (store_rec_ && !recstore_) {
            recstore_ = dalloc<char>(want_rec);
            rec_bytes_ = want_rec;
        }
        if (store_wg_ && segstore_) {  // the states are not kept: give their memory back first
            release(segstore_, seg_slots_ * 4 * nc * dbl);
            segstore_ = nullptr;
            seg_slots_ = 0;
        }
        if (want > wg_slots_) {
            if (wgstore_) release(wgstore_, wg_slots_ * dbl);
            wgstore_ = dalloc<double>(want);
            wg_slots_ = want;
        }
        if (!store_wg_ && (size_t)k * nst > seg_slots_) {
            if (segstore_) release(segstore_, seg_slots_ * 4 * nc * dbl);
            segstore_ = dalloc<double>(need_x);
            seg_slots_ = (size_t)k * nst;
        }
    }
    CUDA_CHECK(cudaMemsetAsync(dc_.flags, 0, sizeof(unsigned) * nc, stream_));
    last_recorded_ = false;
    for (size_t s = 0; s < nseg; s++) {
        CUDA_CHECK(cudaMemcpyAsync(ckpt_ + s * 4 * nc, dc_.A, sizeof(double) * 4 * nc, cudaMemcpyDeviceToDevice,
                                   stream_));
        const int n = std::min<int>(k, nsteps - (int)s * k);
        if (s + 1 == nseg) {
            // the last segment is the first the backward sweep walks: its stages are recorded
            // now (the step's own kernels, so the same bits) instead of being recomputed there
            record_segment(n);
            for (int j = 0; j < n; j++) {
                if (!task_.steady) t_ += tau_;
                steps_++;
            }
            last_recorded_ = true;
            continue;
        }
        for (int j = 0; j < n; j++) {
            if (!task_.steady) t_ += tau_;
            CUDA_CHECK(cudaGraphLaunch(gexec_, stream_));
            steps_++;
        }
    }
    fw_steps_ = nsteps;
    fw_k_ = k;
    CUDA_CHECK(cudaMemcpyAsync(adj_final_, dc_.A, sizeof(double) * 4 * nc, cudaMemcpyDeviceToDevice, stream_));
    launch_objective(dc_, obj_w_, obj_kind_, obj_pref_, obj_partial_, kObjBlocks, stream_);
    std::vector<double> h(kObjBlocks);
    CUDA_CHECK(cudaMemcpyAsync(h.data(), obj_partial_, sizeof(double) * kObjBlocks, cudaMemcpyDeviceToHost, stream_));
    *status = read_status();  // synchronises
    double J = 0.0;
    for (double v : h) J += v;
    return J;
}

void Solver::drop_record_graphs() {
    for (auto& g : rec_graphs_) cudaGraphExecDestroy(g.second.first);
    rec_graphs_.clear();
}

// n forward steps that keep every stage in the segment store (what the backward sweep
// reads), captured once per n into a CUDA graph and replayed.
size_t Solver::rec_stage_bytes() const {
    const size_t fsize = task_.precision == PREC_MIXED ? sizeof(float) : sizeof(double);
    const size_t b = (size_t)dc_.ne * (20 * fsize + sizeof(unsigned));
    return (b + 255) / 256 * 256;
}

FluxRec Solver::rec_at(size_t slot) const {
    const size_t fsize = task_.precision == PREC_MIXED ? sizeof(float) : sizeof(double);
    FluxRec r;
    char* v = recstore_ + slot * rec_stage_bytes();
    r.v = v;
    r.bits = reinterpret_cast<unsigned*>(v + (size_t)dc_.ne * 20 * fsize);
    return r;
}

void Solver::record_segment(int n) {
    const size_t nc = dc_.nc;
    const int nst = n_stages(task_.scheme);
    const size_t fsize = task_.precision == PREC_MIXED ? sizeof(float) : sizeof(double);
    const size_t per_stage = (store_g_ ? 12 : 4) * nc * fsize;
    const int kind = store_rec_ ? 3 : (store_wg_ ? (store_g_ ? 2 : 1) : 0);
    cudaGraphExec_t exec = nullptr;
    for (auto& g : rec_graphs_)
        if (g.first == n && g.second.second == kind) exec = g.second.first;
    if (!exec) {
        cudaGraph_t graph = nullptr;
        CUDA_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            for (int j = 0; j < n; j++)
                record_step(store_wg_ ? nullptr : segstore_ + (size_t)j * nst * 4 * nc,
                            store_wg_ ? reinterpret_cast<char*>(wgstore_) + (size_t)j * nst * per_stage : nullptr,
                            j * nst);
        } catch (...) {
            cudaStreamEndCapture(stream_, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        CUDA_CHECK(cudaStreamEndCapture(stream_, &graph));
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CUDA_CHECK(e);
        rec_graphs_.push_back({n, {exec, kind}});
    }
    CUDA_CHECK(cudaGraphLaunch(exec, stream_));
}

// One forward step that keeps, when given, every stage's input state in
// store[stage] or the stage's primitives (and, with store_g_, gradients) in the
// face precision in wg[stage] (12 or 4 nc values per stage), and with store_rec_ each
// stage's HLLC flux record in the record slot rec_slot + stage.
void Solver::record_step(double* store, void* wg, int rec_slot) {
    const size_t nc = dc_.nc;
    const int nst = n_stages(task_.scheme);
    const int p = task_.precision;
    const size_t fsize = p == PREC_MIXED ? sizeof(float) : sizeof(double);
    const void* W = p == PREC_MIXED ? (const void*)dc_.W32 : (const void*)dc_.W64;
    const void* G = p == PREC_MIXED ? (const void*)dc_.G32 : (const void*)dc_.G64;
    for (int st = 0; st < nst; st++) {
        if (store)
            CUDA_CHECK(cudaMemcpyAsync(store + st * 4 * nc, st == 0 ? dc_.A : dc_.B, sizeof(double) * 4 * nc,
                                       cudaMemcpyDeviceToDevice, stream_));
        if (task_.recon != RECON_NONE) launch_grad(dc_, p, stream_);
        if (wg) {
            char* w = static_cast<char*>(wg) + (size_t)st * (store_g_ ? 12 : 4) * nc * fsize;
            CUDA_CHECK(cudaMemcpyAsync(w, W, fsize * 4 * nc, cudaMemcpyDeviceToDevice, stream_));
            if (task_.recon != RECON_NONE && store_g_)
                CUDA_CHECK(cudaMemcpyAsync(w + 4 * nc * fsize, G, fsize * 8 * nc, cudaMemcpyDeviceToDevice,
                                           stream_));
        }
        if (store_rec_ && rec_slot >= 0) {
            const FluxRec r = rec_at((size_t)rec_slot + st);
            launch_flux_rec(dc_, task_.recon, r, p, stream_);
        } else {
            launch_flux(dc_, p, task_.flux, task_.recon, stream_);
        }
        launch_update(dc_, p, task_.scheme, st, stream_);
    }
    launch_remediate(dc_, p, stream_);
}

void Solver::backward(double* dJdU0, double* dJdbnd) {
    use_device();
    if (fw_steps_ < 1) throw Error(CFD2D_ERR_INVALID_ARG, "run forward() first");
    const size_t nc = dc_.nc;
    {  // the adjoint does not differentiate limiter remediation
        std::vector<unsigned> fl(nc);
        CUDA_CHECK(cudaMemcpyAsync(fl.data(), dc_.flags, sizeof(unsigned) * nc, cudaMemcpyDeviceToHost, stream_));
        CUDA_CHECK(cudaStreamSynchronize(stream_));
        for (unsigned f : fl)
            if (f & 0x2u)
                throw Error(CFD2D_ERR_INVALID_ARG, "limiter flags were raised in the forward run; the adjoint "
                                                   "does not differentiate remediation");
    }
    const int nst = n_stages(task_.scheme);
    const int p = task_.precision;
    const size_t fsize = p == PREC_MIXED ? sizeof(float) : sizeof(double);
    const size_t per_stage = (store_g_ ? 12 : 4) * nc * fsize;
    auto wg_at = [&](int slot) -> void* { return reinterpret_cast<char*>(wgstore_) + (size_t)slot * per_stage; };
    AdjCase a{};
    a.eq = adj_eq_; a.eb = adj_eb_; a.eb2 = adj_eb2_; a.qbar = adj_qbar_; a.gbar = adj_gbar_;
    a.tb = adj_tb_; a.acc = adj_acc_; a.lam = adj_lam_; a.mu = adj_mu_; a.mu_out = adj_mu_;
    a.dbnd = adj_dbnd_; a.n_bnd = (int)task_.bnds.size();
    const size_t nbe = 4 * (size_t)std::max(dc_.ne - dc_.n_int, 1);
    CUDA_CHECK(cudaMemsetAsync(adj_eb_, 0, sizeof(double) * nbe, stream_));
    CUDA_CHECK(cudaMemsetAsync(adj_eb2_, 0, sizeof(double) * nbe, stream_));
    // lambda = dJ/dU of the final state
    {
        DevCase cf = dc_;
        cf.A = adj_final_;
        launch_objective_grad(cf, a, obj_w_, obj_kind_, obj_pref_, stream_);
    }
    double ct_f, ca_f;
    final_coefs(task_.scheme, ct_f, ca_f);
    const int nseg = (fw_steps_ + fw_k_ - 1) / fw_k_;
    // One segment after its checkpoint is restored: recompute its n steps, recording the
    // stages, then walk them backwards. Captured once per segment length into a CUDA
    // graph and replayed, so the host issues one launch per segment.
    // recorded: the segment's stages are in the store already (the forward's last segment)
    auto segment = [&](int n, bool first_step, bool recorded) {  // first_step: the forward's last step
        if (!recorded) {
            launch_prims(dc_, task_.precision, stream_);
            for (int j = 0; j < n; j++)
                record_step(store_wg_ ? nullptr : segstore_ + (size_t)j * nst * 4 * nc,
                            store_wg_ ? wg_at(j * nst) : nullptr, j * nst);
        }
        for (int j = n - 1; j >= 0; j--) {
            // every later step is started by the stage-0 kernel of the step after it
            if (first_step && j == n - 1) launch_adj_step_start(adj_dc_, a, ct_f, ca_f, stream_);
            for (int st = nst - 1; st >= 0; st--) {
                DevCase cx = adj_dc_;
                if (!store_wg_) cx.A = segstore_ + ((size_t)j * nst + st) * 4 * nc;
                if (store_wg_) {  // the recorded stage's own W (and G)
                    char* w = static_cast<char*>(wg_at(j * nst + st));
                    if (p == PREC_MIXED) {
                        cx.W32 = reinterpret_cast<float*>(w);
                        if (store_g_) cx.G32 = cx.W32 + 4 * nc;
                    } else {
                        cx.W64 = reinterpret_cast<double*>(w);
                        if (store_g_) cx.G64 = cx.W64 + 4 * nc;
                    }
                    if (!store_g_ && task_.recon != RECON_NONE) launch_grad(cx, p, stream_);
                } else {  // re-derived by the forward's own kernels from the recorded stage state
                    launch_prims(cx, p, stream_);
                    if (task_.recon != RECON_NONE) launch_grad(cx, p, stream_);
                }
                if (store_rec_) launch_adj_flux_rec(cx, a, task_.recon, rec_at((size_t)j * nst + st), p, stream_);
                else launch_adj_flux(cx, a, task_.flux, task_.recon, p, stream_);
                launch_adj_gather(cx, a, p, stream_);
                double ct = ct_f, ca = ca_f;
                if (st > 0) stage_coefs(task_.scheme, st, ct, ca);
                launch_adj_cell(cx, a, ct, ca, st == 0 ? 1 : 0, p, stream_);
            }
        }
    };
    std::vector<std::pair<int, cudaGraphExec_t>> graphs;  // key: 4 n + 2 (recorded) + (first step)
    auto release = [&]() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
    };
    try {
        for (int seg = nseg - 1; seg >= 0; seg--) {
            const int n = std::min(fw_k_, fw_steps_ - seg * fw_k_);
            const bool first = seg == nseg - 1;
            const bool recorded = first && last_recorded_;
            if (!recorded)
                CUDA_CHECK(cudaMemcpyAsync(dc_.A, ckpt_ + (size_t)seg * 4 * nc, sizeof(double) * 4 * nc,
                                           cudaMemcpyDeviceToDevice, stream_));
            const int key = 4 * n + (recorded ? 2 : 0) + (first ? 1 : 0);
            cudaGraphExec_t exec = nullptr;
            for (auto& g : graphs)
                if (g.first == key) exec = g.second;
            if (!exec) {
                cudaGraph_t graph = nullptr;
                CUDA_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                try {
                    segment(n, first, recorded);
                } catch (...) {
                    cudaStreamEndCapture(stream_, &graph);
                    if (graph) cudaGraphDestroy(graph);
                    throw;
                }
                CUDA_CHECK(cudaStreamEndCapture(stream_, &graph));
                const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                CUDA_CHECK(e);
                graphs.emplace_back(key, exec);
            }
            CUDA_CHECK(cudaGraphLaunch(exec, stream_));
        }
    } catch (...) {
        cudaStreamSynchronize(stream_);
        release();
        throw;
    }
    launch_adj_bnd_reduce(adj_dc_, a, stream_);
    // the solver's state is the forward's final state again
    CUDA_CHECK(cudaMemcpyAsync(dc_.A, adj_final_, sizeof(double) * 4 * nc, cudaMemcpyDeviceToDevice, stream_));
    launch_prims(dc_, task_.precision, stream_);
    if (dJdU0) {
        launch_scatter_state(dc_, adj_lam_, stage_, stream_);
        for (int k = 0; k < 4; k++)
            CUDA_CHECK(cudaMemcpyAsync(dJdU0 + k * nc, stage_ + k * nc, sizeof(double) * nc, cudaMemcpyDeviceToHost,
                                       stream_));
    }
    if (dJdbnd && !task_.bnds.empty())
        CUDA_CHECK(cudaMemcpyAsync(dJdbnd, adj_dbnd_, sizeof(double) * 4 * task_.bnds.size(), cudaMemcpyDeviceToHost,
                                   stream_));
    CUDA_CHECK(cudaStreamSynchronize(stream_));
    release();
}

}  // namespace cfd2d
