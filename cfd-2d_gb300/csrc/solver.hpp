// Host driver of one FVM_TVD instance on the GPU: owns the device arrays, the
// stream and the CUDA graph of one time step.
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cfd2d.h"
#include "kernels.hpp"
#include "mesh.hpp"
#include "task.hpp"

namespace cfd2d {

void log_line(const char* fmt, ...);
// The VTK file of one state (U: 4 x nc conserved, ct: cTau; reference cell order) as
// FVM_TVD::save writes it, or as FVM_TVD_IMPLICIT::save does with implicit_format.
void write_vtk_file(const char* name, const Topo& topo, const std::vector<TaskMaterial>& mats,
                    const std::vector<int>& cell_mat, const double* U, const double* ct, bool implicit_format = false);
void announce_vtk(const char* name);
// The address through which kernels on the current device read or write array p:
// pinned (or registered) or managed memory, pageable memory where the device has
// coherent access to it, or device memory of the current GPU itself; nullptr otherwise
// (the caller then stages through a copy).
void* device_view(const void* p);
void set_verbosity(int v);
void set_log_file(const char* path);

#define CUDA_CHECK(x)                                                                                    \
    do {                                                                                                 \
        cudaError_t e_ = (x);                                                                            \
        if (e_ != cudaSuccess)                                                                           \
            throw ::cfd2d::Error(CFD2D_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));       \
    } while (0)

// One member of a batch: its cells are [cell_off, cell_off + nc) of the union
// mesh (reference order), with its own CFL number and XML time step.
struct Instance {
    int cell_off = 0, nc = 0;
    double tau_xml = 0, cfl = 0, tau = 0, t = 0;
};

// A batch merged into one union mesh and task (solver_batch.cpp).
struct Batch {
    TaskConfig task;
    Topo topo;
    std::vector<int> cell_region, edge_bnd;
    std::vector<Instance> inst;
};
Batch merge_batch(std::vector<TaskConfig>& tasks, std::vector<Topo>& topos, std::vector<std::vector<int>>& cregs,
                  std::vector<std::vector<int>>& ebnds);

class Solver {
public:
    Solver(const TaskConfig& t, Topo&& topo, const std::vector<int>& cell_region, const std::vector<int>& edge_bnd,
           int gauss_points, std::vector<Instance> instances = {});
    ~Solver();
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;

    int step(int n);  // CFD2D_OK, or a warning code from the device error word
    int run();
    void get_state(double* ro, double* ru, double* rv, double* re);
    void set_state(const double* ro, const double* ru, const double* rv, const double* re, bool reset_tau);
    void get_ctau(double* out);
    void get_flags(unsigned* out);
    void residual(double* R);
    void conservation(double sums[4]);
    void save_vtk(int step);
    // restart files: the state, cTau, flags, step count and time
    void save_state(const char* path);
    void load_state(const char* path);
    // run()'s output: snapshot on the stream, file written by a host thread
    void save_vtk_async(int step);
    void vtk_flush();
    // device time of n steps (CUDA events around the graph launches on the solver's stream)
    double timed_steps(int n);
    // n steps launched one kernel at a time with events around each launch;
    // per kind (0 grad, 1 flux, 2 update, 3 remediate): total ms and launch count
    void profile_steps(int n, double ms[4], int launches[4]);

    const TaskConfig& task() const { return task_; }
    const Topo& topo() const { return topo_; }
    const Layout& layout() const { return lay_; }
    int n_steps() const { return steps_; }
    double time() const { return t_; }
    double tau() const { return tau_; }
    size_t device_bytes() const { return bytes_; }
    cudaStream_t stream() const { return stream_; }
    const DevCase& dev() const { return dc_; }
    int precision() const { return task_.precision; }

    // ---- batches and launch shapes (solver_batch.cpp)
    int n_instances() const { return (int)std::max<size_t>(inst_.size(), 1); }
    const Instance& instance(int k) const { return inst_[k]; }
    bool is_batch() const { return !inst_.empty(); }
    // sweep block size x persistent-grid factor per kernel kind; keep the fastest; write JSON when path given
    void autotune(const char* json_path, int reps);
    void load_tuning(const char* json_path);
    const LaunchShape& shape(int kind) const { return dc_.shape[kind]; }

    // ---- discrete adjoint (solver_adjoint.cpp)
    // objective J = sum_i w_i (p_i - p_ref)^2 (kind 0) or sum_i w_i rho_i^2 (kind 1), w in reference cell order
    void set_objective(int kind, const double* w, double p_ref);
    // nsteps steps from the current state, keeping a checkpoint every k steps; returns J of the final state
    double forward(int nsteps, int k, int* status);
    // dJ/dU of the state forward() started from (4 x nc, reference order) and dJ/d(Vx, Vy, T, P) per boundary
    void backward(double* dJdU0, double* dJdbnd);
    void set_boundary_params(int b, const double par[4]);

private:
    template <typename T> T* dalloc(size_t n);
    // free one dalloc'd buffer (after the stream is idle) and forget it
    void release(void* p, size_t bytes);
    void adjoint_setup();
    void record_step(double* store, void* wg, int rec_slot = -1);
    void record_segment(int n);
    void drop_record_graphs();
    // captured recording segments: (n, (graph, store kind 0 states / 1 W / 2 W and G))
    std::vector<std::pair<int, std::pair<cudaGraphExec_t, int>>> rec_graphs_;
    DevCase adj_dc_{};
    bool adj_ready_ = false;
    int obj_kind_ = -1;
    double obj_pref_ = 0;
    double* obj_w_ = nullptr;
    double* obj_partial_ = nullptr;
    double* adj_eq_ = nullptr;
    double* adj_eb_ = nullptr;
    double* adj_eb2_ = nullptr;
    double* adj_qbar_ = nullptr;
    double* adj_gbar_ = nullptr;
    double* adj_tb_ = nullptr;
    double* adj_acc_ = nullptr;
    double* adj_lam_ = nullptr;
    double* adj_mu_ = nullptr;
    double* adj_dbnd_ = nullptr;
    double* adj_final_ = nullptr;
    double* ckpt_ = nullptr;
    double* segstore_ = nullptr;
    double* wgstore_ = nullptr;   // per recorded stage: W (4 nc) then G (8 nc), in the face precision
    size_t wg_slots_ = 0;         // doubles allocated in wgstore_
    bool store_wg_ = false;       // the recorded stages' W are kept
    bool store_g_ = false;        // ... and their G
    bool store_rec_ = false;      // ... and their HLLC flux records (FluxRec per stage)
    char* recstore_ = nullptr;    // per recorded stage: rec_stage_bytes() bytes
    size_t rec_bytes_ = 0;        // bytes allocated in recstore_
    size_t rec_stage_bytes() const;
    FluxRec rec_at(size_t slot) const;
    size_t ckpt_slots_ = 0, seg_slots_ = 0;
    int fw_steps_ = 0, fw_k_ = 0;
    bool last_recorded_ = false;  // forward() left the last segment's stages in the store
    template <typename T> T* upload(const std::vector<T>& v);
    struct VtkJob { int step = 0, buf = 0; };
    void vtk_writer();
    std::thread vtk_thread_;
    std::mutex vtk_mu_;
    std::condition_variable vtk_cv_;
    std::deque<VtkJob> vtk_jobs_;
    bool vtk_stop_ = false;
    bool snap_busy_[2] = {false, false};
    double* snap_host_[2] = {nullptr, nullptr};
    cudaEvent_t snap_ev_[2] = {nullptr, nullptr};
    std::exception_ptr vtk_err_;
    // mixed form, SSP-RK3 / Heun: tiles for the fused stage kernel (solver_tiles.cpp)
    void build_tiles();
    DevTiles tiles_{};
    int fused_ = 0;  // 0 per-kernel stages, 1 one tiled kernel per stage, 2 gradients + tiled flux-and-update,
                     // 3 per-kernel stages whose flux kernel forms the gradients
    float* wrot_[3] = {nullptr, nullptr, nullptr};  // primitives rotated through the stages; wrot_[0] == dc_.W32
    void compute_tau();
    void enqueue_step(cudaEvent_t* ev = nullptr, int* kinds = nullptr, int* nev = nullptr);
    void build_graph();
    int read_status();
    void use_device() const { cudaSetDevice(dev_); }

    TaskConfig task_;
    Topo topo_;
    Layout lay_;
    std::vector<int> cell_mat_;
    int gauss_points_;
    int dev_ = 0;
    DevCase dc_{};
    cudaStream_t stream_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    std::vector<Instance> inst_;
    void compute_tau_batch();
    void rebuild_graph();
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
    double* stage_ = nullptr;     // 4*nc staging for permutations and residuals
    unsigned long long* dtmin_ = nullptr;
    double* partial_ = nullptr;
    double tau_ = 0, t_ = 0;
    int steps_ = 0;
};

// device allocations owned (and freed) by the solver
template <typename T>
inline T* Solver::dalloc(size_t n) {
    void* p = nullptr;
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    CUDA_CHECK(cudaMalloc(&p, b));
    allocs_.push_back(p);
    bytes_ += b;
    return static_cast<T*>(p);
}

template <typename T>
inline T* Solver::upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) CUDA_CHECK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
    return p;
}

}  // namespace cfd2d
