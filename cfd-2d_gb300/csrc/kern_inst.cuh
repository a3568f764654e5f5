// Launchers for one face precision; included once per precision by
// kern_fp64.cu (KT = double) and kern_mixed.cu (KT = float).
#pragma once
#include <algorithm>

#include "kernels.cuh"

namespace cfd2d {
namespace {
inline int nblk(int n, int b) { return (n + b - 1) / b; }
inline int grid_of(const LaunchShape& l, int n) { return l.grid > 0 ? l.grid : nblk(n, l.block); }

template <int FLUX, bool ST>
void flux_by_recon(const DevCase& c, int recon, cudaStream_t s) {
    const LaunchShape& l = c.shape[KIND_FLUX];
    const int g = grid_of(l, c.ne), b = l.block;
    switch (recon) {
    case RECON_NONE: k_flux<KT, FLUX, RECON_NONE, ST><<<g, b, 0, s>>>(c); break;
    case RECON_LINEAR: k_flux<KT, FLUX, RECON_LINEAR, ST><<<g, b, 0, s>>>(c); break;
    default: k_flux<KT, FLUX, RECON_MINMOD, ST><<<g, b, 0, s>>>(c); break;
    }
}

template <bool ST>
void flux_all(const DevCase& c, int flux, int recon, cudaStream_t s) {
    switch (flux) {
    case FLUX_LAX: flux_by_recon<FLUX_LAX, ST>(c, recon, s); break;
    case FLUX_ROE: flux_by_recon<FLUX_ROE, ST>(c, recon, s); break;
    case FLUX_HLLC: flux_by_recon<FLUX_HLLC, ST>(c, recon, s); break;
    default: flux_by_recon<FLUX_GODUNOV, ST>(c, recon, s); break;
    }
}

#ifdef KPIPE
// the pipelined flux kernel: a persistent grid of 256-thread blocks, as many as fit. Its
// shared-memory size needs a function attribute, which cannot be set while a stream is
// being captured, so every instantiation is prepared once beforehand (pipe_prepare_all).
constexpr int kPipeBlock = 256;
template <int FLUX, int RECON> struct PipeGrid { static int grid; };
template <int FLUX, int RECON> int PipeGrid<FLUX, RECON>::grid = 0;
template <int FLUX, int RECON>
void pipe_prepare() {
    if (PipeGrid<FLUX, RECON>::grid) return;
    const size_t smem = 2 * (size_t)kPipeStage * kPipeBlock;
    int per_sm = 0, sms = 0, dev = 0;
    cudaFuncSetAttribute(k_flux_pipe<FLUX, RECON>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_flux_pipe<FLUX, RECON>, kPipeBlock, smem);
    PipeGrid<FLUX, RECON>::grid = std::max(1, per_sm) * std::max(1, sms);
}
template <int FLUX>
void pipe_prepare_flux() {
    pipe_prepare<FLUX, RECON_NONE>();
    pipe_prepare<FLUX, RECON_LINEAR>();
    pipe_prepare<FLUX, RECON_MINMOD>();
}
template <int FLUX, int RECON>
void pipe_launch(const DevCase& c, cudaStream_t s) {
    pipe_prepare<FLUX, RECON>();  // no-op once prepared
    const size_t smem = 2 * (size_t)kPipeStage * kPipeBlock;
    const int g = std::max(1, std::min(PipeGrid<FLUX, RECON>::grid, nblk(c.ne, kPipeBlock)));
    k_flux_pipe<FLUX, RECON><<<g, kPipeBlock, smem, s>>>(c);
}
template <int FLUX>
void flux_pipe_by_recon(const DevCase& c, int recon, cudaStream_t s) {
    switch (recon) {
    case RECON_NONE: pipe_launch<FLUX, RECON_NONE>(c, s); break;
    case RECON_LINEAR: pipe_launch<FLUX, RECON_LINEAR>(c, s); break;
    default: pipe_launch<FLUX, RECON_MINMOD>(c, s); break;
    }
}
inline void flux_pipe_all(const DevCase& c, int flux, int recon, cudaStream_t s) {
    switch (flux) {
    case FLUX_LAX: flux_pipe_by_recon<FLUX_LAX>(c, recon, s); break;
    case FLUX_ROE: flux_pipe_by_recon<FLUX_ROE>(c, recon, s); break;
    case FLUX_HLLC: flux_pipe_by_recon<FLUX_HLLC>(c, recon, s); break;
    default: flux_pipe_by_recon<FLUX_GODUNOV>(c, recon, s); break;
    }
}
#endif

template <bool ST>
void update_all(const DevCase& c, int scheme, int stage, cudaStream_t s) {
    const LaunchShape& l = c.shape[KIND_UPDATE];
    const int g = grid_of(l, c.nc), b = l.block;
    if (scheme == TIME_EULER) k_update<KT, TIME_EULER, 0, ST><<<g, b, 0, s>>>(c);
    else if (scheme == TIME_HEUN) {
        if (stage == 0) k_update<KT, TIME_HEUN, 0, ST><<<g, b, 0, s>>>(c);
        else k_update<KT, TIME_HEUN, 1, ST><<<g, b, 0, s>>>(c);
    } else {
        if (stage == 0) k_update<KT, TIME_SSPRK3, 0, ST><<<g, b, 0, s>>>(c);
        else if (stage == 1) k_update<KT, TIME_SSPRK3, 1, ST><<<g, b, 0, s>>>(c);
        else k_update<KT, TIME_SSPRK3, 2, ST><<<g, b, 0, s>>>(c);
    }
}
}  // namespace

void KFN(grad)(const DevCase& c, cudaStream_t s) {
    const LaunchShape& l = c.shape[KIND_GRAD];
#ifdef KGRAD_MM
    if (c.cf_ax) {  // FP64 with minmod: this project's gradient arithmetic
        if (l.grid > 0) k_grad<KT, true, true><<<l.grid, l.block, 0, s>>>(c);
        else k_grad<KT, false, true><<<grid_of(l, c.nc), l.block, 0, s>>>(c);
        return;
    }
#endif
    if (l.grid > 0) k_grad<KT, true><<<l.grid, l.block, 0, s>>>(c);
    else k_grad<KT, false><<<grid_of(l, c.nc), l.block, 0, s>>>(c);
}

void KFN(flux)(const DevCase& c, int flux, int recon, cudaStream_t s) {
#ifdef KPIPE
    if (c.flux_pipe && c.shape[KIND_FLUX].grid == 0) {
        flux_pipe_all(c, flux, recon, s);
        return;
    }
#endif
    if (c.shape[KIND_FLUX].grid > 0) flux_all<true>(c, flux, recon, s);
    else flux_all<false>(c, flux, recon, s);
}

void KFN(update)(const DevCase& c, int scheme, int stage, cudaStream_t s) {
    if (c.shape[KIND_UPDATE].grid > 0) update_all<true>(c, scheme, stage, s);
    else update_all<false>(c, scheme, stage, s);
}

void KFN(remediate)(const DevCase& c, cudaStream_t s) { k_remediate<KT><<<1, 1024, 0, s>>>(c); }
#ifdef KPIPE
void KFN(flux_prepare)() {
    pipe_prepare_flux<FLUX_GODUNOV>();
    pipe_prepare_flux<FLUX_LAX>();
    pipe_prepare_flux<FLUX_ROE>();
    pipe_prepare_flux<FLUX_HLLC>();
}
#endif
void KFN(prims)(const DevCase& c, cudaStream_t s) { k_prims<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c); }
void KFN(residual)(const DevCase& c, double* R, cudaStream_t s) {
    k_residual<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c, R);
}

}  // namespace cfd2d
