// Launchers for one face precision; included once per precision by
// kern_fp64.cu (KT = double) and kern_mixed.cu (KT = float).
#pragma once
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
    if (l.grid > 0) k_grad<KT, true><<<l.grid, l.block, 0, s>>>(c);
    else k_grad<KT, false><<<grid_of(l, c.nc), l.block, 0, s>>>(c);
}

void KFN(flux)(const DevCase& c, int flux, int recon, cudaStream_t s) {
    if (c.shape[KIND_FLUX].grid > 0) flux_all<true>(c, flux, recon, s);
    else flux_all<false>(c, flux, recon, s);
}

void KFN(update)(const DevCase& c, int scheme, int stage, cudaStream_t s) {
    if (c.shape[KIND_UPDATE].grid > 0) update_all<true>(c, scheme, stage, s);
    else update_all<false>(c, scheme, stage, s);
}

void KFN(remediate)(const DevCase& c, cudaStream_t s) { k_remediate<KT><<<1, 1024, 0, s>>>(c); }
void KFN(prims)(const DevCase& c, cudaStream_t s) { k_prims<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c); }
void KFN(residual)(const DevCase& c, double* R, cudaStream_t s) {
    k_residual<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c, R);
}

}  // namespace cfd2d
