// Launchers for one face precision; included once per precision by
// kern_fp64.cu (KT = double) and kern_mixed.cu (KT = float).
#pragma once
#include "kernels.cuh"

namespace cfd2d {
namespace {
inline int nblk(int n, int b) { return (n + b - 1) / b; }

template <int FLUX>
void flux_by_recon(const DevCase& c, int recon, cudaStream_t s) {
    const int g = nblk(c.ne, 256);
    switch (recon) {
    case RECON_NONE: k_flux<KT, FLUX, RECON_NONE><<<g, 256, 0, s>>>(c); break;
    case RECON_LINEAR: k_flux<KT, FLUX, RECON_LINEAR><<<g, 256, 0, s>>>(c); break;
    default: k_flux<KT, FLUX, RECON_MINMOD><<<g, 256, 0, s>>>(c); break;
    }
}
}  // namespace

void KFN(grad)(const DevCase& c, cudaStream_t s) { k_grad<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c); }

void KFN(flux)(const DevCase& c, int flux, int recon, cudaStream_t s) {
    switch (flux) {
    case FLUX_LAX: flux_by_recon<FLUX_LAX>(c, recon, s); break;
    case FLUX_ROE: flux_by_recon<FLUX_ROE>(c, recon, s); break;
    case FLUX_HLLC: flux_by_recon<FLUX_HLLC>(c, recon, s); break;
    default: flux_by_recon<FLUX_GODUNOV>(c, recon, s); break;
    }
}

void KFN(update)(const DevCase& c, int scheme, int stage, cudaStream_t s) {
    const int g = nblk(c.nc, 256);
    if (scheme == TIME_EULER) k_update<KT, TIME_EULER, 0><<<g, 256, 0, s>>>(c);
    else if (scheme == TIME_HEUN) {
        if (stage == 0) k_update<KT, TIME_HEUN, 0><<<g, 256, 0, s>>>(c);
        else k_update<KT, TIME_HEUN, 1><<<g, 256, 0, s>>>(c);
    } else {
        if (stage == 0) k_update<KT, TIME_SSPRK3, 0><<<g, 256, 0, s>>>(c);
        else if (stage == 1) k_update<KT, TIME_SSPRK3, 1><<<g, 256, 0, s>>>(c);
        else k_update<KT, TIME_SSPRK3, 2><<<g, 256, 0, s>>>(c);
    }
}

void KFN(remediate)(const DevCase& c, cudaStream_t s) { k_remediate<KT><<<1, 1024, 0, s>>>(c); }
void KFN(prims)(const DevCase& c, cudaStream_t s) { k_prims<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c); }
void KFN(residual)(const DevCase& c, double* R, cudaStream_t s) {
    k_residual<KT><<<nblk(c.nc, 256), 256, 0, s>>>(c, R);
}

}  // namespace cfd2d
