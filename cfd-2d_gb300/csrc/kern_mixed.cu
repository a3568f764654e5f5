#include <algorithm>
// Mixed form: reconstruction and Riemann fluxes in FP32; residual sums, state
// update, limits and time steps in FP64 (kernels.cuh, k_update).
#define KT float
#define KFN(name) launch_##name##_mixed
#define KPIPE 1
#include "kern_inst.cuh"

namespace cfd2d {
namespace {
template <int FLUX, int RECON, int SCHEME>
void fused_by_stage(const DevCase& c, const DevTiles& t, int stage, const float* wi, float* wo, cudaStream_t s) {
    const size_t smem = 16 * (2 * (size_t)t.max_cells + 2 * (size_t)t.max_grad + (size_t)t.max_edges);
    auto go = [&](auto kern) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0, sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
        const int grid = std::max(1, std::min(t.n_tiles, std::max(1, per_sm) * std::max(1, sms)));
        kern<<<grid, 256, smem, s>>>(c, t, wi, wo);
    };
    if (stage == 0) go(k_stage_fused<FLUX, RECON, SCHEME, 0>);
    else if (stage == 1) go(k_stage_fused<FLUX, RECON, SCHEME, 1>);
    else if (SCHEME == TIME_SSPRK3) go(k_stage_fused<FLUX, RECON, TIME_SSPRK3, 2>);
}
template <int FLUX, int RECON>
void fused_by_scheme(const DevCase& c, const DevTiles& t, int scheme, int stage, const float* wi, float* wo,
                     cudaStream_t s) {
    if (scheme == TIME_SSPRK3) fused_by_stage<FLUX, RECON, TIME_SSPRK3>(c, t, stage, wi, wo, s);
    else fused_by_stage<FLUX, RECON, TIME_HEUN>(c, t, stage, wi, wo, s);
}
template <int FLUX>
void fused_by_recon(const DevCase& c, const DevTiles& t, int recon, int scheme, int stage, const float* wi,
                    float* wo, cudaStream_t s) {
    if (recon == RECON_NONE) fused_by_scheme<FLUX, RECON_NONE>(c, t, scheme, stage, wi, wo, s);
    else if (recon == RECON_LINEAR) fused_by_scheme<FLUX, RECON_LINEAR>(c, t, scheme, stage, wi, wo, s);
    else fused_by_scheme<FLUX, RECON_MINMOD>(c, t, scheme, stage, wi, wo, s);
}
}  // namespace

namespace {
template <int FLUX, int RECON, int SCHEME>
void fu_by_stage(const DevCase& c, const DevTiles& t, int stage, float* wo, cudaStream_t s) {
    const size_t smem = 16 * (size_t)t.max_edges;
    auto go = [&](auto kern) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<t.n_tiles, t.tile, smem, s>>>(c, t, wo);
    };
    if (stage == 0) go(k_flux_update<FLUX, RECON, SCHEME, 0>);
    else if (stage == 1) go(k_flux_update<FLUX, RECON, SCHEME, 1>);
    else if (SCHEME == TIME_SSPRK3) go(k_flux_update<FLUX, RECON, TIME_SSPRK3, 2>);
}
template <int FLUX, int RECON>
void fu_by_scheme(const DevCase& c, const DevTiles& t, int scheme, int stage, float* wo, cudaStream_t s) {
    if (scheme == TIME_SSPRK3) fu_by_stage<FLUX, RECON, TIME_SSPRK3>(c, t, stage, wo, s);
    else if (scheme == TIME_HEUN) fu_by_stage<FLUX, RECON, TIME_HEUN>(c, t, stage, wo, s);
    else fu_by_stage<FLUX, RECON, TIME_EULER>(c, t, stage, wo, s);
}
template <int FLUX>
void fu_by_recon(const DevCase& c, const DevTiles& t, int recon, int scheme, int stage, float* wo, cudaStream_t s) {
    if (recon == RECON_NONE) fu_by_scheme<FLUX, RECON_NONE>(c, t, scheme, stage, wo, s);
    else if (recon == RECON_LINEAR) fu_by_scheme<FLUX, RECON_LINEAR>(c, t, scheme, stage, wo, s);
    else fu_by_scheme<FLUX, RECON_MINMOD>(c, t, scheme, stage, wo, s);
}
}  // namespace

void launch_flux_grad_mixed(const DevCase& c, int flux, int recon, cudaStream_t s) {
    const int g = (c.ne + 255) / 256;
    auto go = [&](auto kern) { kern<<<g, 256, 0, s>>>(c); };
    const bool mm = recon == RECON_MINMOD;
    switch (flux) {
    case FLUX_LAX: mm ? go(k_flux_grad<FLUX_LAX, RECON_MINMOD>) : go(k_flux_grad<FLUX_LAX, RECON_LINEAR>); break;
    case FLUX_ROE: mm ? go(k_flux_grad<FLUX_ROE, RECON_MINMOD>) : go(k_flux_grad<FLUX_ROE, RECON_LINEAR>); break;
    case FLUX_HLLC: mm ? go(k_flux_grad<FLUX_HLLC, RECON_MINMOD>) : go(k_flux_grad<FLUX_HLLC, RECON_LINEAR>); break;
    default: mm ? go(k_flux_grad<FLUX_GODUNOV, RECON_MINMOD>) : go(k_flux_grad<FLUX_GODUNOV, RECON_LINEAR>); break;
    }
}

// The mixed form's flux and update of one stage per tile (k_flux_update); the stage's
// primitives are c.W32, its gradients c.G32, the new primitives go to w_out.
void launch_flux_update_mixed(const DevCase& c, const DevTiles& t, int flux, int recon, int scheme, int stage,
                              float* w_out, cudaStream_t s) {
    switch (flux) {
    case FLUX_LAX: fu_by_recon<FLUX_LAX>(c, t, recon, scheme, stage, w_out, s); break;
    case FLUX_ROE: fu_by_recon<FLUX_ROE>(c, t, recon, scheme, stage, w_out, s); break;
    case FLUX_HLLC: fu_by_recon<FLUX_HLLC>(c, t, recon, scheme, stage, w_out, s); break;
    default: fu_by_recon<FLUX_GODUNOV>(c, t, recon, scheme, stage, w_out, s); break;
    }
}

// One fused stage of the mixed form (SSP-RK3 or Heun): gradients, fluxes and update per tile.
void launch_stage_fused_mixed(const DevCase& c, const DevTiles& t, int flux, int recon, int scheme, int stage,
                              const float* w_in, float* w_out, cudaStream_t s) {
    switch (flux) {
    case FLUX_LAX: fused_by_recon<FLUX_LAX>(c, t, recon, scheme, stage, w_in, w_out, s); break;
    case FLUX_ROE: fused_by_recon<FLUX_ROE>(c, t, recon, scheme, stage, w_in, w_out, s); break;
    case FLUX_HLLC: fused_by_recon<FLUX_HLLC>(c, t, recon, scheme, stage, w_in, w_out, s); break;
    default: fused_by_recon<FLUX_GODUNOV>(c, t, recon, scheme, stage, w_in, w_out, s); break;
    }
}
}  // namespace cfd2d
