// Mixed form: reconstruction and Riemann fluxes in FP32; residual sums, state
// update, limits and time steps in FP64 (kernels.cuh, k_update).
#define KT float
#define KFN(name) launch_##name##_mixed
#include "kern_inst.cuh"
