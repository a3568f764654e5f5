// FP32-face adjoint kernels of the mixed form, built with the mixed forward
// kernels' flags so that every forward value they recompute is the forward's.
#define KT float
#define KFN(name) launch_##name##_mixed
#include "adj_inst.cuh"
