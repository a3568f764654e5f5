// FP64 face precision: the drop-in. Built with -fmad=false so that, as in the
// reference, no product is fused into a following sum.
#define KT double
#define KFN(name) launch_##name##_fp64
#define KGRAD_MM 1  // the minmod gradient arithmetic (k_grad<double, *, true>)
#include "kern_inst.cuh"
