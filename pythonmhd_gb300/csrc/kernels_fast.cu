// Kernels built with FMA contraction: same source, fewer FP64 instructions;
// results agree with the reference to rounding (checked at 1e-12 per step).
#define MHD_NS fast
#include "godunov2d_kernels.cuh"
