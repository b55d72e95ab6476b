// Kernels built with -fmad=false: every FP64 operation rounds on its own, as in
// the reference's NumPy code, so results match it bit for bit.
#define MHD_NS exact
#include "godunov2d_kernels.cuh"
