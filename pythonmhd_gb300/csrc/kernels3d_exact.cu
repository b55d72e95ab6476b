// 3D step kernels built with -fmad=false: every FP64 operation rounds on its own, as
// in the reference's NumPy code, so results match it bit for bit.
#define MHD_NS exact
#define MHD_BODIES_ONLY
#include "godunov2d_kernels.cuh"
#include "godunov3d_kernels.cuh"
#include "godunov3d_mhd.cuh"
