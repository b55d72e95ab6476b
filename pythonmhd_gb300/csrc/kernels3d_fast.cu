// 3D step kernels with FMA contraction allowed (not bitwise equal to the reference).
#define MHD_NS fast
#define MHD_BODIES_ONLY
#include "godunov2d_kernels.cuh"
#include "godunov3d_kernels.cuh"
#include "godunov3d_mhd.cuh"
