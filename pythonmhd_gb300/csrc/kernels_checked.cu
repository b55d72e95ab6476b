// The bounds-checked build of the 2D kernels (arithmetic mode "checked"): the exact
// build's arithmetic (-fmad=false, bit for bit the reference's) with every global
// index of the per-item bodies checked before use (MHD_GUARD in godunov2d_kernels.cuh).
// A failed check sets a bit of the grid's device error word and records where; the
// advance call then returns MHD_ERR_INDEX.  Nothing traps.
#define MHD_NS checked
#define MHD_CHECKED 1
#include "godunov2d_kernels.cuh"
