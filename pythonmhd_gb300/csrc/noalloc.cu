// CFL timestep of one state with no device allocation.
//
// For callers that cannot allocate device memory themselves: a framework whose
// caching allocator already owns the free device memory, a plugin inside a host
// application that budgets device memory on its own, or a stepping loop that must
// not call cudaMalloc/cudaFree every step (cudaFree synchronises the whole device).
// They pass device pointers to the state and to one output double; the scratch
// this computation needs lives in the static array below, which every GPU that
// loads this library holds until the process exits.
//
// Built with -fmad=false, so the per-cell arithmetic, and with it the result, is
// the same as the exact-arithmetic step's CFL reduction bit for bit.  Maxima and
// minima use the step's order-key compares (mhdk::dmax / dmin), which let a NaN
// signal speed win where a plain `a > b ? a : b` would drop it: a state with a NaN
// gives a NaN dt here, as it makes the step report MHD_ERR_NONFINITE.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pythonmhd_gb300.h"
#include "mhd_math.cuh"

namespace {

constexpr int kMaxRows = MHD2D_NOALLOC_MAX_ROWS;
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;
constexpr double kSmall = 0.000000000001;

// Per-row partial maxima (|vx|+c_x, |vy|+c_y): 2 * kMaxRows doubles = 256 KB.
// Kernel 1 overwrites every slot kernel 2 reads, so contents left by an earlier
// call are never used and nothing needs clearing between calls.
static __device__ __align__(256) double g_row_max[2 * kMaxRows];

std::mutex g_setup_lock;
double* g_scratch[kMaxDevices] = {};

using mhdk::dmax;
using mhdk::dmin;

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ void block_max2(double& mx, double& my, double* sx, double* sy) {
  mx = warp_max(mx);
  my = warp_max(my);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sx[wid] = mx; sy[wid] = my; }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    mx = warp_max(lane < nw ? sx[lane] : 0.0);
    my = warp_max(lane < nw ? sy[lane] : 0.0);
  }
}

// One block per row: the largest signal speeds of the row, in the arithmetic of
// Source/TimestepCalculations_HelperModule.py:67-109 (hydro) and :239-289 (MHD).
__global__ void __launch_bounds__(kThreads) k_row_speeds(int mhd, int ny, int nx, double gamma,
                                                         const double* __restrict__ cons,
                                                         const double* __restrict__ fbx,
                                                         const double* __restrict__ fby,
                                                         double* __restrict__ rows) {
  const int j = blockIdx.x;
  if (j >= ny) return;
  const size_t plane = (size_t)nx * ny;
  double mx = 0.0, my = 0.0;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const size_t idx = (size_t)j * nx + i;
    const double inv_d = 1.0 / cons[idx];
    const double vx = cons[plane + idx] * inv_d;
    const double vy = cons[2 * plane + idx] * inv_d;
    const double vz = cons[3 * plane + idx] * inv_d;
    const double vsq = vx * vx + vy * vy + vz * vz;
    if (mhd) {
      const double c4 = cons[4 * plane + idx], c5 = cons[5 * plane + idx];
      const double bx = c4 + fabs(fbx[(size_t)j * (nx + 1) + i] - c4);
      const double by = c5 + fabs(fby[(size_t)j * nx + i] - c5);
      const double bz = cons[6 * plane + idx];
      const double bsq = bx * bx + by * by + bz * bz;
      const double p = dmax((gamma - 1.0) * (cons[7 * plane + idx] - 0.5 * cons[idx] * vsq - 0.5 * bsq), kSmall);
      const double a2 = gamma * p * inv_d;
      const double ssum = bsq * inv_d + a2;
      const double sdiff = bsq * inv_d - a2;
      const double cfx2 = 0.5 * (ssum + sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d));
      const double cfy2 = 0.5 * (ssum + sqrt(sdiff * sdiff + 4.0 * a2 * (bx * bx + bz * bz) * inv_d));
      mx = dmax(mx, fabs(vx) + sqrt(cfx2));
      my = dmax(my, fabs(vy) + sqrt(cfy2));
    } else {
      const double p = dmax((gamma - 1.0) * (cons[4 * plane + idx] - 0.5 * cons[idx] * vsq), kSmall);
      const double a = sqrt(gamma * p * inv_d);
      mx = dmax(mx, fabs(vx) + a);
      my = dmax(my, fabs(vy) + a);
    }
  }
  __shared__ double sx[kThreads / 32], sy[kThreads / 32];
  block_max2(mx, my, sx, sy);
  if (threadIdx.x == 0) {
    rows[2 * j] = mx;
    rows[2 * j + 1] = my;
  }
}

// One block: reduce the row maxima and form dt as the reference does.
__global__ void __launch_bounds__(kThreads) k_finish_dt(int mhd, int ny, double cfl, double dx, double dy,
                                                        const double* __restrict__ rows, double* dt_out) {
  double mx = 0.0, my = 0.0;
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    mx = dmax(mx, rows[2 * j]);
    my = dmax(my, rows[2 * j + 1]);
  }
  __shared__ double sx[kThreads / 32], sy[kThreads / 32];
  block_max2(mx, my, sx, sy);
  if (threadIdx.x == 0) {
    double dt;
    if (mhd) {
      const double inv = dmax(mx / dx, my / dy);
      dt = cfl / inv;
    } else {
      const double dtx = cfl / (mx / dx);
      const double dty = cfl / (my / dy);
      dt = dmin(dtx, dty);
    }
    *dt_out = dt;
  }
}

// Device address of the static scratch on the current device, looked up once
// per device (cudaGetSymbolAddress) and cached.
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MHD_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MHD_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_setup_lock);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_row_max);
    if (e != cudaSuccess || !p) return MHD_ERR_CUDA;
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return MHD_OK;
}

}  // namespace

extern "C" int mhd2d_cfl_dt_noalloc(int physics, int ny, int nx, double dx, double dy, double gamma,
                                    double cfl, const double* cons, const double* faceBx,
                                    const double* faceBy, double* dt_out, void* stream) {
  if (physics != MHD2D_HYDRO && physics != MHD2D_MHD) return MHD_ERR_ARG;
  if (ny < 1 || nx < 1 || !(dx > 0.0) || !(dy > 0.0) || !cons || !dt_out) return MHD_ERR_ARG;
  if (physics == MHD2D_MHD && (!faceBx || !faceBy)) return MHD_ERR_ARG;
  if (ny > kMaxRows) return MHD_ERR_TOO_LARGE;
  // An error left pending by earlier work on this thread is not ours to clear or
  // to blame on this call: report it and launch nothing.
  if (cudaPeekAtLastError() != cudaSuccess) return MHD_ERR_CUDA;
  double* rows = nullptr;
  const int rc = scratch_for_current_device(&rows);
  if (rc != MHD_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int mhd = physics == MHD2D_MHD ? 1 : 0;
  k_row_speeds<<<ny, kThreads, 0, s>>>(mhd, ny, nx, gamma, cons, faceBx, faceBy, rows);
  k_finish_dt<<<1, kThreads, 0, s>>>(mhd, ny, cfl, dx, dy, rows, dt_out);
  return cudaGetLastError() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}
