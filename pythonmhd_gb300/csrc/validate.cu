// Device-side check of a 2D state before it is advanced: the reference's
// validatePrimVars (Source/SimulationGrid_HelperModule.py:282-410), which the
// reference's simulation constructor runs on the initial primitive state.  Per
// cell it forms the energy in the reference's order of operations
// (:292-297) and counts, for density, pressure and energy, the values below
// zero and the values below the run's floor; it also counts cells holding a NaN
// or Inf (the reference has no such check; an upload could carry one).
//
// Built with -fmad=false so the energy, and with it each comparison, rounds as
// the reference's NumPy expression does.
#include <cuda_runtime.h>

#include "../../include/pythonmhd_gb300.h"
#include "godunov2d_types.h"
#include "mhd_math.cuh"

namespace mhdk {

// counts[0] non-finite cells; [1 + 2v] var v < 0; [2 + 2v] var v < its floor
// (v = 0 density, 1 pressure, 2 energy)
constexpr int kValidateCounts = 7;

__global__ void __launch_bounds__(256) k_validate(int mhd, size_t plane, double gamma, double min_d, double min_p,
                                                  double min_e, const double* __restrict__ prim,
                                                  unsigned long long* __restrict__ counts) {
  unsigned c[kValidateCounts] = {0, 0, 0, 0, 0, 0, 0};
  const int nv = mhd ? 8 : 5;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
    double w[8];
    bool bad = false;
    for (int k = 0; k < nv; ++k) {
      w[k] = prim[k * plane + i];
      bad |= is_nonfinite(w[k]);
    }
    const double rho = w[0], p = w[mhd ? 7 : 4];
    double e = 0.5 * rho * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
    e = e + p / (gamma - 1.0);
    if (mhd) e = e + 0.5 * (w[4] * w[4] + w[5] * w[5] + w[6] * w[6]);
    c[0] += bad ? 1u : 0u;
    const double v[3] = {rho, p, e};
    const double lo[3] = {min_d, min_p, min_e};
    for (int k = 0; k < 3; ++k) {
      c[1 + 2 * k] += is_neg(v[k]) ? 1u : 0u;
      c[2 + 2 * k] += dlt(v[k], lo[k]) ? 1u : 0u;
    }
  }
  for (int k = 0; k < kValidateCounts; ++k)
    if (c[k]) atomicAdd(counts + k, (unsigned long long)c[k]);
}

// Queue the check of `prim` (nvars planes of `plane` cells) on `s`; `counts`
// (kValidateCounts words, device) must be zeroed by the caller.
void enqueue_validate(int mhd, size_t plane, double gamma, double min_d, double min_p, double min_e,
                      const double* prim, unsigned long long* counts, int blocks, cudaStream_t s) {
  k_validate<<<blocks, 256, 0, s>>>(mhd, plane, gamma, min_d, min_p, min_e, prim, counts);
}

}  // namespace mhdk

// ---------------------------------------------------------------------------
// The exact kernels' x / 6 (div6), elementwise, so that it can be compared bit for
// bit with the IEEE division.
// ---------------------------------------------------------------------------
namespace {
__global__ void k_quotient6(const double* __restrict__ x, double* __restrict__ q, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    q[i] = mhdk::div6(x[i]);
}
}  // namespace

// The integer-pipe add, subtract, multiply, divide and square root (softfp.cuh),
// elementwise, so that they can be compared bit for bit with the IEEE operations.
namespace {
__global__ void k_softfp(int op, const double* __restrict__ x, const double* __restrict__ y,
                         double* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = x[i];
    const double b = op == 4 ? 0.0 : y[i];
    out[i] = op == 0 ? sfp::add(a, b) : op == 1 ? sfp::sub(a, b) : op == 2 ? sfp::mul(a, b)
           : op == 3 ? sfp::div(a, b) : sfp::sqrt(a);
  }
}
}  // namespace

extern "C" int mhd_softfp(int op, const double* x, const double* y, double* out, long long n) {
  if (op < 0 || op > 4 || n < 0 || (n > 0 && (!x || !out || (op != 4 && !y)))) return MHD_ERR_ARG;
  if (n == 0) return MHD_OK;
  const long long blocks = (n + 255) / 256 < 152LL * 16 ? (n + 255) / 256 : 152LL * 16;
  k_softfp<<<(unsigned)blocks, 256>>>(op, x, y, out, n);
  if (cudaGetLastError() != cudaSuccess) return MHD_ERR_CUDA;
  return cudaDeviceSynchronize() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}

extern "C" int mhd_quotient6(const double* x, double* q, long long n) {
  if (n < 0 || (n > 0 && (!x || !q))) return MHD_ERR_ARG;
  if (n == 0) return MHD_OK;
  const long long blocks = (n + 255) / 256 < 152LL * 16 ? (n + 255) / 256 : 152LL * 16;
  k_quotient6<<<(unsigned)blocks, 256>>>(x, q, n);
  if (cudaGetLastError() != cudaSuccess) return MHD_ERR_CUDA;
  return cudaDeviceSynchronize() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}
