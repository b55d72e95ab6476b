// Initial states generated on the GPU: the seeded driven-free turbulence state and
// the Orszag-Tang vortex (pythonmhd_gb300/initial_conditions.py states the
// conventions; the vortex is the reference's sample setup,
// InitializationFiles/SampleSimulations/2D_MHD/OrszagTang_InitializationFile.py:134-194).
//
// The turbulence state: the random spectral coefficients are drawn on the host from
// the seeded NumPy stream (so the device state is the host generator's), only the
// few thousand coefficients inside the spectral band are uploaded and scattered
// into the half-spectrum here, the inverse transforms run in cuFFT, and the field
// algebra -- zero mean, unit variance, the rms-Mach and plasma-beta scalings, the
// faces from the vector potential, the cell-averaged B, prim -> cons -- runs in the
// kernels below.  Reductions are two-level and in a fixed order (per-block partial
// sums, then one block), so a state is the same on every run.  Built with
// -fmad=false: every operation rounds as the host generator's NumPy does; the
// transforms and reductions are evaluated differently, so the two states agree to
// rounding, not bit for bit.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/pythonmhd_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 512;       // blocks of every reduction (fixed: the sums' order is fixed)
constexpr int kSums = 4;              // sums per reduction pass (at most)
constexpr double kPi = 3.141592653589793;

// work layout (doubles): [0, kRedBlocks * kSums) partial sums; then results
constexpr long long kWorkWords = (long long)kRedBlocks * kSums + 16;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// per-block partial sums of up to kSums quantities of cell i, then one block adds
// the partials in block order into res[0..nsum)
template <class F>
__global__ void __launch_bounds__(kThreads) k_partials(long long ncell, int nsum, F f, double* partial) {
  __shared__ double sh[kThreads];
  double acc[kSums] = {0.0, 0.0, 0.0, 0.0};
  for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < ncell; i += (long long)gridDim.x * kThreads) {
    double v[kSums];
    f(i, v);
    for (int s = 0; s < nsum; ++s) acc[s] = acc[s] + v[s];
  }
  for (int s = 0; s < nsum; ++s) {
    const double b = block_sum(acc[s], sh);
    if (threadIdx.x == 0) partial[s * kRedBlocks + blockIdx.x] = b;
  }
}

__global__ void __launch_bounds__(kThreads) k_finish(int nsum, const double* partial, double* res) {
  __shared__ double sh[kThreads];
  for (int s = 0; s < nsum; ++s) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < kRedBlocks; b += kThreads) acc = acc + partial[s * kRedBlocks + b];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) res[s] = t;
  }
}

template <class F>
void reduce(long long ncell, int nsum, F f, double* work, double* res, cudaStream_t s) {
  k_partials<<<kRedBlocks, kThreads, 0, s>>>(ncell, nsum, f, work);
  k_finish<<<1, kThreads, 0, s>>>(nsum, work, res);
}

__global__ void k_scatter(long long count, const int* idx, const double* re, const double* im, double* spec) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  spec[2 * (long long)idx[k]] = re[k];
  spec[2 * (long long)idx[k] + 1] = im[k];
}

// the generator's state from the four raw fields (zero-mean shift, scalings, faces)
struct TurbFields {
  int n;
  const double *g, *vx, *vy, *az;
  const double* r;   // results: 0..3 sums of g, vx, vy, az; 4 sum (g-mg)^2; 5 Mach sum; 6 B^2 sum
  double gamma;
  __device__ double mean(int q) const { return r[q] / ((double)n * (double)n); }
};

__global__ void __launch_bounds__(kThreads) k_turb_state(TurbFields T, double mach, double beta, double* prim,
                                                         double* cons, double* fbx, double* fby) {
  const int n = T.n;
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  const long long plane = (long long)n * n;
  if (i >= plane) return;
  const int row = (int)(i / n), col = (int)(i % n);
  const double d = 1.0 / n;
  const double gamma = T.gamma;
  const double mg = T.mean(0), mvx = T.mean(1), mvy = T.mean(2), maz = T.mean(3);
  const double sd = sqrt(T.r[4] / ((double)n * (double)n));
  const double vscale = mach / sqrt(T.r[5] / ((double)n * (double)n));
  const double bscale = sqrt(2.0 * (1.0 / gamma) / beta / (T.r[6] / ((double)n * (double)n)));
  const double rho = exp(0.1 * ((T.g[i] - mg) / sd));
  const double p = 1.0 / gamma;
  const double vx = (T.vx[i] - mvx) * vscale;
  const double vy = (T.vy[i] - mvy) * vscale;
  auto az = [&](int j, int k) { return T.az[(long long)((j + n) % n) * n + (k + n) % n] - maz; };
  // faces of this cell (left x-face, lower y-face) and of its right / upper neighbour
  const double bx_l = ((az(row + 1, col) - az(row, col)) / d) * bscale;
  const double bx_r = ((az(row + 1, col + 1) - az(row, col + 1)) / d) * bscale;
  const double by_b = (-(az(row, col + 1) - az(row, col)) / d) * bscale;
  const double by_t = (-(az(row + 1, col + 1) - az(row + 1, col)) / d) * bscale;
  fbx[(long long)row * (n + 1) + col] = bx_l;
  if (col == 0) fbx[(long long)row * (n + 1) + n] = bx_l;
  fby[(long long)row * n + col] = by_b;
  if (row == 0) fby[(long long)n * n + col] = by_b;
  const double cbx = (bx_l + bx_r) / 2.0;
  const double cby = (by_b + by_t) / 2.0;
  const double w[8] = {rho, vx, vy, 0.0, cbx, cby, 0.0, p};
  double e = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + 0.0 * 0.0);
  e = e + 0.5 * (cbx * cbx + cby * cby + 0.0 * 0.0);
  const double u[8] = {rho, rho * vx, rho * vy, rho * 0.0, cbx, cby, 0.0, e};
  for (int k = 0; k < 8; ++k) {
    prim[k * plane + i] = w[k];
    cons[k * plane + i] = u[k];
  }
}

__global__ void __launch_bounds__(kThreads) k_orszag_tang(int nx, int ny, double gamma, double b0_scale,
                                                          double rho_perturb, const double* noise, double* prim,
                                                          double* cons, double* fbx, double* fby) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  const long long plane = (long long)nx * ny;
  if (i >= plane) return;
  const int row = (int)(i / nx), col = (int)(i % nx);
  const double dx = (1.0 - 0.0) / nx, dy = (1.0 - 0.0) / ny;
  const double b0 = b0_scale / sqrt(4.0 * kPi);
  // corner vector potential at (x_i - dx/2, y_j - dy/2), x_i = (i + 0.5) dx
  auto az = [&](int j, int k) {
    const int jj = (j + ny) % ny, kk = (k + nx) % nx;
    const double X = 0.0 + (kk + 0.5) * dx, Y = 0.0 + (jj + 0.5) * dy;
    return (b0 / (4.0 * kPi)) * cos(4.0 * kPi * (X - dx / 2.0)) + (b0 / (2.0 * kPi)) * cos(2.0 * kPi * (Y - dy / 2.0));
  };
  const double bx_l = (az(row + 1, col) - az(row, col)) / dy;
  const double bx_r = (az(row + 1, col + 1) - az(row, col + 1)) / dy;
  const double by_b = -(az(row, col + 1) - az(row, col)) / dx;
  const double by_t = -(az(row + 1, col + 1) - az(row + 1, col)) / dx;
  fbx[(long long)row * (nx + 1) + col] = bx_l;
  if (col == 0) fbx[(long long)row * (nx + 1) + nx] = bx_l;
  fby[(long long)row * nx + col] = by_b;
  if (row == 0) fby[(long long)ny * nx + col] = by_b;
  const double X = 0.0 + (col + 0.5) * dx, Y = 0.0 + (row + 0.5) * dy;
  double rho = 25.0 / (36.0 * kPi);
  if (noise) rho = rho * (1.0 + rho_perturb * noise[i]);
  const double vx = -sin(2.0 * kPi * Y), vy = sin(2.0 * kPi * X);
  const double cbx = (bx_l + bx_r) / 2.0, cby = (by_b + by_t) / 2.0;
  const double p = 5.0 / (12.0 * kPi);
  const double w[8] = {rho, vx, vy, 0.0, cbx, cby, 0.0, p};
  double e = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + 0.0 * 0.0);
  e = e + 0.5 * (cbx * cbx + cby * cby + 0.0 * 0.0);
  const double u[8] = {rho, rho * vx, rho * vy, rho * 0.0, cbx, cby, 0.0, e};
  for (int k = 0; k < 8; ++k) {
    prim[k * plane + i] = w[k];
    cons[k * plane + i] = u[k];
  }
}

unsigned grid_of(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

extern "C" {

long long mhd_ic_work_words(void) { return kWorkWords; }

int mhd_ic_scatter_spectrum(long long count, const int* idx, const double* re, const double* im, double* spec,
                            void* stream) {
  if (count < 0 || (count > 0 && (!idx || !re || !im)) || !spec) return MHD_ERR_ARG;
  if (count == 0) return MHD_OK;
  k_scatter<<<grid_of(count), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(count, idx, re, im, spec);
  return cudaGetLastError() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}

int mhd_ic_turbulence_2d(int n, double gamma, double mach, double beta, const double* g, const double* vx,
                         const double* vy, const double* az, double* prim, double* cons, double* fbx, double* fby,
                         double* work, long long work_words, void* stream) {
  if (n < 2 || !g || !vx || !vy || !az || !prim || !cons || !fbx || !fby || !work) return MHD_ERR_ARG;
  if (work_words < kWorkWords) return MHD_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long nc = (long long)n * n;
  double* res = work + (long long)kRedBlocks * kSums;
  TurbFields T{n, g, vx, vy, az, res, gamma};
  // means of the four raw fields
  reduce(nc, 4, [=] __device__(long long i, double* v) { v[0] = g[i]; v[1] = vx[i]; v[2] = vy[i]; v[3] = az[i]; },
         work, res, s);
  // variance of g about its mean
  reduce(nc, 1, [=] __device__(long long i, double* v) {
    const double x = g[i] - T.mean(0);
    v[0] = x * x;
  }, work, res + 4, s);
  // <(vx^2 + vy^2) / c_s^2> of the zero-mean velocities, c_s^2 = gamma p / rho
  reduce(nc, 1, [=] __device__(long long i, double* v) {
    const double sd = sqrt(T.r[4] / ((double)n * (double)n));
    const double rho = exp(0.1 * ((g[i] - T.mean(0)) / sd));
    const double p = 1.0 / gamma;
    const double cs2 = gamma * p / rho;
    const double a = vx[i] - T.mean(1), b = vy[i] - T.mean(2);
    v[0] = (a * a + b * b) / cs2;
  }, work, res + 5, s);
  // <Bx^2 + By^2> of the cell-averaged B from the unscaled faces
  reduce(nc, 1, [=] __device__(long long i, double* v) {
    const int row = (int)(i / n), col = (int)(i % n);
    const double d = 1.0 / n, m = T.mean(3);
    auto a = [&](int j, int k) { return az[(long long)((j + n) % n) * n + (k + n) % n] - m; };
    const double cbx = ((a(row + 1, col) - a(row, col)) / d + (a(row + 1, col + 1) - a(row, col + 1)) / d) / 2.0;
    const double cby = (-(a(row, col + 1) - a(row, col)) / d + -(a(row + 1, col + 1) - a(row + 1, col)) / d) / 2.0;
    v[0] = cbx * cbx + cby * cby;
  }, work, res + 6, s);
  k_turb_state<<<grid_of(nc), kThreads, 0, s>>>(T, mach, beta, prim, cons, fbx, fby);
  return cudaGetLastError() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}

int mhd_ic_orszag_tang(int nx, int ny, double gamma, double b0_scale, double rho_perturb, const double* noise,
                       double* prim, double* cons, double* fbx, double* fby, void* stream) {
  if (nx < 2 || ny < 2 || !prim || !cons || !fbx || !fby) return MHD_ERR_ARG;
  k_orszag_tang<<<grid_of((long long)nx * ny), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      nx, ny, gamma, b0_scale, rho_perturb, noise, prim, cons, fbx, fby);
  return cudaGetLastError() == cudaSuccess ? MHD_OK : MHD_ERR_CUDA;
}

}  // extern "C"
