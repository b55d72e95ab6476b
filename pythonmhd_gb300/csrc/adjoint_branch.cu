// The branch-tape forward sweep of the adjoint's stage kernels (adjoint_kernels.cuh):
// one cycle that records (BR 1) or replays (BR 2) every branch decision of every
// stage, for checking the backward pass by finite differences on one smooth piece
// of the step.  A unit of its own so that it builds in parallel with adjoint.cu.
#include "adjoint_kernels.cuh"

namespace mhdadj {

template <int BR>
cudaError_t launch_fwd_branch(const Adj& A, cudaStream_t s) {
  const int nx = A.nx, ny = A.ny;
  Pair serial;
  serial.s = s;
  launch_recon<false, false, BR>(A, serial);
  k_face<0, false, BR><<<g2(nx + 1, ny, 2), kT, 0, s>>>(A);
  k_face<1, false, BR><<<g2(nx, ny + 1, 2), kT, 0, s>>>(A);
  k_roe<0, 1, false, false, BR><<<g1((size_t)(nx + 1) * ny), kT, 0, s>>>(A);
  k_roe<1, 1, false, false, BR><<<g1((size_t)nx * (ny + 1)), kT, 0, s>>>(A);
  k_ez<false><<<g2(nx, ny), kT, 0, s>>>(A);
  k_emf<1, false, BR><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  k_fhalf<0, false, false><<<g2(nx + 1, ny), kT, 0, s>>>(A);
  k_fhalf<1, false, false><<<g2(nx, ny + 1), kT, 0, s>>>(A);
  k_ctu<0, false, false, BR><<<g2(nx + 1, ny, 2), kT, 0, s>>>(A);
  k_ctu<1, false, false, BR><<<g2(nx, ny + 1, 2), kT, 0, s>>>(A);
  k_half<false><<<g2(nx, ny), kT, 0, s>>>(A);
  k_roe<0, 2, false, false, BR><<<g1((size_t)(nx + 1) * ny), kT, 0, s>>>(A);
  k_roe<1, 2, false, false, BR><<<g1((size_t)nx * (ny + 1)), kT, 0, s>>>(A);
  k_emf<2, false, BR><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  k_final<false><<<g2(nx, ny), kT, 0, s>>>(A);
  k_fhalf<0, true, false><<<g2(nx + 1, ny), kT, 0, s>>>(A);
  k_fhalf<1, true, false><<<g2(nx, ny + 1), kT, 0, s>>>(A);
  return cudaGetLastError();
}

template cudaError_t launch_fwd_branch<1>(const Adj& A, cudaStream_t s);
template cudaError_t launch_fwd_branch<2>(const Adj& A, cudaStream_t s);

}  // namespace mhdadj
