// Stage kernels of the adjoint of the MHD step: the stencil around the generated
// pointwise stage functions (adjoint_gen.cuh) for the forward sweep (plain, taped,
// or recording / replaying its branch decisions) and the reverse sweep.  Shared by
// adjoint.cu (forward, taped and reverse sweeps, host side) and adjoint_branch.cu
// (the branch-tape forward sweeps), which build as separate units in parallel.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "adjoint_gen.cuh"

namespace mhdadj {

constexpr int kT = 128;
// resident blocks per SM the heavy reverse kernels are compiled for (1: up to 255
// registers a thread; more blocks cap the registers and trade spills for occupancy)
#ifndef MHD_ADJ_REV_MIN_BLOCKS
#define MHD_ADJ_REV_MIN_BLOCKS 1
#endif
constexpr int kRevMinBlocks = MHD_ADJ_REV_MIN_BLOCKS;
static_assert(g_plm0_NT == g_plm1_NT && g_roe1_0_NT == g_roe1_1_NT && g_roe2_0_NT == g_roe2_1_NT &&
                  g_ctu0_NT == g_ctu1_NT && g_ppmi0_NT == g_ppmi1_NT && g_ppmt0_NT == g_ppmt1_NT &&
                  g_pslope0_NT == g_pslope1_NT &&
                  g_roe1_0_efix_NT == g_roe1_1_efix_NT && g_roe2_0_efix_NT == g_roe2_1_efix_NT,
              "the x and y sweeps of a stage store tapes of the same length");

struct Arr {
  double* v = nullptr;   // values
  double* b = nullptr;   // adjoints
  size_t ps = 0;         // plane stride
  __device__ __forceinline__ double* pv(int slot, size_t i) const { return v + (size_t)slot * ps + i; }
  __device__ __forceinline__ double* pb(int slot, size_t i) const { return b + (size_t)slot * ps + i; }
};

struct Adj {
  int nx, ny, bcx, bcy, recon, efix;
  double dx, dy, gamma, eps, min_d, min_p, min_e;
  double dt;                       // dt of the cycle being processed
  Arr P, C, FX, FY;                // input state
  Arr EX, EY;                      // edge states per cell (lia 7 + ria 7), x and y sweeps
  Arr SX, SY;                      // PPM: limited slopes of the sweep-extended cells and their
                                   // eigensystems' base words (g_pslope0_NO planes)
  Arr E0X, E0Y;                    // PPM: interface values after the monotonicity tests (a 7 + b 7)
  Arr XL, XR, YL, YR;              // reconstructed face states
  Arr F1X, F1Y, EZ, E1, NBX, NBY;  // stage-1 fluxes, cell Ez, corner EMF, half-step faces
  Arr UXL, UXR, UYL, UYR, WXL, WXR, WYL, WYR;  // CTU-corrected face cons / prim
  Arr HEZ, F2X, F2Y, E2;           // half-step Ez, stage-2 fluxes and EMF
  Arr NP, NC, NFX, NFY;            // output state
  double* red;                     // 2 doubles: CFL maxima (bits)
  // tapes of the heavy stages (values their reverse sweeps read), plane-major:
  // PLM per cell and sweep, Roe per face, stage and sweep
  double* tplm[2];
  double* troe[2][2];              // [stage-1][axis]
  double* tctu[2];                 // CTU per (face, side) and sweep
  double* tslope[2];               // PPM slopes per extended cell and sweep
  double* ttrace[2];               // PPM characteristic tracing per cell and sweep
  // branch tapes (32-bit words, item-major planes) of the branch-recording and
  // -replaying forward sweeps: kBt* below
  unsigned int* bt[16];
};

// branch tape of each stage: PPM slopes x/y (extended cells), reconstruction x/y
// (cells; PLM, or the PPM interface values), face states x/y (face, side), Roe stage 1
// x/y and stage 2 x/y (faces), corner EMF stage 1/2 (corners), CTU x/y (face, side),
// PPM tracing x/y (cells)
enum BtSlot {
  kBtSlope = 0, kBtRecon = 2, kBtFace = 4, kBtRoe1 = 6, kBtRoe2 = 8, kBtEmf = 10, kBtCtu = 12, kBtTrace = 14,
  kNumBt = 16
};
static_assert(kNumBt == sizeof(Adj::bt) / sizeof(Adj::bt[0]), "one branch tape per stage slot");

__device__ __forceinline__ int wrapc(int c, int L, int bc) {
  if (bc == 1) {
    int m = c % L;
    return m < 0 ? m + L : m;
  }
  return c < 0 ? 0 : (c >= L ? L - 1 : c);
}

struct IO {
  double* v;
  double* b;
};

__device__ __forceinline__ IO io(const Arr& a, int slot, size_t i) { return IO{a.pv(slot, i), a.pb(slot, i)}; }

// forward: gather inputs, call fwd, write outputs; reverse: gather inputs, read output
// adjoints, call rev, scatter input adjoints.
#define MHD_ADJ_APPLY(NAME, REV, INS, OUTS, PAR)                                  \
  do {                                                                            \
    double x_[g_##NAME##_NI];                                                     \
    _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NI; ++k_) x_[k_] = *INS[k_].v; \
    if constexpr (!(REV)) {                                                       \
      double y_[g_##NAME##_NO];                                                   \
      g_##NAME##_fwd(x_, PAR, y_);                                                \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NO; ++k_) *OUTS[k_].v = y_[k_]; \
    } else {                                                                      \
      double yb_[g_##NAME##_NO], xb_[g_##NAME##_NI];                              \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NO; ++k_) yb_[k_] = *OUTS[k_].b; \
      g_##NAME##_rev(x_, PAR, yb_, xb_);                                          \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NI; ++k_)               \
        if (nz(xb_[k_])) atomicAdd(INS[k_].b, xb_[k_]);                          \
    }                                                                             \
  } while (0)

// the same with a tape: the forward stores what the reverse reads, the reverse
// reads it back instead of recomputing the forward
#define MHD_ADJ_APPLY_T(NAME, REV, INS, OUTS, PAR, TP, ST)                        \
  do {                                                                            \
    double x_[g_##NAME##_NI];                                                     \
    _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NI; ++k_) x_[k_] = *INS[k_].v; \
    if constexpr (!(REV)) {                                                       \
      double y_[g_##NAME##_NO];                                                   \
      g_##NAME##_fwdt(x_, PAR, y_, TP, ST);                                       \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NO; ++k_) *OUTS[k_].v = y_[k_]; \
    } else {                                                                      \
      double yb_[g_##NAME##_NO], xb_[g_##NAME##_NI];                              \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NO; ++k_) yb_[k_] = *OUTS[k_].b; \
      g_##NAME##_revt(x_, PAR, yb_, xb_, TP, ST);                                 \
      _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NI; ++k_)               \
        if (nz(xb_[k_])) atomicAdd(INS[k_].b, xb_[k_]);                          \
    }                                                                             \
  } while (0)

// taped or plain application of a stage
#define MHD_ADJ_STAGE(NAME, REV, TAPE, INS, OUTS, PAR, TP, ST)                    \
  do {                                                                            \
    if constexpr (TAPE) MHD_ADJ_APPLY_T(NAME, REV, INS, OUTS, PAR, TP, ST);       \
    else MHD_ADJ_APPLY(NAME, REV, INS, OUTS, PAR);                                \
  } while (0)

// forward of a stage that records (BR 1) or replays (BR 2) its branch decisions on
// the bit tape BT (words at BT[k * ST])
#define MHD_ADJ_APPLY_B(NAME, BR, INS, OUTS, PAR, BT, ST)                         \
  do {                                                                            \
    double x_[g_##NAME##_NI], y_[g_##NAME##_NO];                                  \
    _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NI; ++k_) x_[k_] = *INS[k_].v; \
    g_##NAME##_fwdb<BR>(x_, PAR, y_, BT, ST);                                     \
    _Pragma("unroll") for (int k_ = 0; k_ < g_##NAME##_NO; ++k_) *OUTS[k_].v = y_[k_]; \
  } while (0)

// plain, taped or branch-tape forward / reverse application of a stage
#define MHD_ADJ_RUN(NAME, REV, TAPE, BR, INS, OUTS, PAR, TP, ST, BT)               \
  do {                                                                            \
    if constexpr (BR != 0) MHD_ADJ_APPLY_B(NAME, BR, INS, OUTS, PAR, BT, ST);      \
    else MHD_ADJ_STAGE(NAME, REV, TAPE, INS, OUTS, PAR, TP, ST);                  \
  } while (0)

// ---------------------------------------------------------------------------
// stage kernels (REV = false: forward with stored intermediates; true: reverse)
// ---------------------------------------------------------------------------
// limited slopes of the sweep-extended cells e = 0 .. L+1 (cell e-1) and the base
// words of each cell's eigensystem, which the PPM edge stage reads (PPM only)
template <int AX, bool REV, bool TAPE, int BR = 0>
__global__ void __launch_bounds__(kT, REV ? kRevMinBlocks : 1) k_slope(Adj A) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
  const int Wd = AX == 0 ? A.nx + 2 : A.nx, H = AX == 0 ? A.ny : A.ny + 2;
  if (col >= Wd || row >= H) return;
  const int e = AX == 0 ? col : row, t = AX == 0 ? row : col;
  const int L = AX == 0 ? A.nx : A.ny;
  const int bc = AX == 0 ? A.bcx : A.bcy;
  const size_t me = (size_t)row * Wd + col;
  const int slots[7] = {0, 1, 2, 3, AX == 0 ? 5 : 6, AX == 0 ? 6 : 4, 7};
  IO in[22];
  IO out[g_pslope0_NO];
#pragma unroll
  for (int o = -1; o <= 1; ++o) {
    const int c = wrapc(e - 1 + o, L, bc);
    const size_t ci = AX == 0 ? (size_t)t * A.nx + c : (size_t)c * A.nx + t;
#pragma unroll
    for (int k = 0; k < 7; ++k) in[(o + 1) * 7 + k] = io(A.P, slots[k], ci);
  }
  {
    const int c = wrapc(e - 1, L, bc);
    in[21] = io(A.P, AX == 0 ? 4 : 5, AX == 0 ? (size_t)t * A.nx + c : (size_t)c * A.nx + t);
  }
  const Arr& S = AX == 0 ? A.SX : A.SY;
#pragma unroll
  for (int k = 0; k < g_pslope0_NO; ++k) out[k] = io(S, k, me);
  const double par[1] = {A.gamma};
  double* tp = A.tslope[AX] + me;
  const size_t st = (size_t)Wd * H;
  unsigned int* bt = BR ? A.bt[kBtSlope + AX] + me : nullptr;
  if (AX == 0) MHD_ADJ_RUN(pslope0, REV, TAPE, BR, in, out, par, tp, st, bt);
  else MHD_ADJ_RUN(pslope1, REV, TAPE, BR, in, out, par, tp, st, bt);
}

// edge states of each cell: first order (copies), PLM (one fused stage), or the PPM
// interface values after the monotonicity tests (into E0X/E0Y; k_trace finishes them)
template <int AX, bool REV, bool TAPE, int RECON, int BR = 0>
__global__ void __launch_bounds__(kT, REV ? kRevMinBlocks : 1) k_recon(Adj A) {
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x, t0 = blockIdx.y;
  if (c0 >= A.nx || t0 >= A.ny) return;
  const size_t me = (size_t)t0 * A.nx + c0;
  const Arr& E = AX == 0 ? A.EX : A.EY;
  const int slots[7] = {0, 1, 2, 3, AX == 0 ? 5 : 6, AX == 0 ? 6 : 4, 7};
  if constexpr (RECON >= 1) {
    const int bc = AX == 0 ? A.bcx : A.bcy;
    constexpr int NI = RECON == 1 ? g_plm0_NI : g_ppmi0_NI;
    static_assert(g_plm0_NI == 22 && g_ppmi0_NI == 42, "edge stage inputs: PLM 3 cells + B_n; PPM 3 cells, 3 slopes");
    IO in[NI];
    IO out[14];
#pragma unroll
    for (int o = -1; o <= 1; ++o) {
      const int jj = AX == 0 ? t0 : wrapc(t0 + o, A.ny, bc);
      const int ii = AX == 0 ? wrapc(c0 + o, A.nx, bc) : c0;
      const size_t ci = (size_t)jj * A.nx + ii;
#pragma unroll
      for (int k = 0; k < 7; ++k) in[(o + 1) * 7 + k] = io(A.P, slots[k], ci);
    }
    if constexpr (RECON == 2) {
      // slopes of cells c-1, c, c+1 sit at extended indices c, c+1, c+2
      const Arr& S = AX == 0 ? A.SX : A.SY;
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        const size_t si = AX == 0 ? (size_t)t0 * (A.nx + 2) + c0 + o : (size_t)(t0 + o) * A.nx + c0;
#pragma unroll
        for (int k = 0; k < 7; ++k) in[21 + o * 7 + k] = io(S, k, si);
      }
    } else {
      in[21] = io(A.P, AX == 0 ? 4 : 5, me);
    }
    const Arr& O = RECON == 2 ? (AX == 0 ? A.E0X : A.E0Y) : E;
#pragma unroll
    for (int k = 0; k < 14; ++k) out[k] = io(O, k, me);
    const double par[2] = {A.gamma, A.dt / (AX == 0 ? A.dx : A.dy)};
    double* tp = A.tplm[AX] + me;
    const size_t st = (size_t)A.nx * A.ny;
    unsigned int* bt = BR ? A.bt[kBtRecon + AX] + me : nullptr;
    if constexpr (RECON == 1) {
      if (AX == 0) MHD_ADJ_RUN(plm0, REV, TAPE, BR, in, out, par, tp, st, bt);
      else MHD_ADJ_RUN(plm1, REV, TAPE, BR, in, out, par, tp, st, bt);
    } else {
      if (AX == 0) MHD_ADJ_RUN(ppmi0, REV, TAPE, BR, in, out, par, tp, st, bt);
      else MHD_ADJ_RUN(ppmi1, REV, TAPE, BR, in, out, par, tp, st, bt);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      if (!REV) {
        *E.pv(k, me) = *A.P.pv(slots[k], me);
        *E.pv(7 + k, me) = *A.P.pv(slots[k], me);
      } else {
        const double g = *E.pb(k, me) + *E.pb(7 + k, me);
        if (nz(g)) atomicAdd(A.P.pb(slots[k], me), g);
      }
    }
  }
}

// PPM: dt/2 characteristic tracing of each cell's interface values (E0X/E0Y -> EX/EY),
// with the eigensystem from the slope stage's base words (extended index c+1)
template <int AX, bool REV, bool TAPE, int BR = 0>
__global__ void __launch_bounds__(kT, REV ? kRevMinBlocks : 1) k_trace(Adj A) {
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x, t0 = blockIdx.y;
  if (c0 >= A.nx || t0 >= A.ny) return;
  const size_t me = (size_t)t0 * A.nx + c0;
  const int slots[7] = {0, 1, 2, 3, AX == 0 ? 5 : 6, AX == 0 ? 6 : 4, 7};
  static_assert(g_ppmt0_NI == 21 + g_pslope0_NO - 7, "tracing inputs: the cell, its interface values, eigensystem words");
  IO in[g_ppmt0_NI];
  IO out[14];
#pragma unroll
  for (int k = 0; k < 7; ++k) in[k] = io(A.P, slots[k], me);
  const Arr& E0 = AX == 0 ? A.E0X : A.E0Y;
#pragma unroll
  for (int k = 0; k < 14; ++k) in[7 + k] = io(E0, k, me);
  const Arr& S = AX == 0 ? A.SX : A.SY;
  const size_t si = AX == 0 ? (size_t)t0 * (A.nx + 2) + c0 + 1 : (size_t)(t0 + 1) * A.nx + c0;
#pragma unroll
  for (int k = 7; k < g_pslope0_NO; ++k) in[21 + k - 7] = io(S, k, si);
  const Arr& E = AX == 0 ? A.EX : A.EY;
#pragma unroll
  for (int k = 0; k < 14; ++k) out[k] = io(E, k, me);
  const double par[2] = {A.gamma, A.dt / (AX == 0 ? A.dx : A.dy)};
  double* tp = A.ttrace[AX] + me;
  const size_t st = (size_t)A.nx * A.ny;
  unsigned int* bt = BR ? A.bt[kBtTrace + AX] + me : nullptr;
  if (AX == 0) MHD_ADJ_RUN(ppmt0, REV, TAPE, BR, in, out, par, tp, st, bt);
  else MHD_ADJ_RUN(ppmt1, REV, TAPE, BR, in, out, par, tp, st, bt);
}

// The x and y kernels of a stage are independent: each writes its own outputs (or,
// in the reverse sweep, reads its own outputs' adjoints and adds into its inputs'
// with atomics).  A Pair runs the second on s2 beside the first and joins it back
// into s, so one kernel's last partial wave overlaps the other; without s2 they run
// one after the other on s.  The first failing stream call is kept in *err.
struct Pair {
  cudaStream_t s = nullptr, s2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaError_t* err = nullptr;
  template <class F, class G>
  void operator()(F first, G second) const {
    if (!s2) {
      first(s);
      second(s);
      return;
    }
    keep(cudaEventRecord(fork, s));
    keep(cudaStreamWaitEvent(s2, fork, 0));
    first(s);
    second(s2);
    keep(cudaEventRecord(join, s2));
    keep(cudaStreamWaitEvent(s, join, 0));
  }
  void keep(cudaError_t e) const {
    if (e != cudaSuccess && err && *err == cudaSuccess) *err = e;
  }
};

// launch the reconstruction of both sweeps (PPM: slopes, interface values, tracing)
template <bool REV, bool TAPE, int BR = 0>
void launch_recon(const Adj& A, const Pair& pair) {
  const int nx = A.nx, ny = A.ny;
  const dim3 gc((unsigned)((nx + kT - 1) / kT), (unsigned)ny);
  const dim3 gsx((unsigned)((nx + 2 + kT - 1) / kT), (unsigned)ny);
  const dim3 gsy((unsigned)((nx + kT - 1) / kT), (unsigned)(ny + 2));
  switch (A.recon) {
    case 0:
      pair([&](cudaStream_t s) { k_recon<0, REV, TAPE, 0, BR><<<gc, kT, 0, s>>>(A); },
           [&](cudaStream_t s) { k_recon<1, REV, TAPE, 0, BR><<<gc, kT, 0, s>>>(A); });
      break;
    case 1:
      pair([&](cudaStream_t s) { k_recon<0, REV, TAPE, 1, BR><<<gc, kT, 0, s>>>(A); },
           [&](cudaStream_t s) { k_recon<1, REV, TAPE, 1, BR><<<gc, kT, 0, s>>>(A); });
      break;
    default:
      if constexpr (!REV) {
        pair([&](cudaStream_t s) { k_slope<0, false, TAPE, BR><<<gsx, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_slope<1, false, TAPE, BR><<<gsy, kT, 0, s>>>(A); });
        pair([&](cudaStream_t s) { k_recon<0, false, TAPE, 2, BR><<<gc, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_recon<1, false, TAPE, 2, BR><<<gc, kT, 0, s>>>(A); });
        pair([&](cudaStream_t s) { k_trace<0, false, TAPE, BR><<<gc, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_trace<1, false, TAPE, BR><<<gc, kT, 0, s>>>(A); });
      } else {
        pair([&](cudaStream_t s) { k_trace<1, true, TAPE><<<gc, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_trace<0, true, TAPE><<<gc, kT, 0, s>>>(A); });
        pair([&](cudaStream_t s) { k_recon<1, true, TAPE, 2><<<gc, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_recon<0, true, TAPE, 2><<<gc, kT, 0, s>>>(A); });
        pair([&](cudaStream_t s) { k_slope<1, true, TAPE><<<gsy, kT, 0, s>>>(A); },
             [&](cudaStream_t s) { k_slope<0, true, TAPE><<<gsx, kT, 0, s>>>(A); });
      }
  }
}

// face states of one sweep: item = (face, side)
template <int AX, bool REV, int BR = 0>
__global__ void __launch_bounds__(kT) k_face(Adj A) {
  const int L = AX == 0 ? A.nx : A.ny;
  const int Wd = AX == 0 ? A.nx + 1 : A.nx;   // row width of the face array
  const int H = AX == 0 ? A.ny : A.ny + 1;
  const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y, side = blockIdx.z;
  if (col >= Wd || row >= H) return;
  const int f = AX == 0 ? col : row;   // face index along the sweep
  const int t = AX == 0 ? row : col;   // transverse index
  const int bc = AX == 0 ? A.bcx : A.bcy;
  int cell, sd, vc, f1, f2;
  if (side == 0) {
    if (bc == 0) {
      cell = f == 0 ? 0 : f - 1; sd = f == 0 ? 0 : 7;
      vc = f == 0 ? 0 : f - 1; f1 = f == 0 ? 0 : f - 1; f2 = f == 0 ? 0 : f;
    } else {
      cell = f == 0 ? L - 1 : f - 1; sd = 7;
      vc = cell; f1 = f == 0 ? L - 1 : f - 1; f2 = f;
    }
  } else {
    if (bc == 0) {
      cell = f == L ? L - 1 : f; sd = f == L ? 7 : 0;
      vc = cell; f1 = f == L ? L : f; f2 = f == L ? L : f + 1;
    } else {
      cell = f == L ? 0 : f; sd = 0;
      vc = cell; f1 = f == L ? L : f; f2 = f == L ? 1 : f + 1;
    }
  }
  const Arr& E = AX == 0 ? A.EX : A.EY;
  const Arr& FB = AX == 0 ? A.FX : A.FY;
  const Arr& OUT = AX == 0 ? (side == 0 ? A.XL : A.XR) : (side == 0 ? A.YL : A.YR);
  const size_t ci = AX == 0 ? (size_t)t * A.nx + cell : (size_t)cell * A.nx + t;
  const size_t vi = AX == 0 ? (size_t)t * A.nx + vc : (size_t)vc * A.nx + t;
  const size_t fi1 = AX == 0 ? (size_t)t * (A.nx + 1) + f1 : (size_t)f1 * A.nx + t;
  const size_t fi2 = AX == 0 ? (size_t)t * (A.nx + 1) + f2 : (size_t)f2 * A.nx + t;
  const size_t me = (size_t)row * Wd + col;
  IO in[10];
  IO out[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) in[k] = io(E, sd + k, ci);
  in[7] = io(A.P, AX == 0 ? 2 : 1, vi);
  in[8] = io(FB, 0, fi1);
  in[9] = io(FB, 0, fi2);
#pragma unroll
  for (int k = 0; k < 7; ++k) out[k] = io(OUT, k, me);
  const double par[4] = {A.min_d, A.min_p, 0.5 * A.dt, 1.0 / (AX == 0 ? A.dx : A.dy)};
  const size_t nfs = (size_t)Wd * H;
  unsigned int* bt = BR ? A.bt[kBtFace + AX] + side * nfs + me : nullptr;
  if (AX == 0) MHD_ADJ_RUN(face0, REV, false, BR, in, out, par, nullptr, 2 * nfs, bt);
  else MHD_ADJ_RUN(face1, REV, false, BR, in, out, par, nullptr, 2 * nfs, bt);
}

template <int AX, int STAGE, bool REV, bool TAPE, int BR = 0>
__global__ void __launch_bounds__(kT, REV ? kRevMinBlocks : 1) k_roe(Adj A) {
  const size_t nf = AX == 0 ? (size_t)(A.nx + 1) * A.ny : (size_t)A.nx * (A.ny + 1);
  const size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const Arr& WL = STAGE == 1 ? (AX == 0 ? A.XL : A.YL) : (AX == 0 ? A.WXL : A.WYL);
  const Arr& WR = STAGE == 1 ? (AX == 0 ? A.XR : A.YR) : (AX == 0 ? A.WXR : A.WYR);
  const Arr& BN = STAGE == 1 ? (AX == 0 ? A.FX : A.FY) : (AX == 0 ? A.NBX : A.NBY);
  const Arr& F = STAGE == 1 ? (AX == 0 ? A.F1X : A.F1Y) : (AX == 0 ? A.F2X : A.F2Y);
  const double par[2] = {A.gamma, A.eps};
  double* tp = A.troe[STAGE - 1][AX] + f;
  unsigned int* bt = BR ? A.bt[(STAGE == 1 ? kBtRoe1 : kBtRoe2) + AX] + f : nullptr;
  IO out[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) out[k] = io(F, k, f);
  if (STAGE == 1) {
    IO in[15];
#pragma unroll
    for (int k = 0; k < 7; ++k) { in[k] = io(WL, k, f); in[7 + k] = io(WR, k, f); }
    in[14] = io(BN, 0, f);
    if (A.efix) {
      if (AX == 0) MHD_ADJ_RUN(roe1_0_efix, REV, TAPE, BR, in, out, par, tp, nf, bt);
      else MHD_ADJ_RUN(roe1_1_efix, REV, TAPE, BR, in, out, par, tp, nf, bt);
    } else {
      if (AX == 0) MHD_ADJ_RUN(roe1_0, REV, TAPE, BR, in, out, par, tp, nf, bt);
      else MHD_ADJ_RUN(roe1_1, REV, TAPE, BR, in, out, par, tp, nf, bt);
    }
  } else {
    const Arr& UL = AX == 0 ? A.UXL : A.UYL;
    const Arr& UR = AX == 0 ? A.UXR : A.UYR;
    IO in[29];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      in[k] = io(WL, k, f); in[7 + k] = io(WR, k, f);
      in[14 + k] = io(UL, k, f); in[21 + k] = io(UR, k, f);
    }
    in[28] = io(BN, 0, f);
    if (A.efix) {
      if (AX == 0) MHD_ADJ_RUN(roe2_0_efix, REV, TAPE, BR, in, out, par, tp, nf, bt);
      else MHD_ADJ_RUN(roe2_1_efix, REV, TAPE, BR, in, out, par, tp, nf, bt);
    } else {
      if (AX == 0) MHD_ADJ_RUN(roe2_0, REV, TAPE, BR, in, out, par, tp, nf, bt);
      else MHD_ADJ_RUN(roe2_1, REV, TAPE, BR, in, out, par, tp, nf, bt);
    }
  }
}

template <bool REV>
__global__ void __launch_bounds__(kT) k_ez(Adj A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= A.nx || j >= A.ny) return;
  const size_t me = (size_t)j * A.nx + i;
  IO in[4] = {io(A.P, 2, me), io(A.P, 4, me), io(A.P, 1, me), io(A.P, 5, me)};
  IO out[1] = {io(A.EZ, 0, me)};
  const double* par = nullptr;
  MHD_ADJ_APPLY(ez, REV, in, out, par);
}

template <int STAGE, bool REV, int BR = 0>
__global__ void __launch_bounds__(kT) k_emf(Adj A) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y;
  const int nx = A.nx, ny = A.ny;
  if (I > nx || J > ny) return;
  const Arr& FXa = STAGE == 1 ? A.F1X : A.F2X;
  const Arr& FYa = STAGE == 1 ? A.F1Y : A.F2Y;
  const Arr& EZa = STAGE == 1 ? A.EZ : A.HEZ;
  const Arr& OUT = STAGE == 1 ? A.E1 : A.E2;
  const int ic = wrapc(I, nx, A.bcx), im = wrapc(I - 1, nx, A.bcx);
  const int jc = wrapc(J, ny, A.bcy), jm = wrapc(J - 1, ny, A.bcy);
  IO in[12] = {io(FYa, 0, (size_t)J * nx + im), io(FYa, 5, (size_t)J * nx + im),
               io(FYa, 0, (size_t)J * nx + ic), io(FYa, 5, (size_t)J * nx + ic),
               io(FXa, 0, (size_t)jc * (nx + 1) + I), io(FXa, 4, (size_t)jc * (nx + 1) + I),
               io(FXa, 0, (size_t)jm * (nx + 1) + I), io(FXa, 4, (size_t)jm * (nx + 1) + I),
               io(EZa, 0, (size_t)jc * nx + ic), io(EZa, 0, (size_t)jc * nx + im),
               io(EZa, 0, (size_t)jm * nx + ic), io(EZa, 0, (size_t)jm * nx + im)};
  IO out[1] = {io(OUT, 0, (size_t)J * (nx + 1) + I)};
  const double* par = nullptr;
  const size_t me = (size_t)J * (nx + 1) + I;
  unsigned int* bt = BR ? A.bt[kBtEmf + STAGE - 1] + me : nullptr;
  MHD_ADJ_RUN(emf, REV, false, BR, in, out, par, nullptr, (size_t)(nx + 1) * (ny + 1), bt);
}

// half-step (FULL=false, from E1 into NBX/NBY) or full-step (FULL=true, from E2 into NFX/NFY) faces
template <int AX, bool FULL, bool REV>
__global__ void __launch_bounds__(kT) k_fhalf(Adj A) {
  const int nx = A.nx, ny = A.ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  const int w = AX == 0 ? nx + 1 : nx, h = AX == 0 ? ny : ny + 1;
  if (i >= w || j >= h) return;
  const Arr& E = FULL ? A.E2 : A.E1;
  const size_t me = (size_t)j * w + i;
  const size_t cw = nx + 1;
  if (AX == 0) {
    IO in[3] = {io(A.FX, 0, me), io(E, 0, (size_t)(j + 1) * cw + i), io(E, 0, (size_t)j * cw + i)};
    IO out[1] = {io(FULL ? A.NFX : A.NBX, 0, me)};
    const double par[1] = {FULL ? A.dt / A.dy : 0.5 * (A.dt / A.dy)};
    MHD_ADJ_APPLY(fhx, REV, in, out, par);
  } else {
    IO in[3] = {io(A.FY, 0, me), io(E, 0, (size_t)j * cw + i + 1), io(E, 0, (size_t)j * cw + i)};
    IO out[1] = {io(FULL ? A.NFY : A.NBY, 0, me)};
    const double par[1] = {FULL ? A.dt / A.dx : 0.5 * (A.dt / A.dx)};
    MHD_ADJ_APPLY(fhy, REV, in, out, par);
  }
}

template <int AX, bool REV, bool TAPE, int BR = 0>
__global__ void __launch_bounds__(kT) k_ctu(Adj A) {
  const int nx = A.nx, ny = A.ny;
  const int Wd = AX == 0 ? nx + 1 : nx, H = AX == 0 ? ny : ny + 1;
  const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y, side = blockIdx.z;
  if (col >= Wd || row >= H) return;
  const int f = AX == 0 ? col : row, t = AX == 0 ? row : col;
  const int L = AX == 0 ? nx : ny;
  const int bc = AX == 0 ? A.bcx : A.bcy;
  const size_t me = (size_t)row * Wd + col;
  const int kpad = f + side;
  int scell, lb, rb;
  if (AX == 0) {
    scell = wrapc(kpad - 1, L, bc);
    if (bc == 0) { lb = kpad - 1 < 0 ? 0 : (kpad - 1 > L ? L : kpad - 1); rb = kpad > L ? L : kpad; }
    else { lb = kpad == 0 ? L - 1 : kpad - 1; rb = kpad == L + 1 ? 1 : kpad; }
  } else {
    if (bc == 0) {
      scell = kpad == 0 ? 1 : (kpad - 1 > L - 1 ? L - 1 : kpad - 1);
      lb = kpad == 0 ? 1 : kpad - 1; rb = kpad == L + 1 ? L - 1 : kpad;
    } else {
      scell = wrapc(kpad - 1, L, bc);
      lb = kpad == 0 ? L - 1 : kpad - 1; rb = kpad == L + 1 ? 1 : kpad;
    }
  }
  const int fc = wrapc(f - 1 + side, L, bc);
  const Arr& W = AX == 0 ? (side == 0 ? A.XL : A.XR) : (side == 0 ? A.YL : A.YR);
  const Arr& U = AX == 0 ? (side == 0 ? A.UXL : A.UXR) : (side == 0 ? A.UYL : A.UYR);
  const Arr& W2 = AX == 0 ? (side == 0 ? A.WXL : A.WXR) : (side == 0 ? A.WYL : A.WYR);
  const Arr& FB = AX == 0 ? A.FX : A.FY;
  const Arr& NB = AX == 0 ? A.NBX : A.NBY;
  const Arr& FT = AX == 0 ? A.F1Y : A.F1X;
  size_t hi, lo, si, lbi, rbi;
  if (AX == 0) {
    hi = (size_t)(t + 1) * nx + fc; lo = (size_t)t * nx + fc;
    si = (size_t)t * nx + scell;
    lbi = (size_t)t * (nx + 1) + lb; rbi = (size_t)t * (nx + 1) + rb;
  } else {
    hi = (size_t)fc * (nx + 1) + t + 1; lo = (size_t)fc * (nx + 1) + t;
    si = (size_t)scell * nx + t;
    lbi = (size_t)lb * nx + t; rbi = (size_t)rb * nx + t;
  }
  IO in[29];
  IO out[14];
#pragma unroll
  for (int k = 0; k < 7; ++k) in[k] = io(W, k, me);
  in[7] = io(FB, 0, me);
#pragma unroll
  for (int k = 0; k < 7; ++k) { in[8 + k] = io(FT, k, hi); in[15 + k] = io(FT, k, lo); }
  in[22] = io(A.P, 4, si); in[23] = io(A.P, 5, si); in[24] = io(A.P, 6, si); in[25] = io(A.P, 3, si);
  in[26] = io(FB, 0, lbi); in[27] = io(FB, 0, rbi);
  in[28] = io(NB, 0, me);
#pragma unroll
  for (int k = 0; k < 7; ++k) { out[k] = io(U, k, me); out[7 + k] = io(W2, k, me); }
  const double par[6] = {A.gamma, 0.5 * A.dt, 1.0 / (AX == 0 ? A.dx : A.dy),
                         0.5 * (A.dt / (AX == 0 ? A.dy : A.dx)), A.min_d, A.min_e};
  const size_t nf = (size_t)H * Wd;
  double* tp = A.tctu[AX] + side * nf + me;
  unsigned int* bt = BR ? A.bt[kBtCtu + AX] + side * nf + me : nullptr;
  if (AX == 0) MHD_ADJ_RUN(ctu0, REV, TAPE, BR, in, out, par, tp, 2 * nf, bt);
  else MHD_ADJ_RUN(ctu1, REV, TAPE, BR, in, out, par, tp, 2 * nf, bt);
}

template <bool REV>
__global__ void __launch_bounds__(kT) k_half(Adj A) {
  const int nx = A.nx;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= nx || j >= A.ny) return;
  const size_t me = (size_t)j * nx + i;
  const size_t xl = (size_t)j * (nx + 1) + i, yt = (size_t)j * nx + i, yb = (size_t)(j + 1) * nx + i;
  IO in[19];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    in[k] = io(A.C, k, me);
    in[3 + k] = io(A.F1X, k, xl);
    in[6 + k] = io(A.F1X, k, xl + 1);
    in[9 + k] = io(A.F1Y, k, yt);
    in[12 + k] = io(A.F1Y, k, yb);
  }
  in[15] = io(A.NBX, 0, xl); in[16] = io(A.NBX, 0, xl + 1);
  in[17] = io(A.NBY, 0, yt); in[18] = io(A.NBY, 0, yb);
  IO out[1] = {io(A.HEZ, 0, me)};
  const double par[2] = {0.5 * (A.dt / A.dx), 0.5 * (A.dt / A.dy)};
  MHD_ADJ_APPLY(half, REV, in, out, par);
}

template <bool REV>
__global__ void __launch_bounds__(kT) k_final(Adj A) {
  const int nx = A.nx;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= nx || j >= A.ny) return;
  const size_t me = (size_t)j * nx + i;
  const size_t xl = (size_t)j * (nx + 1) + i, yt = (size_t)j * nx + i, yb = (size_t)(j + 1) * nx + i;
  const size_t cw = nx + 1;
  const int xs[7] = {0, 1, 2, 3, 5, 6, 7};
  IO in[43];
  in[0] = io(A.FX, 0, xl); in[1] = io(A.FX, 0, xl + 1);
  in[2] = io(A.FY, 0, yt); in[3] = io(A.FY, 0, yb);
  in[4] = io(A.E2, 0, (size_t)j * cw + i); in[5] = io(A.E2, 0, (size_t)(j + 1) * cw + i);
  in[6] = io(A.E2, 0, (size_t)j * cw + i + 1); in[7] = io(A.E2, 0, (size_t)(j + 1) * cw + i + 1);
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    in[8 + k] = io(A.C, xs[k], me);
    in[15 + k] = io(A.F2X, k, xl);
    in[22 + k] = io(A.F2X, k, xl + 1);
    in[29 + k] = io(A.F2Y, k, yt);
    in[36 + k] = io(A.F2Y, k, yb);
  }
  IO out[16];
#pragma unroll
  for (int k = 0; k < 8; ++k) { out[k] = io(A.NP, k, me); out[8 + k] = io(A.NC, k, me); }
  const double par[3] = {A.dt / A.dx, A.dt / A.dy, A.gamma};
  MHD_ADJ_APPLY(final, REV, in, out, par);
}

inline dim3 g2(int w, int h, int z = 1) { return dim3((unsigned)((w + kT - 1) / kT), (unsigned)h, (unsigned)z); }
inline unsigned g1(size_t n) { return (unsigned)((n + kT - 1) / kT); }

// one forward cycle that records (BR 1) or replays (BR 2) its branch decisions on the
// bit tapes A.bt; defined in adjoint_branch.cu
template <int BR>
cudaError_t launch_fwd_branch(const Adj& A, cudaStream_t s);

}  // namespace mhdadj
