// Reverse-mode adjoint of the MHD CTU+CT step (first-order, PLM and PPM reconstruction).
//
// The pointwise stage functions come from adjoint_gen.cuh (generated from
// pythonmhd_gb300/adjoint/stages.py: <stage>_fwd / <stage>_rev).  This file holds
// the stencil around them -- which cell, face or corner feeds each input -- in a
// forward sweep that stores every intermediate array of a cycle and a reverse
// sweep that runs the stages backwards, scattering input adjoints with atomicAdd.
// The gathers mirror the forward kernels in godunov2d_kernels.cuh.
//
// dt is frozen: the forward pass records the CFL dt of every cycle and the
// reverse sweep treats it as a constant.  Long runs keep a state checkpoint every
// K cycles (K ~ sqrt(steps)) and recompute the states inside a segment during the
// backward pass.  The forward statements use non-contracting round-to-nearest
// intrinsics, so the forward sweep reproduces the exact-arithmetic step bit for
// bit although the unit is compiled with FMA contraction for the reverse sweeps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "../../include/pythonmhd_gb300.h"

#include "adjoint_kernels.cuh"

namespace {

using namespace mhdadj;

// ---------------------------------------------------------------------------
// CFL dt of the input state (Source/TimestepCalculations_HelperModule.py:239-289)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dmax2(double a, double b) { return dsl_gt(a, b) ? a : b; }

__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double Ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double Sb(double a, double b) { return __dsub_rn(a, b); }

// The unit is compiled with FMA contraction (for the reverse sweeps), so the
// CFL arithmetic spells out its roundings to match the exact-arithmetic step.
__global__ void __launch_bounds__(256) k_cfl(Adj A) {
  const int nx = A.nx;
  const size_t n = (size_t)A.nx * A.ny, plane = n;
  const double gamma = A.gamma;
  const double* c = A.C.v;
  double mx = 0.0, my = 0.0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const double inv_d = mhdk::ddiv(1.0, c[idx]);
    const double vx = M(c[plane + idx], inv_d);
    const double vy = M(c[2 * plane + idx], inv_d);
    const double vz = M(c[3 * plane + idx], inv_d);
    const double vsq = Ad(Ad(M(vx, vx), M(vy, vy)), M(vz, vz));
    const int j = (int)(idx / nx), i = (int)(idx % nx);
    const double c4 = c[4 * plane + idx], c5 = c[5 * plane + idx];
    const double bx = Ad(c4, fabs(Sb(A.FX.v[(size_t)j * (nx + 1) + i], c4)));
    const double by = Ad(c5, fabs(Sb(A.FY.v[(size_t)j * nx + i], c5)));
    const double bz = c[6 * plane + idx];
    const double bsq = Ad(Ad(M(bx, bx), M(by, by)), M(bz, bz));
    const double e_int = Sb(Sb(c[7 * plane + idx], M(M(0.5, c[idx]), vsq)), M(0.5, bsq));
    const double p = dmax2(M(gamma - 1.0, e_int), 0.000000000001);
    const double a2 = M(M(gamma, p), inv_d);
    const double bd = M(bsq, inv_d);
    const double ssum = Ad(bd, a2);
    const double sdiff = Sb(bd, a2);
    const double dd = M(sdiff, sdiff);
    const double cfx2 = M(0.5, Ad(ssum, mhdk::sqrt(Ad(dd, M(M(M(4.0, a2), Ad(M(by, by), M(bz, bz))), inv_d)))));
    const double cfy2 = M(0.5, Ad(ssum, mhdk::sqrt(Ad(dd, M(M(M(4.0, a2), Ad(M(bx, bx), M(bz, bz))), inv_d)))));
    mx = dmax2(mx, Ad(fabs(vx), mhdk::sqrt(cfx2)));
    my = dmax2(my, Ad(fabs(vy), mhdk::sqrt(cfy2)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = dmax2(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    my = dmax2(my, __shfl_xor_sync(0xffffffffu, my, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned long long*>(A.red), (unsigned long long)__double_as_longlong(mx));
    atomicMax(reinterpret_cast<unsigned long long*>(A.red + 1), (unsigned long long)__double_as_longlong(my));
  }
}

__global__ void k_cfl_finish(Adj A, double cfl, double* dt_slot) {
  const double mx = A.red[0], my = A.red[1];
  const double inv = dmax2(mx / A.dx, my / A.dy);
  *dt_slot = cfl / inv;
  A.red[0] = 0.0;
  A.red[1] = 0.0;
}

// the reverse statements' quotient, elementwise (its error bound is tested against
// the correctly rounded division)
__global__ void k_quotient(const double* __restrict__ b, const double* __restrict__ v, double* __restrict__ q,
                           long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    q[i] = dsl_div(b[i], v[i]);
}


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Every array of a cycle, in arena order: inputs first, outputs last (the
// reverse sweep clears all adjoints below the outputs with one memset).
struct Slot {
  Arr Adj::*arr;
  int planes;
  int kind;   // 0 cell, 1 x-face, 2 y-face, 3 corner, 4 x-extended cell, 5 y-extended cell
};
const Slot kSlots[] = {
    {&Adj::P, 8, 0},   {&Adj::C, 8, 0},   {&Adj::FX, 1, 1},  {&Adj::FY, 1, 2},  {&Adj::EX, 14, 0},
    {&Adj::EY, 14, 0}, {&Adj::SX, g_pslope0_NO, 4},  {&Adj::SY, g_pslope0_NO, 5},  {&Adj::E0X, 14, 0}, {&Adj::E0Y, 14, 0},  {&Adj::XL, 7, 1},  {&Adj::XR, 7, 1},  {&Adj::YL, 7, 2},  {&Adj::YR, 7, 2},
    {&Adj::F1X, 7, 1}, {&Adj::F1Y, 7, 2}, {&Adj::EZ, 1, 0},  {&Adj::E1, 1, 3},  {&Adj::NBX, 1, 1},
    {&Adj::NBY, 1, 2}, {&Adj::UXL, 7, 1}, {&Adj::UXR, 7, 1}, {&Adj::UYL, 7, 2}, {&Adj::UYR, 7, 2},
    {&Adj::WXL, 7, 1}, {&Adj::WXR, 7, 1}, {&Adj::WYL, 7, 2}, {&Adj::WYR, 7, 2}, {&Adj::HEZ, 1, 0},
    {&Adj::F2X, 7, 1}, {&Adj::F2Y, 7, 2}, {&Adj::E2, 1, 3},  {&Adj::NP, 8, 0},  {&Adj::NC, 8, 0},
    {&Adj::NFX, 1, 1}, {&Adj::NFY, 1, 2}};
constexpr int kNumSlots = sizeof(kSlots) / sizeof(kSlots[0]);
constexpr int kFirstOutput = kNumSlots - 4;

struct Handle {
  Adj A{};
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;              // the second kernel of each x/y pair (Pair)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  size_t off[kNumSlots] = {};  // word offset of each array in an arena
  size_t ps[kNumSlots] = {};   // plane stride of each array
  size_t W = 0;                // words of one arena (all arrays of one cycle)
  double* bars = nullptr;      // one adjoint arena
  size_t bars_cap = 0, vals_cap = 0, tapes_cap = 0;   // words held
  double* vals = nullptr;      // nsets value arenas
  size_t TW = 0;               // words of one tape arena
  double* tapes = nullptr;     // nsets tape arenas
  size_t toff[12] = {};        // tape offsets: recon x, recon y, roe1 x, roe1 y, roe2 x, roe2 y, ctu x, ctu y,
                               // PPM slopes x, y, PPM tracing x, y
  int nsets = 0;
  double* red = nullptr;       // CFL maxima (2) + dt (1)
  size_t budget = 0;           // bytes the stored-segment mode may use (0: 85% of free memory)
  // forward record: uniform segments of `every` cycles over the first steps - tail
  // cycles, then (stored mode) a tail segment whose cycles the forward pass runs with
  // the taped kernels and leaves resident, so the backward pass reverses them at once
  int steps = 0, every = 0;
  int tail = 0;                // cycles of the tail segment (0: none)
  int tail_max = -1;           // -1: as many as the segment budget holds; 0: no tail
  bool tail_resident = false;  // the tail's arrays and tapes are still in the arenas
  double* dtlog = nullptr;     // device log of the production solver's dts
  size_t dtlog_cap = 0;
  bool stored = false;         // backward keeps every cycle of a segment resident
  std::vector<double> dts;
  double* ckpt = nullptr;      // one packed state per segment
  bool ckpt_owned = true;      // false: the caller's memory (mhd2d_adj_restore)
  double* seg = nullptr;       // recompute mode: packed states of the current segment
  size_t ckpt_bytes = 0, seg_bytes = 0;
  size_t state_words = 0;
  void* solver = nullptr;      // exact-arithmetic production step: the CFL forward pass
  // branch arena of the branch-recording / -replaying forward sweeps: BW words per
  // cycle (offsets btoff per stage slot), recorded for br_steps cycles
  unsigned int* br = nullptr;
  size_t br_cap = 0, BW = 0, btoff[kNumBt] = {};
  int br_steps = 0;
};

int fail(cudaError_t e) { return e == cudaErrorMemoryAllocation ? MHD_ERR_NOMEM : MHD_ERR_CUDA; }
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return fail(e_); } while (0)

size_t state_words(const Adj& A) {
  const size_t cp = (size_t)A.nx * A.ny;
  return 16 * cp + (size_t)(A.nx + 1) * A.ny + (size_t)A.nx * (A.ny + 1);
}

// point the Arr views of h->A at value arena k (adjoints always in the one bar arena)
void select_set(Handle* h, int k) {
  double* base = h->vals + (size_t)k * h->W;
  for (int i = 0; i < kNumSlots; ++i) {
    Arr& a = h->A.*(kSlots[i].arr);
    a.v = base + h->off[i];
    a.b = h->bars + h->off[i];
    a.ps = h->ps[i];
  }
  double* tb = h->tapes + (size_t)k * h->TW;
  h->A.tplm[0] = tb + h->toff[0];
  h->A.tplm[1] = tb + h->toff[1];
  h->A.troe[0][0] = tb + h->toff[2];
  h->A.troe[0][1] = tb + h->toff[3];
  h->A.troe[1][0] = tb + h->toff[4];
  h->A.troe[1][1] = tb + h->toff[5];
  h->A.tctu[0] = tb + h->toff[6];
  h->A.tctu[1] = tb + h->toff[7];
  h->A.tslope[0] = tb + h->toff[8];
  h->A.tslope[1] = tb + h->toff[9];
  h->A.ttrace[0] = tb + h->toff[10];
  h->A.ttrace[1] = tb + h->toff[11];
}

// n value+tape arenas of the current layout.  Memory is kept while it is large
// enough (fewer arenas, or a handle reshaped to a smaller grid, reuse it) and
// released when the handle is destroyed.
int alloc_sets(Handle* h, int n) {
  const size_t need_v = (size_t)n * h->W, need_t = (size_t)n * h->TW;
  if (need_v > h->vals_cap || need_t > h->tapes_cap) {
    cudaFree(h->vals);
    cudaFree(h->tapes);
    h->vals = h->tapes = nullptr;
    h->vals_cap = h->tapes_cap = 0;
    h->nsets = 0;
    CK(cudaMalloc(&h->vals, need_v * sizeof(double)));
    h->vals_cap = need_v;
    CK(cudaMalloc(&h->tapes, (need_t ? need_t : 1) * sizeof(double)));
    h->tapes_cap = need_t;
  }
  h->nsets = n;
  select_set(h, 0);
  return MHD_OK;
}

size_t device_bytes(const Handle* h) {
  return (h->bars_cap + h->vals_cap + h->tapes_cap + 4 + h->dtlog_cap) * sizeof(double) + h->ckpt_bytes +
         h->seg_bytes + h->br_cap * sizeof(unsigned int);
}

// Words of one cycle's branch tapes and each stage slot's offset (items x words of
// the stage, 128-byte aligned).
void branch_layout(int nx, int ny, int recon, int efix, size_t* off, size_t* BW) {
  const size_t cells = (size_t)nx * ny, xf = (size_t)(nx + 1) * ny, yf = (size_t)nx * (ny + 1);
  const size_t corners = (size_t)(nx + 1) * (ny + 1);
  const int nb_recon = recon == 1 ? std::max(g_plm0_NB, g_plm1_NB) : (recon == 2 ? std::max(g_ppmi0_NB, g_ppmi1_NB) : 0);
  const int nb_trace = recon == 2 ? std::max(g_ppmt0_NB, g_ppmt1_NB) : 0;
  const int nb_slope = recon == 2 ? std::max(g_pslope0_NB, g_pslope1_NB) : 0;
  const int nb_roe1 = efix ? std::max(g_roe1_0_efix_NB, g_roe1_1_efix_NB) : std::max(g_roe1_0_NB, g_roe1_1_NB);
  const int nb_roe2 = efix ? std::max(g_roe2_0_efix_NB, g_roe2_1_efix_NB) : std::max(g_roe2_0_NB, g_roe2_1_NB);
  const size_t items[kNumBt] = {(size_t)(nx + 2) * ny, (size_t)nx * (ny + 2), cells, cells, 2 * xf, 2 * yf,
                                xf, yf, xf, yf, corners, corners, 2 * xf, 2 * yf, cells, cells};
  const int words[kNumBt] = {nb_slope, nb_slope, nb_recon, nb_recon, std::max(g_face0_NB, g_face1_NB),
                             std::max(g_face0_NB, g_face1_NB), nb_roe1, nb_roe1, nb_roe2, nb_roe2, g_emf_NB, g_emf_NB,
                             std::max(g_ctu0_NB, g_ctu1_NB), std::max(g_ctu0_NB, g_ctu1_NB), nb_trace, nb_trace};
  size_t w = 0;
  for (int i = 0; i < kNumBt; ++i) {
    off[i] = w;
    w += items[i] * (size_t)words[i];
    w = (w + 31) & ~(size_t)31;
  }
  *BW = w;
}


// segments of a record: ceil(head / every) uniform segments over the first
// head = steps - tail cycles, then the tail segment when tail > 0
int head_segments(const Handle* h) { return (h->steps - h->tail + h->every - 1) / h->every; }
int num_segments(const Handle* h) { return head_segments(h) + (h->tail > 0 ? 1 : 0); }
void segment(const Handle* h, int s, int* c0, int* len) {
  const int head = h->steps - h->tail;
  if (s < head_segments(h)) {
    *c0 = s * h->every;
    *len = std::min(h->every, head - *c0);
  } else {
    *c0 = head;
    *len = h->tail;
  }
}

// copy a packed state [prim 8 | cons 8 | fbx | fby] into / out of four arrays
int pack(Handle* h, double* dst, const Arr& P, const Arr& C, const Arr& FX, const Arr& FY, bool bars) {
  const Adj& A = h->A;
  const size_t cp = (size_t)A.nx * A.ny, xp = (size_t)(A.nx + 1) * A.ny, yp = (size_t)A.nx * (A.ny + 1);
  auto src = [&](const Arr& a) { return bars ? a.b : a.v; };
  CK(cudaMemcpyAsync(dst, src(P), 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst + 8 * cp, src(C), 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst + 16 * cp, src(FX), xp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst + 16 * cp + xp, src(FY), yp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return MHD_OK;
}

int unpack(Handle* h, const double* src, Arr& P, Arr& C, Arr& FX, Arr& FY, bool bars) {
  const Adj& A = h->A;
  const size_t cp = (size_t)A.nx * A.ny, xp = (size_t)(A.nx + 1) * A.ny, yp = (size_t)A.nx * (A.ny + 1);
  auto dst = [&](Arr& a) { return bars ? a.b : a.v; };
  CK(cudaMemcpyAsync(dst(P), src, 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst(C), src + 8 * cp, 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst(FX), src + 16 * cp, xp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(dst(FY), src + 16 * cp + xp, yp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return MHD_OK;
}


// the handle's streams and events as a Pair (x/y kernels of a stage side by side)
Pair pair_of(Handle* h, cudaError_t* err) {
  Pair p;
  p.s = h->stream;
  p.s2 = h->stream2;
  p.fork = h->ev_fork;
  p.join = h->ev_join;
  p.err = err;
  return p;
}

// forward sweep of one cycle from the input arrays (P, C, FX, FY) with A.dt set;
// TAPE: the PLM and Roe stages also write the tapes their reverse sweeps read
template <bool TAPE>
int fwd_cycle_t(Handle* h) {
  Adj& A = h->A;
  const int nx = A.nx, ny = A.ny;
  cudaError_t err = cudaSuccess;
  const Pair pair = pair_of(h, &err);
  cudaStream_t s = h->stream;
  launch_recon<false, TAPE>(A, pair);
  pair([&](cudaStream_t t) { k_face<0, false><<<g2(nx + 1, ny, 2), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_face<1, false><<<g2(nx, ny + 1, 2), kT, 0, t>>>(A); });
  pair([&](cudaStream_t t) { k_roe<0, 1, false, TAPE><<<g1((size_t)(nx + 1) * ny), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_roe<1, 1, false, TAPE><<<g1((size_t)nx * (ny + 1)), kT, 0, t>>>(A); });
  k_ez<false><<<g2(nx, ny), kT, 0, s>>>(A);
  k_emf<1, false><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_fhalf<0, false, false><<<g2(nx + 1, ny), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_fhalf<1, false, false><<<g2(nx, ny + 1), kT, 0, t>>>(A); });
  pair([&](cudaStream_t t) { k_ctu<0, false, TAPE><<<g2(nx + 1, ny, 2), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_ctu<1, false, TAPE><<<g2(nx, ny + 1, 2), kT, 0, t>>>(A); });
  k_half<false><<<g2(nx, ny), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_roe<0, 2, false, TAPE><<<g1((size_t)(nx + 1) * ny), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_roe<1, 2, false, TAPE><<<g1((size_t)nx * (ny + 1)), kT, 0, t>>>(A); });
  k_emf<2, false><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  k_final<false><<<g2(nx, ny), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_fhalf<0, true, false><<<g2(nx + 1, ny), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_fhalf<1, true, false><<<g2(nx, ny + 1), kT, 0, t>>>(A); });
  CK(err);
  CK(cudaGetLastError());
  return MHD_OK;
}

int fwd_cycle(Handle* h, bool tape) { return tape ? fwd_cycle_t<true>(h) : fwd_cycle_t<false>(h); }

// forward sweep of one cycle that records (BR 1) or replays (BR 2) every branch
// decision on the bit tapes A.bt (set to the cycle's region of the branch arena)
template <int BR>
int fwd_cycle_b(Handle* h) {
  CK(launch_fwd_branch<BR>(h->A, h->stream));
  return MHD_OK;
}

// reverse sweep: output adjoints in NP/NC/NFX/NFY .b -> input adjoints in P/C/FX/FY .b
// (reads the tapes of the last taped forward sweep of the selected arena)
int rev_cycle(Handle* h) {
  Adj& A = h->A;
  cudaStream_t s = h->stream;
  const int nx = A.nx, ny = A.ny;
  cudaError_t err = cudaSuccess;
  const Pair pair = pair_of(h, &err);
  // zero every adjoint except the outputs' (they sit at the end of the arena)
  CK(cudaMemsetAsync(h->bars, 0, h->off[kFirstOutput] * sizeof(double), s));
  pair([&](cudaStream_t t) { k_fhalf<1, true, true><<<g2(nx, ny + 1), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_fhalf<0, true, true><<<g2(nx + 1, ny), kT, 0, t>>>(A); });
  k_final<true><<<g2(nx, ny), kT, 0, s>>>(A);
  k_emf<2, true><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_roe<1, 2, true, true><<<g1((size_t)nx * (ny + 1)), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_roe<0, 2, true, true><<<g1((size_t)(nx + 1) * ny), kT, 0, t>>>(A); });
  k_half<true><<<g2(nx, ny), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_ctu<1, true, true><<<g2(nx, ny + 1, 2), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_ctu<0, true, true><<<g2(nx + 1, ny, 2), kT, 0, t>>>(A); });
  pair([&](cudaStream_t t) { k_fhalf<1, false, true><<<g2(nx, ny + 1), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_fhalf<0, false, true><<<g2(nx + 1, ny), kT, 0, t>>>(A); });
  k_emf<1, true><<<g2(nx + 1, ny + 1), kT, 0, s>>>(A);
  k_ez<true><<<g2(nx, ny), kT, 0, s>>>(A);
  pair([&](cudaStream_t t) { k_roe<1, 1, true, true><<<g1((size_t)nx * (ny + 1)), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_roe<0, 1, true, true><<<g1((size_t)(nx + 1) * ny), kT, 0, t>>>(A); });
  pair([&](cudaStream_t t) { k_face<1, true><<<g2(nx, ny + 1, 2), kT, 0, t>>>(A); },
       [&](cudaStream_t t) { k_face<0, true><<<g2(nx + 1, ny, 2), kT, 0, t>>>(A); });
  launch_recon<true, true>(A, pair);
  CK(err);
  CK(cudaGetLastError());
  return MHD_OK;
}

int cfl_dt(Handle* h, double cfl, double* host_dt) {
  Adj& A = h->A;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_cfl<<<sms * 4, 256, 0, h->stream>>>(A);
  k_cfl_finish<<<1, 1, 0, h->stream>>>(A, cfl, h->red + 2);
  CK(cudaMemcpyAsync(host_dt, h->red + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

// inputs of value arena `to` <- outputs of value arena `from` (the state after that cycle)
int output_to_input(Handle* h, int from, int to) {
  const double* src = h->vals + (size_t)from * h->W;
  double* dst = h->vals + (size_t)to * h->W;
  for (int i = 0; i < 4; ++i) {
    const size_t n = (size_t)kSlots[i].planes * h->ps[i];
    CK(cudaMemcpyAsync(dst + h->off[i], src + h->off[kFirstOutput + i], n * sizeof(double),
                       cudaMemcpyDeviceToDevice, h->stream));
  }
  return MHD_OK;
}

int bars_in_to_out(Handle* h) {
  Adj& A = h->A;
  const size_t cp = (size_t)A.nx * A.ny;
  CK(cudaMemcpyAsync(A.NP.b, A.P.b, 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(A.NC.b, A.C.b, 8 * cp * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(A.NFX.b, A.FX.b, A.FX.ps * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(A.NFY.b, A.FY.b, A.FY.ps * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return MHD_OK;
}

// `steps` cycles with the host dts `dt` from state_in, recording (mode 1) or
// replaying (mode 2) every branch decision; the final state goes to state_out.
int run_branches(Handle* h, int mode, const double* state_in, int steps, const double* dt, double* state_out) {
  Adj& A = h->A;
  int rc;
  if (mode == 1) {
    const size_t need = (size_t)std::max(steps, 1) * h->BW;
    if (need > h->br_cap) {
      cudaFree(h->br);
      h->br = nullptr;
      h->br_cap = 0;
      CK(cudaMalloc(&h->br, need * sizeof(unsigned int)));
      h->br_cap = need;
    }
    h->br_steps = 0;
  } else if (steps > h->br_steps) {
    return MHD_ERR_STATE;
  }
  if (h->nsets < 1 && (rc = alloc_sets(h, 1))) return rc;
  h->tail_resident = false;   // arena 0 is reused: a pending tail is recomputed from its checkpoint
  select_set(h, 0);
  if ((rc = unpack(h, state_in, A.P, A.C, A.FX, A.FY, false))) return rc;
  if (steps == 0) {
    if ((rc = pack(h, state_out, A.P, A.C, A.FX, A.FY, false))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return MHD_OK;
  }
  for (int c = 0; c < steps; ++c) {
    if (!std::isfinite(dt[c])) return MHD_ERR_ARG;
    for (int i = 0; i < kNumBt; ++i) A.bt[i] = h->br + (size_t)c * h->BW + h->btoff[i];
    A.dt = dt[c];
    rc = mode == 1 ? fwd_cycle_b<1>(h) : fwd_cycle_b<2>(h);
    if (rc) return rc;
    if (c + 1 < steps && (rc = output_to_input(h, 0, 0))) return rc;
  }
  if ((rc = pack(h, state_out, A.NP, A.NC, A.NFX, A.NFY, false))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  if (mode == 1) h->br_steps = steps;
  return MHD_OK;
}

// Arena layout of one cycle for an nx x ny grid: value/adjoint arena offsets and
// plane strides (W words), and the tape arena offsets (TW words).
void layout(int nx, int ny, int recon, int efix, size_t* off, size_t* ps, size_t* W, size_t* toff, size_t* TW) {
  const size_t plane[6] = {(size_t)nx * ny, (size_t)(nx + 1) * ny, (size_t)nx * (ny + 1),
                           (size_t)(nx + 1) * (ny + 1), (size_t)(nx + 2) * ny, (size_t)nx * (ny + 2)};
  size_t w = 0;
  for (int i = 0; i < kNumSlots; ++i) {
    off[i] = w;
    ps[i] = plane[kSlots[i].kind];
    // the slope arrays (sweep-extended cells) and the interface values exist only for PPM
    const bool ppm_only = kSlots[i].kind == 4 || kSlots[i].kind == 5 || kSlots[i].arr == &Adj::E0X ||
                          kSlots[i].arr == &Adj::E0Y;
    w += (size_t)(ppm_only && recon != 2 ? 0 : kSlots[i].planes) * ps[i];
    w = (w + 31) & ~(size_t)31;   // 256-byte aligned plane groups
  }
  *W = w;
  // tapes: PLM / PPM interface values per cell and sweep (first order has no reconstruction stage), Roe per
  // face, stage and sweep, CTU per face side and sweep, PLM/PPM slopes per extended cell and sweep
  const int nt_plm = recon == 1 ? g_plm0_NT : (recon == 2 ? g_ppmi0_NT : 0);
  const int nt_trace = recon == 2 ? g_ppmt0_NT : 0;
  const int nt_slope = recon == 2 ? g_pslope0_NT : 0;
  const int nt_roe[2] = {efix ? g_roe1_0_efix_NT : g_roe1_0_NT, efix ? g_roe2_0_efix_NT : g_roe2_0_NT};
  const size_t items[12] = {plane[0], plane[0], plane[1], plane[2], plane[1], plane[2], 2 * plane[1], 2 * plane[2],
                            plane[4], plane[5], plane[0], plane[0]};
  const int words[12] = {nt_plm, nt_plm, nt_roe[0], nt_roe[0], nt_roe[1], nt_roe[1], g_ctu0_NT, g_ctu0_NT,
                         nt_slope, nt_slope, nt_trace, nt_trace};
  size_t tw = 0;
  for (int i = 0; i < 12; ++i) {
    toff[i] = tw;
    tw += items[i] * (size_t)words[i];
    tw = (tw + 31) & ~(size_t)31;
  }
  *TW = tw;
}

// Size the record of a run of `steps` cycles: the checkpoint interval, the
// checkpoint store (owned, or borrowed from the caller), and the backward mode --
// all `every` cycles of a segment resident when they fit the budget, else one
// cycle's arrays plus the segment's states.  In stored mode with `allow_tail`, the
// last segment is a tail of as many cycles as the budget holds (at most tail_max).
int prepare_record(Handle* h, int steps, int& every, bool own_ckpt, bool allow_tail) {
  if (every <= 0) every = (int)std::ceil(std::sqrt((double)steps));
  every = std::min(every, steps);
  h->steps = 0;
  h->tail = 0;
  h->tail_resident = false;
  if (h->ckpt_owned) cudaFree(h->ckpt);
  cudaFree(h->seg);
  h->ckpt = h->seg = nullptr;
  h->ckpt_bytes = h->seg_bytes = 0;
  h->ckpt_owned = own_ckpt;
  if (own_ckpt) {
    // one state per segment: at most ceil(steps / every) + 1 with a tail
    const int nck = (steps + every - 1) / every + (allow_tail ? 1 : 0);
    CK(cudaMalloc(&h->ckpt, (size_t)nck * h->state_words * sizeof(double)));
    h->ckpt_bytes = (size_t)nck * h->state_words * sizeof(double);
  }
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  // (arenas this handle already holds count as free)
  const size_t set_bytes = (h->W + h->TW) * sizeof(double);
  const size_t held_all = (h->vals_cap + h->tapes_cap) * sizeof(double);
  const size_t held = held_all > set_bytes ? held_all - set_bytes : 0;
  const size_t budget = h->budget ? h->budget : (size_t)(0.85 * (double)(free_b + held));
  const size_t extra = ((size_t)every - 1) * set_bytes;
  h->stored = every > 1 && extra <= budget;
  int tail = 0;
  if (allow_tail && h->stored && h->tail_max != 0) {
    const size_t fit = 1 + budget / set_bytes;
    tail = (int)std::min<size_t>(fit, (size_t)steps);
    if (h->tail_max > 0) tail = std::min(tail, h->tail_max);
    if (tail < every) tail = 0;   // no longer than a plain segment: keep the uniform record
  }
  int rc;
  if (h->stored) {
    const int sets = std::max(every, tail);
    if (h->nsets < sets && (rc = alloc_sets(h, sets))) return rc;
  } else {
    if ((rc = alloc_sets(h, 1))) return rc;
    CK(cudaMalloc(&h->seg, (size_t)every * h->state_words * sizeof(double)));
    h->seg_bytes = (size_t)every * h->state_words * sizeof(double);
  }
  h->every = every;
  h->tail = tail;
  h->steps = steps;   // the segment helpers read it; callers reset it if the record fails
  return MHD_OK;
}

// Run the tail segment from the state in value arena 0's inputs: per cycle the CFL
// dt (the production step's arithmetic, bit for bit), then the taped forward sweep
// into arena k, whose outputs become arena k+1's inputs.  The arrays and tapes stay
// resident for the backward pass.
int run_tail(Handle* h, int c0, double cfl, const double* fixed_dt) {
  Adj& A = h->A;
  int rc;
  for (int k = 0; k < h->tail; ++k) {
    select_set(h, k);
    double dt = 0.0;
    if (fixed_dt) dt = fixed_dt[c0 + k];
    else if ((rc = cfl_dt(h, cfl, &dt))) return rc;
    if (!std::isfinite(dt)) return MHD_ERR_NONFINITE;
    h->dts[c0 + k] = dt;
    A.dt = dt;
    if ((rc = fwd_cycle(h, true))) return rc;
    if (k + 1 < h->tail && (rc = output_to_input(h, k, k + 1))) return rc;
  }
  h->tail_resident = true;
  return MHD_OK;
}

// Forward pass with the CFL dt on the production exact-arithmetic step (the same
// arithmetic as the stage kernels, bit for bit, and faster): one advance call per
// segment, each cycle's dt logged on the device; then the tail, if any, on the
// taped stage kernels.
int forward_on_solver(Handle* h, const double* state_in, int steps, double cfl, double* state_out) {
  Adj& A = h->A;
  const size_t cp = (size_t)A.nx * A.ny, xp = (size_t)(A.nx + 1) * A.ny;
  if (!h->solver) {
    int rc = mhd2d_create(A.ny, A.nx, A.dx, A.dy, A.bcx, A.bcy, A.gamma, MHD2D_MHD, A.recon, A.efix, A.eps,
                          A.min_d, A.min_p, A.min_e, MHD2D_ARITH_EXACT, &h->solver);
    if (rc) return rc;
  }
  if (h->dtlog_cap < (size_t)steps) {
    cudaFree(h->dtlog);
    h->dtlog = nullptr;
    h->dtlog_cap = 0;
    CK(cudaMalloc(&h->dtlog, (size_t)steps * sizeof(double)));
    h->dtlog_cap = steps;
  }
  int rc = mhd2d_set_dt_log(h->solver, h->dtlog, (long long)h->dtlog_cap);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  rc = mhd2d_upload_device(h->solver, state_in, state_in + 8 * cp, state_in + 16 * cp, state_in + 16 * cp + xp);
  if (rc) return rc;
  auto save = [&](double* dst) -> int {
    double *p = nullptr, *c = nullptr, *bx = nullptr, *by = nullptr;
    int r = mhd2d_state_ptrs(h->solver, 0, &p, &c, &bx, &by);
    if (r) return r;
    Arr P, C, FX, FY;
    P.v = p; C.v = c; FX.v = bx; FY.v = by;
    return pack(h, dst, P, C, FX, FY, false);
  };
  const int nh = head_segments(h);
  const int head = steps - h->tail;
  for (int s = 0; s < nh; ++s) {
    int c0 = 0, len = 0;
    segment(h, s, &c0, &len);
    if ((rc = save(h->ckpt + (size_t)s * h->state_words))) return rc;
    // the copy above is on this handle's stream; the solver runs on its own
    CK(cudaStreamSynchronize(h->stream));
    double t = 0.0;
    long long cyc = 0;
    if ((rc = mhd2d_advance(h->solver, 0.0, 1e300, c0, c0 + len, cfl, &t, &cyc, nullptr))) return rc;
    if (cyc != c0 + len || !std::isfinite(t)) return MHD_ERR_NONFINITE;
  }
  if (head > 0) {
    CK(cudaMemcpy(h->dts.data(), h->dtlog, (size_t)head * sizeof(double), cudaMemcpyDeviceToHost));
    for (int c = 0; c < head; ++c)
      if (!std::isfinite(h->dts[c])) return MHD_ERR_NONFINITE;
  }
  if (h->tail > 0) {
    double* ck = h->ckpt + (size_t)nh * h->state_words;
    if ((rc = save(ck))) return rc;
    select_set(h, 0);
    if ((rc = unpack(h, ck, A.P, A.C, A.FX, A.FY, false))) return rc;
    if ((rc = run_tail(h, head, cfl, nullptr))) return rc;
    select_set(h, h->tail - 1);
    rc = pack(h, state_out, A.NP, A.NC, A.NFX, A.NFY, false);
    select_set(h, 0);
    return rc;
  }
  return save(state_out);
}

int forward_record(Handle* h, Adj& A, const double* state_in, int steps, double cfl, const double* fixed_dt,
                   double* state_out);

}  // namespace

extern "C" {

int mhd2d_adj_create(int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma, int recon,
                     int entropy_fix, double eps, double min_d, double min_p, double min_e, void** handle) {
  if (!handle) return MHD_ERR_ARG;
  *handle = nullptr;
  if (nx < 2 || ny < 2 || !(dx > 0.0) || !(dy > 0.0) || recon < 0 || recon > 2) return MHD_ERR_ARG;
  if ((bcx != 0 && bcx != 1) || (bcy != 0 && bcy != 1)) return MHD_ERR_ARG;
  Handle* h = new (std::nothrow) Handle();
  if (!h) return MHD_ERR_NOMEM;
  Adj& A = h->A;
  A.nx = nx; A.ny = ny; A.dx = dx; A.dy = dy; A.bcx = bcx; A.bcy = bcy; A.recon = recon;
  A.efix = entropy_fix ? 1 : 0; A.gamma = gamma; A.eps = eps; A.min_d = min_d; A.min_p = min_p; A.min_e = min_e;
  layout(nx, ny, recon, A.efix, h->off, h->ps, &h->W, h->toff, &h->TW);
  branch_layout(nx, ny, recon, A.efix, h->btoff, &h->BW);
  h->state_words = state_words(A);
  int rc = MHD_OK;
  cudaError_t e = cudaMalloc(&h->bars, h->W * sizeof(double));
  h->bars_cap = e == cudaSuccess ? h->W : 0;
  if (e == cudaSuccess) e = cudaMalloc(&h->red, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->red, 0, 4 * sizeof(double), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) rc = fail(e);
  if (rc == MHD_OK) rc = alloc_sets(h, 1);
  A.red = h->red;
  if (rc != MHD_OK) {
    cudaFree(h->bars);
    cudaFree(h->red);
    cudaFree(h->vals);
    cudaFree(h->tapes);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream2) cudaStreamDestroy(h->stream2);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return rc;
  }
  *handle = h;
  return MHD_OK;
}

void mhd2d_adj_destroy(void* handle) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->bars);
  cudaFree(h->vals);
  cudaFree(h->tapes);
  cudaFree(h->red);
  cudaFree(h->dtlog);
  if (h->ckpt_owned) cudaFree(h->ckpt);
  cudaFree(h->seg);
  cudaFree(h->br);
  if (h->solver) mhd2d_destroy(h->solver);
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int mhd2d_adj_reshape(void* handle, int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || nx < 2 || ny < 2 || !(dx > 0.0) || !(dy > 0.0)) return MHD_ERR_ARG;
  if ((bcx != 0 && bcx != 1) || (bcy != 0 && bcy != 1)) return MHD_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  Adj& A = h->A;
  A.nx = nx; A.ny = ny; A.dx = dx; A.dy = dy; A.bcx = bcx; A.bcy = bcy; A.gamma = gamma;
  layout(nx, ny, A.recon, A.efix, h->off, h->ps, &h->W, h->toff, &h->TW);
  branch_layout(nx, ny, A.recon, A.efix, h->btoff, &h->BW);
  h->br_steps = 0;
  h->state_words = state_words(A);
  if (h->W > h->bars_cap) {
    cudaFree(h->bars);
    h->bars = nullptr;
    h->bars_cap = 0;
    CK(cudaMalloc(&h->bars, h->W * sizeof(double)));
    h->bars_cap = h->W;
  }
  // the record, the segment states and the production solver belong to the old grid
  h->steps = 0;
  h->tail = 0;
  h->tail_resident = false;
  if (h->ckpt_owned) cudaFree(h->ckpt);
  cudaFree(h->seg);
  h->ckpt = h->seg = nullptr;
  h->ckpt_bytes = h->seg_bytes = 0;
  h->ckpt_owned = true;
  if (h->solver) {
    mhd2d_destroy(h->solver);
    h->solver = nullptr;
  }
  h->nsets = 0;
  return alloc_sets(h, 1);
}

int mhd2d_adj_cycle_bytes(int ny, int nx, int recon, int entropy_fix, size_t* bytes) {
  if (!bytes || nx < 2 || ny < 2 || recon < 0 || recon > 2) return MHD_ERR_ARG;
  size_t off[kNumSlots], ps[kNumSlots], toff[12], W = 0, TW = 0;
  layout(nx, ny, recon, entropy_fix ? 1 : 0, off, ps, &W, toff, &TW);
  *bytes = (W + TW) * sizeof(double);
  return MHD_OK;
}

int mhd2d_adj_configure(void* handle, size_t segment_bytes) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  h->budget = segment_bytes;
  return MHD_OK;
}

int mhd2d_adj_cycle(void* handle, double dt, const double* state_in, double* state_out) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !state_in || !state_out) return MHD_ERR_ARG;
  Adj& A = h->A;
  h->tail_resident = false;   // arena 0 is overwritten
  select_set(h, 0);
  A.dt = dt;
  int rc = unpack(h, state_in, A.P, A.C, A.FX, A.FY, false);
  if (rc) return rc;
  if ((rc = fwd_cycle(h, false))) return rc;
  if ((rc = pack(h, state_out, A.NP, A.NC, A.NFX, A.NFY, false))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd2d_adj_cycle_reverse(void* handle, double dt, const double* state_in, const double* bar_out,
                            double* bar_in) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !state_in || !bar_out || !bar_in) return MHD_ERR_ARG;
  Adj& A = h->A;
  h->tail_resident = false;   // arena 0 is overwritten
  select_set(h, 0);
  A.dt = dt;
  int rc = unpack(h, state_in, A.P, A.C, A.FX, A.FY, false);
  if (rc) return rc;
  if ((rc = fwd_cycle(h, true))) return rc;
  if ((rc = unpack(h, bar_out, A.NP, A.NC, A.NFX, A.NFY, true))) return rc;
  if ((rc = rev_cycle(h))) return rc;
  if ((rc = pack(h, bar_in, A.P, A.C, A.FX, A.FY, true))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd2d_adj_forward(void* handle, const double* state_in, int steps, double cfl, const double* fixed_dt,
                      int every, double* state_out, double* dt_log) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !state_in || !state_out || steps < 1) return MHD_ERR_ARG;
  Adj& A = h->A;
  int rc = prepare_record(h, steps, every, true, true);
  if (rc) {
    h->steps = 0;
    return rc;
  }
  h->dts.assign(steps, 0.0);
  rc = forward_record(h, A, state_in, steps, cfl, fixed_dt, state_out);
  if (rc) {
    h->steps = 0;
    h->tail_resident = false;
    return rc;
  }
  if (dt_log) std::copy(h->dts.begin(), h->dts.end(), dt_log);
  return MHD_OK;
}

}  // extern "C"

namespace {
// the body of mhd2d_adj_forward once the record is sized
int forward_record(Handle* h, Adj& A, const double* state_in, int steps, double cfl, const double* fixed_dt,
                   double* state_out) {
  int rc;
  if (!fixed_dt) {
    if ((rc = forward_on_solver(h, state_in, steps, cfl, state_out))) return rc;
  } else {
    select_set(h, 0);
    if ((rc = unpack(h, state_in, A.P, A.C, A.FX, A.FY, false))) return rc;
    const int nh = head_segments(h);
    for (int s = 0; s < nh; ++s) {
      int c0 = 0, len = 0;
      segment(h, s, &c0, &len);
      if ((rc = pack(h, h->ckpt + (size_t)s * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
      for (int c = c0; c < c0 + len; ++c) {
        const double dt = fixed_dt[c];
        if (!std::isfinite(dt)) return MHD_ERR_NONFINITE;
        h->dts[c] = dt;
        A.dt = dt;
        if ((rc = fwd_cycle(h, false))) return rc;
        if ((rc = output_to_input(h, 0, 0))) return rc;
      }
    }
    if (h->tail > 0) {
      if ((rc = pack(h, h->ckpt + (size_t)nh * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
      if ((rc = run_tail(h, steps - h->tail, cfl, fixed_dt))) return rc;
      select_set(h, h->tail - 1);
      if ((rc = pack(h, state_out, A.NP, A.NC, A.NFX, A.NFY, false))) return rc;
      select_set(h, 0);
    } else if ((rc = pack(h, state_out, A.P, A.C, A.FX, A.FY, false))) {
      return rc;
    }
  }
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}
}  // namespace

extern "C" {

int mhd2d_adj_restore(void* handle, const double* checkpoints, int steps, int every, const double* dt) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !checkpoints || !dt || steps < 1 || every < 1) return MHD_ERR_ARG;
  int rc = prepare_record(h, steps, every, false, false);
  if (rc) {
    h->steps = 0;
    return rc;
  }
  h->ckpt = const_cast<double*>(checkpoints);
  h->dts.assign(dt, dt + steps);
  for (int c = 0; c < steps; ++c)
    if (!std::isfinite(h->dts[c])) {
      h->steps = 0;
      return MHD_ERR_NONFINITE;
    }
  return MHD_OK;
}

int mhd2d_adj_backward(void* handle, const double* bar_final, double* bar_initial) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !bar_final || !bar_initial) return MHD_ERR_ARG;
  if (!h->ckpt || h->steps < 1) return MHD_ERR_STATE;
  Adj& A = h->A;
  const int nseg = num_segments(h);
  select_set(h, 0);
  int rc = unpack(h, bar_final, A.NP, A.NC, A.NFX, A.NFY, true);
  if (rc) return rc;
  for (int s = nseg - 1; s >= 0; --s) {
    int c0 = 0, len = 0;
    segment(h, s, &c0, &len);
    const bool resident = h->tail > 0 && s == nseg - 1 && h->tail_resident;
    if (h->stored) {
      // recompute the segment once, keeping every cycle's arrays, then sweep back
      // (the tail left resident by the forward pass needs no recomputation)
      if (!resident) {
        select_set(h, 0);
        if ((rc = unpack(h, h->ckpt + (size_t)s * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
        for (int k = 0; k < len; ++k) {
          select_set(h, k);
          A.dt = h->dts[c0 + k];
          if ((rc = fwd_cycle(h, true))) return rc;
          if (k + 1 < len && (rc = output_to_input(h, k, k + 1))) return rc;
        }
      }
      h->tail_resident = false;   // the arenas now hold this segment
      for (int k = len - 1; k >= 0; --k) {
        select_set(h, k);
        A.dt = h->dts[c0 + k];
        if ((rc = rev_cycle(h))) return rc;
        if ((rc = bars_in_to_out(h))) return rc;
      }
    } else {
      // recompute the segment's states, then each cycle again before its reverse sweep
      select_set(h, 0);
      if ((rc = unpack(h, h->ckpt + (size_t)s * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
      for (int k = 0; k < len; ++k) {
        if ((rc = pack(h, h->seg + (size_t)k * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
        if (k + 1 < len) {
          A.dt = h->dts[c0 + k];
          if ((rc = fwd_cycle(h, false))) return rc;
          if ((rc = output_to_input(h, 0, 0))) return rc;
        }
      }
      for (int k = len - 1; k >= 0; --k) {
        A.dt = h->dts[c0 + k];
        if ((rc = unpack(h, h->seg + (size_t)k * h->state_words, A.P, A.C, A.FX, A.FY, false))) return rc;
        if ((rc = fwd_cycle(h, true))) return rc;
        if ((rc = rev_cycle(h))) return rc;
        if ((rc = bars_in_to_out(h))) return rc;
      }
    }
  }
  select_set(h, 0);
  if ((rc = pack(h, bar_initial, A.NP, A.NC, A.NFX, A.NFY, true))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd2d_adj_branches(void* handle, int mode, const double* state_in, int steps, const double* dt,
                       double* state_out) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || (mode != 1 && mode != 2) || steps < 0 || !state_in || !state_out || (steps > 0 && !dt)) return MHD_ERR_ARG;
  return run_branches(h, mode, state_in, steps, dt, state_out);
}

int mhd2d_adj_set_tail(void* handle, int max_cycles) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || max_cycles < -1) return MHD_ERR_ARG;
  h->tail_max = max_cycles;
  return MHD_OK;
}

int mhd2d_adj_record(void* handle, int* steps, int* every, int* tail) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (steps) *steps = h->steps;
  if (every) *every = h->every;
  if (tail) *tail = h->tail;
  return MHD_OK;
}

int mhd2d_adj_info(void* handle, size_t* state_words_out, size_t* device_bytes_out, int* segment_sets) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (state_words_out) *state_words_out = h->state_words;
  if (device_bytes_out) {
    size_t solver_bytes = 0;
    if (h->solver) mhd2d_device_bytes(h->solver, &solver_bytes);
    *device_bytes_out = device_bytes(h) + solver_bytes;
  }
  if (segment_sets) *segment_sets = h->stored ? h->every : 1;
  return MHD_OK;
}

int mhd2d_adj_quotient(const double* b, const double* v, double* q, long long n) {
  if (n < 0 || (n > 0 && (!b || !v || !q))) return MHD_ERR_ARG;
  if (n == 0) return MHD_OK;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  k_quotient<<<(unsigned)blocks, 256>>>(b, v, q, n);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return MHD_OK;
}

}  // extern "C"
