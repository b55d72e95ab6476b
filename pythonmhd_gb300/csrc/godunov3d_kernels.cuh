// Kernels of one 3D CTU cycle of hydrodynamics (Source/EvolveFunctions_Hydro.py:607-792).
// Included, after godunov2d_kernels.cuh with MHD_BODIES_ONLY defined, by two
// translation units that define MHD_NS: `exact` (-fmad=false, the reference's
// NumPy arithmetic bit for bit) and `fast` (FMA contraction allowed).
//
// A cycle:
//   dt_reduce -> begin -> for x, y, z: [slopes] -> faces
//   -> roe(x, y, z) -> ctu(x, y, z) -> roe(x, y, z) -> final -> end
// The sweeps reuse the 2D sweep policies (HydroSweep<0/1/2>), the limited-slope and
// edge-state math and the Roe flux; only the indexing is 3D.  Work items are linear
// indices of the [y][x][z] arrays, so consecutive threads touch consecutive z and
// every sweep's loads coalesce.  Every kernel returns at once when the loop state
// says the cycle is not a real one, as in 2D.
#pragma once
#include "godunov3d_types.h"

namespace mhdk {
namespace MHD_NS {

// linear index of cell / face / extended-cell coordinates c[3] (c[0] x, c[1] y, c[2] z)
// in an array whose extent along DIR is ADD cells larger
template <int DIR, int ADD>
__device__ __forceinline__ size_t lin3(const Grid3& G, const int* c) {
  return ((size_t)c[1] * (size_t)ext_n(G, 0, DIR, ADD) + (size_t)c[0]) * (size_t)ext_n(G, 2, DIR, ADD) + (size_t)c[2];
}
template <int DIR, int ADD>
__device__ __forceinline__ void unlin3(const Grid3& G, unsigned i, int* c) {
  const unsigned nz = (unsigned)ext_n(G, 2, DIR, ADD), nx = (unsigned)ext_n(G, 0, DIR, ADD);
  c[2] = (int)(i % nz);
  const unsigned r = i / nz;
  c[0] = (int)(r % nx);
  c[1] = (int)(r / nx);
}
// stride of direction A in an array whose extent along DIR is ADD cells larger
template <int DIR, int ADD, int A>
__device__ __forceinline__ size_t stride3(const Grid3& G) {
  return A == 2 ? (size_t)1
       : A == 0 ? (size_t)ext_n(G, 2, DIR, ADD)
                : (size_t)ext_n(G, 0, DIR, ADD) * (size_t)ext_n(G, 2, DIR, ADD);
}

__device__ __forceinline__ unsigned item3() { return blockIdx.x * blockDim.x + threadIdx.x; }

// The sweep's cells around c along D (wrapped or clamped by the boundary condition).
template <class S, int D>
struct Line3 {
  size_t base, cs, plane;
  int L, bc;
  __device__ Line3(const Grid3& G, const int* c, int bc_line = -1) {
    int c0[3] = {c[0], c[1], c[2]};
    c0[D] = 0;
    base = lin3<D, 0>(G, c0);
    cs = stride3<D, 0, D>(G);
    plane = cells3(G);
    L = G.n[D];
    bc = bc_line >= 0 ? bc_line : G.bc[D];
  }
  __device__ void load(const double* prim, int cell, double* w) const {
    const size_t idx = base + (size_t)wrapc(cell, L, bc) * cs;
#pragma unroll
    for (int k = 0; k < S::NV; ++k) w[k] = __ldg(prim + S::src(k) * plane + idx);
  }
  // one plane's value at cell `cell` of the line
  __device__ double at(const double* a, int slot, int cell) const {
    return __ldg(a + (size_t)slot * plane + base + (size_t)wrapc(cell, L, bc) * cs);
  }
};

// ----------------------------------------------------------------------------
// Reconstruction: limited slopes over the cells -1..L of direction D, then the
// edge states and face writes of every cell (the 2D bodies' math).
// ----------------------------------------------------------------------------
template <class S, int D>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k3_slopes(Grid3 G, StateBuf3 in) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  if (i >= plane3(G, D, 2)) return;
  int c[3];
  unlin3<D, 2>(G, i, c);
  const int cc = c[D] - 1;
  const Line3<S, D> ln(G, c);
  constexpr int NV = S::NV;
  double wl[NV], wc[NV], wr[NV];
  ln.load(in.prim, cc - 1, wl);
  ln.load(in.prim, cc, wc);
  ln.load(in.prim, cc + 1, wr);
  double bn = 0.0;
  if (S::BN >= 0) bn = ln.at(in.prim, S::BN >= 0 ? S::BN : 0, cc);
  typename S::Eig e;
  S::eig(wc, bn, G.gamma, e);
  double ps[NV];
  limited_slopes<S>(wl, wc, wr, e, ps);
  const size_t es = G.ext_plane;
#pragma unroll
  for (int k = 0; k < NV; ++k) G.slopes[k * es + i] = ps[k];
  S::store(e, G.eig + i, es);
}

template <class S, int D, int MODE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k3_faces(Grid3 G, StateBuf3 in) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  if (i >= cells3(G)) return;
  int c[3];
  unlin3<D, 0>(G, i, c);
  const int cc = c[D];
  const Line3<S, D> ln(G, c);
  constexpr int NV = S::NV;
  double lia[NV], ria[NV], wc[NV], wl[NV], wr[NV];
  ln.load(in.prim, cc, wc);
  if (MODE != 0) {
    ln.load(in.prim, cc - 1, wl);
    ln.load(in.prim, cc + 1, wr);
  }
  {
    int ce[3] = {c[0], c[1], c[2]};
    ce[D] = cc + 1;
    const size_t xe = lin3<D, 2>(G, ce);
    const ptrdiff_t step = (ptrdiff_t)stride3<D, 2, D>(G);
    const size_t es = G.ext_plane;
    const double* sl = G.slopes;
    const double* eg = G.eig;
    edge_states<S, MODE>(
        wl, wc, wr, [&](int k, int d) { return sl[k * es + xe + (ptrdiff_t)d * step]; },
        [&](typename S::Eig& e) { S::load(e, eg + xe, es); }, G.loop->dt, G.d[D], lia, ria);
  }
  // cell cc gives the plus-side state of face cc and the minus-side state of face
  // cc+1; the boundary cells also fill face 0 / face L (the reference's padding,
  // Source/Reconstruction_PPM_Hydro_HelperModule.py:1207-1226, EvolveFunctions_Hydro.py:622-664)
  const size_t fp = plane3(G, D, 1);
  const int L = G.n[D];
  auto fidx = [&](int f) {
    int cf[3] = {c[0], c[1], c[2]};
    cf[D] = f;
    return lin3<D, 1>(G, cf);
  };
  put_face<S>(G.wr[D], fp, fidx(cc), lia, G.min_d, G.min_p, 0.0, false);
  put_face<S>(G.wl[D], fp, fidx(cc + 1), ria, G.min_d, G.min_p, 0.0, false);
  if (cc == 0) {
    if (G.bc[D] == OUTFLOW) put_face<S>(G.wl[D], fp, fidx(0), lia, G.min_d, G.min_p, 0.0, false);
    else put_face<S>(G.wr[D], fp, fidx(L), lia, G.min_d, G.min_p, 0.0, false);
  }
  if (cc == L - 1) {
    if (G.bc[D] == OUTFLOW) put_face<S>(G.wr[D], fp, fidx(L), ria, G.min_d, G.min_p, 0.0, false);
    else put_face<S>(G.wl[D], fp, fidx(0), ria, G.min_d, G.min_p, 0.0, false);
  }
}

// ----------------------------------------------------------------------------
// Roe fluxes at every face of direction D from the face prim states
// (Source/RiemannSolvers_Hydro_Roe_HelperModule.py:68-869).
// ----------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k3_roe_hydro(Grid3 G) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t fp = plane3(G, D, 1);
  if (i >= fp) return;
  double wl[5], wr[5], flux[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    wl[k] = G.wl[D][k * fp + i];
    wr[k] = G.wr[D][k * fp + i];
  }
  hroe_flux<D>(wl, wr, G.gamma, G.efix != 0, G.eps, flux);
#pragma unroll
  for (int k = 0; k < 5; ++k) G.f[D][k * fp + i] = flux[k];
}

// ----------------------------------------------------------------------------
// CTU predictor (Source/EvolveFunctions_Hydro.py:694-756): each face state of
// direction D, in conserved form, takes half-dt flux differences of the two other
// directions' stage-1 fluxes at its cell, in ascending direction order; then back
// to primitives for the stage-2 solve.
// ----------------------------------------------------------------------------
template <int D, int E>
__device__ __forceinline__ void ctu3_take(const Grid3& G, const int* cell, double half, double* u) {
  const size_t lo = lin3<E, 1>(G, cell);
  const size_t hi = lo + stride3<E, 1, E>(G);
  const size_t fp = plane3(G, E, 1);
  const double* F = G.f[E];
#pragma unroll
  for (int k = 0; k < 5; ++k) u[k] = u[k] - half * (F[k * fp + hi] - F[k * fp + lo]);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k3_ctu_hydro(Grid3 G) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t fp = plane3(G, D, 1);
  if (i >= fp) return;
  int c[3];
  unlin3<D, 1>(G, i, c);
  const int f = c[D];
  const double dt = G.loop->dt;
  constexpr int E1 = D == 0 ? 1 : 0;
  constexpr int E2 = D == 2 ? 1 : 2;
  const double h1 = 0.5 * ddiv(dt, G.d[E1]);
  const double h2 = 0.5 * ddiv(dt, G.d[E2]);
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double* W = side == 0 ? G.wl[D] : G.wr[D];
    double w[5], u[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) w[k] = W[k * fp + i];
    hprim_to_cons<D>(w, G.gamma, u);
    int cell[3] = {c[0], c[1], c[2]};
    cell[D] = wrapc(f - 1 + side, G.n[D], G.bc[D]);
    ctu3_take<D, E1>(G, cell, h1, u);
    ctu3_take<D, E2>(G, cell, h2, u);
    hcons_to_prim<D>(u, G.gamma, w);
#pragma unroll
    for (int k = 0; k < 5; ++k) W[k * fp + i] = w[k];
  }
}

// ----------------------------------------------------------------------------
// Conservative update with the stage-2 fluxes, x then y then z, and back to
// primitives (Source/EvolveFunctions_Hydro.py:776-784).
// ----------------------------------------------------------------------------
template <int E>
__device__ __forceinline__ double final3_take(const Grid3& G, const int* c, int k, double dtde, double v) {
  const size_t lo = lin3<E, 1>(G, c);
  const size_t hi = lo + stride3<E, 1, E>(G);
  const size_t fp = plane3(G, E, 1);
  return v - dtde * (G.f[E][k * fp + hi] - G.f[E][k * fp + lo]);
}

__global__ void __launch_bounds__(kBlock) k3_final_hydro(Grid3 G, StateBuf3 in, StateBuf3 out) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t plane = cells3(G);
  if (i >= plane) return;
  int c[3];
  unlin3<0, 0>(G, i, c);
  const double dt = G.loop->dt;
  const double dtdx = ddiv(dt, G.d[0]), dtdy = ddiv(dt, G.d[1]), dtdz = ddiv(dt, G.d[2]);
  double u[5], w[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double v = __ldg(in.cons + k * plane + i);
    v = final3_take<0>(G, c, k, dtdx, v);
    v = final3_take<1>(G, c, k, dtdy, v);
    v = final3_take<2>(G, c, k, dtdz, v);
    u[k] = v;
  }
  hcons_to_prim<0>(u, G.gamma, w);
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    out.prim[k * plane + i] = w[k];
    out.cons[k * plane + i] = u[k];
  }
}

// ----------------------------------------------------------------------------
// CFL timestep (Source/TimestepCalculations_HelperModule.py:121-181): the largest
// |v_d| + c per direction over the cells, then dt = min(dt_x, min(dt_y, dt_z)).
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3_dt_reduce_hydro(Grid3 G, StateBuf3 in) {
  if (!loop_running(G.loop)) return;
  const size_t n = cells3(G);
  const double gamma = G.gamma;
  const double* c = in.cons;
  double m[3] = {0.0, 0.0, 0.0};
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const double inv_d = ddiv(1.0, c[idx]);
    const double vx = c[n + idx] * inv_d;
    const double vy = c[2 * n + idx] * inv_d;
    const double vz = c[3 * n + idx] * inv_d;
    const double vsq = vx * vx + vy * vy + vz * vz;
    const double p = dmax((gamma - 1.0) * (c[4 * n + idx] - 0.5 * c[idx] * vsq), SMALL_VALUE);
    const double a = sqrt(gamma * p * inv_d);
    m[0] = dmax(m[0], fabs(vx) + a);
    m[1] = dmax(m[1], fabs(vy) + a);
    m[2] = dmax(m[2], fabs(vz) + a);
  }
  __shared__ double sm[3][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    m[a] = warp_max(m[a]);
    if (lane == 0) sm[a][wid] = m[a];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    unsigned long long* dst[3] = {&G.loop->max_sx, &G.loop->max_sy, &G.loop->max_sz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double v = lane < nw ? sm[a][lane] : 0.0;
      v = warp_max(v);
      if (lane == 0) atomicMax(dst[a], (unsigned long long)__double_as_longlong(v));
    }
  }
}

__global__ void k3_begin_hydro(Grid3 G) {
  LoopState* L = G.loop;
  const int act = loop_running(L) ? 1 : 0;
  L->active = act;
  if (act) {
    const double mx = __longlong_as_double((long long)L->max_sx);
    const double my = __longlong_as_double((long long)L->max_sy);
    const double mz = __longlong_as_double((long long)L->max_sz);
    const double dtx = ddiv(L->cfl, ddiv(mx, G.d[0]));
    const double dty = ddiv(L->cfl, ddiv(my, G.d[1]));
    const double dtz = ddiv(L->cfl, ddiv(mz, G.d[2]));
    double dt = dmin(dtx, dmin(dty, dtz));
    if (L->t + dt > L->t_end) dt = L->t_end - L->t;
    L->dt = dt;
  }
  L->max_sx = 0ull;
  L->max_sy = 0ull;
  L->max_sz = 0ull;
}

__global__ void k3_end(Grid3 G) {
  LoopState* L = G.loop;
  if (!L->active) return;
  L->t_prev = L->t;
  L->t = L->t + L->dt;
  L->cycle = L->cycle + 1;
  L->cycles_run = L->cycles_run + 1;
  L->cur ^= 1;
  L->active = 0;
}

// ----------------------------------------------------------------------------
// Host-side enqueue of one 3D cycle reading state buffer `parity`.
// ----------------------------------------------------------------------------
inline unsigned grid3(size_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

template <int D>
void enqueue_recon3(const Grid3& g, const StateBuf3& in, cudaStream_t s) {
  using S = HydroSweep<D>;
  if (g.recon >= 1) k3_slopes<S, D><<<grid3(plane3(g, D, 2)), kBlock, 0, s>>>(g, in);
  if (g.recon == 2) k3_faces<S, D, 2><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  else if (g.recon == 1) k3_faces<S, D, 1><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  else k3_faces<S, D, 0><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
}

void enqueue_cycle3_mhd(const Grid3& g, int parity, int dt_blocks, cudaStream_t s);

void enqueue_cycle3(const Grid3& g, int parity, int dt_blocks, cudaStream_t s) {
  if (g.physics == MHD) {
    enqueue_cycle3_mhd(g, parity, dt_blocks, s);
    return;
  }
  const StateBuf3 in = g.st[parity];
  const StateBuf3 out = g.st[parity ^ 1];
  k3_dt_reduce_hydro<<<dt_blocks, 256, 0, s>>>(g, in);
  k3_begin_hydro<<<1, 1, 0, s>>>(g);
  enqueue_recon3<0>(g, in, s);
  enqueue_recon3<1>(g, in, s);
  enqueue_recon3<2>(g, in, s);
  k3_roe_hydro<0><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g);
  k3_roe_hydro<1><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g);
  k3_roe_hydro<2><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g);
  k3_ctu_hydro<0><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g);
  k3_ctu_hydro<1><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g);
  k3_ctu_hydro<2><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g);
  k3_roe_hydro<0><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g);
  k3_roe_hydro<1><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g);
  k3_roe_hydro<2><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g);
  k3_final_hydro<<<grid3(cells3(g)), kBlock, 0, s>>>(g, in, out);
  k3_end<<<1, 1, 0, s>>>(g);
}

}  // namespace MHD_NS
}  // namespace mhdk
