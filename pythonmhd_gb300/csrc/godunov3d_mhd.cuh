// Kernels of one 3D CTU+CT cycle of ideal MHD (Source/EvolveFunctions_MHD.py:750-1157).
// Included after godunov3d_kernels.cuh by the 3D translation units.
//
// A cycle:
//   dt_reduce -> begin -> for x, y, z: [slopes] -> faces (edge states, floors, the 3D
//   B corrections, conversion with the face B) -> roe(x, y, z) -> cell E -> EMF
//   (three edge components) -> half CT (x, y, z) -> ctu(x, y, z) (transverse
//   fluxes, EMF terms, source vector, back to prims with the half-step face B)
//   -> half-step cell E -> roe(x, y, z) -> EMF -> full CT (x, y, z) -> final -> end
// Sweep vectors are [rho, v, B_t1, B_t2, p] in the frames x (vx, vy, vz), y (vy, vz,
// vx), z (vz, vx, vy) (MhdSweep<0/1/2>); the PPM, eigensystem and Roe math is the
// 2D bodies'.  Reference quirks kept: first-order z faces and the z B corrections
// take the x boundary condition; the y B correction zeroes its z term when dBz == 0;
// the z predictor's outflow ghost above the last cell takes face nz-1.  The x
// predictor's y terms, which the reference computes in long double, are FP64 here.
#pragma once
#include "godunov3d_kernels.cuh"

namespace mhdk {
namespace MHD_NS {

// face-state conversions with the kinetic sum in the frame order (n, t1, t2)
// (Source/PrimCons_HelperModule.py:232-468)
template <int N, int T1, int T2>
__device__ __forceinline__ void p2c_frame(const double w[7], double bn, double gamma, double u[7]) {
  u[0] = w[0];
  u[1] = w[0] * w[1];
  u[2] = w[0] * w[2];
  u[3] = w[0] * w[3];
  u[4] = w[4];
  u[5] = w[5];
  u[6] = ddiv(w[6], gamma - 1.0) + 0.5 * w[0] * (w[N] * w[N] + w[T1] * w[T1] + w[T2] * w[T2]);
  u[6] = u[6] + 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5]);
}
template <int N, int T1, int T2>
__device__ __forceinline__ void c2p_frame(const double u[7], double bn, double gamma, double w[7]) {
  const double inv_d = ddiv(1.0, u[0]);
  w[0] = u[0];
  w[1] = u[1] * inv_d;
  w[2] = u[2] * inv_d;
  w[3] = u[3] * inv_d;
  w[4] = u[4];
  w[5] = u[5];
  double e = u[6] - 0.5 * (u[N] * u[N] + u[T1] * u[T1] + u[T2] * u[T2]) * inv_d;
  e = e - 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5]);
  w[6] = e * (gamma - 1.0);
}

__device__ __forceinline__ size_t edge3(const Grid3& G, int y, int x, int z) {
  return ((size_t)y * (size_t)(G.n[0] + 1) + (size_t)x) * (size_t)(G.n[2] + 1) + (size_t)z;
}

// index of point p (p[0] x, p[1] y, p[2] z) in the face array of direction A
template <int A>
__device__ __forceinline__ size_t face3(const Grid3& G, const int* p) { return lin3<A, 1>(G, p); }

// ----------------------------------------------------------------------------
// CFL timestep (Source/TimestepCalculations_HelperModule.py:305-361)
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3m_dt_reduce(Grid3 G, StateBuf3 in) {
  if (!loop_running(G.loop)) return;
  const size_t n = cells3(G);
  const double gamma = G.gamma;
  const double* c = in.cons;
  double m[3] = {0.0, 0.0, 0.0};
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    int p[3];
    unlin3<0, 0>(G, (unsigned)idx, p);
    const double inv_d = ddiv(1.0, c[idx]);
    const double vx = c[n + idx] * inv_d;
    const double vy = c[2 * n + idx] * inv_d;
    const double vz = c[3 * n + idx] * inv_d;
    const double vsq = vx * vx + vy * vy + vz * vz;
    const double c4 = c[4 * n + idx], c5 = c[5 * n + idx], c6 = c[6 * n + idx];
    const double bx = c4 + fabs(in.fb[0][face3<0>(G, p)] - c4);
    const double by = c5 + fabs(in.fb[1][face3<1>(G, p)] - c5);
    const double bz = c6 + fabs(in.fb[2][face3<2>(G, p)] - c6);
    const double bsq = bx * bx + by * by + bz * bz;
    const double pr = dmax((gamma - 1.0) * (c[7 * n + idx] - 0.5 * c[idx] * vsq - 0.5 * bsq), SMALL_VALUE);
    const double a2 = gamma * pr * inv_d;
    const double ssum = bsq * inv_d + a2;
    const double sdiff = bsq * inv_d - a2;
    const double dd = sdiff * sdiff;
    const double cfx = 0.5 * (ssum + sqrt(dd + 4.0 * a2 * (by * by + bz * bz) * inv_d));
    const double cfy = 0.5 * (ssum + sqrt(dd + 4.0 * a2 * (bx * bx + bz * bz) * inv_d));
    const double cfz = 0.5 * (ssum + sqrt(dd + 4.0 * a2 * (bx * bx + by * by) * inv_d));
    m[0] = dmax(m[0], fabs(vx) + sqrt(cfx));
    m[1] = dmax(m[1], fabs(vy) + sqrt(cfy));
    m[2] = dmax(m[2], fabs(vz) + sqrt(cfz));
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

// dt = cfl / max(mx/dx, my/dy, mz/dz), clipped to the stop time as evolve_3D_mhd
// does (Source/EvolveFunctions_MHD.py:829-833)
__global__ void k3m_begin(Grid3 G) {
  LoopState* L = G.loop;
  const int act = loop_running(L) ? 1 : 0;
  L->active = act;
  if (act) {
    const double mx = __longlong_as_double((long long)L->max_sx);
    const double my = __longlong_as_double((long long)L->max_sy);
    const double mz = __longlong_as_double((long long)L->max_sz);
    const double inv = dmax(ddiv(mx, G.d[0]), dmax(ddiv(my, G.d[1]), ddiv(mz, G.d[2])));
    double dt = ddiv(L->cfl, inv);
    if (L->t_end - L->t < dt) dt = L->t_end - L->t;
    L->dt = dt;
  }
  L->max_sx = 0ull;
  L->max_sy = 0ull;
  L->max_sz = 0ull;
}

// ----------------------------------------------------------------------------
// 3D corrections of the reconstructed transverse B
// (Source/Reconstruction_PPM_MHD_HelperModule.py:1351-1434, :1543-1628, :1743-1824)
// ----------------------------------------------------------------------------
__device__ __forceinline__ double b3_limit(double nch, double tch, bool zero_when_t_zero) {
  double r = 0.0;
  if (is_nonneg(nch)) {
    if (dlt(nch, -tch)) r = nch;
    else r = (zero_when_t_zero && is_zero(tch)) ? 0.0 : -tch;
    if (is_neg(r)) r = 0.0;
  } else {
    if (dgt(nch, -tch)) r = nch;
    else r = (zero_when_t_zero && is_zero(tch)) ? 0.0 : -tch;
    if (is_pos(r)) r = 0.0;
  }
  return r;
}

// change of face B of direction A across the cell at p: (fb[hi] - fb[lo]) * inv
template <int A>
__device__ __forceinline__ double own_change(const Grid3& G, const double* fb, const int* p, double h, bool divide) {
  const size_t lo = face3<A>(G, p);
  const double d = fb[lo + stride3<A, 1, A>(G)] - fb[lo];
  return divide ? ddiv(d, h) : d * h;
}

// normal change of face B of direction D at the sweep-extended cell e (-1..L) of the
// line through p: the reference's ghost faces (outflow: the end faces, a zero change;
// periodic: faces L-1 and 1); hi_face is the outflow ghost above the last cell
template <int D>
__device__ __forceinline__ double normal_change(const Grid3& G, const double* fb, const int* p, int e, int bc,
                                                double h, bool divide, int hi_face) {
  const int L = G.n[D];
  int lo, hi;
  if (e < 0) { lo = bc == OUTFLOW ? 0 : L - 1; hi = 0; }
  else if (e >= L) { lo = L; hi = bc == OUTFLOW ? hi_face : 1; }
  else { lo = e; hi = e + 1; }
  int q[3] = {p[0], p[1], p[2]};
  q[D] = lo;
  const double b_lo = fb[face3<D>(G, q)];
  q[D] = hi;
  const double b_hi = fb[face3<D>(G, q)];
  const double d = b_hi - b_lo;
  return divide ? ddiv(d, h) : d * h;
}

__device__ __forceinline__ double own_change_dyn(const Grid3& G, const double* const* fb, int a, const int* p,
                                                 double h, bool divide) {
  return a == 0 ? own_change<0>(G, fb[0], p, h, divide)
       : a == 1 ? own_change<1>(G, fb[1], p, h, divide)
                : own_change<2>(G, fb[2], p, h, divide);
}

// the two corrections (slots 4 and 5) of the sweep-extended cell e of the line through p
template <int D>
__device__ __forceinline__ void b3_corr(const Grid3& G, const StateBuf3& in, const int* p, int e, int bc,
                                        double dt, double out[2]) {
  using S = MhdSweep<D>;
  const int L = G.n[D];
  const double nch = normal_change<D>(G, in.fb[D], p, e, bc, ddiv(1.0, G.d[D]), false, L);
  int q[3] = {p[0], p[1], p[2]};
  q[D] = wrapc(e, L, bc);
  const size_t cell = lin3<0, 0>(G, q);
  const size_t plane = cells3(G);
  const double dens = __ldg(in.prim + cell);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int a = (s == 0 ? S::T1 : S::T2) - 1;
    const double tch = own_change_dyn(G, in.fb, a, q, ddiv(1.0, G.d[a]), false);
    const double v = ddiv(__ldg(in.cons + (size_t)(1 + a) * plane + cell), dens);
    const double term = b3_limit(nch, tch, D == 1 && s == 0);
    out[s] = 0.5 * dt * (v * term);
  }
}

// ----------------------------------------------------------------------------
// Reconstruction of direction D: edge states (the 2D bodies' math), floors, the B
// corrections and the conversion with the face B; writes prim (wl/wr) and cons
// (ul/ur) face states.
// ----------------------------------------------------------------------------
template <int D, int MODE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k3m_faces(Grid3 G, StateBuf3 in) {
  using S = MhdSweep<D>;
  if (!G.loop->active) return;
  const unsigned i = item3();
  if (i >= cells3(G)) return;
  int c[3];
  unlin3<D, 0>(G, i, c);
  const int cc = c[D];
  // face padding: the reconstruction's boundary condition (the first-order z faces
  // take BcX, Source/EvolveFunctions_MHD.py:867-884); corrections: BcX for z (:921-922)
  const int rbc = (D == 2 && MODE == 0) ? G.bc[0] : G.bc[D];
  const int cbc = D == 2 ? G.bc[0] : G.bc[D];
  const Line3<S, D> ln(G, c, rbc);
  double lia[7], ria[7], wc[7], wl[7], wr[7];
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
  const double dt = G.loop->dt;
  const size_t fp = plane3(G, D, 1);
  const int L = G.n[D];
  double corr[2];
  b3_corr<D>(G, in, c, cc, cbc, dt, corr);
  auto emit = [&](const double* v, int f, int side, const double* cr) {
    int q[3] = {c[0], c[1], c[2]};
    q[D] = f;
    const size_t fi = face3<D>(G, q);
    double w[7], u[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) w[k] = v[k];
    if (dlt(w[0], G.min_d)) w[0] = G.min_d;
    if (dlt(w[6], G.min_p)) w[6] = G.min_p;
    w[4] = w[4] + cr[0];
    w[5] = w[5] + cr[1];
    p2c_frame<S::N, S::T1, S::T2>(w, in.fb[D][fi], G.gamma, u);
    double* W = side == 0 ? G.wl[D] : G.wr[D];
    double* U = side == 0 ? G.ul[D] : G.ur[D];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      W[k * fp + fi] = w[k];
      U[k * fp + fi] = u[k];
    }
  };
  emit(lia, cc, 1, corr);
  emit(ria, cc + 1, 0, corr);
  if (cc == 0 || cc == L - 1) {
    double g_lo[2], g_hi[2];
    b3_corr<D>(G, in, c, -1, cbc, dt, g_lo);
    b3_corr<D>(G, in, c, L, cbc, dt, g_hi);
    if (cc == 0) {
      if (rbc == OUTFLOW) emit(lia, 0, 0, g_lo);
      else emit(lia, L, 1, g_hi);
    }
    if (cc == L - 1) {
      if (rbc == OUTFLOW) emit(ria, L, 1, g_hi);
      else emit(ria, 0, 0, g_lo);
    }
  }
}


// ----------------------------------------------------------------------------
// Roe fluxes of direction D (stage 1: the state's face B; stage 2: the half-step face B)
// ----------------------------------------------------------------------------
template <int D, int STAGE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k3m_roe(Grid3 G, StateBuf3 in) {
  using S = MhdSweep<D>;
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t fp = plane3(G, D, 1);
  if (i >= fp) return;
  double wl[7], wr[7], ul[7], ur[7], flux[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    wl[k] = G.wl[D][k * fp + i];
    wr[k] = G.wr[D][k * fp + i];
    ul[k] = G.ul[D][k * fp + i];
    ur[k] = G.ur[D][k * fp + i];
  }
  const double bn = STAGE == 1 ? in.fb[D][i] : G.nfb[D][i];
  roe_flux<S::N, S::T1, S::T2>(wl, wr, ul, ur, bn, G.gamma, G.efix != 0, G.eps, flux);
#pragma unroll
  for (int k = 0; k < 7; ++k) G.f[D][k * fp + i] = flux[k];
}

// stage-1 cell E = -v x B from the cell state (Source/EvolveFunctions_MHD.py:961-963)
__global__ void __launch_bounds__(kBlock) k3m_cell_e(Grid3 G, StateBuf3 in) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t n = cells3(G);
  if (i >= n) return;
  const double* p = in.prim;
  const double* c = in.cons;
  const double d = c[i];
  G.ce[0][i] = ddiv(p[5 * n + i] * c[3 * n + i] - p[6 * n + i] * c[2 * n + i], d);
  G.ce[1][i] = ddiv(p[6 * n + i] * c[n + i] - p[4 * n + i] * c[3 * n + i], d);
  G.ce[2][i] = ddiv(p[4 * n + i] * c[2 * n + i] - p[5 * n + i] * c[n + i], d);
}

// ----------------------------------------------------------------------------
// Edge EMFs: the three components on the (ny+1, nx+1, nz+1) edge grid, each the
// average of its two adjacent face fluxes and two upwinded terms per transverse
// direction (Source/CornerEMF_HelperModule.py:546-951)
// ----------------------------------------------------------------------------
__device__ __forceinline__ double upwind3(double s, double pos, double neg, double zero) {
  return is_pos(s) ? pos : (is_neg(s) ? neg : (is_zero(s) ? zero : 0.0));
}

// slot k of the flux of direction A at point (x, y, z) of its face array
template <int A>
__device__ __forceinline__ double flux3(const Grid3& G, int k, int x, int y, int z) {
  const int p[3] = {x, y, z};
  return G.f[A][(size_t)k * plane3(G, A, 1) + face3<A>(G, p)];
}
__device__ __forceinline__ double cell3(const Grid3& G, const double* a, int x, int y, int z) {
  const int p[3] = {x, y, z};
  return a[lin3<0, 0>(G, p)];
}

__global__ void __launch_bounds__(kBlock) k3m_emf(Grid3 G) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  if (i >= edges3(G)) return;
  const int nx = G.n[0], ny = G.n[1], nz = G.n[2];
  const int K = (int)(i % (unsigned)(nz + 1));
  const unsigned r = i / (unsigned)(nz + 1);
  const int I = (int)(r % (unsigned)(nx + 1));
  const int J = (int)(r / (unsigned)(nx + 1));
  const int bx = G.bc[0], by = G.bc[1], bz = G.bc[2];
  const int wI = wrapc(I, nx, bx), wI1 = wrapc(I - 1, nx, bx);
  const int wJ = wrapc(J, ny, by), wJ1 = wrapc(J - 1, ny, by);
  const int wK = wrapc(K, nz, bz), wK1 = wrapc(K - 1, nz, bz);
  {  // z component at (y-corner J, x-corner I, z-cell K)
    const double* E = G.ce[2];
    const double t0 = flux3<1>(G, 0, wI, J, wK), t5 = flux3<1>(G, 5, wI, J, wK);
    const double lt0 = flux3<1>(G, 0, wI1, J, wK), lt5 = flux3<1>(G, 5, wI1, J, wK);
    const double l0 = flux3<0>(G, 0, I, wJ, wK), l4 = flux3<0>(G, 4, I, wJ, wK);
    const double ul0 = flux3<0>(G, 0, I, wJ1, wK), ul4 = flux3<0>(G, 4, I, wJ1, wK);
    const double cE = cell3(G, E, wI, wJ, wK), lE = cell3(G, E, wI1, wJ, wK);
    const double uE = cell3(G, E, wI, wJ1, wK), ulE = cell3(G, E, wI1, wJ1, wK);
    const double x1 = upwind3(lt0, -ul4 - ulE, -l4 - lE, -0.5 * (l4 + ul4 + lE + ulE));
    const double x2 = upwind3(t0, -ul4 - uE, -l4 - cE, -0.5 * (l4 + ul4 + cE + uE));
    const double y1 = upwind3(ul0, lt5 - ulE, t5 - uE, 0.5 * (lt5 + t5 - ulE - uE));
    const double y2 = upwind3(l0, lt5 - lE, t5 - cE, 0.5 * (lt5 + t5 - lE - cE));
    G.emf[2][i] = 0.25 * (lt5 + t5 - ul4 - l4 + x1 + x2 + y1 + y2);
  }
  {  // x component at (y-corner J, x-cell I, z-corner K)
    const double* E = G.ce[0];
    const double b0 = flux3<2>(G, 0, wI, wJ, K), b5 = flux3<2>(G, 5, wI, wJ, K);
    const double ub0 = flux3<2>(G, 0, wI, wJ1, K), ub5 = flux3<2>(G, 5, wI, wJ1, K);
    const double t0 = flux3<1>(G, 0, wI, J, wK), t4 = flux3<1>(G, 4, wI, J, wK);
    const double bt0 = flux3<1>(G, 0, wI, J, wK1), bt4 = flux3<1>(G, 4, wI, J, wK1);
    const double cE = cell3(G, E, wI, wJ, wK), bE = cell3(G, E, wI, wJ, wK1);
    const double uE = cell3(G, E, wI, wJ1, wK), ubE = cell3(G, E, wI, wJ1, wK1);
    const double z1 = upwind3(bt0, ub5 - ubE, b5 - bE, 0.5 * (ub5 + b5 - ubE - bE));
    const double z2 = upwind3(t0, ub5 - uE, b5 - cE, 0.5 * (ub5 + b5 - uE - cE));
    const double y1 = upwind3(ub0, -bt4 - ubE, -t4 - uE, 0.5 * (-bt4 - t4 - ubE - uE));
    const double y2 = upwind3(b0, -bt4 - bE, -t4 - cE, 0.5 * (-bt4 - t4 - bE - cE));
    G.emf[0][i] = 0.25 * (b5 + ub5 - t4 - bt4 + y1 + y2 + z1 + z2);
  }
  {  // y component at (y-cell J, x-corner I, z-corner K)
    const double* E = G.ce[1];
    const double b0 = flux3<2>(G, 0, wI, wJ, K), b4 = flux3<2>(G, 4, wI, wJ, K);
    const double lb0 = flux3<2>(G, 0, wI1, wJ, K), lb4 = flux3<2>(G, 4, wI1, wJ, K);
    const double l0 = flux3<0>(G, 0, I, wJ, wK), l5 = flux3<0>(G, 5, I, wJ, wK);
    const double bl0 = flux3<0>(G, 0, I, wJ, wK1), bl5 = flux3<0>(G, 5, I, wJ, wK1);
    const double cE = cell3(G, E, wI, wJ, wK), bE = cell3(G, E, wI, wJ, wK1);
    const double lE = cell3(G, E, wI1, wJ, wK), blE = cell3(G, E, wI1, wJ, wK1);
    const double z1 = upwind3(bl0, -lb4 - blE, -b4 - bE, 0.5 * (-lb4 - b4 - blE - bE));
    const double z2 = upwind3(l0, -lb4 - lE, -b4 - cE, 0.5 * (-lb4 - b4 - lE - cE));
    const double x1 = upwind3(lb0, bl5 - blE, l5 - lE, 0.5 * (bl5 + l5 - blE - lE));
    const double x2 = upwind3(b0, bl5 - bE, l5 - cE, 0.5 * (bl5 + l5 - bE - cE));
    G.emf[1][i] = 0.25 * (l5 + bl5 - b4 - lb4 + x1 + x2 + z1 + z2);
  }
}

// ----------------------------------------------------------------------------
// CT update of the face B of direction D from the edge EMFs with factors
// h = (dt/dx, dt/dy, dt/dz), halved for the half step (Source/EvolveFunctions_MHD.py:1005-1029,
// :1082-1104): FULL writes the new state's faces, else the half-step faces.
// ----------------------------------------------------------------------------
template <int D, bool FULL>
__global__ void __launch_bounds__(kBlock) k3m_ct(Grid3 G, StateBuf3 in, StateBuf3 out) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  if (i >= plane3(G, D, 1)) return;
  int p[3];
  unlin3<D, 1>(G, i, p);
  const int x = p[0], y = p[1], z = p[2];
  const double dt = G.loop->dt;
  const double h0 = FULL ? ddiv(dt, G.d[0]) : 0.5 * ddiv(dt, G.d[0]);
  const double h1 = FULL ? ddiv(dt, G.d[1]) : 0.5 * ddiv(dt, G.d[1]);
  const double h2 = FULL ? ddiv(dt, G.d[2]) : 0.5 * ddiv(dt, G.d[2]);
  const double* ex = G.emf[0];
  const double* ey = G.emf[1];
  const double* ez = G.emf[2];
  double v = in.fb[D][i];
  if (D == 0) v = v + (h2 * (ey[edge3(G, y, x, z + 1)] - ey[edge3(G, y, x, z)]) -
                       h1 * (ez[edge3(G, y + 1, x, z)] - ez[edge3(G, y, x, z)]));
  if (D == 1) v = v + (h0 * (ez[edge3(G, y, x + 1, z)] - ez[edge3(G, y, x, z)]) -
                       h2 * (ex[edge3(G, y, x, z + 1)] - ex[edge3(G, y, x, z)]));
  if (D == 2) v = v + (h1 * (ex[edge3(G, y + 1, x, z)] - ex[edge3(G, y, x, z)]) -
                       h0 * (ey[edge3(G, y, x + 1, z)] - ey[edge3(G, y, x, z)]));
  (FULL ? out.fb[D] : G.nfb[D])[i] = v;
}

// ----------------------------------------------------------------------------
// 3D CTU predictor of direction D (Source/CTU_HelperModule.py:451-1078): each face
// state (conserved) takes, for each transverse direction in the reference's order,
// the half-dt flux difference at its cell (B slots zeroed) and the EMF term of the
// edge EMF parallel to D; then the source vector of its sweep-extended cell; then
// back to prims with the half-step face B.
// ----------------------------------------------------------------------------
__device__ __forceinline__ double minmod3(double nch, double tch) {
  if (is_pos(nch) && is_neg(tch)) return dgt(tch, -nch) ? tch : -nch;
  if (is_neg(nch) && is_pos(tch)) return dlt(tch, -nch) ? tch : -nch;
  return 0.0;
}

// transverse step of direction E (other transverse direction O) on u at cell p: flux
// difference, then the EMF term of the D-parallel edge EMF on `slot` with `sign`
template <int D, int E>
__device__ __forceinline__ void ctu3m_step(const Grid3& G, const int* p, double half, int slot, double sign,
                                           double* u) {
  constexpr int O = 3 - D - E;
  const size_t lo = face3<E>(G, p);
  const size_t hi = lo + stride3<E, 1, E>(G);
  const size_t fp = plane3(G, E, 1);
  const double* F = G.f[E];
#pragma unroll
  for (int k = 0; k < 7; ++k)
    if (k != 4 && k != 5) u[k] = u[k] - half * (F[k * fp + hi] - F[k * fp + lo]);
  // the four D-parallel edges around the cell in the (E, O) plane
  int q[3] = {p[0], p[1], p[2]};
  auto em = [&](int de, int dof) {
    int r[3] = {q[0], q[1], q[2]};
    r[E] += de;
    r[O] += dof;
    return G.emf[D][edge3(G, r[1], r[0], r[2])];
  };
  const double delta = ((em(1, 0) - em(0, 0)) + em(1, 1)) - em(0, 1);
  const double upd = (half * 0.5) * delta;
  u[slot] = is_pos(sign) ? u[slot] + upd : u[slot] - upd;
}

template <int D>
__global__ void __launch_bounds__(kBlock) k3m_ctu(Grid3 G, StateBuf3 in) {
  using S = MhdSweep<D>;
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t fp = plane3(G, D, 1);
  if (i >= fp) return;
  int c[3];
  unlin3<D, 1>(G, i, c);
  const int f = c[D];
  const int L = G.n[D];
  const int bc = G.bc[D];
  const double dt = G.loop->dt;
  constexpr int E1 = D == 0 ? 1 : 0;
  constexpr int E2 = D == 2 ? 1 : 2;
  // (slot, sign) of each step's EMF term: x: (5, +), (4, -); y: (4, -), (5, +); z: (5, +), (4, -)
  constexpr int SL1 = D == 1 ? 4 : 5, SL2 = D == 1 ? 5 : 4;
  constexpr double SG1 = D == 1 ? -1.0 : 1.0, SG2 = D == 1 ? 1.0 : -1.0;
  const double h1 = 0.5 * ddiv(dt, G.d[E1]);
  const double h2 = 0.5 * ddiv(dt, G.d[E2]);
  // the source vector's changes: x with products by 1/dn, y and z with quotients by dn
  const bool divide = D != 0;
  const size_t n = cells3(G);
  const double* pr = in.prim;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double* U = side == 0 ? G.ul[D] : G.ur[D];
    double u[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) u[k] = U[k * fp + i];
    int p[3] = {c[0], c[1], c[2]};
    p[D] = wrapc(f - 1 + side, L, bc);
    ctu3m_step<D, E1>(G, p, h1, SL1, SG1, u);
    ctu3m_step<D, E2>(G, p, h2, SL2, SG2, u);
    // source vector of the sweep-extended cell e = f - 1 + side
    const int e = f - 1 + side;
    const double hn = divide ? G.d[D] : ddiv(1.0, G.d[D]);
    const double nch = normal_change<D>(G, in.fb[D], c, e, bc, hn, divide, D == 2 ? L - 1 : L);
    const int a = S::T1 - 1, b = S::T2 - 1;
    const double ta = own_change_dyn(G, in.fb, a, p, divide ? G.d[a] : ddiv(1.0, G.d[a]), divide);
    const double tb = own_change_dyn(G, in.fb, b, p, divide ? G.d[b] : ddiv(1.0, G.d[b]), divide);
    const size_t cell = lin3<0, 0>(G, p);
    const double bx = pr[4 * n + cell], by = pr[5 * n + cell], bz = pr[6 * n + cell];
    const double va = pr[(size_t)(1 + a) * n + cell], vb = pr[(size_t)(1 + b) * n + cell];
    const double ba = pr[(size_t)(4 + a) * n + cell], bb = pr[(size_t)(4 + b) * n + cell];
    const double hdt = 0.5 * dt;
    const double mmb = minmod3(nch, tb), mma = minmod3(nch, ta);
    u[0] = u[0] + 0.0;
    u[1] = u[1] + hdt * bx * nch;
    u[2] = u[2] + hdt * by * nch;
    u[3] = u[3] + hdt * bz * nch;
    u[4] = u[4] + hdt * va * (-mmb);
    u[5] = u[5] + hdt * vb * (-mma);
    u[6] = u[6] + hdt * (ba * va * (-mmb) + bb * vb * (-mma));
    double w[7];
    c2p_frame<S::N, S::T1, S::T2>(u, G.nfb[D][i], G.gamma, w);
    double* W = side == 0 ? G.wl[D] : G.wr[D];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      U[k * fp + i] = u[k];
      W[k * fp + i] = w[k];
    }
  }
}

// ----------------------------------------------------------------------------
// Half-step cell E from the stage-1 fluxes and the half-step face B
// (Source/EvolveFunctions_MHD.py:1038-1062)
// ----------------------------------------------------------------------------
template <int A>
__device__ __forceinline__ double fdiff3(const Grid3& G, int k, const int* p) {
  const size_t lo = face3<A>(G, p);
  const size_t fp = plane3(G, A, 1);
  return G.f[A][k * fp + lo + stride3<A, 1, A>(G)] - G.f[A][k * fp + lo];
}
template <int A>
__device__ __forceinline__ double favg3(const Grid3& G, const double* fb, const int* p) {
  const size_t lo = face3<A>(G, p);
  return 0.5 * (fb[lo] + fb[lo + stride3<A, 1, A>(G)]);
}

__global__ void __launch_bounds__(kBlock) k3m_half_e(Grid3 G, StateBuf3 in) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t n = cells3(G);
  if (i >= n) return;
  int p[3];
  unlin3<0, 0>(G, i, p);
  const double dt = G.loop->dt;
  const double hx = 0.5 * ddiv(dt, G.d[0]), hy = 0.5 * ddiv(dt, G.d[1]), hz = 0.5 * ddiv(dt, G.d[2]);
  double h[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double v = in.cons[(size_t)k * n + i] - hx * fdiff3<0>(G, k, p);
    v = v - hy * fdiff3<1>(G, k, p);
    v = v - hz * fdiff3<2>(G, k, p);
    h[k] = v;
  }
  const double bx = favg3<0>(G, G.nfb[0], p), by = favg3<1>(G, G.nfb[1], p), bz = favg3<2>(G, G.nfb[2], p);
  G.ce[0][i] = ddiv(by * h[3] - bz * h[2], h[0]);
  G.ce[1][i] = ddiv(bz * h[1] - bx * h[3], h[0]);
  G.ce[2][i] = ddiv(bx * h[2] - by * h[1], h[0]);
}

// ----------------------------------------------------------------------------
// Conservative update with the stage-2 fluxes (7-vectors in their sweep orders, as
// the reference subtracts them), cell B from the new faces, prims
// (Source/EvolveFunctions_MHD.py:1106-1152)
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k3m_final(Grid3 G, StateBuf3 in, StateBuf3 out) {
  if (!G.loop->active) return;
  const unsigned i = item3();
  const size_t n = cells3(G);
  if (i >= n) return;
  int p[3];
  unlin3<0, 0>(G, i, p);
  const double dt = G.loop->dt;
  const double dtdx = ddiv(dt, G.d[0]), dtdy = ddiv(dt, G.d[1]), dtdz = ddiv(dt, G.d[2]);
  constexpr int src[7] = {0, 1, 2, 3, 5, 6, 7};
  double u[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) u[k] = in.cons[(size_t)src[k] * n + i];
#pragma unroll
  for (int k = 0; k < 7; ++k) u[k] = u[k] - dtdx * fdiff3<0>(G, k, p);
#pragma unroll
  for (int k = 0; k < 7; ++k) u[k] = u[k] - dtdy * fdiff3<1>(G, k, p);
#pragma unroll
  for (int k = 0; k < 7; ++k) u[k] = u[k] - dtdz * fdiff3<2>(G, k, p);
  const double cbx = favg3<0>(G, out.fb[0], p), cby = favg3<1>(G, out.fb[1], p), cbz = favg3<2>(G, out.fb[2], p);
  u[4] = cby;
  u[5] = cbz;
  double w[7];
  cons_to_prim7(u, cbx, G.gamma, w);
  const double pw[8] = {w[0], w[1], w[2], w[3], cbx, w[4], w[5], w[6]};
  const double cw[8] = {u[0], u[1], u[2], u[3], cbx, u[4], u[5], u[6]};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    out.prim[(size_t)k * n + i] = pw[k];
    out.cons[(size_t)k * n + i] = cw[k];
  }
}

// ----------------------------------------------------------------------------
// Host-side enqueue of one 3D MHD cycle reading state buffer `parity`.
// ----------------------------------------------------------------------------
template <int D>
void enqueue_recon3m(const Grid3& g, const StateBuf3& in, cudaStream_t s) {
  using S = MhdSweep<D>;
  if (g.recon >= 1) k3_slopes<S, D><<<grid3(plane3(g, D, 2)), kBlock, 0, s>>>(g, in);
  if (g.recon == 2) k3m_faces<D, 2><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  else if (g.recon == 1) k3m_faces<D, 1><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  else k3m_faces<D, 0><<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
}

void enqueue_cycle3_mhd(const Grid3& g, int parity, int dt_blocks, cudaStream_t s) {
  const StateBuf3 in = g.st[parity];
  const StateBuf3 out = g.st[parity ^ 1];
  k3m_dt_reduce<<<dt_blocks, 256, 0, s>>>(g, in);
  k3m_begin<<<1, 1, 0, s>>>(g);
  enqueue_recon3m<0>(g, in, s);
  enqueue_recon3m<1>(g, in, s);
  enqueue_recon3m<2>(g, in, s);
  k3m_roe<0, 1><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g, in);
  k3m_roe<1, 1><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g, in);
  k3m_roe<2, 1><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g, in);
  k3m_cell_e<<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  k3m_emf<<<grid3(edges3(g)), kBlock, 0, s>>>(g);
  k3m_ct<0, false><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_ct<1, false><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_ct<2, false><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_ctu<0><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g, in);
  k3m_ctu<1><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g, in);
  k3m_ctu<2><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g, in);
  k3m_half_e<<<grid3(cells3(g)), kBlock, 0, s>>>(g, in);
  k3m_roe<0, 2><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g, in);
  k3m_roe<1, 2><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g, in);
  k3m_roe<2, 2><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g, in);
  k3m_emf<<<grid3(edges3(g)), kBlock, 0, s>>>(g);
  k3m_ct<0, true><<<grid3(plane3(g, 0, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_ct<1, true><<<grid3(plane3(g, 1, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_ct<2, true><<<grid3(plane3(g, 2, 1)), kBlock, 0, s>>>(g, in, out);
  k3m_final<<<grid3(cells3(g)), kBlock, 0, s>>>(g, in, out);
  k3_end<<<1, 1, 0, s>>>(g);
}

}  // namespace MHD_NS
}  // namespace mhdk
