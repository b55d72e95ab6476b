// Kernels of one 2D CTU(+CT) cycle.  Included by two translation units that
// define MHD_NS: `exact` (built with -fmad=false: reproduces the reference's
// NumPy arithmetic bit for bit) and `fast` (FMA contraction allowed).
//
// A cycle (Source/EvolveFunctions_MHD.py:464-692, Source/EvolveFunctions_Hydro.py:390-513):
//   dt_reduce -> begin -> [slopes_x] -> faces_x -> [slopes_y] -> faces_y   (slopes: PLM/PPM)
//   -> roe_x(1) -> roe_y(1) -> [MHD: emf(1)] -> ctu_x -> ctu_y
//   -> [MHD: half] -> roe_x(2) -> roe_y(2) -> [MHD: emf(2)] -> final -> end
// Every kernel returns at once when the loop state says the cycle is not a real
// one (t >= t_end or cycle >= max_cycles), so a captured graph can be replayed
// past the end of a run without changing the state.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "godunov2d_types.h"
#include "mhd_math.cuh"

#ifndef MHD_NS
#error "define MHD_NS"
#endif

namespace mhdk {
namespace MHD_NS {

constexpr int kBlock = 128;
#ifndef MHD_MIN_BLOCKS
#define MHD_MIN_BLOCKS 2
#endif
#ifndef MHD_MIN_BLOCKS_SLOPES
#define MHD_MIN_BLOCKS_SLOPES MHD_MIN_BLOCKS
#endif
#ifndef MHD_MIN_BLOCKS_FACES
#define MHD_MIN_BLOCKS_FACES MHD_MIN_BLOCKS
#endif
#ifndef MHD_MIN_BLOCKS_ROE
#define MHD_MIN_BLOCKS_ROE MHD_MIN_BLOCKS
#endif
// resident blocks per SM the heavy FP64 kernels are compiled for (caps registers):
// the batched kernels, and per kernel the slope, face and Roe kernels of the single grid
constexpr int kMinBlocks = MHD_MIN_BLOCKS;
constexpr int kMinBlocksSlopes = MHD_MIN_BLOCKS_SLOPES;
constexpr int kMinBlocksFaces = MHD_MIN_BLOCKS_FACES;
constexpr int kMinBlocksRoe = MHD_MIN_BLOCKS_ROE;

__device__ __forceinline__ int wrapc(int c, int L, int bc) {
  if (bc == PERIODIC) {
    int m = c % L;
    return m < 0 ? m + L : m;
  }
  return c < 0 ? 0 : (c >= L ? L - 1 : c);
}

// ----------------------------------------------------------------------------
// Checked build (MHD_CHECKED, the "checked" arithmetic mode): every global access
// of the per-item bodies below is preceded by MHD_GUARD(G, base, idx), which
// requires the in-plane index idx to lie inside one plane of the array that starts
// at `base` (each access is base[k * plane + idx] with k a compile-time slot below
// the array's plane count).  A violation sets kStatusIndex in the grid's error
// word, records the first offending source line and index, and skips the item: it
// never traps and never touches memory outside the array.  In the other builds
// MHD_GUARD is empty.
// ----------------------------------------------------------------------------
#ifdef MHD_CHECKED
// elements in one plane of the grid array that starts at base (0: not an array of G)
__device__ __forceinline__ size_t plane_extent(const Grid& G, const void* base) {
  const size_t cp = cell_plane(G), xp = xface_plane(G), yp = yface_plane(G), kp = corner_plane(G);
  for (int b = 0; b < 2; ++b) {
    if (base == G.st[b].prim || base == G.st[b].cons) return cp;
    if (base == G.st[b].fbx) return xp;
    if (base == G.st[b].fby) return yp;
  }
  if (base == G.xl || base == G.xr || base == G.fx || base == G.uxl || base == G.uxr || base == G.nfbx) return xp;
  if (base == G.yl || base == G.yr || base == G.fy || base == G.uyl || base == G.uyr || base == G.nfby) return yp;
  if (base == G.emf) return kp;
  if (base == G.hez) return cp;
  if (base == G.slopes || base == G.eig || base == G.slopes_y || base == G.eig_y) return G.ext_plane;
  if (base == G.dt_log) return (size_t)G.dt_log_cap;
  return 0;
}
__device__ __noinline__ void report_index(const Grid& G, int line, size_t idx) {
  if (G.status) atomicOr(G.status, kStatusIndex);
  if (G.bad && atomicCAS(reinterpret_cast<unsigned long long*>(G.bad), 0ull, (unsigned long long)line) == 0ull)
    G.bad[1] = (long long)idx;
}
#define MHD_GUARD(G, base, idx)                                               \
  do {                                                                        \
    const size_t i_ = (idx);                                                  \
    if (!(i_ < plane_extent((G), (base)))) { report_index((G), __LINE__, i_); return; } \
  } while (0)
#define MHD_GUARD_RET(G, base, idx, ret)                                      \
  do {                                                                        \
    const size_t i_ = (idx);                                                  \
    if (!(i_ < plane_extent((G), (base)))) { report_index((G), __LINE__, i_); return (ret); } \
  } while (0)
#else
#define MHD_GUARD(G, base, idx) do {} while (0)
#define MHD_GUARD_RET(G, base, idx, ret) do {} while (0)
#endif

// ----------------------------------------------------------------------------
// Sweep policies
// ----------------------------------------------------------------------------
// Sweep vectors [rho, v, B_t1, B_t2, p] in the frame (n, t1, t2): x (vx, vy, vz) with
// (By, Bz), y (vy, vz, vx) with (Bz, Bx), z (vz, vx, vy) with (Bx, By) -- the z frame
// serves the 3D step.
template <int AX>
struct MhdSweep {
  static constexpr int NV = 7;
  static constexpr int NW = kPrimEigWords;
  static constexpr int N = AX + 1;
  static constexpr int T1 = AX == 0 ? 2 : (AX == 1 ? 3 : 1);
  static constexpr int T2 = AX == 0 ? 3 : (AX == 1 ? 1 : 2);
  static constexpr int BN = 4 + AX;            // prim8 slot of the cell normal B
  static constexpr int SB = AX == 0 ? 4 : 5;   // 2D: sweep slot that gets the B source term
  __device__ static constexpr int src(int k) {
    return k < 4 ? k : (k == 6 ? 7 : 3 + (k == 4 ? T1 : T2));
  }
  __device__ static constexpr int ord(int k) {
    return k == 0 ? 0 : k == 1 ? N : k == 2 ? T1 : k == 3 ? T2 : k == 4 ? 6 : k == 5 ? 4 : 5;
  }
  using Eig = PrimEig;
  __device__ static void eig(const double* w, double bn, double gamma, Eig& e) {
    prim_eigensystem<N, T1, T2>(w, bn, gamma, e);
  }
  __device__ static bool Lnz(int i, int j) { return prim_L_nz<N, T1, T2>(i, j); }
  __device__ static bool Rnz(int i, int j) { return prim_R_nz<N, T1, T2>(i, j); }
  __device__ static double L(const Eig& e, int i, int j) { return prim_L<N, T1, T2>(e, i, j); }
  __device__ static double R(const Eig& e, int i, int j) { return prim_R<N, T1, T2>(e, i, j); }
  __device__ static double* lam(Eig& e) { return e.lam; }
  __device__ static void store(const Eig& e, double* p, size_t stride) {
    const double* s = reinterpret_cast<const double*>(&e);
#pragma unroll
    for (int k = 0; k < NW; ++k) p[k * stride] = s[k];
  }
  __device__ static void load(Eig& e, const double* p, size_t stride) {
    double* s = reinterpret_cast<double*>(&e);
#pragma unroll
    for (int k = 0; k < NW; ++k) s[k] = p[k * stride];
  }
};

template <int AX>
struct HydroSweep {
  static constexpr int NV = 5;
  static constexpr int NW = 10;
  static constexpr int BN = -1;
  static constexpr int SB = -1;
  __device__ static constexpr int src(int k) { return k; }
  __device__ static constexpr int ord(int k) { return k; }
  using Eig = HPrimEig;
  __device__ static void eig(const double* w, double, double gamma, Eig& e) { hprim_eigensystem<AX>(w, gamma, e); }
  __device__ static bool Lnz(int i, int j) { return hprim_L_nz<AX>(i, j); }
  __device__ static bool Rnz(int i, int j) { return hprim_R_nz<AX>(i, j); }
  __device__ static double L(const Eig& e, int i, int j) { return hprim_L<AX>(e, i, j); }
  __device__ static double R(const Eig& e, int i, int j) { return hprim_R<AX>(e, i, j); }
  __device__ static double* lam(Eig& e) { return e.lam; }
  __device__ static void store(const Eig& e, double* p, size_t stride) {
    const double* s = reinterpret_cast<const double*>(&e);
#pragma unroll
    for (int k = 0; k < NW; ++k) p[k * stride] = s[k];
  }
  __device__ static void load(Eig& e, const double* p, size_t stride) {
    double* s = reinterpret_cast<double*>(&e);
#pragma unroll
    for (int k = 0; k < NW; ++k) s[k] = p[k * stride];
  }
};

// Row i of L times v in the reference's accumulation order.
template <class S>
__device__ __forceinline__ double project(const typename S::Eig& e, int i, const double* v) {
  double acc = 0.0;
  bool first = true;
#pragma unroll
  for (int k = 0; k < S::NV; ++k) {
    const int j = S::ord(k);
    if (S::Lnz(i, j)) {
      const double t = S::L(e, i, j) * v[j];
      acc = first ? t : acc + t;
      first = false;
    }
  }
  return acc;
}

struct SweepGeom {
  int Ls, Lt, nx;  // sweep length, transverse length, row stride of the cell grid
  int bc;
};

template <int AX>
__device__ __forceinline__ size_t cell_index(int c, int t, int nx) {
  return AX == 0 ? (size_t)t * nx + c : (size_t)c * nx + t;
}
template <int AX>
__device__ __forceinline__ size_t ext_index(int c, int t, int nx) {
  // c in [-1, Ls]; extended grid has Ls+2 cells along the sweep
  return AX == 0 ? (size_t)t * (nx + 2) + (c + 1) : (size_t)(c + 1) * nx + t;
}
template <int AX>
__device__ __forceinline__ size_t face_index(int f, int t, int nx) {
  return AX == 0 ? (size_t)t * (nx + 1) + f : (size_t)f * nx + t;
}

template <class S, int AX>
__device__ __forceinline__ void load_sweep_cell(const Grid& G, const double* prim, size_t plane, int c, int t,
                                                const SweepGeom& g, double* w) {
  const size_t idx = cell_index<AX>(wrapc(c, g.Ls, g.bc), t, g.nx);
  MHD_GUARD(G, prim, idx);
#pragma unroll
  for (int k = 0; k < S::NV; ++k) w[k] = __ldg(prim + S::src(k) * plane + idx);
}

// Characteristic-limited slope of one cell from its two neighbours, in primitive
// variables: the differences projected on the left eigenvectors, limited (van Leer
// weight, 2x one-sided and centred bounds), and mapped back with the right
// eigenvectors (Source/Reconstruction_PPM_MHD_HelperModule.py:317-389, Hydro :86-200).
template <class S>
__device__ __forceinline__ void limited_slopes(const double* wl, const double* wc, const double* wr,
                                               const typename S::Eig& e, double* out) {
  constexpr int NV = S::NV;
  double dc[NV], dl[NV], dr[NV], wt[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    dc[k] = wr[k] - wl[k];
    dl[k] = wc[k] - wl[k];
    dr[k] = wr[k] - wc[k];
    wt[k] = is_pos(dl[k] * dr[k]) ? ddiv(2.0 * dl[k] * dr[k], dl[k] + dr[k]) : 0.0;
  }
  double sc[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double cc = project<S>(e, i, dc);
    const double cl = project<S>(e, i, dl);
    const double cr = project<S>(e, i, dr);
    const double cw = project<S>(e, i, wt);
    double s = 0.0;
    if (is_pos(cl * cr)) {
      const double lim1 = dmin(fabs(cl), fabs(cr));
      const double lim2 = dmin(0.5 * fabs(cc), fabs(cw));
      s = signed_mag(cc, dmin(2.0 * lim1, lim2));
    }
    sc[i] = s;
  }
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      if (S::Rnz(i, j)) {
        const double tt = sc[j] * S::R(e, i, j);
        acc = first ? tt : acc + tt;
        first = false;
      }
    }
    out[i] = acc;
  }
}

// ----------------------------------------------------------------------------
// PPM phase A: eigensystem + monotonised characteristic slopes for cells -1..Ls
// (Source/Reconstruction_PPM_MHD_HelperModule.py:317-389, Hydro :86-200)
// ----------------------------------------------------------------------------
// work item (x, y) of the sweep-extended cell space: (Ls+2) x Lt along the sweep
template <class S, int AX>
__device__ __forceinline__ void b_ppm_slopes(const Grid& G, const StateBuf& in, int x, int y) {
  if (!G.loop->active) return;
  SweepGeom g;
  g.nx = G.nx;
  g.Ls = AX == 0 ? G.nx : G.ny;
  g.Lt = AX == 0 ? G.ny : G.nx;
  g.bc = AX == 0 ? G.bcx : G.bcy;
  int c, t;
  if (AX == 0) { c = x - 1; t = y; }
  else { t = x; c = y - 1; }
  if (c > g.Ls || t >= g.Lt) return;
  const size_t plane = cell_plane(G);
  constexpr int NV = S::NV;
  double wl[NV], wc[NV], wr[NV];
  load_sweep_cell<S, AX>(G, in.prim, plane, c - 1, t, g, wl);
  load_sweep_cell<S, AX>(G, in.prim, plane, c, t, g, wc);
  load_sweep_cell<S, AX>(G, in.prim, plane, c + 1, t, g, wr);
  double bn = 0.0;
  MHD_GUARD(G, in.prim, cell_index<AX>(wrapc(c, g.Ls, g.bc), t, g.nx));
  if (S::BN >= 0)
    bn = G.one_d ? G.bx1d
                 : __ldg(in.prim + (size_t)(S::BN >= 0 ? S::BN : 0) * plane + cell_index<AX>(wrapc(c, g.Ls, g.bc), t, g.nx));
  typename S::Eig e;
  S::eig(wc, bn, G.gamma, e);
  double ps[NV];
  limited_slopes<S>(wl, wc, wr, e, ps);
  const size_t xi = ext_index<AX>(c, t, g.nx);
  const size_t es = G.ext_plane;
  MHD_GUARD(G, AX == 0 ? G.slopes : G.slopes_y, xi);
  MHD_GUARD(G, AX == 0 ? G.eig : G.eig_y, xi);
#pragma unroll
  for (int i = 0; i < NV; ++i) (AX == 0 ? G.slopes : G.slopes_y)[i * es + xi] = ps[i];
  S::store(e, (AX == 0 ? G.eig : G.eig_y) + xi, es);
}

// Write one reconstructed state to a face: floors (Source/PrimCons_HelperModule.py:499-554),
// then the transverse-B source term (Source/EvolveFunctions_MHD.py:524-535).  Returns how
// many of its values the floors raised (the reference counts them for a warning it
// then discards; here they reach mhd2d_stats).
template <class S>
__device__ __forceinline__ unsigned put_face(double* buf, size_t fplane, size_t fidx, const double* v,
                                             double min_d, double min_p, double bsrc, bool add_src = true) {
  constexpr int NV = S::NV;
  unsigned hits = 0;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
    if (k == 0 && dlt(x, min_d)) { x = min_d; ++hits; }
    if (k == NV - 1 && dlt(x, min_p)) { x = min_p; ++hits; }
    if (k == S::SB && add_src) x = x + bsrc;
    buf[k * fplane + fidx] = x;
  }
  return hits;
}

// Publish a thread's floor hits / a non-finite output with one atomic (rare events).
__device__ __forceinline__ void note_floor_hits(const Grid& G, unsigned hits) {
  if (hits && G.floor_hits) atomicAdd(G.floor_hits, (unsigned long long)hits);
}
__device__ __forceinline__ void note_nonfinite(const Grid& G, bool bad) {
  if (bad && G.status) atomicOr(G.status, kStatusNonfinite);
}

// B source term of one face state: half_dt * v_t(cell) * ((fb[f2] - fb[f1]) * inv_dn)
// (Source/Reconstruction_PPM_MHD_HelperModule.py:1193-1239)
template <int AX>
__device__ __forceinline__ double bsource(const Grid& G, const double* prim, const double* fb, size_t plane, int cell,
                                          int f1, int f2, int t, int nx, double half_dt, double inv_dn) {
  const int vslot = AX == 0 ? 2 : 1;
  MHD_GUARD_RET(G, prim, cell_index<AX>(cell, t, nx), 0.0);
  MHD_GUARD_RET(G, fb, face_index<AX>(f2, t, nx), 0.0);
  MHD_GUARD_RET(G, fb, face_index<AX>(f1, t, nx), 0.0);
  const double vt = __ldg(prim + vslot * plane + cell_index<AX>(cell, t, nx));
  const double b2 = __ldg(fb + face_index<AX>(f2, t, nx));
  const double b1 = __ldg(fb + face_index<AX>(f1, t, nx));
  return half_dt * vt * ((b2 - b1) * inv_dn);
}

// Edge states of one cell along a sweep from the cell, its two neighbours and
// (PLM/PPM) the limited slopes: MODE 2 = PPM interfaces, monotonicity and
// characteristic tracing (Source/Reconstruction_PPM_MHD_HelperModule.py:391-548,
// Hydro :202-371), MODE 1 = PLM (no reference counterpart: the reference's limited
// slope taken as a linear profile W -/+ s/2, clamped to the neighbours, traced with
// the reference's own tracing with the parabolic coefficient zero -- Stone et al.
// 2008 eqs. 38-42), MODE 0 = first order (the cell value on both sides).
// slope_at(k, d) returns slot k's slope at cell offset d in {-1, 0, 1}; eig_at(e)
// loads the cell's stored eigensystem.  lia / ria: the states at the cell's minus /
// plus interface.
template <class S, int MODE, class SlopeAt, class EigAt>
__device__ __forceinline__ void edge_states(const double* wl, const double* wc, const double* wr,
                                            SlopeAt slope_at, EigAt eig_at, double dt, double dn, double* lia,
                                            double* ria) {
  constexpr int NV = S::NV;
  if (MODE == 1) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double s_c = slope_at(k, 0);
      double a = wc[k] - 0.5 * s_c;
      double b = wc[k] + 0.5 * s_c;
      a = dmax(dmin(wc[k], wl[k]), a);
      a = dmin(dmax(wc[k], wl[k]), a);
      b = dmax(dmin(wc[k], wr[k]), b);
      b = dmin(dmax(wc[k], wr[k]), b);
      lia[k] = a;
      ria[k] = b;
    }
    typename S::Eig e;
    eig_at(e);
    const double* lam = S::lam(e);
    const double dtdx = ddiv(dt, dn);
    double c1[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) c1[k] = ria[k] - lia[k];
    const double c3 = 0.5 * dmax(lam[NV - 1], 0.0) * dtdx;
    const double c4 = -0.5 * dmin(lam[0], 0.0) * dtdx;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      lia[k] = lia[k] + c4 * c1[k];
      ria[k] = ria[k] - c3 * c1[k];
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        if (side == 0 ? is_nonpos(lam[i]) : is_nonneg(lam[i])) {
          const double v3 = 0.5 * dtdx * lam[side == 0 ? 0 : NV - 1] - 0.5 * dtdx * lam[i];
          double fac = 0.0;
          bool first = true;
#pragma unroll
          for (int k = 0; k < NV; ++k) {
            const int j = S::ord(k);
            if (S::Lnz(i, j)) {
              const double tt = S::L(e, i, j) * (v3 * c1[j]);
              fac = first ? tt : fac + tt;
              first = false;
            }
          }
          double* edge = side == 0 ? lia : ria;
#pragma unroll
          for (int j = 0; j < NV; ++j)
            if (S::Rnz(j, i)) edge[j] = edge[j] + fac * S::R(e, j, i);
        }
      }
    }
  } else if (MODE == 2) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double s_l = slope_at(k, -1);
      const double s_c = slope_at(k, 0);
      const double s_r = slope_at(k, 1);
      double a = 0.5 * (wc[k] + wl[k]) - div6(s_c - s_l);
      double b = 0.5 * (wr[k] + wc[k]) - div6(s_r - s_c);
      const double dprod = (b - wc[k]) * (wc[k] - a);
      const double idiff = b - a;
      const double adiff = 6.0 * (wc[k] - 0.5 * (a + b));
      if (is_nonpos(dprod)) {
        a = wc[k];
        b = wc[k];
      } else if (dgt(idiff * adiff, sq(idiff))) {
        a = (6.0 * wc[k] - 4.0 * b) * 0.5;   // x / 2 exactly
      } else if (dlt(idiff * adiff, -1.0 * sq(idiff))) {
        b = (6.0 * wc[k] - 4.0 * a) * 0.5;
      }
      a = dmax(dmin(wc[k], wl[k]), a);
      a = dmin(dmax(wc[k], wl[k]), a);
      b = dmax(dmin(wc[k], wr[k]), b);
      b = dmin(dmax(wc[k], wr[k]), b);
      lia[k] = a;
      ria[k] = b;
    }
    typename S::Eig e;
    eig_at(e);
    const double* lam = S::lam(e);
    const double dtdx = ddiv(dt, dn);
    double c1[NV], c2[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      c1[k] = ria[k] - lia[k];
      c2[k] = 6.0 * (wc[k] - 0.5 * (lia[k] + ria[k]));
    }
    const double c3 = 0.5 * dmax(lam[NV - 1], 0.0) * dtdx;
    const double c4 = -0.5 * dmin(lam[0], 0.0) * dtdx;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      lia[k] = lia[k] + c4 * (c1[k] + (1.0 - FOUR_THIRDS * c4) * c2[k]);
      ria[k] = ria[k] - c3 * (c1[k] - (1.0 - FOUR_THIRDS * c3) * c2[k]);
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (is_nonpos(lam[i])) {
        const double v1 = 0.5 * dtdx * lam[0];
        const double v2 = 0.5 * dtdx * lam[i];
        const double v3 = v1 - v2;
        const double v4 = FOUR_THIRDS * (sq(v1) - sq(v2));
        double fac = 0.0;
        bool first = true;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const int j = S::ord(k);
          if (S::Lnz(i, j)) {
            const double tt = S::L(e, i, j) * (v3 * (c1[j] + c2[j]) + v4 * c2[j]);
            fac = first ? tt : fac + tt;
            first = false;
          }
        }
#pragma unroll
        for (int j = 0; j < NV; ++j)
          if (S::Rnz(j, i)) lia[j] = lia[j] + fac * S::R(e, j, i);
      }
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (is_nonneg(lam[i])) {
        const double v1 = 0.5 * dtdx * lam[NV - 1];
        const double v2 = 0.5 * dtdx * lam[i];
        const double v3 = v1 - v2;
        const double v4 = FOUR_THIRDS * (sq(v1) - sq(v2));
        double fac = 0.0;
        bool first = true;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const int j = S::ord(k);
          if (S::Lnz(i, j)) {
            const double tt = S::L(e, i, j) * (v3 * (c1[j] - c2[j]) + v4 * c2[j]);
            fac = first ? tt : fac + tt;
            first = false;
          }
        }
#pragma unroll
        for (int j = 0; j < NV; ++j)
          if (S::Rnz(j, i)) ria[j] = ria[j] + fac * S::R(e, j, i);
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) { lia[k] = wc[k]; ria[k] = wc[k]; }
  }

}

// ----------------------------------------------------------------------------
// Reconstruction phase B: edge values, monotonicity, characteristic tracing and
// face states.  MODE 2 = PPM (Source/Reconstruction_PPM_MHD_HelperModule.py:391-548),
// MODE 1 = PLM (no reference counterpart: the reference's limited slope taken as a
// linear profile W -/+ s/2, clamped to the neighbours, traced with the reference's
// own tracing with the parabolic coefficient zero -- Stone et al. 2008 eqs. 38-42),
// MODE 0 = first order (cell values copied to both faces, :489-511).
// ----------------------------------------------------------------------------
// work item (x, y) of the cell space nx x ny
template <class S, int AX, int MODE>
__device__ __forceinline__ void b_faces(const Grid& G, const StateBuf& in, int x, int y) {
  if (!G.loop->active) return;
  SweepGeom g;
  g.nx = G.nx;
  g.Ls = AX == 0 ? G.nx : G.ny;
  g.Lt = AX == 0 ? G.ny : G.nx;
  g.bc = AX == 0 ? G.bcx : G.bcy;
  int c, t;
  if (AX == 0) { c = x; t = y; }
  else { t = x; c = y; }
  if (c >= g.Ls || t >= g.Lt) return;
  const size_t plane = cell_plane(G);
  constexpr int NV = S::NV;
  const double dt = G.loop->dt;
  const double dn = AX == 0 ? G.dx : G.dy;
  double lia[NV], ria[NV];
  double wc[NV], wl[NV], wr[NV];
  load_sweep_cell<S, AX>(G, in.prim, plane, c, t, g, wc);
  if (MODE != 0) {
    load_sweep_cell<S, AX>(G, in.prim, plane, c - 1, t, g, wl);
    load_sweep_cell<S, AX>(G, in.prim, plane, c + 1, t, g, wr);
  }
  {
    const size_t es = G.ext_plane;
    const size_t xc = ext_index<AX>(c, t, g.nx);
    const double* sl = AX == 0 ? G.slopes : G.slopes_y;
    const double* eg = AX == 0 ? G.eig : G.eig_y;
    const size_t step = AX == 0 ? 1 : (size_t)g.nx;
    if (MODE != 0) {
      MHD_GUARD(G, sl, xc - step);
      MHD_GUARD(G, sl, xc + step);
      MHD_GUARD(G, eg, xc);
    }
    edge_states<S, MODE>(
        wl, wc, wr, [&](int k, int d) { return sl[k * es + xc + (ptrdiff_t)d * (ptrdiff_t)step]; },
        [&](typename S::Eig& e) { S::load(e, eg + xc, es); }, dt, dn, lia, ria);
  }

  // Face writes: cell c gives the right state of face c and the left state of face c+1;
  // the boundary cells also fill face 0 / face Ls (reference :529-548).
  double* outL = AX == 0 ? G.xl : G.yl;
  double* outR = AX == 0 ? G.xr : G.yr;
  const size_t fplane = AX == 0 ? xface_plane(G) : yface_plane(G);
  const int Ls = g.Ls;
  double s_mid = 0.0, s_lo = 0.0, s_hi = 0.0;
  const bool src = S::SB >= 0 && !G.one_d;   // 1D MHD has no B source terms
  if (src) {
    const double* fb = AX == 0 ? in.fbx : in.fby;
    const double half_dt = 0.5 * dt;
    const double inv_dn = ddiv(1.0, dn);
    s_mid = bsource<AX>(G, in.prim, fb, plane, c, c, c + 1, t, g.nx, half_dt, inv_dn);
    if (c == 0) {
      if (g.bc == OUTFLOW) s_lo = bsource<AX>(G, in.prim, fb, plane, 0, 0, 0, t, g.nx, half_dt, inv_dn);
      else s_hi = bsource<AX>(G, in.prim, fb, plane, 0, Ls, 1, t, g.nx, half_dt, inv_dn);
    }
    if (c == Ls - 1) {
      if (g.bc == OUTFLOW) s_hi = bsource<AX>(G, in.prim, fb, plane, Ls - 1, Ls, Ls, t, g.nx, half_dt, inv_dn);
      else s_lo = bsource<AX>(G, in.prim, fb, plane, Ls - 1, Ls - 1, 0, t, g.nx, half_dt, inv_dn);
    }
  }
  MHD_GUARD(G, outR, face_index<AX>(c, t, g.nx));
  MHD_GUARD(G, outL, face_index<AX>(c + 1, t, g.nx));
  MHD_GUARD(G, outL, face_index<AX>(0, t, g.nx));
  MHD_GUARD(G, outR, face_index<AX>(Ls, t, g.nx));
  unsigned hits = put_face<S>(outR, fplane, face_index<AX>(c, t, g.nx), lia, G.min_d, G.min_p, s_mid, src);
  hits += put_face<S>(outL, fplane, face_index<AX>(c + 1, t, g.nx), ria, G.min_d, G.min_p, s_mid, src);
  if (c == 0) {
    if (g.bc == OUTFLOW) hits += put_face<S>(outL, fplane, face_index<AX>(0, t, g.nx), lia, G.min_d, G.min_p, s_lo, src);
    else hits += put_face<S>(outR, fplane, face_index<AX>(Ls, t, g.nx), lia, G.min_d, G.min_p, s_hi, src);
  }
  if (c == Ls - 1) {
    if (g.bc == OUTFLOW) hits += put_face<S>(outR, fplane, face_index<AX>(Ls, t, g.nx), ria, G.min_d, G.min_p, s_hi, src);
    else hits += put_face<S>(outL, fplane, face_index<AX>(0, t, g.nx), ria, G.min_d, G.min_p, s_lo, src);
  }
  note_floor_hits(G, hits);
}

// ----------------------------------------------------------------------------
// Roe fluxes at every face of one direction.  Stage 1 converts the reconstructed
// prim states with the current face B; stage 2 reads the CTU-corrected cons and
// prim states (converted with the half-step face B in k_ctu_mhd).
// ----------------------------------------------------------------------------
// work item: linear face index f of the x-face (AX 0) or y-face (AX 1) space
template <int AX, int STAGE>
__device__ __forceinline__ void b_roe_mhd(const Grid& G, const StateBuf& in, size_t f) {
  if (!G.loop->active) return;
  const size_t nf = AX == 0 ? xface_plane(G) : yface_plane(G);
  if (f >= nf) return;
  constexpr int N = AX == 0 ? 1 : 2, T1 = AX == 0 ? 2 : 3, T2 = AX == 0 ? 3 : 1;
  const double* WL = AX == 0 ? G.xl : G.yl;
  const double* WR = AX == 0 ? G.xr : G.yr;
  MHD_GUARD(G, WL, f);
  MHD_GUARD(G, WR, f);
  MHD_GUARD(G, AX == 0 ? G.fx : G.fy, f);
  MHD_GUARD(G, STAGE == 1 ? (AX == 0 ? in.fbx : in.fby) : (AX == 0 ? G.nfbx : G.nfby), f);
  if (STAGE == 2) {
    MHD_GUARD(G, AX == 0 ? G.uxl : G.uyl, f);
    MHD_GUARD(G, AX == 0 ? G.uxr : G.uyr, f);
  }
  double wl[7], wr[7], ul[7], ur[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) { wl[k] = WL[k * nf + f]; wr[k] = WR[k * nf + f]; }
  double bn;
  if (STAGE == 1) {
    bn = (AX == 0 ? in.fbx : in.fby)[f];
    prim_to_cons7(wl, bn, G.gamma, ul);
    prim_to_cons7(wr, bn, G.gamma, ur);
  } else {
    bn = (AX == 0 ? G.nfbx : G.nfby)[f];
    const double* UL = AX == 0 ? G.uxl : G.uyl;
    const double* UR = AX == 0 ? G.uxr : G.uyr;
#pragma unroll
    for (int k = 0; k < 7; ++k) { ul[k] = UL[k * nf + f]; ur[k] = UR[k * nf + f]; }
  }
  double flux[7];
  roe_flux<N, T1, T2>(wl, wr, ul, ur, bn, G.gamma, G.efix != 0, G.eps, flux);
  double* F = AX == 0 ? G.fx : G.fy;
#pragma unroll
  for (int k = 0; k < 7; ++k) F[k * nf + f] = flux[k];
}

template <int AX>
__device__ __forceinline__ void b_roe_hydro(const Grid& G, size_t f) {
  if (!G.loop->active) return;
  const size_t nf = AX == 0 ? xface_plane(G) : yface_plane(G);
  if (f >= nf) return;
  const double* WL = AX == 0 ? G.xl : G.yl;
  const double* WR = AX == 0 ? G.xr : G.yr;
  MHD_GUARD(G, WL, f);
  MHD_GUARD(G, WR, f);
  MHD_GUARD(G, AX == 0 ? G.fx : G.fy, f);
  double wl[5], wr[5], flux[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) { wl[k] = WL[k * nf + f]; wr[k] = WR[k * nf + f]; }
  hroe_flux<AX>(wl, wr, G.gamma, G.efix != 0, G.eps, flux);
  double* F = AX == 0 ? G.fx : G.fy;
#pragma unroll
  for (int k = 0; k < 5; ++k) F[k * nf + f] = flux[k];
}

// ----------------------------------------------------------------------------
// Corner EMF (Source/CornerEMF_HelperModule.py:440-529)
// STAGE 1 takes the cell Ez = vy*Bx - vx*By from the primitives
// (Source/EvolveFunctions_MHD.py:541); STAGE 2 the half-step Ez.
// ----------------------------------------------------------------------------
template <int STAGE>
__device__ __forceinline__ double cell_ez(const Grid& G, const StateBuf& in, int j, int i) {
  const size_t idx = (size_t)j * G.nx + i;
  MHD_GUARD_RET(G, G.hez, idx, 0.0);
  if (STAGE == 2) return G.hez[idx];
  const size_t plane = cell_plane(G);
  return __ldg(in.prim + 2 * plane + idx) * __ldg(in.prim + 4 * plane + idx)
       - __ldg(in.prim + 1 * plane + idx) * __ldg(in.prim + 5 * plane + idx);
}

// work item (I, J) of the corner space (nx+1) x (ny+1)
template <int STAGE>
__device__ __forceinline__ void b_emf(const Grid& G, const StateBuf& in, int I, int J) {
  if (!G.loop->active) return;
  const int nx = G.nx, ny = G.ny;
  if (I > nx || J > ny) return;
  const int ic = wrapc(I, nx, G.bcx), im = wrapc(I - 1, nx, G.bcx);
  const int jc = wrapc(J, ny, G.bcy), jm = wrapc(J - 1, ny, G.bcy);
  const size_t yfp = yface_plane(G), xfp = xface_plane(G);
  MHD_GUARD(G, G.fy, (size_t)J * nx + ic);
  MHD_GUARD(G, G.fy, (size_t)J * nx + im);
  MHD_GUARD(G, G.fx, (size_t)jc * (nx + 1) + I);
  MHD_GUARD(G, G.fx, (size_t)jm * (nx + 1) + I);
  MHD_GUARD(G, G.emf, (size_t)J * (nx + 1) + I);
  // y-face fluxes of row J at columns I (top) and I-1 (ltop)
  const double top0 = G.fy[0 * yfp + (size_t)J * nx + ic];
  const double top5 = G.fy[5 * yfp + (size_t)J * nx + ic];
  const double lt0 = G.fy[0 * yfp + (size_t)J * nx + im];
  const double lt5 = G.fy[5 * yfp + (size_t)J * nx + im];
  // x-face fluxes of column I at rows J (left) and J-1 (uleft)
  const double l0 = G.fx[0 * xfp + (size_t)jc * (nx + 1) + I];
  const double l4 = G.fx[4 * xfp + (size_t)jc * (nx + 1) + I];
  const double ul0 = G.fx[0 * xfp + (size_t)jm * (nx + 1) + I];
  const double ul4 = G.fx[4 * xfp + (size_t)jm * (nx + 1) + I];
  const double ec = cell_ez<STAGE>(G, in, jc, ic);
  const double el = cell_ez<STAGE>(G, in, jc, im);
  const double eu = cell_ez<STAGE>(G, in, jm, ic);
  const double eul = cell_ez<STAGE>(G, in, jm, im);
  double x1 = 0.0, x2 = 0.0, y1 = 0.0, y2 = 0.0;
  if (is_pos(lt0)) x1 = lt5 - ul4 - eul;
  else if (is_neg(lt0)) x1 = lt5 - l4 - el;
  else if (is_zero(lt0)) x1 = lt5 - 0.5 * (l4 + ul4 + el + eul);
  if (is_pos(top0)) x2 = top5 - ul4 - eu;
  else if (is_neg(top0)) x2 = top5 - l4 - ec;
  else if (is_zero(top0)) x2 = top5 - 0.5 * (l4 + ul4 + ec + eu);
  if (is_pos(ul0)) y1 = -ul4 + lt5 - eul;
  else if (is_neg(ul0)) y1 = -ul4 + top5 - eu;
  else if (is_zero(ul0)) y1 = -ul4 + 0.5 * (lt5 + top5 - eul - eu);
  if (is_pos(l0)) y2 = -l4 + lt5 - el;
  else if (is_neg(l0)) y2 = -l4 + top5 - ec;
  else if (is_zero(l0)) y2 = -l4 + 0.5 * (lt5 + top5 - el - ec);
  G.emf[(size_t)J * (nx + 1) + I] = 0.25 * (x1 + x2 + y1 + y2);
}

// ----------------------------------------------------------------------------
// CTU transverse predictor for MHD face states (Source/CTU_HelperModule.py:282-444,
// Source/EvolveFunctions_MHD.py:557-592): cons += transverse flux difference +
// source, cons floors, half-step face B, prim with the half-step face B.
// ----------------------------------------------------------------------------
template <int AX>
__device__ __forceinline__ void b_ctu_mhd(const Grid& G, const StateBuf& in, size_t fl) {
  if (!G.loop->active) return;
  const int nx = G.nx, ny = G.ny;
  const size_t nf = AX == 0 ? xface_plane(G) : yface_plane(G);
  if (fl >= nf) return;
  const int width = AX == 0 ? nx + 1 : nx;
  const int row = (int)(fl / width), col = (int)(fl % width);
  // sweep-face index f and transverse index t
  const int f = AX == 0 ? col : row;
  const int t = AX == 0 ? row : col;
  const int Ls = AX == 0 ? nx : ny;
  const int bc = AX == 0 ? G.bcx : G.bcy;
  const double dt = G.loop->dt;
  const double half_dt = 0.5 * dt;
  const double inv_dn = ddiv(1.0, AX == 0 ? G.dx : G.dy);
  const double half_dtdt = 0.5 * ddiv(dt, AX == 0 ? G.dy : G.dx);   // transverse
  const size_t plane = cell_plane(G);
  const double* fb = AX == 0 ? in.fbx : in.fby;
  auto fbv = [&](int ff) -> double {
    const size_t ii = face_index<AX>(ff, t, nx);
#ifdef MHD_CHECKED
    if (!(ii < plane_extent(G, fb))) { report_index(G, __LINE__, ii); return 0.0; }
#endif
    return fb[ii];
  };
  MHD_GUARD(G, fb, fl);
  MHD_GUARD(G, AX == 0 ? G.nfbx : G.nfby, fl);
  MHD_GUARD(G, AX == 0 ? G.xl : G.yl, fl);
  MHD_GUARD(G, AX == 0 ? G.xr : G.yr, fl);
  MHD_GUARD(G, AX == 0 ? G.uxl : G.uyl, fl);
  MHD_GUARD(G, AX == 0 ? G.uxr : G.uyr, fl);
  if (AX == 0) {
    MHD_GUARD(G, G.emf, (size_t)(row + 1) * (nx + 1) + col);
    MHD_GUARD(G, G.emf, (size_t)row * (nx + 1) + col);
  } else {
    MHD_GUARD(G, G.emf, (size_t)row * (nx + 1) + col + 1);
    MHD_GUARD(G, G.emf, (size_t)row * (nx + 1) + col);
  }
  const double bn = fb[fl];

  // half-step face B from the stage-1 corner EMF (Source/EvolveFunctions_MHD.py:579-586)
  double nb;
  if (AX == 0) {
    const double lo = G.emf[(size_t)(row + 1) * (nx + 1) + col];
    const double up = G.emf[(size_t)row * (nx + 1) + col];
    nb = bn - half_dtdt * (lo - up);
    G.nfbx[fl] = nb;
  } else {
    const double r = G.emf[(size_t)row * (nx + 1) + col + 1];
    const double l = G.emf[(size_t)row * (nx + 1) + col];
    nb = bn + half_dtdt * (r - l);
    G.nfby[fl] = nb;
  }

  double* Wout[2] = {AX == 0 ? G.xl : G.yl, AX == 0 ? G.xr : G.yr};
  double* Uout[2] = {AX == 0 ? G.uxl : G.uyl, AX == 0 ? G.uxr : G.uyr};
  unsigned hits = 0;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double w[7], u[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) w[k] = Wout[side][k * nf + fl];
    prim_to_cons7(w, bn, G.gamma, u);

    // padded cell index kpad and its source cell / dB (Source/CTU_HelperModule.py:293-345, :377-430)
    const int kpad = f + side;
    int scell;
    double lb, rb;
    if (AX == 0) {
      scell = wrapc(kpad - 1, Ls, bc);
      if (bc == OUTFLOW) {
        lb = fbv(kpad - 1 < 0 ? 0 : (kpad - 1 > Ls ? Ls : kpad - 1));
        rb = fbv(kpad > Ls ? Ls : kpad);
      } else {
        lb = fbv(kpad == 0 ? Ls - 1 : kpad - 1);
        rb = fbv(kpad == Ls + 1 ? 1 : kpad);
      }
    } else {
      if (bc == OUTFLOW) {
        scell = kpad == 0 ? 1 : (kpad - 1 > Ls - 1 ? Ls - 1 : kpad - 1);
        lb = fbv(kpad == 0 ? 1 : kpad - 1);
        rb = fbv(kpad == Ls + 1 ? Ls - 1 : kpad);
      } else {
        scell = wrapc(kpad - 1, Ls, bc);
        lb = fbv(kpad == 0 ? Ls - 1 : kpad - 1);
        rb = fbv(kpad == Ls + 1 ? 1 : kpad);
      }
    }
    const double dB = rb - lb;
    const size_t sidx = cell_index<AX>(scell, t, nx);
    MHD_GUARD(G, in.prim, sidx);
    const double cbx = __ldg(in.prim + 4 * plane + sidx);
    const double cby = __ldg(in.prim + 5 * plane + sidx);
    const double cbz = __ldg(in.prim + 6 * plane + sidx);
    const double cvz = __ldg(in.prim + 3 * plane + sidx);
    double src[7];
    src[0] = 0.0;
    src[1] = cbx * dB * inv_dn;
    src[2] = cby * dB * inv_dn;
    src[3] = cbz * dB * inv_dn;
    src[4] = AX == 0 ? 0.0 : cvz * dB * inv_dn;
    src[5] = AX == 0 ? cvz * dB * inv_dn : 0.0;
    src[6] = (cbz * cvz) * dB * inv_dn;

    // transverse flux difference of the cell on this side (standard wrap/clamp)
    const int fc = wrapc(f - 1 + side, Ls, bc);
    const double* F = AX == 0 ? G.fy : G.fx;
    const size_t tfp = AX == 0 ? yface_plane(G) : xface_plane(G);
    size_t i_lo, i_hi;  // lower/upper transverse face of cell (fc, t)
    if (AX == 0) { i_lo = (size_t)t * nx + fc; i_hi = (size_t)(t + 1) * nx + fc; }
    else { i_lo = (size_t)fc * (nx + 1) + t; i_hi = (size_t)fc * (nx + 1) + t + 1; }
    MHD_GUARD(G, F, i_lo);
    MHD_GUARD(G, F, i_hi);
    double fh[7], flo[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) { fh[k] = F[k * tfp + i_hi]; flo[k] = F[k * tfp + i_lo]; }
    // remap: x-sweep takes the y-flux Bz (slot 4) into slot 5 and zeroes slot 4;
    // y-sweep takes the x-flux Bz (slot 5) into slot 4 and zeroes slot 5
    if (AX == 0) { fh[5] = fh[4]; fh[4] = 0.0; flo[5] = flo[4]; flo[4] = 0.0; }
    else { fh[4] = fh[5]; fh[5] = 0.0; flo[4] = flo[5]; flo[5] = 0.0; }
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const bool zero_src = (k == 0) || (AX == 0 ? k == 4 : k == 5);
      const double corr = zero_src ? (-half_dtdt * (fh[k] - flo[k]))
                                   : (-half_dtdt * (fh[k] - flo[k]) + half_dt * src[k]);
      u[k] = u[k] + corr;
    }
    if (dlt(u[0], G.min_d)) { u[0] = G.min_d; ++hits; }
    if (dlt(u[6], G.min_e)) { u[6] = G.min_e; ++hits; }
    double w2[7];
    cons_to_prim7(u, nb, G.gamma, w2);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      Uout[side][k * nf + fl] = u[k];
      Wout[side][k * nf + fl] = w2[k];
    }
  }
  note_floor_hits(G, hits);
}

// Hydro CTU (Source/EvolveFunctions_Hydro.py:460-489): cons -= half dt/dn * transverse
// flux difference, back to prim.
template <int AX>
__device__ __forceinline__ void b_ctu_hydro(const Grid& G, size_t fl) {
  if (!G.loop->active) return;
  const int nx = G.nx;
  const size_t nf = AX == 0 ? xface_plane(G) : yface_plane(G);
  if (fl >= nf) return;
  const int width = AX == 0 ? nx + 1 : nx;
  const int row = (int)(fl / width), col = (int)(fl % width);
  const int f = AX == 0 ? col : row;
  const int t = AX == 0 ? row : col;
  const int Ls = AX == 0 ? G.nx : G.ny;
  const int bc = AX == 0 ? G.bcx : G.bcy;
  const double dt = G.loop->dt;
  const double half_dtdt = 0.5 * ddiv(dt, AX == 0 ? G.dy : G.dx);
  double* Wout[2] = {AX == 0 ? G.xl : G.yl, AX == 0 ? G.xr : G.yr};
  const double* F = AX == 0 ? G.fy : G.fx;
  const size_t tfp = AX == 0 ? yface_plane(G) : xface_plane(G);
  MHD_GUARD(G, Wout[0], fl);
  MHD_GUARD(G, Wout[1], fl);
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double w[5], u[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) w[k] = Wout[side][k * nf + fl];
    hprim_to_cons<AX>(w, G.gamma, u);
    const int fc = wrapc(f - 1 + side, Ls, bc);
    size_t i_lo, i_hi;
    if (AX == 0) { i_lo = (size_t)t * nx + fc; i_hi = (size_t)(t + 1) * nx + fc; }
    else { i_lo = (size_t)fc * (nx + 1) + t; i_hi = (size_t)fc * (nx + 1) + t + 1; }
    MHD_GUARD(G, F, i_lo);
    MHD_GUARD(G, F, i_hi);
#pragma unroll
    for (int k = 0; k < 5; ++k) u[k] = u[k] - half_dtdt * (F[k * tfp + i_hi] - F[k * tfp + i_lo]);
    hcons_to_prim<AX>(u, G.gamma, w);
#pragma unroll
    for (int k = 0; k < 5; ++k) Wout[side][k * nf + fl] = w[k];
  }
}

// ----------------------------------------------------------------------------
// Half-step cell Ez (Source/EvolveFunctions_MHD.py:594-624)
// ----------------------------------------------------------------------------
__device__ __forceinline__ void b_half_ez(const Grid& G, const StateBuf& in, int i, int j) {
  if (!G.loop->active) return;
  const int nx = G.nx;
  if (i >= nx || j >= G.ny) return;
  const double dt = G.loop->dt;
  const double hx = 0.5 * ddiv(dt, G.dx), hy = 0.5 * ddiv(dt, G.dy);
  const size_t plane = cell_plane(G), xfp = xface_plane(G), yfp = yface_plane(G);
  const size_t idx = (size_t)j * nx + i;
  const size_t xr = (size_t)j * (nx + 1) + i + 1, xlf = (size_t)j * (nx + 1) + i;
  const size_t yb = (size_t)(j + 1) * nx + i, yt = (size_t)j * nx + i;
  MHD_GUARD(G, in.cons, idx);
  MHD_GUARD(G, G.hez, idx);
  MHD_GUARD(G, G.fx, xr);
  MHD_GUARD(G, G.fx, xlf);
  MHD_GUARD(G, G.fy, yb);
  MHD_GUARD(G, G.fy, yt);
  MHD_GUARD(G, G.nfbx, xr);
  MHD_GUARD(G, G.nfbx, xlf);
  MHD_GUARD(G, G.nfby, yb);
  MHD_GUARD(G, G.nfby, yt);
  double hu[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double u = __ldg(in.cons + k * plane + idx);
    u = u - hx * (G.fx[k * xfp + xr] - G.fx[k * xfp + xlf]);
    u = u - hy * (G.fy[k * yfp + yb] - G.fy[k * yfp + yt]);
    hu[k] = u;
  }
  const double hbx = (G.nfbx[xlf] + G.nfbx[xr]) * 0.5;   // x / 2 exactly
  const double hby = (G.nfby[yt] + G.nfby[yb]) * 0.5;
  const double hvx = ddiv(hu[1], hu[0]);
  const double hvy = ddiv(hu[2], hu[0]);
  G.hez[idx] = hvy * hbx - hvx * hby;
}

// ----------------------------------------------------------------------------
// Final update (Source/EvolveFunctions_MHD.py:643-687; Hydro :502-506)
// ----------------------------------------------------------------------------
__device__ __forceinline__ void b_final_mhd(const Grid& G, const StateBuf& in, const StateBuf& out, int i,
                                            int j) {
  if (!G.loop->active) return;
  const int nx = G.nx, ny = G.ny;
  if (i >= nx || j >= ny) return;
  const double dt = G.loop->dt;
  const double dtdy = ddiv(dt, G.dy), dtdx = ddiv(dt, G.dx);
  const size_t plane = cell_plane(G), xfp = xface_plane(G), yfp = yface_plane(G);
  const size_t idx = (size_t)j * nx + i;
  const size_t xlf = (size_t)j * (nx + 1) + i, xr = xlf + 1;
  const size_t yt = (size_t)j * nx + i, yb = (size_t)(j + 1) * nx + i;
  const size_t cw = nx + 1;
  const double* E = G.emf;
  MHD_GUARD(G, in.cons, idx);
  MHD_GUARD(G, out.prim, idx);
  MHD_GUARD(G, out.cons, idx);
  MHD_GUARD(G, in.fbx, xlf);
  MHD_GUARD(G, in.fbx, xr);
  MHD_GUARD(G, in.fby, yt);
  MHD_GUARD(G, in.fby, yb);
  MHD_GUARD(G, out.fbx, xlf);
  MHD_GUARD(G, out.fbx, xr);
  MHD_GUARD(G, out.fby, yt);
  MHD_GUARD(G, out.fby, yb);
  MHD_GUARD(G, G.fx, xlf);
  MHD_GUARD(G, G.fx, xr);
  MHD_GUARD(G, G.fy, yt);
  MHD_GUARD(G, G.fy, yb);
  MHD_GUARD(G, E, (size_t)j * cw + i);
  MHD_GUARD(G, E, (size_t)(j + 1) * cw + i + 1);
  // full-step face B (Source/EvolveFunctions_MHD.py:644-645)
  const double bxl = in.fbx[xlf] - dtdy * (E[(size_t)(j + 1) * cw + i] - E[(size_t)j * cw + i]);
  const double bxr = in.fbx[xr] - dtdy * (E[(size_t)(j + 1) * cw + i + 1] - E[(size_t)j * cw + i + 1]);
  const double byt = in.fby[yt] + dtdx * (E[(size_t)j * cw + i + 1] - E[(size_t)j * cw + i]);
  const double byb = in.fby[yb] + dtdx * (E[(size_t)(j + 1) * cw + i + 1] - E[(size_t)(j + 1) * cw + i]);
  out.fbx[xlf] = bxl;
  if (i == nx - 1) out.fbx[xr] = bxr;
  out.fby[yt] = byt;
  if (j == ny - 1) out.fby[yb] = byb;
  const double cbx = (bxl + bxr) * 0.5;   // x / 2 exactly
  const double cby = (byt + byb) * 0.5;
  // conservative update of the x-sweep cons vector [rho, mx, my, mz, By, Bz, E]
  const int cslot[7] = {0, 1, 2, 3, 5, 6, 7};
  double u[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) u[k] = __ldg(in.cons + cslot[k] * plane + idx);
  const double bz = u[5] - dtdx * (G.fx[5 * xfp + xr] - G.fx[5 * xfp + xlf])
                         - dtdy * (G.fy[4 * yfp + yb] - G.fy[4 * yfp + yt]);
  const int upd[5] = {0, 1, 2, 3, 6};
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    const int k = upd[q];
    double v = u[k] - dtdx * (G.fx[k * xfp + xr] - G.fx[k * xfp + xlf]);
    v = v - dtdy * (G.fy[k * yfp + yb] - G.fy[k * yfp + yt]);
    u[k] = v;
  }
  u[5] = bz;
  u[4] = cby;
  double w[7];
  cons_to_prim7(u, cbx, G.gamma, w);
  const double po[8] = {w[0], w[1], w[2], w[3], cbx, w[4], w[5], w[6]};
  const double co[8] = {u[0], u[1], u[2], u[3], cbx, u[4], u[5], u[6]};
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    out.prim[k * plane + idx] = po[k];
    out.cons[k * plane + idx] = co[k];
    bad |= is_nonfinite(co[k]) | is_nonfinite(po[k]);
  }
  if (i == nx - 1) bad |= is_nonfinite(bxr);
  if (j == ny - 1) bad |= is_nonfinite(byb);
  note_nonfinite(G, bad | is_nonfinite(bxl) | is_nonfinite(byt));
}

__device__ __forceinline__ void b_final_hydro(const Grid& G, const StateBuf& in, const StateBuf& out, int i,
                                              int j) {
  if (!G.loop->active) return;
  const int nx = G.nx;
  if (i >= nx || j >= G.ny) return;
  const double dt = G.loop->dt;
  const double dtdx = ddiv(dt, G.dx), dtdy = ddiv(dt, G.dy);
  const size_t plane = cell_plane(G), xfp = xface_plane(G), yfp = yface_plane(G);
  const size_t idx = (size_t)j * nx + i;
  const size_t xlf = (size_t)j * (nx + 1) + i, xr = xlf + 1;
  const size_t yt = (size_t)j * nx + i, yb = (size_t)(j + 1) * nx + i;
  MHD_GUARD(G, in.cons, idx);
  MHD_GUARD(G, out.prim, idx);
  MHD_GUARD(G, out.cons, idx);
  MHD_GUARD(G, G.fx, xlf);
  MHD_GUARD(G, G.fx, xr);
  MHD_GUARD(G, G.fy, yt);
  MHD_GUARD(G, G.fy, yb);
  double u[5], w[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double v = __ldg(in.cons + k * plane + idx);
    v = v - dtdx * (G.fx[k * xfp + xr] - G.fx[k * xfp + xlf]);
    v = v - dtdy * (G.fy[k * yfp + yb] - G.fy[k * yfp + yt]);
    u[k] = v;
  }
  hcons_to_prim<0>(u, G.gamma, w);
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    out.prim[k * plane + idx] = w[k];
    out.cons[k * plane + idx] = u[k];
    bad |= is_nonfinite(u[k]) | is_nonfinite(w[k]);
  }
  note_nonfinite(G, bad);
}

// ----------------------------------------------------------------------------
// CFL reduction (Source/TimestepCalculations_HelperModule.py:67-109, :239-289):
// per-cell max signal speeds, warp-shuffle + block max, one atomicMax per block on
// the bit pattern (non-negative doubles order like their 64-bit integers).
// ----------------------------------------------------------------------------
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// largest signal speeds of cell idx folded into (mx, my)
template <int PHYS>
__device__ __forceinline__ void b_dt_cell(const Grid& G, const StateBuf& in, size_t idx, double& mx, double& my) {
  const int nx = G.nx;
  const size_t plane = cell_plane(G);
  const double gamma = G.gamma;
  const double* c = in.cons;
  MHD_GUARD(G, c, idx);
  if (PHYS == MHD) {
    MHD_GUARD(G, in.fbx, (size_t)(idx / nx) * (nx + 1) + idx % nx);
    MHD_GUARD(G, in.fby, idx);
  }
  const double inv_d = ddiv(1.0, c[idx]);
  const double vx = c[plane + idx] * inv_d;
  const double vy = c[2 * plane + idx] * inv_d;
  const double vz = c[3 * plane + idx] * inv_d;
  const double vsq = vx * vx + vy * vy + vz * vz;
  if (PHYS == MHD) {
    const int j = (int)(idx / nx), i = (int)(idx % nx);
    const double c4 = c[4 * plane + idx], c5 = c[5 * plane + idx];
    const double bx = c4 + fabs(in.fbx[(size_t)j * (nx + 1) + i] - c4);
    const double by = c5 + fabs(in.fby[(size_t)j * nx + i] - c5);
    const double bz = c[6 * plane + idx];
    const double bsq = bx * bx + by * by + bz * bz;
    const double p = dmax((gamma - 1.0) * (c[7 * plane + idx] - 0.5 * c[idx] * vsq - 0.5 * bsq), SMALL_VALUE);
    const double a2 = gamma * p * inv_d;
    const double ssum = bsq * inv_d + a2;
    const double sdiff = bsq * inv_d - a2;
    const double cfx2 = 0.5 * (ssum + sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d));
    const double cfy2 = 0.5 * (ssum + sqrt(sdiff * sdiff + 4.0 * a2 * (bx * bx + bz * bz) * inv_d));
    mx = dmax(mx, fabs(vx) + sqrt(cfx2));
    my = dmax(my, fabs(vy) + sqrt(cfy2));
  } else {
    const double p = dmax((gamma - 1.0) * (c[4 * plane + idx] - 0.5 * c[idx] * vsq), SMALL_VALUE);
    const double a = sqrt(gamma * p * inv_d);
    mx = dmax(mx, fabs(vx) + a);
    my = dmax(my, fabs(vy) + a);
  }
}

// block max of (mx, my), then one atomicMax per block on the loop state
__device__ __forceinline__ void block_max_to_loop(double mx, double my, LoopState* L) {
  __shared__ double sx[32], sy[32];
  mx = warp_max(mx);
  my = warp_max(my);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sx[wid] = mx; sy[wid] = my; }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    mx = lane < nw ? sx[lane] : 0.0;
    my = lane < nw ? sy[lane] : 0.0;
    mx = warp_max(mx);
    my = warp_max(my);
    if (lane == 0) {
      atomicMax(&L->max_sx, (unsigned long long)__double_as_longlong(mx));
      atomicMax(&L->max_sy, (unsigned long long)__double_as_longlong(my));
    }
  }
  __syncthreads();
}

__device__ __forceinline__ bool loop_running(const LoopState* L) {
  return L->t < L->t_end && L->cycle < L->max_cycles;
}

// dt from the reduced speeds, the tEnd clip, and the loop condition
// (Source/EvolveFunctions_MHD.py:466-479).
template <int PHYS>
__device__ __forceinline__ void b_begin(const Grid& G) {
  LoopState* L = G.loop;
  const int act = loop_running(L) ? 1 : 0;
  L->active = act;
  if (act) {
    const double mx = __longlong_as_double((long long)L->max_sx);
    const double my = __longlong_as_double((long long)L->max_sy);
    double dt;
    if (is_pos(L->dt_fixed)) {
      dt = L->dt_fixed;
    } else if (PHYS == MHD) {
      const double inv = dmax(ddiv(mx, G.dx), ddiv(my, G.dy));
      dt = ddiv(L->cfl, inv);
    } else {
      const double dtx = ddiv(L->cfl, ddiv(mx, G.dx));
      const double dty = ddiv(L->cfl, ddiv(my, G.dy));
      dt = dmin(dtx, dty);
    }
    if (L->t + dt > L->t_end) dt = L->t_end - L->t;
    L->dt = dt;
  }
  L->max_sx = 0ull;
  L->max_sy = 0ull;
}

__device__ __forceinline__ void b_end(const Grid& G) {
  LoopState* L = G.loop;
  if (!L->active) return;
  if (G.dt_log && L->cycle >= 0 && L->cycle < G.dt_log_cap) {
#ifdef MHD_CHECKED
    // (no early return here: the loop bookkeeping below must run)
    if (!((size_t)L->cycle < plane_extent(G, G.dt_log))) report_index(G, __LINE__, (size_t)L->cycle);
    else
#endif
    G.dt_log[L->cycle] = L->dt;
  }
  L->t_prev = L->t;
  L->t = L->t + L->dt;
  L->cycle = L->cycle + 1;
  L->cycles_run = L->cycles_run + 1;
  L->cur ^= 1;
  L->active = 0;
}

// MHD_BODIES_ONLY: a translation unit that wants the sweep policies and the
// per-item bodies above without these kernels (the 3D step) defines it.
#ifndef MHD_BODIES_ONLY
// ============================================================================
// Plain kernels: one grid per launch, work item from the block/thread index.
// ============================================================================
template <int PHYS>
__global__ void __launch_bounds__(256) k_dt_reduce(Grid G, StateBuf in) {
  if (!loop_running(G.loop)) return;
  const size_t n = cell_plane(G);
  double mx = 0.0, my = 0.0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x)
    b_dt_cell<PHYS>(G, in, idx, mx, my);
  block_max_to_loop(mx, my, G.loop);
}
template <int PHYS>
__global__ void k_begin(Grid G) { b_begin<PHYS>(G); }
__global__ void k_end(Grid G) { b_end(G); }

template <class S, int AX>
__global__ void __launch_bounds__(kBlock, kMinBlocksSlopes) k_ppm_slopes(Grid G, StateBuf in) {
  b_ppm_slopes<S, AX>(G, in, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}
template <class S, int AX, int MODE>
__global__ void __launch_bounds__(kBlock, kMinBlocksFaces) k_faces(Grid G, StateBuf in) {
  b_faces<S, AX, MODE>(G, in, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}
template <int AX, int STAGE>
__global__ void __launch_bounds__(kBlock, kMinBlocksRoe) k_roe_mhd(Grid G, StateBuf in) {
  b_roe_mhd<AX, STAGE>(G, in, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int AX>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_roe_hydro(Grid G) {
  b_roe_hydro<AX>(G, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int STAGE>
__global__ void __launch_bounds__(kBlock) k_emf(Grid G, StateBuf in) {
  b_emf<STAGE>(G, in, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}
template <int AX>
__global__ void __launch_bounds__(kBlock) k_ctu_mhd(Grid G, StateBuf in) {
  b_ctu_mhd<AX>(G, in, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int AX>
__global__ void __launch_bounds__(kBlock) k_ctu_hydro(Grid G) {
  b_ctu_hydro<AX>(G, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(kBlock) k_half_ez(Grid G, StateBuf in) {
  b_half_ez(G, in, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(kBlock) k_final_mhd(Grid G, StateBuf in, StateBuf out) {
  b_final_mhd(G, in, out, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(kBlock) k_final_hydro(Grid G, StateBuf in, StateBuf out) {
  b_final_hydro(G, in, out, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// ----------------------------------------------------------------------------
// 1D grids (ny = 1): the reference's evolve_1D_mhd / evolve_1D_hydro
// (Source/EvolveFunctions_MHD.py:195-340, Source/EvolveFunctions_Hydro.py:232-305):
// x-sweep reconstruction and Roe fluxes, then cons -= dt/dx (F_right - F_left).
// ----------------------------------------------------------------------------
// largest x signal speed of cell i (Source/TimestepCalculations_HelperModule.py:24-56,
// :183-225: B from the cell's conserved B, no face B)
template <int PHYS>
__device__ __forceinline__ void b_dt_cell_1d(const Grid& G, const StateBuf& in, size_t i, double& mx) {
  const size_t plane = cell_plane(G);
  const double gamma = G.gamma;
  const double* c = in.cons;
  MHD_GUARD(G, c, i);
  const double inv_d = ddiv(1.0, c[i]);
  const double vx = c[plane + i] * inv_d;
  const double vy = c[2 * plane + i] * inv_d;
  const double vz = c[3 * plane + i] * inv_d;
  const double vsq = vx * vx + vy * vy + vz * vz;
  if (PHYS == MHD) {
    const double bx = c[4 * plane + i], by = c[5 * plane + i], bz = c[6 * plane + i];
    const double bsq = bx * bx + by * by + bz * bz;
    const double p = dmax((gamma - 1.0) * (c[7 * plane + i] - 0.5 * c[i] * vsq - 0.5 * bsq), SMALL_VALUE);
    const double a2 = gamma * p * inv_d;
    const double ssum = bsq * inv_d + a2;
    const double sdiff = bsq * inv_d - a2;
    const double cf2 = 0.5 * (ssum + sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d));
    mx = dmax(mx, fabs(vx) + sqrt(cf2));
  } else {
    const double p = dmax((gamma - 1.0) * (c[4 * plane + i] - 0.5 * c[i] * vsq), SMALL_VALUE);
    mx = dmax(mx, fabs(vx) + sqrt(gamma * p * inv_d));
  }
}

template <int PHYS>
__global__ void __launch_bounds__(256) k_dt_reduce_1d(Grid G, StateBuf in) {
  if (!loop_running(G.loop)) return;
  double mx = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)G.nx; i += (size_t)gridDim.x * blockDim.x)
    b_dt_cell_1d<PHYS>(G, in, i, mx);
  // the y maximum stays 0, so the 2D dt rule reduces to cfl / (max_x / dx)
  block_max_to_loop(mx, 0.0, G.loop);
}

template <int PHYS>
__global__ void __launch_bounds__(kBlock) k_update_1d(Grid G, StateBuf in, StateBuf out) {
  if (!G.loop->active) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nx) return;
  const double dtdx = ddiv(G.loop->dt, G.dx);
  const size_t plane = cell_plane(G), fp = xface_plane(G);
  MHD_GUARD(G, in.cons, (size_t)i);
  MHD_GUARD(G, out.prim, (size_t)i);
  MHD_GUARD(G, out.cons, (size_t)i);
  MHD_GUARD(G, G.fx, (size_t)i + 1);
  if (PHYS == MHD) {
    constexpr int src[7] = {0, 1, 2, 3, 5, 6, 7};
    double u[7], w[7];
#pragma unroll
    for (int k = 0; k < 7; ++k)
      u[k] = __ldg(in.cons + src[k] * plane + i) - dtdx * (G.fx[k * fp + i + 1] - G.fx[k * fp + i]);
    cons_to_prim7(u, G.bx1d, G.gamma, w);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      out.prim[src[k] * plane + i] = w[k];
      out.cons[src[k] * plane + i] = u[k];
      bad |= is_nonfinite(u[k]) | is_nonfinite(w[k]);
    }
    out.prim[4 * plane + i] = G.bx1d;
    out.cons[4 * plane + i] = G.bx1d;
    note_nonfinite(G, bad);
  } else {
    double u[5], w[5];
#pragma unroll
    for (int k = 0; k < 5; ++k)
      u[k] = __ldg(in.cons + k * plane + i) - dtdx * (G.fx[k * fp + i + 1] - G.fx[k * fp + i]);
    hcons_to_prim<0>(u, G.gamma, w);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      out.prim[k * plane + i] = w[k];
      out.cons[k * plane + i] = u[k];
      bad |= is_nonfinite(u[k]) | is_nonfinite(w[k]);
    }
    note_nonfinite(G, bad);
  }
}

// ----------------------------------------------------------------------------
// Host-side enqueue of one cycle reading state buffer `parity`.
// ----------------------------------------------------------------------------
inline dim3 row_grid(int n, int rows) { return dim3((unsigned)((n + kBlock - 1) / kBlock), (unsigned)rows); }
inline unsigned lin_grid(size_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

template <int PHYS>
void enqueue_recon(const Grid& g, const StateBuf& in, cudaStream_t s) {
  using SX = typename std::conditional<PHYS == MHD, MhdSweep<0>, HydroSweep<0>>::type;
  using SY = typename std::conditional<PHYS == MHD, MhdSweep<1>, HydroSweep<1>>::type;
  if (g.recon == 2) {
    k_ppm_slopes<SX, 0><<<row_grid(g.nx + 2, g.ny), kBlock, 0, s>>>(g, in);
    k_faces<SX, 0, 2><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
    k_ppm_slopes<SY, 1><<<row_grid(g.nx, g.ny + 2), kBlock, 0, s>>>(g, in);
    k_faces<SY, 1, 2><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
  } else if (g.recon == 1) {
    k_ppm_slopes<SX, 0><<<row_grid(g.nx + 2, g.ny), kBlock, 0, s>>>(g, in);
    k_faces<SX, 0, 1><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
    k_ppm_slopes<SY, 1><<<row_grid(g.nx, g.ny + 2), kBlock, 0, s>>>(g, in);
    k_faces<SY, 1, 1><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
  } else {
    k_faces<SX, 0, 0><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
    k_faces<SY, 1, 0><<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
  }
}

template <int PHYS>
void enqueue_cycle_1d(const Grid& g, const StateBuf& in, const StateBuf& out, int dt_blocks, cudaStream_t s) {
  using SX = typename std::conditional<PHYS == MHD, MhdSweep<0>, HydroSweep<0>>::type;
  k_dt_reduce_1d<PHYS><<<dt_blocks, 256, 0, s>>>(g, in);
  k_begin<PHYS><<<1, 1, 0, s>>>(g);
  if (g.recon >= 1) k_ppm_slopes<SX, 0><<<row_grid(g.nx + 2, 1), kBlock, 0, s>>>(g, in);
  if (g.recon == 2) k_faces<SX, 0, 2><<<row_grid(g.nx, 1), kBlock, 0, s>>>(g, in);
  else if (g.recon == 1) k_faces<SX, 0, 1><<<row_grid(g.nx, 1), kBlock, 0, s>>>(g, in);
  else k_faces<SX, 0, 0><<<row_grid(g.nx, 1), kBlock, 0, s>>>(g, in);
  if (PHYS == MHD) k_roe_mhd<0, 1><<<lin_grid(xface_plane(g)), kBlock, 0, s>>>(g, in);
  else k_roe_hydro<0><<<lin_grid(xface_plane(g)), kBlock, 0, s>>>(g);
  k_update_1d<PHYS><<<lin_grid(g.nx), kBlock, 0, s>>>(g, in, out);
  k_end<<<1, 1, 0, s>>>(g);
}

void enqueue_cycle(const Grid& g, int parity, int dt_blocks, cudaStream_t s) {
  const StateBuf in = g.st[parity];
  const StateBuf out = g.st[parity ^ 1];
  if (g.one_d) {
    if (g.physics == MHD) enqueue_cycle_1d<MHD>(g, in, out, dt_blocks, s);
    else enqueue_cycle_1d<HYDRO>(g, in, out, dt_blocks, s);
    return;
  }
  const size_t nxf = xface_plane(g), nyf = yface_plane(g);
  if (g.physics == MHD) {
    k_dt_reduce<MHD><<<dt_blocks, 256, 0, s>>>(g, in);
    k_begin<MHD><<<1, 1, 0, s>>>(g);
    enqueue_recon<MHD>(g, in, s);
    k_roe_mhd<0, 1><<<lin_grid(nxf), kBlock, 0, s>>>(g, in);
    k_roe_mhd<1, 1><<<lin_grid(nyf), kBlock, 0, s>>>(g, in);
    k_emf<1><<<row_grid(g.nx + 1, g.ny + 1), kBlock, 0, s>>>(g, in);
    k_ctu_mhd<0><<<lin_grid(nxf), kBlock, 0, s>>>(g, in);
    k_ctu_mhd<1><<<lin_grid(nyf), kBlock, 0, s>>>(g, in);
    k_half_ez<<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in);
    k_roe_mhd<0, 2><<<lin_grid(nxf), kBlock, 0, s>>>(g, in);
    k_roe_mhd<1, 2><<<lin_grid(nyf), kBlock, 0, s>>>(g, in);
    k_emf<2><<<row_grid(g.nx + 1, g.ny + 1), kBlock, 0, s>>>(g, in);
    k_final_mhd<<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in, out);
  } else {
    k_dt_reduce<HYDRO><<<dt_blocks, 256, 0, s>>>(g, in);
    k_begin<HYDRO><<<1, 1, 0, s>>>(g);
    enqueue_recon<HYDRO>(g, in, s);
    k_roe_hydro<0><<<lin_grid(nxf), kBlock, 0, s>>>(g);
    k_roe_hydro<1><<<lin_grid(nyf), kBlock, 0, s>>>(g);
    k_ctu_hydro<0><<<lin_grid(nxf), kBlock, 0, s>>>(g);
    k_ctu_hydro<1><<<lin_grid(nyf), kBlock, 0, s>>>(g);
    k_roe_hydro<0><<<lin_grid(nxf), kBlock, 0, s>>>(g);
    k_roe_hydro<1><<<lin_grid(nyf), kBlock, 0, s>>>(g);
    k_final_hydro<<<row_grid(g.nx, g.ny), kBlock, 0, s>>>(g, in, out);
  }
  k_end<<<1, 1, 0, s>>>(g);
}

// ============================================================================
// Batched persistent kernels: many grids (instances) in one launch per stage.
// Each launch walks a work list of tiles -- int4 {instance, row, x0, 0}: one
// row segment of kBlock work items of one instance's index space -- with a
// grid of resident blocks striding through the list.  The per-item bodies are
// the ones above, so a batched cycle computes exactly what the plain cycle
// computes for every instance.  Instances keep their own dt, time, cycle count
// and current state buffer in their own LoopState.
// ============================================================================
#define MHD_TILE_LOOP(space)                                                  \
  for (int ti = blockIdx.x; ti < V.ntiles[space]; ti += gridDim.x)           \
    if (const int4 tl = V.tiles[space][ti]; true)

template <int PHYS>
__global__ void __launch_bounds__(kBlock) kb_dt_reduce(BatchView V) {
  MHD_TILE_LOOP(SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    if (!loop_running(G.loop)) continue;   // uniform across the block
    double mx = 0.0, my = 0.0;
    const int i = tl.z + threadIdx.x;
    if (i < G.nx) b_dt_cell<PHYS>(G, G.st[G.loop->cur], (size_t)tl.y * G.nx + i, mx, my);
    block_max_to_loop(mx, my, G.loop);
  }
}
template <int PHYS>
__global__ void kb_begin(BatchView V) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < V.ninst) b_begin<PHYS>(V.grids[k]);
}
__global__ void kb_end(BatchView V) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < V.ninst) b_end(V.grids[k]);
}
template <class S, int AX>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_ppm_slopes(BatchView V) {
  MHD_TILE_LOOP(AX == 0 ? SPACE_EXT_X : SPACE_EXT_Y) {
    const Grid& G = V.grids[tl.x];
    b_ppm_slopes<S, AX>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
template <class S, int AX, int MODE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_faces(BatchView V) {
  MHD_TILE_LOOP(SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    b_faces<S, AX, MODE>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
template <int AX, int STAGE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_roe_mhd(BatchView V) {
  MHD_TILE_LOOP(AX == 0 ? SPACE_XFACE : SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int w = AX == 0 ? G.nx + 1 : G.nx;
    const int x = tl.z + threadIdx.x;
    if (x < w) b_roe_mhd<AX, STAGE>(G, G.st[G.loop->cur], (size_t)tl.y * w + x);
  }
}
template <int AX>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_roe_hydro(BatchView V) {
  MHD_TILE_LOOP(AX == 0 ? SPACE_XFACE : SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int w = AX == 0 ? G.nx + 1 : G.nx;
    const int x = tl.z + threadIdx.x;
    if (x < w) b_roe_hydro<AX>(G, (size_t)tl.y * w + x);
  }
}
template <int STAGE>
__global__ void __launch_bounds__(kBlock) kb_emf(BatchView V) {
  MHD_TILE_LOOP(SPACE_CORNER) {
    const Grid& G = V.grids[tl.x];
    b_emf<STAGE>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
template <int AX>
__global__ void __launch_bounds__(kBlock) kb_ctu_mhd(BatchView V) {
  MHD_TILE_LOOP(AX == 0 ? SPACE_XFACE : SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int w = AX == 0 ? G.nx + 1 : G.nx;
    const int x = tl.z + threadIdx.x;
    if (x < w) b_ctu_mhd<AX>(G, G.st[G.loop->cur], (size_t)tl.y * w + x);
  }
}
template <int AX>
__global__ void __launch_bounds__(kBlock) kb_ctu_hydro(BatchView V) {
  MHD_TILE_LOOP(AX == 0 ? SPACE_XFACE : SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int w = AX == 0 ? G.nx + 1 : G.nx;
    const int x = tl.z + threadIdx.x;
    if (x < w) b_ctu_hydro<AX>(G, (size_t)tl.y * w + x);
  }
}
__global__ void __launch_bounds__(kBlock) kb_half_ez(BatchView V) {
  MHD_TILE_LOOP(SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    b_half_ez(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
__global__ void __launch_bounds__(kBlock) kb_final_mhd(BatchView V) {
  MHD_TILE_LOOP(SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    b_final_mhd(G, G.st[G.loop->cur], G.st[G.loop->cur ^ 1], tl.z + threadIdx.x, tl.y);
  }
}
__global__ void __launch_bounds__(kBlock) kb_final_hydro(BatchView V) {
  MHD_TILE_LOOP(SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    b_final_hydro(G, G.st[G.loop->cur], G.st[G.loop->cur ^ 1], tl.z + threadIdx.x, tl.y);
  }
}

// ---- fusion depth 2: the independent x and y launches of a stage in one launch,
// walking the x work list and then the y work list.
#define MHD_PAIR_LOOP(SA, SB)                                                       \
  for (int ti = blockIdx.x; ti < V.ntiles[SA] + V.ntiles[SB]; ti += gridDim.x)      \
    if (const bool first = ti < V.ntiles[SA]; true)                                 \
      if (const int4 tl = first ? V.tiles[SA][ti] : V.tiles[SB][ti - V.ntiles[SA]]; true)

template <class SX, class SY>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_ppm_slopes_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_EXT_X, SPACE_EXT_Y) {
    const Grid& G = V.grids[tl.x];
    if (first) b_ppm_slopes<SX, 0>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
    else b_ppm_slopes<SY, 1>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
template <class SX, class SY, int MODE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_faces_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_CELL, SPACE_CELL) {
    const Grid& G = V.grids[tl.x];
    if (first) b_faces<SX, 0, MODE>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
    else b_faces<SY, 1, MODE>(G, G.st[G.loop->cur], tl.z + threadIdx.x, tl.y);
  }
}
template <int STAGE>
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_roe_mhd_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_XFACE, SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int x = tl.z + threadIdx.x;
    if (first) {
      if (x < G.nx + 1) b_roe_mhd<0, STAGE>(G, G.st[G.loop->cur], (size_t)tl.y * (G.nx + 1) + x);
    } else {
      if (x < G.nx) b_roe_mhd<1, STAGE>(G, G.st[G.loop->cur], (size_t)tl.y * G.nx + x);
    }
  }
}
__global__ void __launch_bounds__(kBlock, kMinBlocks) kb_roe_hydro_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_XFACE, SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int x = tl.z + threadIdx.x;
    if (first) {
      if (x < G.nx + 1) b_roe_hydro<0>(G, (size_t)tl.y * (G.nx + 1) + x);
    } else {
      if (x < G.nx) b_roe_hydro<1>(G, (size_t)tl.y * G.nx + x);
    }
  }
}
__global__ void __launch_bounds__(kBlock) kb_ctu_mhd_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_XFACE, SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int x = tl.z + threadIdx.x;
    if (first) {
      if (x < G.nx + 1) b_ctu_mhd<0>(G, G.st[G.loop->cur], (size_t)tl.y * (G.nx + 1) + x);
    } else {
      if (x < G.nx) b_ctu_mhd<1>(G, G.st[G.loop->cur], (size_t)tl.y * G.nx + x);
    }
  }
}
__global__ void __launch_bounds__(kBlock) kb_ctu_hydro_xy(BatchView V) {
  MHD_PAIR_LOOP(SPACE_XFACE, SPACE_YFACE) {
    const Grid& G = V.grids[tl.x];
    const int x = tl.z + threadIdx.x;
    if (first) {
      if (x < G.nx + 1) b_ctu_hydro<0>(G, (size_t)tl.y * (G.nx + 1) + x);
    } else {
      if (x < G.nx) b_ctu_hydro<1>(G, (size_t)tl.y * G.nx + x);
    }
  }
}

template <int PHYS>
void enqueue_recon_batch(const BatchView& V, int recon, unsigned blocks, unsigned tw, cudaStream_t s) {
  using SX = typename std::conditional<PHYS == MHD, MhdSweep<0>, HydroSweep<0>>::type;
  using SY = typename std::conditional<PHYS == MHD, MhdSweep<1>, HydroSweep<1>>::type;
  if (recon == 2) {
    kb_ppm_slopes<SX, 0><<<blocks, tw, 0, s>>>(V);
    kb_faces<SX, 0, 2><<<blocks, tw, 0, s>>>(V);
    kb_ppm_slopes<SY, 1><<<blocks, tw, 0, s>>>(V);
    kb_faces<SY, 1, 2><<<blocks, tw, 0, s>>>(V);
  } else if (recon == 1) {
    kb_ppm_slopes<SX, 0><<<blocks, tw, 0, s>>>(V);
    kb_faces<SX, 0, 1><<<blocks, tw, 0, s>>>(V);
    kb_ppm_slopes<SY, 1><<<blocks, tw, 0, s>>>(V);
    kb_faces<SY, 1, 1><<<blocks, tw, 0, s>>>(V);
  } else {
    kb_faces<SX, 0, 0><<<blocks, tw, 0, s>>>(V);
    kb_faces<SY, 1, 0><<<blocks, tw, 0, s>>>(V);
  }
}

void enqueue_cycle_batch(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw, cudaStream_t s);

template <int PHYS>
void enqueue_recon_batch_xy(const BatchView& V, int recon, unsigned blocks, unsigned tw, cudaStream_t s) {
  using SX = typename std::conditional<PHYS == MHD, MhdSweep<0>, HydroSweep<0>>::type;
  using SY = typename std::conditional<PHYS == MHD, MhdSweep<1>, HydroSweep<1>>::type;
  if (recon >= 1) kb_ppm_slopes_xy<SX, SY><<<blocks, tw, 0, s>>>(V);
  if (recon == 2) kb_faces_xy<SX, SY, 2><<<blocks, tw, 0, s>>>(V);
  else if (recon == 1) kb_faces_xy<SX, SY, 1><<<blocks, tw, 0, s>>>(V);
  else kb_faces_xy<SX, SY, 0><<<blocks, tw, 0, s>>>(V);
}

// One batched cycle of every instance; each instance reads the state buffer its
// loop state names as current.  `blocks` = blocks of a persistent launch (a
// multiple of the SM count); `tw` = tile width = threads per block (the work
// lists must be built for it); `fuse` = 2 runs the x and y launches of a stage
// as one launch.
void enqueue_cycle_batch_tuned(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw,
                               int fuse, cudaStream_t s) {
  const unsigned ib = (unsigned)((V.ninst + 127) / 128);
  if (fuse == 2) {
    if (physics == MHD) {
      kb_dt_reduce<MHD><<<blocks, tw, 0, s>>>(V);
      kb_begin<MHD><<<ib, 128, 0, s>>>(V);
      enqueue_recon_batch_xy<MHD>(V, recon, blocks, tw, s);
      kb_roe_mhd_xy<1><<<blocks, tw, 0, s>>>(V);
      kb_emf<1><<<blocks, tw, 0, s>>>(V);
      kb_ctu_mhd_xy<<<blocks, tw, 0, s>>>(V);
      kb_half_ez<<<blocks, tw, 0, s>>>(V);
      kb_roe_mhd_xy<2><<<blocks, tw, 0, s>>>(V);
      kb_emf<2><<<blocks, tw, 0, s>>>(V);
      kb_final_mhd<<<blocks, tw, 0, s>>>(V);
    } else {
      kb_dt_reduce<HYDRO><<<blocks, tw, 0, s>>>(V);
      kb_begin<HYDRO><<<ib, 128, 0, s>>>(V);
      enqueue_recon_batch_xy<HYDRO>(V, recon, blocks, tw, s);
      kb_roe_hydro_xy<<<blocks, tw, 0, s>>>(V);
      kb_ctu_hydro_xy<<<blocks, tw, 0, s>>>(V);
      kb_roe_hydro_xy<<<blocks, tw, 0, s>>>(V);
      kb_final_hydro<<<blocks, tw, 0, s>>>(V);
    }
    kb_end<<<ib, 128, 0, s>>>(V);
    return;
  }
  enqueue_cycle_batch(V, physics, recon, blocks, tw, s);
}

void enqueue_cycle_batch(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw, cudaStream_t s) {
  const unsigned ib = (unsigned)((V.ninst + 127) / 128);
  if (physics == MHD) {
    kb_dt_reduce<MHD><<<blocks, tw, 0, s>>>(V);
    kb_begin<MHD><<<ib, 128, 0, s>>>(V);
    enqueue_recon_batch<MHD>(V, recon, blocks, tw, s);
    kb_roe_mhd<0, 1><<<blocks, tw, 0, s>>>(V);
    kb_roe_mhd<1, 1><<<blocks, tw, 0, s>>>(V);
    kb_emf<1><<<blocks, tw, 0, s>>>(V);
    kb_ctu_mhd<0><<<blocks, tw, 0, s>>>(V);
    kb_ctu_mhd<1><<<blocks, tw, 0, s>>>(V);
    kb_half_ez<<<blocks, tw, 0, s>>>(V);
    kb_roe_mhd<0, 2><<<blocks, tw, 0, s>>>(V);
    kb_roe_mhd<1, 2><<<blocks, tw, 0, s>>>(V);
    kb_emf<2><<<blocks, tw, 0, s>>>(V);
    kb_final_mhd<<<blocks, tw, 0, s>>>(V);
  } else {
    kb_dt_reduce<HYDRO><<<blocks, tw, 0, s>>>(V);
    kb_begin<HYDRO><<<ib, 128, 0, s>>>(V);
    enqueue_recon_batch<HYDRO>(V, recon, blocks, tw, s);
    kb_roe_hydro<0><<<blocks, tw, 0, s>>>(V);
    kb_roe_hydro<1><<<blocks, tw, 0, s>>>(V);
    kb_ctu_hydro<0><<<blocks, tw, 0, s>>>(V);
    kb_ctu_hydro<1><<<blocks, tw, 0, s>>>(V);
    kb_roe_hydro<0><<<blocks, tw, 0, s>>>(V);
    kb_roe_hydro<1><<<blocks, tw, 0, s>>>(V);
    kb_final_hydro<<<blocks, tw, 0, s>>>(V);
  }
  kb_end<<<ib, 128, 0, s>>>(V);
}

#endif  // MHD_BODIES_ONLY

}  // namespace MHD_NS
}  // namespace mhdk
