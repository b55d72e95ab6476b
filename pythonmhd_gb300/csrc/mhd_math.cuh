// Pointwise FP64 physics of the 2D Godunov step: primitive eigensystem, Roe
// fluxes, prim<->cons conversions and the PPM per-cell pieces.
//
// Every expression keeps the operation order of the reference
// (PythonMHD Source/*.py, cited per function) so that a build without FMA
// contraction reproduces the reference's NumPy results bit for bit.  Structural
// zeros of the eigenmatrices are skipped: adding a +-0 product to an
// accumulator that never holds -0 leaves it unchanged, so skipping changes at
// most the sign of an exact zero.
//
// Sweep vectors (7 slots) follow the reference's x/y orderings
// (Source/EvolveFunctions_MHD.py:415-438):
//   x: [rho, vx, vy, vz, By, Bz, p]    y: [rho, vx, vy, vz, Bz, Bx, p]
// and a sweep is described by its normal (N) and transverse (T1, T2) velocity
// slots: x = (1,2,3), y = (2,3,1).
#pragma once
#include <cstdint>

#include "softfp.cuh"

namespace mhdk {

constexpr double SMALL_VALUE = 0.000000000001;   // Source/PythonMHD_Constants.py:7
constexpr double FOUR_THIRDS = 1.333333333333333;  // Source/PythonMHD_Constants.py:8 (truncated)

__device__ __forceinline__ double sq(double x) { return x * x; }

// ---------------------------------------------------------------------------
// Division and square root, correctly rounded.  As FP64 instructions each costs
// about ten FP64-pipe slots, and that pipe bounds every kernel of the step; these
// compute the same bits by integer Newton-Raphson with an exact remainder check
// (softfp.cuh), on the integer pipes.  The unqualified sqrt() of every kernel in
// this namespace resolves here.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double ddiv(double a, double b) { return sfp::div(a, b); }
__host__ __device__ __forceinline__ double sqrt(double x) { return sfp::sqrt(x); }

// ---------------------------------------------------------------------------
// Operations the compiler never fuses into a multiply-add.  The fast build lets
// nvcc contract a*b+c into one rounding; these keep two.  They are used for the
// scalars that decide the reference's branches (wave speeds, the Roe-averaged
// sound speed, the fast/slow normalisations) so that both builds take the same
// branch from the same inputs; in the exact build they are the plain operators.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double nadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double nsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double nsq(double x) { return __dmul_rn(x, x); }

// ---------------------------------------------------------------------------
// x / 6, correctly rounded, in one multiply and two FMAs (Markstein's remainder
// correction, IBM J. Res. Dev. 34(1), 1990), against about ten FP64 slots for an
// IEEE division.  With z = RN(1/6) = (1 - 2^-54) / 6, let u = ulp(x/6); x lies two
// or three binades above x/6, so it is a multiple of 4u.
//  * q0 = RN(x z) lies within 1.5u of x/6 (x z is within u/2 of x/6, and the
//    rounding adds at most another ulp of q0's binade);
//  * r = x - 6 q0 is then a multiple of 2u of magnitude <= 9u, so it is a double and
//    the FMA computes it exactly;
//  * q0 + r z = x/6 - r 2^-54 / 6 exactly, within 1.5u 2^-54 of x/6, and the final
//    FMA rounds it once.
// x/6 is never that close to a rounding boundary: a midpoint m = (2k+1) u/2 of the
// binade of x/6 gives 6m - x = u (6k + 3 - x/u), an odd multiple of u, so
// |x/6 - m| >= u/6 (and the boundary below the binade is u/4 away from it).  The
// rounding of q0 + r z therefore equals that of x/6.  The argument needs x/6 and q0
// in the normal range; a zero is returned as it is (+-0 / 6 = +-0), and other
// exponents (subnormals, huge values, inf, NaN) take the IEEE division.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double div6(double x) {
  const unsigned int ex = ((unsigned int)__double2hiint(x) >> 20) & 0x7ffu;
  if (ex - 24u > 1998u)
    return (static_cast<unsigned long long>(__double_as_longlong(x)) << 1) == 0ULL ? x : x / 6.0;
  const double z = 0.16666666666666666;   // RN(1/6)
  const double q0 = __dmul_rn(x, z);
  return __fma_rn(__fma_rn(-6.0, q0, x), z, q0);
}

// ---------------------------------------------------------------------------
// Comparisons on the IEEE-754 bit pattern.  An FP64 compare (DSETP, and the
// select of an FP64 max/min) issues on the FP64 pipe at the DFMA rate, and that
// pipe bounds every kernel of the step; the same test on the 64-bit pattern runs
// on the integer pipe at about 7x the rate.  Each helper equals the IEEE
// comparison for every non-NaN operand, zeros of either sign included.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
// order key: okey(a) < okey(b) <=> a < b for non-NaN a, b; +0 and -0 both map to 0
__device__ __forceinline__ long long okey(double x) {
  const long long b = dbits(x);
  return b < 0 ? (-0x7fffffffffffffffLL - 1) - b : b;
}
__device__ __forceinline__ bool is_pos(double x) { return dbits(x) > 0; }       // x > 0
__device__ __forceinline__ bool is_nonpos(double x) { return dbits(x) <= 0; }   // x <= 0
__device__ __forceinline__ bool is_neg(double x) { return okey(x) < 0; }        // x < 0
__device__ __forceinline__ bool is_nonneg(double x) { return okey(x) >= 0; }    // x >= 0
__device__ __forceinline__ bool is_zero(double x) {                             // x == 0
  return (static_cast<unsigned long long>(dbits(x)) << 1) == 0ULL;
}
// x is NaN or +-Inf (exponent field all ones), tested on the integer pipe
__device__ __forceinline__ bool is_nonfinite(double x) {
  return (static_cast<unsigned long long>(dbits(x)) & 0x7ff0000000000000ULL) == 0x7ff0000000000000ULL;
}
__device__ __forceinline__ bool dgt(double a, double b) { return okey(a) > okey(b); }  // a > b
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }  // a < b

// np.sign(x) with 0 -> 1 (Source/RiemannSolvers_MHD_Roe_HelperModule.py:286-287)
__device__ __forceinline__ double sign_one(double x) { return is_neg(x) ? -1.0 : 1.0; }
// np.sign(x) * m for m >= 0 (0 for x == 0)
__device__ __forceinline__ double signed_mag(double x, double m) {
  return is_pos(x) ? m : (is_neg(x) ? -m : 0.0);
}
// numpy maximum / minimum (a > b ? a : b, a < b ? a : b; finite data)
__device__ __forceinline__ double dmax(double a, double b) { return dgt(a, b) ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return dlt(a, b) ? a : b; }

// ---------------------------------------------------------------------------
// Structural non-zero patterns of the eigenmatrices (row i, column j)
// ---------------------------------------------------------------------------
template <int N, int T1, int T2>
__host__ __device__ constexpr bool prim_L_nz(int i, int j) {
  return (i == 0 || i == 2 || i == 4 || i == 6) ? (j == N || j == T1 || j == T2 || j == 4 || j == 5 || j == 6)
       : (i == 1 || i == 5) ? (j == T1 || j == T2 || j == 4 || j == 5)
       : (j == 0 || j == 6);  // i == 3
}
template <int N, int T1, int T2>
__host__ __device__ constexpr bool prim_R_nz(int i, int j) {
  return (i == 0) ? (j == 0 || j == 2 || j == 3 || j == 4 || j == 6)
       : (i == N || i == 6) ? (j == 0 || j == 2 || j == 4 || j == 6)
       : (j != 3);  // rows T1, T2, 4, 5
}
template <int N, int T1, int T2>
__host__ __device__ constexpr bool roe_L_nz(int i, int j) {
  return (i == 1 || i == 5) ? (j == 0 || j == T1 || j == T2 || j == 4 || j == 5) : true;
}
template <int N, int T1, int T2>
__host__ __device__ constexpr bool roe_R_nz(int i, int j) {
  return (i == 0 || i == N) ? (j != 1 && j != 5)
       : (i == 4 || i == 5) ? (j != 3)
       : true;
}

// ---------------------------------------------------------------------------
// Cell-centred primitive eigensystem, compact form.
// Source/ReconstructionEigenmatrices_MHD_HelperModule.py:27-207 (x), :220-396 (y)
// Rows 4, 5, 6 of L are +- rows 2, 1, 0; R repeats entries likewise. The
// struct keeps each distinct value once; L()/R() expand them.
// ---------------------------------------------------------------------------
struct PrimEig {
  double lam[7];
  // R distinct values
  double r00, r02, rn0, rn2, qsb1, qfb1, qsb2, qfb2, b1, b2, r60, r62, r40, r41, r42, r50, r51, r52;
  // L distinct values
  double l0n, l0t1, l0t2, l06, l04, l05, l1t1, l1t2, l14, l15, l2n, l2t1, l2t2, l26, l24, l25, l36;
};
constexpr int kPrimEigWords = 7 + 18 + 17;

template <int N, int T1, int T2>
__device__ __forceinline__ double prim_L(const PrimEig& e, int i, int j) {
  // rows 0/6: (N, T1, T2, 6, 4, 5) ; rows 6 = (-,-,-,+,+,+) of row 0
  if (i == 0 || i == 6) {
    if (j == N) return i == 6 ? -e.l0n : e.l0n;
    if (j == T1) return i == 6 ? -e.l0t1 : e.l0t1;
    if (j == T2) return i == 6 ? -e.l0t2 : e.l0t2;
    if (j == 6) return e.l06;
    if (j == 4) return e.l04;
    return e.l05;
  }
  if (i == 2 || i == 4) {
    if (j == N) return i == 4 ? -e.l2n : e.l2n;
    if (j == T1) return i == 4 ? -e.l2t1 : e.l2t1;
    if (j == T2) return i == 4 ? -e.l2t2 : e.l2t2;
    if (j == 6) return e.l26;
    if (j == 4) return e.l24;
    return e.l25;
  }
  if (i == 1 || i == 5) {
    if (j == T1) return i == 5 ? -e.l1t1 : e.l1t1;
    if (j == T2) return i == 5 ? -e.l1t2 : e.l1t2;
    if (j == 4) return e.l14;
    return e.l15;
  }
  // i == 3
  if (j == 0) return 1.0;
  return e.l36;
}

template <int N, int T1, int T2>
__device__ __forceinline__ double prim_R(const PrimEig& e, int i, int j) {
  if (i == 0) {
    if (j == 0 || j == 6) return e.r00;
    if (j == 3) return 1.0;
    return e.r02;  // j == 2, 4
  }
  if (i == N) {
    if (j == 0) return e.rn0;
    if (j == 6) return -e.rn0;
    if (j == 2) return e.rn2;
    return -e.rn2;  // j == 4
  }
  if (i == 6) {
    if (j == 0 || j == 6) return e.r60;
    return e.r62;
  }
  if (i == T1) {
    if (j == 0) return e.qsb1;
    if (j == 6) return -e.qsb1;
    if (j == 1) return -e.b2;
    if (j == 5) return e.b2;
    if (j == 2) return -e.qfb1;
    return e.qfb1;  // j == 4
  }
  if (i == T2) {
    if (j == 0) return e.qsb2;
    if (j == 6) return -e.qsb2;
    if (j == 1) return e.b1;
    if (j == 5) return -e.b1;
    if (j == 2) return -e.qfb2;
    return e.qfb2;
  }
  if (i == 4) {
    if (j == 0 || j == 6) return e.r40;
    if (j == 1 || j == 5) return e.r41;
    return e.r42;  // j == 2, 4
  }
  // i == 5
  if (j == 0 || j == 6) return e.r50;
  if (j == 1 || j == 5) return e.r51;
  return e.r52;
}

template <int N, int T1, int T2>
__device__ __forceinline__ void prim_eigensystem(const double w[7], double bn, double gamma, PrimEig& e) {
  const double bt2 = nadd(nsq(w[4]), nsq(w[5]));
  const double bt = sqrt(bt2);
  const double gp = gamma * w[6];
  const double inv_d = ddiv(1.0, w[0]);
  const double sqrt_d = sqrt(w[0]);
  const double red_bt2 = bt2 * inv_d;
  const double a2 = gp * inv_d;
  const double a = sqrt(a2);
  const double ca2 = bn * bn * inv_d;
  const double ca = sqrt(ca2);
  const double ssum = ca2 + red_bt2 + a2;
  const double sdiff = ca2 + red_bt2 - a2;
  const double ssqrt = sqrt(nadd(nsq(sdiff), nmul(4.0 * a2, red_bt2)));
  const double cf2 = 0.5 * (ssum + ssqrt);
  const double cf = sqrt(cf2);
  const double cs2 = ddiv(a2 * ca2, cf2);
  const double cs = sqrt(cs2);

  double b1 = 0.0, b2 = 0.0;
  if (is_zero(bt)) b1 = 1.0;
  if (is_pos(bt)) { b1 = ddiv(w[4], bt); b2 = ddiv(w[5], bt); }

  double fa = 0.0, sa = 0.0;
  if (is_zero(ssqrt)) {
    fa = 1.0;
  } else if (is_nonpos(a2 - cs2)) {
    sa = 1.0;
  } else if (is_nonpos(cf2 - a2)) {
    fa = 1.0;
  } else {
    fa = sqrt(ddiv(a2 - cs2, ssqrt));
    sa = sqrt(ddiv(cf2 - a2, ssqrt));
  }
  const double sgn = sign_one(bn);
  const double qf = cf * fa * sgn;
  const double qs = cs * sa * sgn;
  const double af = a * fa * sqrt_d;
  const double as = a * sa * sqrt_d;

  const double vn = w[N];
  e.lam[0] = vn - cf; e.lam[1] = vn - ca; e.lam[2] = vn - cs; e.lam[3] = vn;
  e.lam[4] = vn + cs; e.lam[5] = vn + ca; e.lam[6] = vn + cf;

  e.r00 = w[0] * fa;
  e.r02 = w[0] * sa;
  e.rn0 = -cf * fa;
  e.rn2 = -cs * sa;
  e.qsb1 = qs * b1;
  e.qfb1 = qf * b1;
  e.qsb2 = qs * b2;
  e.qfb2 = qf * b2;
  e.b1 = b1;
  e.b2 = b2;
  e.r60 = w[0] * a2 * fa;
  e.r62 = w[0] * a2 * sa;
  e.r40 = as * b1;
  e.r41 = -b2 * sgn * sqrt_d;
  e.r42 = -af * b1;
  e.r50 = as * b2;
  e.r51 = b1 * sgn * sqrt_d;
  e.r52 = -af * b2;

  const double nf = ddiv(0.5, a2);
  const double qf_n = nf * qf;
  const double qs_n = nf * qs;
  const double afp = nf * af * inv_d;
  const double asp = nf * as * inv_d;
  e.l0n = -nf * cf * fa;
  e.l0t1 = qs_n * b1;
  e.l0t2 = qs_n * b2;
  e.l06 = nf * fa * inv_d;
  e.l04 = asp * b1;
  e.l05 = asp * b2;
  e.l1t1 = -0.5 * b2;
  e.l1t2 = 0.5 * b1;
  e.l14 = ddiv(-0.5 * b2 * sgn, sqrt_d);
  e.l15 = ddiv(0.5 * b1 * sgn, sqrt_d);
  e.l2n = -nf * cs * sa;
  e.l2t1 = -qf_n * b1;
  e.l2t2 = -qf_n * b2;
  e.l26 = nf * sa * inv_d;
  e.l24 = -afp * b1;
  e.l25 = -afp * b2;
  e.l36 = ddiv(-1.0, a2);
}

// Row i of L times v, accumulated in the reference order (0, N, T1, T2, 6, 4, 5).
template <int N, int T1, int T2>
__device__ __forceinline__ double prim_project(const PrimEig& e, int i, const double v[7]) {
  const int order[7] = {0, N, T1, T2, 6, 4, 5};
  double acc = 0.0;
  bool first = true;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const int j = order[k];
    if (prim_L_nz<N, T1, T2>(i, j)) {
      const double t = prim_L<N, T1, T2>(e, i, j) * v[j];
      acc = first ? t : acc + t;
      first = false;
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// prim <-> cons for a 7-slot sweep vector (Source/PrimCons_HelperModule.py:208-229, :358-380)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void prim_to_cons7(const double w[7], double bn, double gamma, double u[7]) {
  u[0] = w[0];
  u[1] = w[0] * w[1];
  u[2] = w[0] * w[2];
  u[3] = w[0] * w[3];
  u[4] = w[4];
  u[5] = w[5];
  double e = ddiv(w[6], gamma - 1.0) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  e = e + 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5]);
  u[6] = e;
}

__device__ __forceinline__ void cons_to_prim7(const double u[7], double bn, double gamma, double w[7]) {
  const double inv_d = ddiv(1.0, u[0]);
  w[0] = u[0];
  w[1] = u[1] * inv_d;
  w[2] = u[2] * inv_d;
  w[3] = u[3] * inv_d;
  w[4] = u[4];
  w[5] = u[5];
  double p = u[6] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * inv_d;
  p = p - 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5]);
  w[6] = p * (gamma - 1.0);
}

// ---------------------------------------------------------------------------
// Roe flux (Source/RiemannSolvers_MHD_Roe_HelperModule.py:74-576 for x, :595-1071 for y)
// ---------------------------------------------------------------------------
template <int N, int T1, int T2>
__device__ __forceinline__ void cell_flux7(const double w[7], const double u[7], double bn, double hb, double F[7]) {
  const double p = w[6];
  F[0] = u[N];
#pragma unroll
  for (int k = 1; k <= 3; ++k) F[k] = u[N] * w[k];
  F[N] = F[N] + p;
  F[6] = (u[6] + p) * w[N];
  F[N] = F[N] - 0.5 * (bn * bn - sq(w[4]) - sq(w[5]));
  F[T1] = F[T1] - bn * w[4];
  F[T2] = F[T2] - bn * w[5];
  F[6] = F[6] + (hb * w[N] - bn * (bn * w[N] + w[4] * w[T1] + w[5] * w[T2]));
  F[4] = w[4] * w[N] - bn * w[T1];
  F[5] = w[5] * w[N] - bn * w[T2];
}

template <int N, int T1, int T2>
__device__ __forceinline__ void roe_flux(const double wl[7], const double wr[7], const double ul[7],
                                         const double ur[7], double bn, double gamma, bool efix,
                                         double eps, double flux[7]) {
  const double sl = sqrt(wl[0]);
  const double sr = sqrt(wr[0]);
  const double isum = ddiv(1.0, sl + sr);
  const double rd = sl * sr;
  double v[4];
#pragma unroll
  for (int k = 1; k <= 3; ++k) v[k] = nadd(nmul(sl, wl[k]), nmul(sr, wr[k])) * isum;
  const double vsq = nadd(nadd(nsq(v[N]), nsq(v[T1])), nsq(v[T2]));
  const double b1 = nadd(nmul(sr, wl[4]), nmul(sl, wr[4])) * isum;
  const double b2 = nadd(nmul(sr, wl[5]), nmul(sl, wr[5])) * isum;
  const double hbl = 0.5 * nadd(nadd(nsq(bn), nsq(wl[4])), nsq(wl[5]));
  const double hbr = 0.5 * nadd(nadd(nsq(bn), nsq(wr[4])), nsq(wr[5]));
  const double H = (ddiv(ul[6] + wl[6] + hbl, sl) + ddiv(ur[6] + wr[6] + hbr, sr)) * isum;

  const double ird = ddiv(1.0, rd);
  const double btc = ddiv(0.5 * nadd(nsq(wl[4] - wr[4]), nsq(wl[5] - wr[5])), sq(sl + sr));
  const double rc = ddiv(0.5 * (wl[0] + wr[0]), rd);
  const double bt2 = nadd(nsq(b1), nsq(b2));
  const double bt = sqrt(bt2);
  const double bts2 = nsub(gamma - 1.0, nmul(gamma - 2.0, rc)) * bt2;
  const double bts = sqrt(bts2);
  const double rbts2 = bts2 * ird;
  const double ca2 = bn * bn * ird;
  const double ca = sqrt(ca2);
  const double hmb = H - nadd(ca2, nmul(bt2, ird));
  const double a2 = dmax(nsub(nmul(gamma - 1.0, hmb - 0.5 * vsq), nmul(gamma - 2.0, btc)), SMALL_VALUE);
  const double a = sqrt(a2);
  const double ssum = ca2 + rbts2 + a2;
  const double sdiff = ca2 + rbts2 - a2;
  const double ssqrt = sqrt(nadd(nsq(sdiff), nmul(4.0 * a2, rbts2)));
  const double cf2 = 0.5 * (ssum + ssqrt);
  const double cf = sqrt(cf2);
  const double cs2 = ddiv(a2 * ca2, cf2);
  const double cs = sqrt(cs2);

  const double vn = v[N];
  double lam[7] = {vn - cf, vn - ca, vn - cs, vn, vn + cs, vn + ca, vn + cf};
  if (efix) {
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const double x = lam[k];
      if (dlt(fabs(x), 2.0 * eps) && !is_zero(x)) {
        const double corr = eps + ddiv(sq(x), 4.0 * eps);
        lam[k] = is_pos(x) ? x + corr : x - corr;
      }
    }
  }

  double fa = 0.0, sa = 0.0;
  if (is_zero(cf2 - cs2)) {
    fa = 1.0;
  } else if (is_nonpos(a2 - cs2)) {
    sa = 1.0;
  } else if (is_nonpos(cf2 - a2)) {
    fa = 1.0;
  } else {
    fa = sqrt(ddiv(a2 - cs2, cf2 - cs2));
    sa = sqrt(ddiv(cf2 - a2, cf2 - cs2));
  }
  const double sgn = sign_one(bn);
  const double srd = sqrt(rd);
  const double isrd = ddiv(1.0, srd);
  const double qf = cf * fa * sgn;
  const double qs = cs * sa * sgn;
  const double afp = a * fa * isrd;
  const double asp = a * sa * isrd;

  double bh1 = 0.0, bh2 = 0.0;
  if (is_zero(bt)) bh1 = 1.0;
  if (is_pos(bt)) { bh1 = ddiv(b1, bt); bh2 = ddiv(b2, bt); }
  const double den = sqrt(nsub(gamma - 1.0, nmul(gamma - 2.0, rc)));
  const double b1s = ddiv(bh1, den);
  const double b2s = ddiv(bh2, den);
  const double vb = v[T1] * b1s + v[T2] * b2s;
  const double bs2 = b1s * b1s + b2s * b2s;
  const double afb = afp * bts * bs2;
  const double asb = asp * bts * bs2;

  double fl[7], fr[7];
  cell_flux7<N, T1, T2>(wl, ul, bn, hbl, fl);
  cell_flux7<N, T1, T2>(wr, ur, bn, hbr, fr);
  if (is_nonpos(lam[6])) {
#pragma unroll
    for (int i = 0; i < 7; ++i) flux[i] = fr[i];
    return;
  }
  if (is_nonneg(lam[0])) {
#pragma unroll
    for (int i = 0; i < 7; ++i) flux[i] = fl[i];
    return;
  }
  // L, the wave amplitudes, then R: each matrix is formed where it is used, after
  // the supersonic exits (the same expressions, so the same roundings)
  double nf = ddiv(0.5, a2);
  const double cff = nf * fa * cf;
  const double css = nf * sa * cs;
  const double qfn = qf * nf;
  const double qsn = qs * nf;
  const double af_ = nf * afp * rd;
  const double as_ = nf * asp * rd;
  const double afb2 = nf * afp * bts;
  const double asb2 = nf * asp * bts;
  nf = nf * (gamma - 1.0);
  const double fan = fa * nf;
  const double san = sa * nf;
  const double b1c = ddiv(b1s, bs2);
  const double b2c = ddiv(b2s, bs2);
  const double vbs = v[T1] * b1c + v[T2] * b2c;
  nf = nf * 2.0;

  double L[7][7];
  L[0][0] = fan * (vsq - hmb) + cff * (cf + vn) - qsn * vbs - asb2;
  L[0][N] = -1.0 * fan * vn - cff;
  L[0][T1] = -1.0 * fan * v[T1] + qsn * b1c;
  L[0][T2] = -1.0 * fan * v[T2] + qsn * b2c;
  L[0][6] = fan;
  L[0][4] = as_ * b1c - fan * b1;
  L[0][5] = as_ * b2c - fan * b2;
  L[1][0] = 0.5 * (v[T1] * bh2 - v[T2] * bh1);
  L[1][T1] = -0.5 * bh2;
  L[1][T2] = 0.5 * bh1;
  L[1][4] = -0.5 * srd * bh2 * sgn;
  L[1][5] = 0.5 * srd * bh1 * sgn;
  L[2][0] = san * (vsq - hmb) + css * (cs + vn) + qfn * vbs + afb2;
  L[2][N] = -san * vn - css;
  L[2][T1] = -san * v[T1] - qfn * b1c;
  L[2][T2] = -san * v[T2] - qfn * b2c;
  L[2][6] = san;
  L[2][4] = -af_ * b1c - san * b1;
  L[2][5] = -af_ * b2c - san * b2;
  L[3][0] = 1.0 - nf * (0.5 * vsq - ddiv((gamma - 2.0) * btc, gamma - 1.0));
  L[3][1] = nf * v[1];
  L[3][2] = nf * v[2];
  L[3][3] = nf * v[3];
  L[3][6] = -1.0 * nf;
  L[3][4] = nf * b1;
  L[3][5] = nf * b2;
  L[4][0] = san * (vsq - hmb) + css * (cs - vn) - qfn * vbs + afb2;
  L[4][N] = -san * vn + css;
  L[4][T1] = -san * v[T1] + qfn * b1c;
  L[4][T2] = -san * v[T2] + qfn * b2c;
  L[4][6] = san;
  L[4][4] = L[2][4];
  L[4][5] = L[2][5];
  L[5][0] = -L[1][0];
  L[5][T1] = -L[1][T1];
  L[5][T2] = -L[1][T2];
  L[5][4] = L[1][4];
  L[5][5] = L[1][5];
  L[6][0] = fan * (vsq - hmb) + cff * (cf - vn) + qsn * vbs - asb2;
  L[6][N] = -fan * vn + cff;
  L[6][T1] = -fan * v[T1] - qsn * b1c;
  L[6][T2] = -fan * v[T2] - qsn * b2c;
  L[6][6] = fan;
  L[6][4] = L[0][4];
  L[6][5] = L[0][5];

  double du[7];
#pragma unroll
  for (int i = 0; i < 7; ++i) du[i] = ur[i] - ul[i];
  const int order[7] = {0, N, T1, T2, 6, 4, 5};
  double amps[7];
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const int j = order[k];
      if (roe_L_nz<N, T1, T2>(i, j)) {
        const double t = L[i][j] * du[j];
        acc = first ? t : acc + t;
        first = false;
      }
    }
    amps[i] = 0.5 * fabs(lam[i]) * acc;
  }
  double R[7][7];
  R[0][0] = fa; R[0][2] = sa; R[0][3] = 1.0; R[0][4] = sa; R[0][6] = fa;
  R[N][0] = fa * lam[0]; R[N][2] = sa * lam[2]; R[N][3] = vn; R[N][4] = sa * lam[4]; R[N][6] = fa * lam[6];
  {
    const double fv = fa * v[T1], sv = sa * v[T1], qsb = qs * b1s, qfb = qf * b1s;
    R[T1][0] = fv + qsb; R[T1][1] = -bh2; R[T1][2] = sv - qfb; R[T1][3] = v[T1];
    R[T1][4] = sv + qfb; R[T1][5] = bh2; R[T1][6] = fv - qsb;
  }
  {
    const double fv = fa * v[T2], sv = sa * v[T2], qsb = qs * b2s, qfb = qf * b2s;
    R[T2][0] = fv + qsb; R[T2][1] = bh1; R[T2][2] = sv - qfb; R[T2][3] = v[T2];
    R[T2][4] = sv + qfb; R[T2][5] = -bh1; R[T2][6] = fv - qsb;
  }
  R[6][0] = fa * (hmb - vn * cf) + qs * vb + asb;
  R[6][1] = -(v[T1] * bh2 - v[T2] * bh1);
  R[6][2] = sa * (hmb - vn * cs) - qf * vb - afb;
  R[6][3] = 0.5 * vsq + ddiv((gamma - 2.0) * btc, gamma - 1.0);
  R[6][4] = sa * (hmb + vn * cs) + qf * vb - afb;
  R[6][5] = -R[6][1];
  R[6][6] = fa * (hmb + vn * cf) - qs * vb + asb;
  R[4][0] = asp * b1s; R[4][1] = -bh2 * sgn * isrd; R[4][2] = -afp * b1s;
  R[4][4] = R[4][2]; R[4][5] = R[4][1]; R[4][6] = R[4][0];
  R[5][0] = asp * b2s; R[5][1] = bh1 * sgn * isrd; R[5][2] = -afp * b2s;
  R[5][4] = R[5][2]; R[5][5] = R[5][1]; R[5][6] = R[5][0];

#pragma unroll
  for (int i = 0; i < 7; ++i) {
    double acc = 0.5 * (fl[i] + fr[i]);
#pragma unroll
    for (int j = 0; j < 7; ++j)
      if (roe_R_nz<N, T1, T2>(i, j)) acc = acc - amps[j] * R[i][j];
    flux[i] = acc;
  }
}

// ---------------------------------------------------------------------------
// Hydro (5 slots: [rho, vx, vy, vz, p] in every sweep); template argument A is
// the sweep direction (0 x, 1 y, 2 z).
// Source/PrimCons_HelperModule.py:46-114, :135-196 ; the y forms sum the kinetic
// terms in the order (vy, vz, vx), the z forms in the order (vz, vx, vy).
// ---------------------------------------------------------------------------
template <int A>
__device__ __forceinline__ double hkin(double a1, double a2, double a3) {
  return A == 2 ? (sq(a3) + sq(a1) + sq(a2)) : A == 1 ? (sq(a2) + sq(a3) + sq(a1)) : (sq(a1) + sq(a2) + sq(a3));
}

template <int A>
__device__ __forceinline__ void hprim_to_cons(const double w[5], double gamma, double u[5]) {
  u[0] = w[0];
  u[1] = w[0] * w[1];
  u[2] = w[0] * w[2];
  u[3] = w[0] * w[3];
  const double ke = hkin<A>(w[1], w[2], w[3]);
  u[4] = ddiv(w[4], gamma - 1.0) + 0.5 * w[0] * ke;
}

template <int A>
__device__ __forceinline__ void hcons_to_prim(const double u[5], double gamma, double w[5]) {
  w[0] = u[0];
  const double inv_d = ddiv(1.0, w[0]);
  w[1] = u[1] * inv_d;
  w[2] = u[2] * inv_d;
  w[3] = u[3] * inv_d;
  const double m2 = hkin<A>(u[1], u[2], u[3]);
  const double p = u[4] - 0.5 * m2 * inv_d;
  w[4] = p * (gamma - 1.0);
}

// Hydro primitive eigensystem (Source/ReconstructionEigenmatrices_Hydro_HelperModule.py:25-151,
// :230-282).  Wave order x = (a-, entropy, vy, vz, a+), y = (a-, vx, entropy, vz, a+),
// z = (a-, vx, vy, entropy, a+): the entropy wave sits at the normal velocity's slot
// n = A + 1 and shear wave k carries velocity slot k.
struct HPrimEig {
  double lam[5];
  double rn0;   // R[n][0] = -a/rho ; R[n][4] = -rn0
  double a2;    // R[4][0] = R[4][4]
  double l0n;   // L[0][n] = -0.5 rho / a ; L[4][n] = -l0n
  double l04;   // L[0][4] = L[4][4] = 0.5/a2
  double le4;   // L[ent][4] = -1/a2
};

template <int A>
__host__ __device__ constexpr bool hprim_L_nz(int i, int j) {
  return (i == 0 || i == 4) ? (j == A + 1 || j == 4) : (i == A + 1) ? (j == 0 || j == 4) : (j == i);
}
template <int A>
__host__ __device__ constexpr bool hprim_R_nz(int i, int j) {
  return (j == 0 || j == 4) ? (i == 0 || i == A + 1 || i == 4) : (j == A + 1) ? (i == 0) : (i == j);
}
template <int A>
__device__ __forceinline__ double hprim_L(const HPrimEig& e, int i, int j) {
  if (i == 0) return j == 4 ? e.l04 : e.l0n;
  if (i == 4) return j == 4 ? e.l04 : -e.l0n;
  if (i == A + 1) return j == 0 ? 1.0 : e.le4;
  return 1.0;
}
template <int A>
__device__ __forceinline__ double hprim_R(const HPrimEig& e, int i, int j) {
  if (j == 0 || j == 4) {
    if (i == 0) return 1.0;
    if (i == 4) return e.a2;
    return j == 0 ? e.rn0 : -e.rn0;
  }
  return 1.0;
}
template <int A>
__device__ __forceinline__ void hprim_eigensystem(const double w[5], double gamma, HPrimEig& e) {
  const int n = A + 1;
  const double gp = gamma * w[4];
  const double a2 = ddiv(gp, w[0]);
  const double a = sqrt(a2);
  const double vn = w[n];
  e.lam[0] = vn - a; e.lam[1] = vn; e.lam[2] = vn; e.lam[3] = vn; e.lam[4] = vn + a;
  e.rn0 = ddiv(-a, w[0]);
  e.a2 = a2;
  e.l0n = ddiv(-0.5 * w[0], a);
  e.l04 = ddiv(0.5, a2);
  e.le4 = ddiv(-1.0, a2);
}
template <int A>
__device__ __forceinline__ double hprim_project(const HPrimEig& e, int i, const double v[5]) {
  double acc = 0.0;
  bool first = true;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    if (hprim_L_nz<A>(i, j)) {
      const double t = hprim_L<A>(e, i, j) * v[j];
      acc = first ? t : acc + t;
      first = false;
    }
  }
  return acc;
}

// Hydro Roe flux (Source/RiemannSolvers_Hydro_Roe_HelperModule.py:68-328, :342-596, :614-869).
// Wave order x = (a-, vy, vz, entropy, a+), y = (a-, entropy, vz, vx, a+),
// z = (a-, vy, entropy, vx, a+).
template <int A>
__device__ __forceinline__ void hroe_flux(const double wl[5], const double wr[5], double gamma, bool efix,
                                          double eps, double flux[5]) {
  constexpr int n = A + 1;
  double ul[5], ur[5];
  hprim_to_cons<A>(wl, gamma, ul);
  hprim_to_cons<A>(wr, gamma, ur);
  const double sl = sqrt(wl[0]);
  const double sr = sqrt(wr[0]);
  const double isum = ddiv(1.0, sl + sr);
  double v[4];
#pragma unroll
  for (int k = 1; k <= 3; ++k) v[k] = (sl * wl[k] + sr * wr[k]) * isum;
  const double vsq = A == 2 ? (v[3] * v[3] + v[1] * v[1] + v[2] * v[2])
                   : A == 1 ? (v[2] * v[2] + v[3] * v[3] + v[1] * v[1])
                            : (v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
  const double H = (ddiv(ul[4] + wl[4], sl) + ddiv(ur[4] + wr[4], sr)) * isum;
  const double a2 = (gamma - 1.0) * dmax(H - 0.5 * vsq, SMALL_VALUE);
  const double a = sqrt(a2);
  const double vn = v[n];
  double lam[5] = {vn - a, vn, vn, vn, vn + a};
  if (efix) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double x = lam[k];
      if (dlt(fabs(x), 2.0 * eps) && !is_zero(x)) {
        const double corr = eps + ddiv(sq(x), 4.0 * eps);
        lam[k] = is_pos(x) ? x + corr : x - corr;
      }
    }
  }
  double fl[5], fr[5];
  fl[0] = ul[n]; fr[0] = ur[n];
  fl[1] = ul[n] * wl[1]; fr[1] = ur[n] * wr[1];
  fl[2] = ul[n] * wl[2]; fr[2] = ur[n] * wr[2];
  fl[3] = ul[n] * wl[3]; fr[3] = ur[n] * wr[3];
  fl[n] = fl[n] + wl[4]; fr[n] = fr[n] + wr[4];
  fl[4] = (ul[4] + wl[4]) * wl[n]; fr[4] = (ur[4] + wr[4]) * wr[n];
  if (is_nonpos(lam[4])) {
#pragma unroll
    for (int i = 0; i < 5; ++i) flux[i] = fr[i];
    return;
  }
  if (is_nonneg(lam[0])) {
#pragma unroll
    for (int i = 0; i < 5; ++i) flux[i] = fl[i];
    return;
  }
  const double nf = ddiv(0.5, a2);
  const double g1 = gamma - 1.0;
  const double gn = ddiv(g1, a2);
  double du[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) du[i] = ur[i] - ul[i];
  double c[5];  // L . du in the reference order j = 0..4 (structural zeros skipped)
  if (A == 0) {
    const double l00 = nf * (0.5 * g1 * vsq + v[1] * a);
    const double l01 = -nf * (g1 * v[1] + a);
    const double l02 = -nf * g1 * v[2];
    const double l03 = -nf * g1 * v[3];
    const double l04 = nf * g1;
    c[0] = l00 * du[0] + l01 * du[1] + l02 * du[2] + l03 * du[3] + l04 * du[4];
    c[1] = -v[2] * du[0] + 1.0 * du[2];
    c[2] = -v[3] * du[0] + 1.0 * du[3];
    c[3] = (1.0 - nf * g1 * vsq) * du[0] + gn * v[1] * du[1] + gn * v[2] * du[2] + gn * v[3] * du[3] + -gn * du[4];
    const double l40 = nf * (0.5 * g1 * vsq - v[1] * a);
    const double l41 = -nf * (g1 * v[1] - a);
    c[4] = l40 * du[0] + l41 * du[1] + l02 * du[2] + l03 * du[3] + l04 * du[4];
  } else if (A == 1) {
    const double l00 = nf * (0.5 * g1 * vsq + v[2] * a);
    const double l01 = -nf * g1 * v[1];
    const double l02 = -nf * (g1 * v[2] + a);
    const double l03 = -nf * g1 * v[3];
    const double l04 = nf * g1;
    c[0] = l00 * du[0] + l01 * du[1] + l02 * du[2] + l03 * du[3] + l04 * du[4];
    c[1] = (1.0 - nf * g1 * vsq) * du[0] + gn * v[1] * du[1] + gn * v[2] * du[2] + gn * v[3] * du[3] + -gn * du[4];
    c[2] = -v[3] * du[0] + 1.0 * du[3];
    c[3] = -v[1] * du[0] + 1.0 * du[1];
    const double l40 = nf * (0.5 * g1 * vsq - v[2] * a);
    const double l42 = -nf * (g1 * v[2] - a);
    c[4] = l40 * du[0] + l01 * du[1] + l42 * du[2] + l03 * du[3] + l04 * du[4];
  } else {
    const double l00 = nf * (0.5 * g1 * vsq + v[3] * a);
    const double l01 = -nf * g1 * v[1];
    const double l02 = -nf * g1 * v[2];
    const double l03 = -nf * (g1 * v[3] + a);
    const double l04 = nf * g1;
    c[0] = l00 * du[0] + l01 * du[1] + l02 * du[2] + l03 * du[3] + l04 * du[4];
    c[1] = -v[2] * du[0] + 1.0 * du[2];
    c[2] = (1.0 - nf * g1 * vsq) * du[0] + gn * v[1] * du[1] + gn * v[2] * du[2] + gn * v[3] * du[3] + -gn * du[4];
    c[3] = -v[1] * du[0] + 1.0 * du[1];
    const double l40 = nf * (0.5 * g1 * vsq - v[3] * a);
    const double l43 = -nf * (g1 * v[3] - a);
    c[4] = l40 * du[0] + l01 * du[1] + l02 * du[2] + l43 * du[3] + l04 * du[4];
  }
  double amps[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) amps[k] = 0.5 * fabs(lam[k]) * c[k];
  double R[5][5];
  // non-zero entries only; R[i][j] for wave j
  if (A == 0) {
    R[0][0] = 1.0; R[1][0] = v[1] - a; R[2][0] = v[2]; R[3][0] = v[3]; R[4][0] = H - v[1] * a;
    R[2][1] = 1.0; R[4][1] = v[2];
    R[3][2] = 1.0; R[4][2] = v[3];
    R[0][3] = 1.0; R[1][3] = v[1]; R[2][3] = v[2]; R[3][3] = v[3]; R[4][3] = 0.5 * vsq;
    R[0][4] = 1.0; R[1][4] = v[1] + a; R[2][4] = v[2]; R[3][4] = v[3]; R[4][4] = H + v[1] * a;
  } else if (A == 1) {
    R[0][0] = 1.0; R[1][0] = v[1]; R[2][0] = v[2] - a; R[3][0] = v[3]; R[4][0] = H - v[2] * a;
    R[0][1] = 1.0; R[1][1] = v[1]; R[2][1] = v[2]; R[3][1] = v[3]; R[4][1] = 0.5 * vsq;
    R[3][2] = 1.0; R[4][2] = v[3];
    R[1][3] = 1.0; R[4][3] = v[1];
    R[0][4] = 1.0; R[1][4] = v[1]; R[2][4] = v[2] + a; R[3][4] = v[3]; R[4][4] = H + v[2] * a;
  } else {
    R[0][0] = 1.0; R[1][0] = v[1]; R[2][0] = v[2]; R[3][0] = v[3] - a; R[4][0] = H - v[3] * a;
    R[2][1] = 1.0; R[4][1] = v[2];
    R[0][2] = 1.0; R[1][2] = v[1]; R[2][2] = v[2]; R[3][2] = v[3]; R[4][2] = 0.5 * vsq;
    R[1][3] = 1.0; R[4][3] = v[1];
    R[0][4] = 1.0; R[1][4] = v[1]; R[2][4] = v[2]; R[3][4] = v[3] + a; R[4][4] = H + v[3] * a;
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    double acc = 0.5 * (fl[i] + fr[i]);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const bool nz = A == 0 ? ((j == 0 || j == 3 || j == 4) || (j == 1 && (i == 2 || i == 4)) || (j == 2 && (i == 3 || i == 4)))
                    : A == 1 ? ((j == 0 || j == 1 || j == 4) || (j == 2 && (i == 3 || i == 4)) || (j == 3 && (i == 1 || i == 4)))
                             : ((j == 0 || j == 2 || j == 4) || (j == 1 && (i == 2 || i == 4)) || (j == 3 && (i == 1 || i == 4)));
      if (nz) acc = acc - amps[j] * R[i][j];
    }
    flux[i] = acc;
  }
}

}  // namespace mhdk
