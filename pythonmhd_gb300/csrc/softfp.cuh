// IEEE-754 binary64 addition, subtraction and multiplication, rounded to nearest
// even, computed with 32/64-bit integer instructions.
//
// GB300 issues FP64 adds and multiplies at about 1.6 lanes per SM per clock, while
// its integer pipes run some forty times faster.  Every operation here returns the
// same bits as the FP64 instruction for every pair of operands, so a kernel can send
// any subset of its adds and multiplies through these functions, keep the other
// pipe busy instead of leaving it idle, and still reproduce the FP64 results bit for
// bit.  Only the common case is done in integers: both operands normal (or, for the
// sum, one of them a zero) and a normal, finite result; every other case (subnormal
// operands or results, infinities, NaN, overflow of the product) takes the FP64
// instruction.
//
// The same code compiles for the host, where the tests compare it bit for bit with
// the host's IEEE arithmetic.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SFP_FN __host__ __device__ __forceinline__
#else
#define SFP_FN inline
#endif

namespace sfp {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

SFP_FN uint64_t to_bits(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

SFP_FN double from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(b));
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// The FP64 instructions, for the cases the integer paths leave out.
SFP_FN double hw_add(double x, double y) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(x, y);
#else
  return x + y;
#endif
}

SFP_FN double hw_mul(double x, double y) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(x, y);
#else
  return x * y;
#endif
}

SFP_FN double hw_div(double x, double y) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(x, y);
#else
  return x / y;
#endif
}

SFP_FN double hw_sqrt(double x) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(x);
#else
  return __builtin_sqrt(x);
#endif
}

SFP_FN uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

SFP_FN float u2f(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// Seeds for the Newton iterations: a few correct bits are all they must give (one
// FP32 Newton step follows each).  On the GPU they are the SFU's approximate
// reciprocal and reciprocal square root.
struct ApproxSeed {
  SFP_FN float rcp(float f) const {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
#else
    return 1.0f / f;
#endif
  }
  SFP_FN float rsqrt(float f) const {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
#else
    return 1.0f / __builtin_sqrtf(f);
#endif
  }
};

SFP_FN float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}

// floor(x * y / 2^64)
SFP_FN uint64_t mulhi64(uint64_t x, uint64_t y) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(x, y);
#else
  return static_cast<uint64_t>((static_cast<unsigned __int128>(x) * y) >> 64);
#endif
}

SFP_FN int clz64(uint64_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(x));
#else
  return __builtin_clzll(x);
#endif
}

// Full product of two 53-bit significands, P = hi * 2^64 + lo, from 32-bit limbs
// (x1, y1 < 2^21): three wide multiplies for the partial products and one carry.
SFP_FN void mul53(uint64_t x, uint64_t y, uint64_t& hi, uint64_t& lo) {
  const uint32_t x0 = static_cast<uint32_t>(x), x1 = static_cast<uint32_t>(x >> 32);
  const uint32_t y0 = static_cast<uint32_t>(y), y1 = static_cast<uint32_t>(y >> 32);
  const uint64_t p00 = static_cast<uint64_t>(x0) * y0;
  const uint64_t mid = static_cast<uint64_t>(x1) * y0 + static_cast<uint64_t>(x0) * y1;  // < 2^54
  const uint64_t p11 = static_cast<uint64_t>(x1) * y1;                                    // < 2^42
  lo = p00 + (mid << 32);
  hi = p11 + (mid >> 32) + (lo < p00 ? 1u : 0u);
}

// x * y.  With biased exponents ea, eb in [1, 2046] the product of the significands
// P = ma * mb lies in [2^104, 2^106) and the result's biased exponent is
// e = ea + eb - 1023, plus one when P >= 2^105, plus one more when rounding carries
// out of the significand.  e in [1, 2044] keeps all of those normal and finite.
SFP_FN double mul(double x, double y) {
  const uint64_t a = to_bits(x), b = to_bits(y);
  const uint32_t ea = static_cast<uint32_t>(a >> 52) & 0x7ffu;
  const uint32_t eb = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  const uint32_t e = ea + eb - 1023u;  // wraps when ea + eb < 1023
  if (ea - 1u > 2045u || eb - 1u > 2045u || e - 1u > 2043u) return hw_mul(x, y);
  uint64_t hi, lo;
  mul53((a & kFrac) | kHidden, (b & kFrac) | kHidden, hi, lo);
  const uint64_t t = (hi << 12) | (lo >> 52);  // P >> 52, in [2^52, 2^54)
  const uint64_t r = lo << 12;                 // the 52 bits below, left-aligned
  const uint32_t norm = static_cast<uint32_t>(t >> 53);
  uint64_t m;
  uint32_t rnd, sticky;
  if (norm) {
    m = t >> 1;
    rnd = static_cast<uint32_t>(t) & 1u;
    sticky = r != 0;
  } else {
    m = t;
    rnd = static_cast<uint32_t>(r >> 63);
    sticky = (r << 1) != 0;
  }
  m += rnd & (sticky | (static_cast<uint32_t>(m) & 1u));
  // m carries the hidden bit, so adding it to (exponent - 1) << 52 also propagates a
  // rounding carry (m = 2^53) into the exponent field.
  return from_bits(((a ^ b) & kSign) | ((static_cast<uint64_t>(e + norm - 1u) << 52) + m));
}

// x + y.  Operands are ordered by magnitude, |L| >= |S|.  The significands are
// placed with the hidden bit at bit 62 and ten zero bits below; S is shifted right by
// the exponent difference with the bits shifted out ORed into bit 0 ("sticky
// jamming").  Because L's low ten bits are zero, the jammed sum or difference is odd
// exactly when bits were lost and agrees with the exact one in every bit from 1
// upward, and after normalisation the rounding bit sits at bit 9, so the rounding
// decision (round bit, and sticky = any bit below it) is the exact one.
SFP_FN double add(double x, double y) {
  const uint64_t a = to_bits(x), b = to_bits(y);
  const uint64_t aa = a & ~kSign, bb = b & ~kSign;
  const bool swap = aa < bb;
  const uint64_t L = swap ? b : a;
  const uint64_t LL = swap ? bb : aa, SS = swap ? aa : bb;
  const uint32_t eL = static_cast<uint32_t>(LL >> 52), eS = static_cast<uint32_t>(SS >> 52);
  if (eL - 1u > 2044u || eS == 0u) {
    // a zero operand with a finite other one: the other one, and for two zeros
    // +0 unless both are -0
    if (SS == 0u && eL < 2047u) return from_bits(LL == 0u ? (a & b) : L);
    return hw_add(x, y);
  }
  const uint32_t d = eL - eS;
  const uint64_t mL = ((LL & kFrac) | kHidden) << 10;
  const uint64_t mS0 = ((SS & kFrac) | kHidden) << 10;
  uint64_t mS;
  if (d == 0u) {
    mS = mS0;
  } else if (d < 64u) {
    mS = (mS0 >> d) | ((mS0 << (64u - d)) != 0u ? 1u : 0u);
  } else {
    mS = 1u;
  }
  const bool sub = static_cast<int64_t>(a ^ b) < 0;
  uint64_t R = sub ? mL - mS : mL + mS;
  if (R == 0u) return 0.0;  // x == -y: +0 when rounding to nearest
  int e = static_cast<int>(eL);
  if (R >> 63) {
    R = (R >> 1) | (R & 1u);
    e += 1;
  } else {
    const int lz = clz64(R) - 1;
    R <<= lz;
    e -= lz;
  }
  if (e <= 0) return hw_add(x, y);  // subnormal result
  uint64_t m = R >> 10;
  const uint32_t rnd = static_cast<uint32_t>(R >> 9) & 1u;
  const uint32_t sticky = (R & 0x1ffu) != 0u;
  m += rnd & (sticky | (static_cast<uint32_t>(m) & 1u));
  return from_bits((L & kSign) | ((static_cast<uint64_t>(e - 1) << 52) + m));
}

SFP_FN double sub(double x, double y) { return add(x, from_bits(to_bits(y) ^ kSign)); }

// x / y by integer Newton-Raphson division with an exact remainder check.
//  * With significands mx, my in [2^52, 2^53), N = mx or 2 mx so that N / my is in
//    [1, 2); the result is Q = floor(N 2^53 / my), 54 bits (53 of significand and the
//    rounding bit), and the remainder R = N 2^53 - Q my decides the sticky bit.
//  * Z approximates 2^115 / my in (2^62, 2^63] from below.  Seed: the FP32 reciprocal
//    of my's top 24 bits, sharpened by one FP32 Newton step to within about 2^-22,
//    then lowered by 2^-21 so that it lies below, with relative error eps < 2^-20.
//  * Each fixed-point Newton step Z' = Z + Z (2^115 - my Z) / 2^115 (truncated
//    products) keeps Z' below the target and gives eps' <= eps^2 + 2^-61; two steps
//    leave eps < 2^-60.9.
//  * Q0 = floor(N Z / 2^62) then lies within two of Q from below; the remainder is
//    computed exactly modulo 2^64 (it is below 3 my < 2^55) and two conditional steps
//    correct Q0.
// Fast path: normal operands and a normal result (biased exponent 1..2045 before a
// rounding carry), and a zero over a normal divisor; everything else takes the FP64
// division.
template <class Seed>
SFP_FN double div_seeded(double x, double y, const Seed& seed) {
  const uint64_t a = to_bits(x), b = to_bits(y);
  const uint32_t ex = static_cast<uint32_t>(a >> 52) & 0x7ffu;
  const uint32_t ey = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  const uint64_t mx = (a & kFrac) | kHidden, my = (b & kFrac) | kHidden;
  const uint32_t lt = mx < my ? 1u : 0u;
  const uint32_t e = ex - ey + 1023u - lt;  // wraps below zero
  if (ex - 1u > 2045u || ey - 1u > 2045u || e - 1u > 2044u) {
    // a zero dividend over a normal divisor: a zero with the sign of the quotient
    if ((a << 1) == 0u && ey - 1u <= 2045u) return from_bits((a ^ b) & kSign);
    return hw_div(x, y);
  }
  // seed: my's top 24 bits as a float (exact), its reciprocal, one FP32 Newton step
  const float f = u2f(static_cast<uint32_t>(my >> 29) - 0x800000u + (150u << 23));
  float r = seed.rcp(f);
  r = ffma(r, ffma(-f, r, 1.0f), r);  // r ~ 1/f in (2^-24, 2^-23]
  const uint32_t rb = f2u(r);
  uint64_t Z = static_cast<uint64_t>((rb & 0x7fffffu) | 0x800000u) << ((rb >> 23) - 64u);  // r 2^86
  Z -= (Z >> 21) + 1u;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    uint64_t hi, lo;
    mul53(my, Z, hi, lo);  // my Z < 2^116 (Z < 2^63: the limb product still fits)
    // E = 2^115 - my Z > 0 ; take E >> 51
    const uint64_t ehi = (1ull << 51) - hi - (lo != 0u ? 1u : 0u);
    const uint64_t elo = 0u - lo;
    const uint64_t E = (ehi << 13) | (elo >> 51);
    Z += mulhi64(Z, E);
  }
  const uint64_t N = mx << lt;
  uint64_t hi, lo;
  mul53(N, Z, hi, lo);
  uint64_t Q = (hi << 2) | (lo >> 62);
  uint64_t R = (N << 53) - Q * my;
  if (R >= my) { R -= my; ++Q; }
  if (R >= my) { R -= my; ++Q; }
  uint64_t m = Q >> 1;
  const uint32_t rnd = static_cast<uint32_t>(Q) & 1u;
  const uint32_t sticky = R != 0u;
  m += rnd & (sticky | (static_cast<uint32_t>(m) & 1u));
  return from_bits(((a ^ b) & kSign) | ((static_cast<uint64_t>(e - 1u) << 52) + m));
}

// sqrt(x) by integer Newton-Raphson on the reciprocal square root with an exact
// remainder check.
//  * For x = mx 2^(ex-1075) > 0 normal, K = mx 2^54 (ex odd) or mx 2^55 (ex even),
//    K in [2^106, 2^108); the result is S = floor(sqrt K), 54 bits, with sticky
//    = (K != S^2), and biased exponent floor((ex - 1023) / 2) + 1023, always normal.
//  * With u = K / 2^106 in [1, 4), Y approximates 2^63 / sqrt(u) in (2^62, 2^63] from
//    below.  Seed: the FP32 reciprocal square root of u (K's top 24 bits), sharpened
//    by one FP32 Newton step, lowered by 2^-21.  Each fixed-point step
//    Y' = Y + Y h / 2 with h = 1 - u Y^2 / 2^126 rounds u Y^2 up and the update down,
//    so Y stays below and the error goes from eps to 1.5 eps^2 + 2^-58.5.
//  * S0 = floor(K Y / 2^116) then lies within two of S from below; K - S0^2 is
//    computed exactly modulo 2^64 (its magnitude is below 2^57) and two conditional
//    steps correct S0.
// Fast path: positive normal x, and zeros (returned as they are); negative numbers,
// subnormals, infinities and NaN take the FP64 square root.
template <class Seed>
SFP_FN double sqrt_seeded(double x, const Seed& seed) {
  const uint64_t a = to_bits(x);
  const uint32_t ex = static_cast<uint32_t>(a >> 52);  // sign included: negative x fails below
  if (ex - 1u > 2045u) return (a << 1) == 0u ? x : hw_sqrt(x);  // sqrt(+-0) = +-0
  const uint64_t mx = (a & kFrac) | kHidden;
  const uint32_t odd = (ex & 1u) ^ 1u;  // 1 when ex - 1023 is odd
  const uint64_t M = mx << odd;         // K = M 2^54, u = M / 2^52
  // seed: u from M's top 24 bits as a float (within 2^-23)
  const uint32_t top = static_cast<uint32_t>(M >> (29u + odd));  // in [2^23, 2^24)
  const float f = u2f(top - 0x800000u + ((127u + odd) << 23));
  float r = seed.rsqrt(f);
  r = r * ffma(-0.5f * f * r, r, 1.5f);  // one FP32 Newton step: r ~ 1/sqrt(u) in (0.5, 1]
  const uint32_t rb = f2u(r);
  uint64_t Y = static_cast<uint64_t>((rb & 0x7fffffu) | 0x800000u) << ((rb >> 23) - 87u);  // r 2^63
  Y -= (Y >> 21) + 1u;
  const uint64_t U = M << 10;  // u 2^62, exact
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const uint64_t Y2 = mulhi64(Y, Y) + 1u;   // y^2 2^62, rounded up
    const uint64_t UY = mulhi64(U, Y2) + 1u;  // u y^2 2^60, rounded up
    const uint64_t H = UY < (1ull << 60) ? (1ull << 60) - UY : 0u;  // h 2^60
    Y += mulhi64(Y, H) << 3;                  // y h / 2, in units of 2^-63
  }
  // S0 = floor(K Y / 2^116) = floor(M Y / 2^62)
  const uint64_t Sh = mulhi64(M, Y), Sl = M * Y;
  uint64_t S = (Sh << 2) | (Sl >> 62);
  int64_t R = static_cast<int64_t>((M << 54) - S * S);  // K - S^2, exact modulo 2^64
  if (R > static_cast<int64_t>(2u * S)) { R -= static_cast<int64_t>(2u * S + 1u); ++S; }
  if (R > static_cast<int64_t>(2u * S)) { R -= static_cast<int64_t>(2u * S + 1u); ++S; }
  uint64_t m = S >> 1;
  const uint32_t rnd = static_cast<uint32_t>(S) & 1u;
  const uint32_t sticky = R != 0;
  m += rnd & (sticky | (static_cast<uint32_t>(m) & 1u));
  const uint32_t e = ((ex + 1025u) >> 1) - 1u;  // floor((ex - 1023) / 2) + 1023
  return from_bits((static_cast<uint64_t>(e - 1u) << 52) + m);
}

SFP_FN double div(double x, double y) { return div_seeded(x, y, ApproxSeed()); }
SFP_FN double sqrt(double x) { return sqrt_seeded(x, ApproxSeed()); }

}  // namespace sfp
