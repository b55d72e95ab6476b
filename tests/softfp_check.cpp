// Host check of the integer-pipe FP64 add, subtract and multiply (softfp.cuh):
// every result is compared bit for bit with the host's IEEE-754 arithmetic (NaN
// results only as NaN).  Operand pairs come from generators aimed at the cases the
// integer paths must get right: random bit patterns (specials, subnormals), close
// magnitudes and cancellation, every exponent difference, significands with long
// runs of ones or zeros (rounding ties and carries), products near the overflow and
// underflow limits.
//
// Division and square root are checked the same way, once with the host's seed
// reciprocals and once with seeds perturbed by up to 2^-12 relative (the integer Newton
// steps must absorb any seed within that of the true value).
//
// usage: softfp_check <pairs per generator> <seed>
// prints one line per generator and "mismatches N" last; exit status 1 on a mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "softfp.cuh"

namespace {

struct Rng {  // splitmix64
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  uint32_t below(uint32_t n) { return static_cast<uint32_t>(next() % n); }
};

double make(uint64_t sign, uint64_t exp, uint64_t frac) {
  return sfp::from_bits((sign << 63) | ((exp & 0x7ffu) << 52) | (frac & sfp::kFrac));
}

// a significand with runs of equal bits (ties, carries and long borrows)
uint64_t runs(Rng& r) {
  uint64_t f = 0;
  int pos = 0;
  while (pos < 52) {
    const int len = 1 + static_cast<int>(r.below(20));
    if (r.next() & 1) f |= ((len >= 64 ? ~0ull : ((1ull << len) - 1)) << pos);
    pos += len;
  }
  return f & sfp::kFrac;
}

uint64_t mismatches = 0;

// seeds off by a pseudo-random relative error in [-2^-12, 2^-12]
struct JitterSeed {
  mutable uint64_t s;
  float jitter() const {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return 1.0f + (static_cast<float>(static_cast<int32_t>(s >> 32)) / 2147483648.0f) * (1.0f / 4096.0f);
  }
  float rcp(float f) const { return (1.0f / f) * jitter(); }
  float rsqrt(float f) const { return (1.0f / std::sqrt(f)) * jitter(); }
};
JitterSeed jitter_seed{12345};

bool same(double got, double want) {
  if (std::isnan(want)) return std::isnan(got);
  return sfp::to_bits(got) == sfp::to_bits(want);
}

void check(double x, double y) {
  const double s = sfp::add(x, y), d = sfp::sub(x, y), p = sfp::mul(x, y);
  const double ws = x + y, wd = x - y, wp = x * y;
  const double q = sfp::div(x, y), wq = x / y, qj = sfp::div_seeded(x, y, jitter_seed);
  const double r = sfp::sqrt(x), wr = std::sqrt(x), rj = sfp::sqrt_seeded(x, jitter_seed);
  if (!same(q, wq) || !same(qj, wq) || !same(r, wr) || !same(rj, wr)) {
    if (mismatches < 20)
      std::printf("mismatch x=%016llx y=%016llx div %016llx/%016llx/%016llx sqrt %016llx/%016llx/%016llx\n",
                  (unsigned long long)sfp::to_bits(x), (unsigned long long)sfp::to_bits(y),
                  (unsigned long long)sfp::to_bits(q), (unsigned long long)sfp::to_bits(qj),
                  (unsigned long long)sfp::to_bits(wq), (unsigned long long)sfp::to_bits(r),
                  (unsigned long long)sfp::to_bits(rj), (unsigned long long)sfp::to_bits(wr));
    ++mismatches;
  }
  if (!same(s, ws) || !same(d, wd) || !same(p, wp)) {
    if (mismatches < 20)
      std::printf("mismatch x=%016llx y=%016llx add %016llx/%016llx sub %016llx/%016llx mul %016llx/%016llx\n",
                  (unsigned long long)sfp::to_bits(x), (unsigned long long)sfp::to_bits(y),
                  (unsigned long long)sfp::to_bits(s), (unsigned long long)sfp::to_bits(ws),
                  (unsigned long long)sfp::to_bits(d), (unsigned long long)sfp::to_bits(wd),
                  (unsigned long long)sfp::to_bits(p), (unsigned long long)sfp::to_bits(wp));
    ++mismatches;
  }
}

}  // namespace

int main(int argc, char** argv) {
  const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1000000;
  Rng r{argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1};
  const char* names[] = {"random bits", "moderate exponents", "close magnitudes", "exponent differences 0-70",
                         "runs of equal bits", "near overflow/underflow", "zeros, subnormals, specials",
                         "small integers and halves", "exact and near-tie quotients, squares"};
  // fixed operands at known hard spots: halfway cases of the sum and product, rounding carries
  // into the exponent, overflow and underflow thresholds, exact quotients and squares
  {
    const double e = std::ldexp(1.0, -52), m = 1.7976931348623157e308, tiny = std::ldexp(1.0, -1022);
    const double fixed[] = {1.0, 1.0 + e, 1.0 - e / 2, 1.5, 2.0, 3.0, 1.0 / 3.0, 0.1, 0.2, 0.3, std::ldexp(1.0, -53),
                            3 * std::ldexp(1.0, -53), m, m / 2, std::ldexp(1.0, 1023), tiny, tiny * (1 + e), 2 * tiny,
                            std::ldexp(1.0, 511), std::ldexp(1.0, -511), std::ldexp(1.0 + e, 600),
                            std::ldexp(1.0, -600), 0.0, -0.0, 4.0, 9.0, 1e-300, 1e300, -1.0, -(1.0 + e)};
    const uint64_t before = mismatches;
    for (double x : fixed)
      for (double y : fixed) check(x, y);
    std::printf("%-30s %llu pairs, %llu mismatches\n", "fixed hard operands",
                (unsigned long long)(sizeof(fixed) / sizeof(fixed[0]) * (sizeof(fixed) / sizeof(fixed[0]))),
                (unsigned long long)(mismatches - before));
  }
  for (int g = 0; g < 9; ++g) {
    const uint64_t before = mismatches;
    for (uint64_t i = 0; i < n; ++i) {
      double x, y;
      switch (g) {
        case 0:
          x = sfp::from_bits(r.next());
          y = sfp::from_bits(r.next());
          break;
        case 1:
          x = make(r.next() & 1, 1023 - 40 + r.below(81), r.next());
          y = make(r.next() & 1, 1023 - 40 + r.below(81), r.next());
          break;
        case 2: {  // y = -x perturbed in its last bits, or an exponent apart
          const uint64_t e = 1 + r.below(2046);
          x = make(r.next() & 1, e, r.next());
          uint64_t yb = sfp::to_bits(x) ^ (r.next() & ((1ull << (1 + r.below(53))) - 1));
          if (r.next() & 1) yb ^= sfp::kSign;
          if ((r.next() & 3) == 0) yb -= (1ull << 52);
          y = sfp::from_bits(yb);
          break;
        }
        case 3: {
          const uint64_t e = 100 + r.below(1848);
          x = make(r.next() & 1, e, r.next() & 1 ? r.next() : runs(r));
          y = make(r.next() & 1, e - r.below(71), r.next() & 1 ? r.next() : runs(r));
          if (r.next() & 1) { const double t = x; x = y; y = t; }
          break;
        }
        case 4:
          x = make(r.next() & 1, 1023 - 60 + r.below(121), runs(r));
          y = make(r.next() & 1, 1023 - 60 + r.below(121), runs(r));
          break;
        case 5: {  // exponent sums near the limits of the product and the sum
          const uint64_t ea = 1 + r.below(2046);
          const int64_t target = (r.next() & 1) ? 2046 - static_cast<int64_t>(r.below(6))
                                                : 1 + static_cast<int64_t>(r.below(6));
          int64_t eb = target + 1023 - static_cast<int64_t>(ea) + static_cast<int64_t>(r.below(3)) - 1;
          if (eb < 0) eb = r.below(3);
          if (eb > 2047) eb = 2046 - r.below(3);
          x = make(r.next() & 1, ea, r.next() & 1 ? r.next() : runs(r));
          y = make(r.next() & 1, static_cast<uint64_t>(eb), r.next() & 1 ? r.next() : runs(r));
          if (r.next() & 1) {  // or a sum at the top of the range
            x = make(r.next() & 1, 2046 - r.below(2), r.next() | (r.next() & 1 ? sfp::kFrac : 0));
            y = make(r.next() & 1, 2046 - r.below(60), r.next() | (r.next() & 1 ? sfp::kFrac : 0));
          }
          break;
        }
        case 6: {
          const uint64_t pick[] = {0, 0x8000000000000000ull, 0x7ff0000000000000ull, 0xfff0000000000000ull,
                                   0x7ff8000000000000ull, 0x0000000000000001ull, 0x000fffffffffffffull,
                                   0x0010000000000000ull, 0x8010000000000000ull, 0x7fefffffffffffffull};
          x = sfp::from_bits(r.next() & 1 ? pick[r.below(10)] : (r.next() & 0x800fffffffffffffull) | (static_cast<uint64_t>(r.below(4)) << 52));
          y = sfp::from_bits(r.next() & 1 ? pick[r.below(10)] : r.next());
          if (r.next() & 1) { const double t = x; x = y; y = t; }
          break;
        }
        case 8: {  // y * k with k short (exact or one-off quotients); x = k^2 (+-1 ulp)
          const uint64_t k = (r.next() >> (11 + r.below(40))) | 1u;
          y = make(r.next() & 1, 1 + r.below(2046), r.next() & 1 ? r.next() : runs(r));
          const double kd = static_cast<double>(k) * (r.next() & 1 ? 1.0 : 0.5);
          x = y * kd;
          if (r.next() & 1) x = sfp::from_bits(sfp::to_bits(x) + (r.next() & 1 ? 1 : -1));
          if (r.next() & 1) {
            const uint64_t s2 = (r.next() >> (12 + r.below(30))) | 1u;
            x = static_cast<double>(s2) * static_cast<double>(s2) * std::ldexp(1.0, static_cast<int>(r.below(200)) - 100);
            if (r.next() & 1) x = sfp::from_bits(sfp::to_bits(x) + (r.next() & 1 ? 1 : -1));
          }
          break;
        }
        default: {
          x = static_cast<double>(static_cast<int>(r.below(2001)) - 1000) * (r.next() & 1 ? 0.5 : 1.0);
          y = static_cast<double>(static_cast<int>(r.below(2001)) - 1000) * (r.next() & 1 ? 0.25 : 1.0);
          break;
        }
      }
      check(x, y);
    }
    std::printf("%-30s %llu pairs, %llu mismatches\n", names[g], (unsigned long long)n,
                (unsigned long long)(mismatches - before));
  }
  std::printf("mismatches %llu\n", (unsigned long long)mismatches);
  return mismatches ? 1 : 0;
}
