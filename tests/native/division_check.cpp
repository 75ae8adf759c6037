// Host restatement of the erosion kernel's quotient (neg_div_rn_bits in
// fs_kernels.cu): q0 = RN(num * R) with R = RN(1/D), r0 = num - q0*D by a
// fused multiply-add, q1 = RN(q0 + r0*R), accepted when q0 is not a power of
// two, its exponent is far from the range limits, D and D*ulp(q0) are
// positive normal numbers and |r0| < D*ulp(q0) --
// then q0 is within one ulp of num/D, r0 is exact, and by Markstein's theorem
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990) q1 = RN(num/D). The check
// compares every accepted q1 with the IEEE quotient on random operands and
// on operands built next to rounding midpoints (num = RN(D * midpoint)),
// D of all significand shapes and exponents (below 1, huge, negative, the
// receiver slopes' divisors), and reports the acceptance rate.
// It checks the integer form the kernel uses the same way: q0 = RN(num * R)
// and the residual num - q0*D exactly in integer arithmetic, in units of
// ulp(q0)*ulp(D): R' = mn*2^k - mq*mD from the significands (implicit bit
// set) and k = en - eq - eD + 1075 from the biased exponents. Because
// |q0 - num/D| <= 2^-52 |num/D| (1 + 2^-52), |R'| < 2.01 mD < 2^55 and the
// difference taken modulo 2^64 is exact; num/D = q0 + (R'/mD) ulp(q0) in
// magnitude, so RN(num/D) is q0 when 2|R'| < mD and q0 one ulp up or down
// when mD < 2|R'| < 3 mD (a quotient is never a rounding midpoint).
// A third form divides by any denominator (the n = 2 erosion's, which has no
// tabled reciprocal): the FP32 reciprocal of |den| truncated to FP32 as the
// seed (IEEE round to nearest, as __frcp_rn), one FP64 Newton step
// r1 = r0 + r0*(1 - |den|*r0) by fused multiply-adds, q0 = RN(|num|*r1)
// within ~2^8.2 ulp, then round_quotient_bits (fs_bits.h), the integer
// rounding the kernel uses.
// Usage: division_check <cases> <seed>; exit 1 on the first mismatch.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../../barnes2019-landscape_gb300/csrc/fs_bits.h"

static double dbl(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }

// Returns true and *q = RN(num/D) when the fast path accepts.
static bool fast_quotient(double num, double D, double R, double *q) {
  const double Rn = -R;
  const double q0n = num * Rn;
  const double r0 = std::fma(q0n, D, num);
  const uint64_t q0b = bits(q0n);
  const int e = (int)((q0b << 1) >> 53);
  const int ed = (int)(bits(D) >> 52);
  const int et = ed + e - 1075;
  if (e >= 64 && e <= 1980 && ed >= 1 && ed <= 2046 && et >= 1 && et <= 2046 &&
      (q0b << 12) != 0) {
    const uint64_t thr = (uint64_t)((int64_t)bits(D) + ((int64_t)(e - 1075) << 52));
    if ((bits(r0) << 1) < (thr << 1)) {
      *q = -std::fma(r0, Rn, q0n);
      return true;
    }
  }
  return false;
}

// Returns true and *q = RN(num/D) when the integer form accepts.
static bool int_quotient(double num, double D, double R, double *q) {
  const uint64_t kMant = (1ull << 52) - 1, kHidden = 1ull << 52;
  const uint64_t numb = bits(num), Db = bits(D);
  const uint64_t q0b = bits(num * -R);
  const int eq = (int)((q0b << 1) >> 53);
  const int en = (int)((numb << 1) >> 53);
  const int ed = (int)((Db << 1) >> 53);
  const int k = en - eq - ed + 1075;
  if ((unsigned)(eq - 64) <= 1980u - 64u && (unsigned)(en - 1) <= 2045u &&
      (unsigned)(ed - 1) <= 2043u && (unsigned)(k - 48) <= 12u && (q0b << 12) != 0) {
    const uint64_t mq = (q0b & kMant) | kHidden, mn = (numb & kMant) | kHidden,
                   md = (Db & kMant) | kHidden;
    const int64_t r = (int64_t)((mn << k) - mq * md);
    const uint64_t a2 = (uint64_t)(r < 0 ? -r : r) << 1;
    uint64_t qb;
    if (a2 < md) qb = q0b;
    else if (a2 > md && a2 < 3 * md) qb = r > 0 ? q0b + 1 : q0b - 1;
    else return false;
    *q = -dbl(qb);
    return true;
  }
  return false;
}

// Returns true and *q = RN(num/den) when the general form accepts.
static bool gen_quotient(double num, double den, double *q) {
  const uint64_t kSign = 1ull << 63;
  const uint64_t an = bits(num) & ~kSign, ad = bits(den) & ~kSign;
  const int en = (int)(an >> 52), ed = (int)(ad >> 52);
  if ((unsigned)(en - 924) > 200u || (unsigned)(ed - 924) > 200u) return false;
  const float rf = 1.0f / fs::trunc_bits_to_float(ad);
  const double r0 = (double)rf;
  const double e = std::fma(-dbl(ad), r0, 1.0);
  const double r1 = std::fma(r0, e, r0);
  const uint64_t qb = fs::round_quotient_bits(an, ad, bits(dbl(an) * r1));
  if (!qb) return false;
  *q = dbl(qb | ((bits(num) ^ bits(den)) & kSign));
  return true;
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 10000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  long accepted = 0, accepted_int = 0, accepted_gen = 0;
  for (long i = 0; i < n; i++) {
    // D = 1 + F, F from tiny to huge; significands of every shape; also the
    // receiver slopes' divisors (dx, dx*sqrt(2)), D below 1, huge D (where
    // the threshold's exponent leaves the range) and negative D
    double D;
    switch (i % 7) {
      case 0: D = 1.0 + std::ldexp((double)(g() >> 11), -53 + (int)(g() % 80) - 40); break;
      case 1: D = dbl((uint64_t)(1023 + g() % 40) << 52 | (g() & ((1ull << 52) - 1))); break;
      case 2: D = dbl((uint64_t)(1023 + g() % 40) << 52 | (((1ull << 52) - 1) ^ ((1ull << (g() % 52)) - 1))); break;
      case 3: D = dbl((uint64_t)(1023 + g() % 40) << 52 | ((1ull << (g() % 52)) | (g() & 0xFF))); break;
      case 4: D = (g() & 1) ? 100.0 : 100.0 * 1.4142135623730951; break;
      case 5: D = dbl((uint64_t)(1 + g() % 2046) << 52 | (g() & ((1ull << 52) - 1))); break;
      default: D = -dbl((uint64_t)(1023 + g() % 40) << 52 | (g() & ((1ull << 52) - 1))); break;
    }
    if (D == 0 || !std::isfinite(D)) continue;
    const double R = 1.0 / D;
    double num;
    if (i & 1) {
      // next to a midpoint: num = RN(D * (m + ulp(m)/2)), m a double
      const double m = dbl((uint64_t)(1023 + (int)(g() % 200) - 100) << 52 | (g() & ((1ull << 52) - 1)));
      int e; std::frexp(m, &e);
      num = std::fma(D, m, D * std::ldexp(1.0, e - 54));
      if (i % 3 == 0) num = dbl(bits(num) + (int)(g() % 5) - 2);
    } else if (i % 5 == 0) {
      num = dbl((uint64_t)(1 + g() % 2046) << 52 | (g() & ((1ull << 52) - 1)));  // any exponent
    } else {
      num = dbl((uint64_t)(1023 + (int)(g() % 400) - 200) << 52 | (g() & ((1ull << 52) - 1)));
    }
    if (g() & 1) num = -num;
    double q;
    if (gen_quotient(num, D, &q)) {
      accepted_gen++;
      const double ex = num / D;
      if (bits(q) != bits(ex)) {
        std::printf("MISMATCH (general form) num=%a D=%a gen=%a ieee=%a\n", num, D, q, ex);
        return 1;
      }
    }
    if (int_quotient(num, D, R, &q)) {
      accepted_int++;
      const double ex = num / D;
      if (bits(q) != bits(ex)) {
        std::printf("MISMATCH (integer form) num=%a D=%a int=%a ieee=%a\n", num, D, q, ex);
        return 1;
      }
    }
    if (fast_quotient(num, D, R, &q)) {
      accepted++;
      const double ex = num / D;
      if (bits(q) != bits(ex)) {
        std::printf("MISMATCH num=%a D=%a fast=%a ieee=%a\n", num, D, q, ex);
        return 1;
      }
    }
  }
  std::printf("%ld cases, %ld accepted by the fast path, %ld by the integer form, %ld by the "
              "general form, all equal to the IEEE quotient\n",
              n, accepted, accepted_int, accepted_gen);
  return 0;
}
