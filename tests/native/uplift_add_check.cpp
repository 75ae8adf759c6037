// Host check of fs::add_pos_rn_bits, fs::sub_near_bits and fs::sub_far_bits
// (barnes2019-landscape_gb300/csrc/fs_bits.h), the integer restatements of
// the erosion kernel's additions and subtractions of elevations: every
// operand pair the kernel sends to them must give the bits of the hardware's
// RN result, and a declined pair must be one the function does not cover.
// Cases: random significands at every exponent difference, operands next to
// rounding ties (the discarded part exactly half an ulp, or half an ulp plus
// or minus one unit), significands of all ones (carry through the rounding),
// deep cancellation, low bits clear (the sticky-free subtraction's declined
// cases), the top of the exponent range (overflow to +Inf), the operand
// filter itself, and elevations of the workload's range.
// Usage: uplift_add_check <cases> <seed>; exit 1 on the first mismatch.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "fs_bits.h"

static double dbl(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }

static long mismatches = 0;

static void check(uint64_t x, uint64_t y) {
  if (!fs::add_pos_operand(x) || !fs::add_pos_operand(y)) return;
  const uint64_t want = bits(dbl(x) + dbl(y));
  const uint64_t got = fs::add_pos_rn_bits(x, y);
  if (want != got && mismatches++ < 10)
    std::printf("mismatch: %016" PRIx64 " + %016" PRIx64 ": %016" PRIx64 " want %016" PRIx64 "\n",
                x, y, got, want);
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 10000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  const uint64_t kFrac = (1ull << 52) - 1;
  // The operand filter: positive, biased exponent 1..2045.
  const uint64_t edge[] = {0, 1, kFrac, 1ull << 52, (2045ull << 52) | kFrac, 2046ull << 52,
                           0x7FF0000000000000ull, 0x7FF8000000000000ull, 0x8000000000000000ull,
                           0x8010000000000000ull, 0xBFF0000000000000ull};
  const bool edge_ok[] = {false, false, false, true, true, false, false, false, false, false, false};
  for (int i = 0; i < (int)(sizeof edge / sizeof edge[0]); i++) {
    if (fs::add_pos_operand(edge[i]) != edge_ok[i]) {
      std::printf("operand filter wrong for %016" PRIx64 "\n", edge[i]);
      return 1;
    }
  }
  long tested = 0;
  for (long i = 0; i < n; i++) {
    const int ea = 1 + (int)(g() % 2045);
    const int d = (int)(g() % 71);
    const int eb = ea - d >= 1 ? ea - d : 1 + (int)(g() % 2045);
    uint64_t fa = g() & kFrac, fb = g() & kFrac;
    switch (i % 6) {
      case 1: fa = kFrac; break;                        // carry through the rounding
      case 2: fb = kFrac; fa = kFrac ^ (g() & 0xF); break;
      case 3: fb &= ~((1ull << (g() % 53)) - 1); break;  // short significands
      default: break;
    }
    const uint64_t x = (uint64_t)ea << 52 | fa, y = (uint64_t)eb << 52 | fb;
    check(x, y);
    check(y, x);
    // Ties: y's bits below the kept part of the sum are exactly 100..0 (half
    // an ulp of x when no renormalisation happens), optionally +-1 unit.
    if (d >= 1 && d <= 53 && ea - d >= 1) {
      const uint64_t low = (1ull << d) - 1;               // bits of y below x's ulp
      const uint64_t m = ((fb | (1ull << 52)) & ~low) | (1ull << (d - 1));
      const uint64_t yb = ((uint64_t)(ea - d) << 52) | (m & kFrac);
      check(x, yb);
      check(x, yb + 1);
      check(x, yb - 1);
      tested += 3;
    }
    tested += 2;
  }
  // Top of the range: sums that overflow to +Inf or stay just below it.
  for (long i = 0; i < n / 100; i++) {
    const uint64_t x = (uint64_t)(2040 + g() % 6) << 52 | (g() & kFrac);
    const uint64_t y = (uint64_t)(2040 + g() % 6) << 52 | (g() & kFrac);
    check(x, y);
    ++tested;
  }
  // The workload's own operands: elevations 0..5000 m plus U*dt = 2.
  for (long i = 0; i < n / 10; i++) {
    const double h = std::ldexp(1.0, -(int)(g() % 40)) * (double)(g() >> 11) * 0x1p-53 * 5000.0;
    check(bits(h), bits(2.0));
    ++tested;
  }
  // The special cases: sub_near_bits (Sterbenz, exact) and sub_far_bits
  // (exponent difference >= 2, no sticky bit). A declined pair (0) must be
  // one the function does not cover; an accepted one must be exact.
  long near_taken = 0, far_taken = 0, far_declined = 0;
  for (long i = 0; i < n; i++) {
    const int ea = 1 + (int)(g() % 2045);
    const int d = (i % 3 == 0) ? (int)(g() % 3) : (int)(g() % 64);
    const int eb = ea - d >= 1 ? ea - d : 1 + (int)(g() % 2045);
    uint64_t fa = g() & kFrac, fb = g() & kFrac;
    switch (i % 5) {
      case 1: fb = fa ^ (g() & ((1ull << (g() % 52)) - 1)); break;
      case 2: fb &= ~((1ull << (g() % 53)) - 1); break;
      case 3: fa = (fa & ~0xFFFull); fb = (fb & ~((1ull << (g() % 40)) - 1)); break;  // thresholds
      default: break;
    }
    uint64_t x = (uint64_t)ea << 52 | fa, y = (uint64_t)eb << 52 | fb;
    if (x < y) { const uint64_t t = x; x = y; y = t; }
    if (x == y || !fs::add_pos_operand(x) || !fs::add_pos_operand(y)) continue;
    const uint64_t want = bits(dbl(x) - dbl(y));
    const int dd = (int)(x >> 52) - (int)(y >> 52);
    const uint64_t rn = fs::sub_near_bits(x, y), rf = fs::sub_far_bits(x, y);
    const bool sterbenz = dbl(y) >= dbl(x) / 2;
    tested += 2;
    if (rn) {
      ++near_taken;
      if (rn != want && mismatches++ < 10)
        std::printf("near mismatch: %016" PRIx64 " - %016" PRIx64 "\n", x, y);
    } else if (sterbenz && ((want << 1) >> 53) != 0 && mismatches++ < 10) {
      std::printf("near declined a Sterbenz pair: %016" PRIx64 " - %016" PRIx64 "\n", x, y);
    }
    if (rf) {
      ++far_taken;
      if (rf != want && mismatches++ < 10)
        std::printf("far mismatch: %016" PRIx64 " - %016" PRIx64 ": %016" PRIx64 " want %016" PRIx64 "\n",
                    x, y, rf, want);
    } else if (dd >= 2) {
      ++far_declined;
      if (dd <= 10 && mismatches++ < 10)
        std::printf("far declined an exact alignment: %016" PRIx64 " - %016" PRIx64 "\n", x, y);
    }
  }
  std::printf("near taken %ld, far taken %ld, far declined %ld\n", near_taken, far_taken,
              far_declined);
  // The workload's own differences: elevation minus a lower elevation.
  for (long i = 0; i < n / 10; i++) {
    const double h0 = 2.0 + (double)(g() >> 11) * 0x1p-53 * 5000.0;
    const double hn = h0 * (double)(g() >> 11) * 0x1p-53;
    if (!(h0 > hn) || !fs::add_pos_operand(bits(hn))) continue;
    const uint64_t rn = fs::sub_near_bits(bits(h0), bits(hn));
    const uint64_t rf = fs::sub_far_bits(bits(h0), bits(hn));
    tested += 2;
    if ((rn && rn != bits(h0 - hn)) || (rf && rf != bits(h0 - hn))) {
      if (mismatches++ < 10) std::printf("workload special-case mismatch: %.17g - %.17g\n", h0, hn);
    }
  }
  if (mismatches) {
    std::printf("%ld mismatches in %ld results\n", mismatches, tested);
    return 1;
  }
  std::printf("%ld results, all equal to the hardware operation\n", tested);
  return 0;
}
