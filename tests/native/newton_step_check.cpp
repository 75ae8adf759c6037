// Host check of fs::newton_step_in_spacing (barnes2019-landscape_gb300/csrc/
// fs_bits.h): the erosion's second Newton iterate x2 = RN(x - RN(num/D))
// decided from an FP32 estimate of |num/D| in units of x's spacing. Every
// decision must equal the exact double computation. The estimate is formed
// like the kernel's (truncated operands, FP32 quotient) and then perturbed
// by -2^-20, 0 and +2^-20 relative -- more than the device's approximate
// division can be off -- so the check covers its error too. Cases: iterates
// of every exponent the function accepts, powers of two and their
// neighbours, D from 1 to 2^99, corrections concentrated around half a
// spacing and around 1.2 spacings, both signs.
// Usage: newton_step_check <cases> <seed>; exit 1 on the first mismatch.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "fs_bits.h"

static double dbl(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 10000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  const uint64_t kFrac = (1ull << 52) - 1;
  long decided = 0, checked = 0, bad = 0;
  for (long i = 0; i < n; i++) {
    const int ex = 995 + (int)(g() % 170);  // a few outside [1000, 1160]
    uint64_t fx = g() & kFrac;
    switch (i % 5) {
      case 1: fx = 0; break;            // a power of two
      case 2: fx = 1; break;            // just above one
      case 3: fx = kFrac; break;        // just below the next
      default: break;
    }
    const uint64_t x = (uint64_t)ex << 52 | fx;
    double D;
    switch (i % 3) {
      case 0: D = 1.0 + std::ldexp((double)(g() >> 11), -53) * 1000.0; break;
      case 1: D = 1.0 + std::ldexp((double)(g() >> 11), -53 - (int)(g() % 40)); break;
      default: D = std::ldexp(1.0 + std::ldexp((double)(g() >> 11), -53), (int)(g() % 100)); break;
    }
    // |num/D| = rho spacings on its side, rho near the thresholds or anywhere
    const bool down = g() & 1;
    const double spacing = (down && fx == 0) ? std::ldexp(1.0, ex - 1076) : std::ldexp(1.0, ex - 1075);
    double rho;
    const double u = std::ldexp((double)(g() >> 11), -53);
    switch (i % 4) {
      case 0: rho = 0.5 + (u - 0.5) * std::ldexp(1.0, -(int)(g() % 30)); break;
      case 1: rho = 1.2 + (u - 0.5) * std::ldexp(1.0, -(int)(g() % 30)); break;
      default: rho = 1.5 * u; break;
    }
    double num = rho * spacing * D;
    if (!down) num = -num;
    if (num == 0 || !std::isfinite(num)) continue;
    const double q = num / D;
    const uint64_t want = bits(dbl(x) - q);
    const float nf = std::fabs(fs::trunc_bits_to_float(bits(num)));
    const float Df = fs::trunc_bits_to_float(bits(D));
    for (int k = -1; k <= 1; k++) {
      const float qe = (nf / Df) * (1.f + (float)k * 0x1p-20f);
      int step = 7;
      float ulp = 0;
      ++checked;
      if (!fs::newton_step_in_spacing(bits(num), bits(D), x, qe, &step, &ulp)) continue;
      ++decided;
      if (x + (uint64_t)(int64_t)step != want && bad++ < 10)
        std::printf("mismatch: x %016" PRIx64 " num %.17g D %.17g step %d want %016" PRIx64 "\n", x,
                    num, D, step, want);
      if (ulp != (float)std::ldexp(1.0, ex - 1075) && bad++ < 10)
        std::printf("spacing wrong for x %016" PRIx64 "\n", x);
    }
  }
  std::printf("%ld decided of %ld\n", decided, checked);
  if (bad) {
    std::printf("%ld mismatches\n", bad);
    return 1;
  }
  std::printf("all decisions equal to the exact iterate\n");
  return 0;
}
