// Host check of fs::fixed_in_binade (barnes2019-landscape_gb300/csrc/fs_bits.h),
// the receiver filter's staging of high ground relative to a tile's first
// value: with et the tile's largest biased exponent and u = 2^(et-1084),
//   f = RN32(X - X_ref) * u,  X = fixed_in_binade(h, et),
// must satisfy |f - (h - X_ref*u)| <= 2^-24 |h - X_ref*u| + 1.01 u, and
// |X| < 2^62 (so X - X_ref cannot overflow). Checked exactly in 128-bit
// integers in units of v = 2^(et-1137) = u * 2^-53, over random tiles with
// mixed signs, exponents down to 70 binades below et, zeros and subnormals.
// The scale factors the kernel builds from bit patterns (u and 2^22 u as
// FP32) are checked against ldexp over the kernel's range of et.
// Usage: tile_fixed_check <cases> <seed>; exit 1 on the first failure.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "fs_bits.h"

using i128 = __int128;

static i128 iabs(i128 x) { return x < 0 ? -x : x; }

// h / v for h = bits b (|h| < 2^(et-1022)), exactly when et - e <= 62, else
// truncated toward zero (then |error| < 1).
static i128 in_v_units(uint64_t b, int et) {
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0;  // zeros and subnormals: below 1 unit of v for et >= 1030
  const uint64_t mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
  const int d = et - e;
  const i128 mag = d <= 62 ? ((i128)mant << (62 - d)) : (d - 62 < 64 ? (i128)(mant >> (d - 62)) : 0);
  return (b >> 63) ? -mag : mag;
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  for (int et = 1030; et <= 1123; et++) {
    if (fs::float_from_bits((uint32_t)(et - 1084 + 127) << 23) != std::ldexp(1.0f, et - 1084) ||
        fs::float_from_bits((uint32_t)(et - 1062 + 127) << 23) != std::ldexp(1.0f, et - 1062)) {
      std::printf("scale factor wrong at et %d\n", et);
      return 1;
    }
  }
  long checked = 0;
  for (long c = 0; c < n; c++) {
    const int et = 1030 + (int)(g() % 94);
    auto draw = [&]() -> uint64_t {
      const unsigned kind = (unsigned)(g() % 16);
      if (kind == 0) return (g() & 1) << 63;                         // +-0
      if (kind == 1) return ((g() & 1) << 63) | (g() & ((1ull << 52) - 1));  // subnormal
      const int e = kind < 8 ? et - (int)(g() % 3) : et - (int)(g() % 71);
      if (e < 1) return 0;
      return ((g() & 1) << 63) | ((uint64_t)e << 52) | (g() & ((1ull << 52) - 1));
    };
    const uint64_t ref = draw(), h = draw();
    const long long xr = fs::fixed_in_binade(ref, et), x = fs::fixed_in_binade(h, et);
    if (x >= (1ll << 62) || x <= -(1ll << 62) || xr >= (1ll << 62) || xr <= -(1ll << 62)) {
      std::printf("fixed value out of range: %016" PRIx64 " at et %d\n", h, et);
      return 1;
    }
    const float f = (float)(x - xr);  // the kernel's RN32(X - X_ref), before the exact scaling by u
    // exact h - X_ref*u in units of v (u = 2^53 v)
    const i128 H = in_v_units(h, et) - ((i128)xr << 53);
    const i128 F = (i128)(double)f << 53;  // f is integral and below 2^63
    const int e = (int)((h >> 52) & 0x7FF);
    const i128 slack = (e != 0 && et - e > 62) ? 1 : 0;
    const i128 bound = (iabs(H) >> 24) + 1 + (((i128)1 << 53) + ((i128)1 << 53) / 100) + slack;
    if (iabs(F - H) > bound) {
      std::printf("bound exceeded: h %016" PRIx64 " ref %016" PRIx64 " et %d\n", h, ref, et);
      return 1;
    }
    ++checked;
  }
  std::printf("%ld values, all within the staging bound\n", checked);
  return 0;
}
