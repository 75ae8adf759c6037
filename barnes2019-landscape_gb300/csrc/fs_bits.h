// fs_bits.h -- IEEE binary64 operations restated in integer arithmetic on bit
// patterns, for kernels whose FP64 pipe is the bottleneck while their integer
// pipes are idle. Shared by the kernels and the host check
// tests/native/uplift_add_check.cpp, which compares every result with the
// hardware addition.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define FS_BITS_FN __host__ __device__ __forceinline__
#else
#define FS_BITS_FN inline
#endif

namespace fs {

// True when x is positive, normal and at most 2^1023 (biased exponent in
// [1, 2045]): the operands add_pos_rn_bits accepts.
FS_BITS_FN bool add_pos_operand(uint64_t x) {
  return x - (1ull << 52) < (2045ull << 52);
}

// RN(x + y) (round to nearest, ties to even) for two operands accepted by
// add_pos_operand, as bits. Same-sign addition: no cancellation, so the sum's
// exponent is the larger operand's or one more. Significands are held with 10
// guard bits; the smaller one is aligned with its shifted-out bits folded
// into a sticky bit, the sum is renormalised by at most one place, and the
// rounding adds half an ulp less one plus the kept significand's last bit
// (which turns an exact tie into ties-to-even). A carry out of the rounding
// moves into the exponent field by the final addition; a sum rounding past
// the largest double gives the bits of +Inf, as the hardware does.
FS_BITS_FN uint64_t add_pos_rn_bits(uint64_t x, uint64_t y) {
  const uint64_t a = x > y ? x : y;  // positive doubles order like their bits
  const uint64_t b = x > y ? y : x;
  int ea = (int)(a >> 52);
  const int eb = (int)(b >> 52);
  int d = ea - eb;
  d = d < 63 ? d : 63;
  constexpr uint64_t kFrac = (1ull << 52) - 1, kOne = 1ull << 52;
  const uint64_t ma = ((a & kFrac) | kOne) << 10;  // [2^62, 2^63)
  const uint64_t mb = ((b & kFrac) | kOne) << 10;
  const uint64_t sh = mb >> d;
  const uint64_t sticky = (sh << d) != mb ? 1u : 0u;
  uint64_t s = ma + (sh | sticky);  // < 2^64
  if (s >> 63) {
    s = (s >> 1) | (s & 1);
    ++ea;
  }
  const uint64_t r = (s + 0x1FF + ((s >> 10) & 1)) >> 10;  // [2^52, 2^53]
  return ((uint64_t)(ea - 1) << 52) + r;
}

FS_BITS_FN int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// x - y for x > y, both accepted by add_pos_operand, when y >= x/2: the
// difference is then exact (Sterbenz's lemma), so it is the integer
// difference of the aligned significands (exponent difference 0, or 1 with
// y's significand at least x's), renormalised by a count of leading zeros.
// 0 when the lemma does not apply or the difference is below the normal
// range (the caller then subtracts otherwise).
FS_BITS_FN uint64_t sub_near_bits(uint64_t x, uint64_t y) {
  const int ex = (int)(x >> 52), ey = (int)(y >> 52);
  constexpr uint64_t kFrac = (1ull << 52) - 1, kOne = 1ull << 52;
  const uint64_t mx = (x & kFrac) | kOne, my = (y & kFrac) | kOne;
  uint64_t dm;  // the difference in units of y's last place, in (0, 2^53)
  if (ex == ey) dm = mx - my;
  else if (ex == ey + 1 && my >= mx) dm = (mx << 1) - my;
  else return 0;
  const int lz = clz64(dm) - 11;
  const int e = ey - lz;
  if (e <= 0) return 0;
  return ((uint64_t)(e - 1) << 52) + (dm << lz);
}

// RN(x - y) for x > y, both accepted by add_pos_operand, when x's exponent
// exceeds y's by at least 2 (so y < x/2 and the difference keeps its leading
// bit at one of two places). The aligned y is truncated without a sticky
// bit: the exact difference lies in (s - 1, s], and every rounding threshold
// is a multiple of 2^8 of these units, so s rounds like the exact difference
// unless s is itself such a multiple after bits were shifted out -- then 0
// is returned and the caller subtracts otherwise.
FS_BITS_FN uint64_t sub_far_bits(uint64_t x, uint64_t y) {
  const int ex = (int)(x >> 52), ey = (int)(y >> 52);
  int d = ex - ey;
  if (d < 2) return 0;
  d = d < 63 ? d : 63;
  constexpr uint64_t kFrac = (1ull << 52) - 1, kOne = 1ull << 52;
  const uint64_t mx = ((x & kFrac) | kOne) << 10;  // [2^62, 2^63)
  const uint64_t my = ((y & kFrac) | kOne) << 10;
  uint64_t s = mx - (my >> d);                     // (2^61, 2^63)
  if (d > 10 && (s & 0xFF) == 0) return 0;
  const int lz = 1 - (int)(s >> 62);               // 0 or 1
  s <<= lz;
  const uint64_t r = (s + 0x1FF + ((s >> 10) & 1)) >> 10;  // [2^52, 2^53]
  return ((uint64_t)(ex - lz - 1) << 52) + r;
}

}  // namespace fs
