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

FS_BITS_FN float float_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}

// Correctly rounded quotient from an approximate one: an = |num|, ad = |den|
// (bits of positive normal doubles) and q0 = bits of an approximation of
// an/ad within 2^9 ulp. The residual an - q0*ad is exact in integer
// arithmetic in units of ulp(q0)*ulp(ad): r = mn*2^k - mq*md from the
// significands (implicit bit set) and k = en - eq - ed + 1075; |r| < 2^62,
// so the difference of the products' low 64 bits is r itself. With
// an/ad = (mq + r/md) ulp(q0), n = the nearest integer to r/md (from the top
// bits of r and md, within one of it) and r' = r - n*md, the correctly
// rounded quotient's significand is mq + n when 2|r'| < md, one more or
// one less when md < 2|r'| < 3md (a quotient is never a rounding midpoint),
// as long as it stays in q0's binade (a result at the binade's lower edge
// with the quotient below it may round into the binade beneath). Returns
// the quotient's bits, or 0 where this does not decide (the caller then
// divides).
FS_BITS_FN uint64_t round_quotient_bits(uint64_t an, uint64_t ad, uint64_t q0) {
  constexpr uint64_t kMant = (1ull << 52) - 1, kHidden = 1ull << 52;
  const int en = (int)(an >> 52), ed = (int)(ad >> 52), eq = (int)(q0 >> 52);
  const int k = en - eq - ed + 1075;
  if ((unsigned)(k - 48) > 12u || (unsigned)(eq - 64) > 1916u) return 0;
  const uint64_t mq = (q0 & kMant) | kHidden, mn = (an & kMant) | kHidden,
                 md = (ad & kMant) | kHidden;
  long long r = (long long)((mn << k) - mq * md);
  // any integer n keeps the result exact (the checks below decide); the
  // estimate's accuracy only sets how often they do
#if defined(__CUDA_ARCH__)
  const float t = __fdividef((float)(int)(r >> 32), (float)(int)(md >> 32));
#else
  const float t = (float)(int)(r >> 32) / (float)(int)(md >> 32);
#endif
  const long long n = (long long)(t < 0.0f ? -(int)(0.5f - t) : (int)(t + 0.5f));
  if (n > 1024 || n < -1024) return 0;
  r -= n * (long long)md;
  long long m = (long long)mq + n;
  const uint64_t a2 = (uint64_t)(r < 0 ? -r : r) << 1;
  if (a2 > md) {
    if (a2 >= 3 * md) return 0;
    m += r > 0 ? 1 : -1;
    r -= r > 0 ? (long long)md : -(long long)md;
  } else if (a2 == md) {
    return 0;
  }
  if (m < (long long)kHidden || m >= 2 * (long long)kHidden) return 0;
  if (m == (long long)kHidden && r < 0) return 0;
  return ((uint64_t)eq << 52) | ((uint64_t)m & kMant);
}

// Truncation of a double (as bits) to FP32 with integer operations only:
// rebias the exponent, keep the top 23 fraction bits. Values below 2^-126
// flush to signed zero; |x| >= 2^128, Inf and NaN give NaN.
FS_BITS_FN float trunc_bits_to_float(uint64_t b) {
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  const uint32_t frac = (uint32_t)(b >> 29) & 0x7FFFFFu;
  if (e <= 0) return float_from_bits(sign);
  if (e >= 255) return float_from_bits(0x7FC00000u);
  return float_from_bits(sign | ((uint32_t)e << 23) | frac);
}

// Fixed-point value of a double (bits b) in units of 2^(et - 1084), et a
// biased exponent at least b's: the significand with 9 guard bits, shifted
// right by et - e (bits below the unit truncated toward zero), signed.
// |result| < 2^62, so the difference of two such values fits an int64.
// Zeros, subnormals and values 63 or more binades below 2^(et-1023) give 0.
FS_BITS_FN long long fixed_in_binade(uint64_t b, int et) {
  const int e = (int)((b >> 52) & 0x7FF);
  const int d = et - e;
  if (e == 0 || d > 62) return 0;
  const uint64_t mag = (((b & ((1ull << 52) - 1)) | (1ull << 52)) << 9) >> d;
  return (b >> 63) ? -(long long)mag : (long long)mag;
}

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

// A Newton correction far below its iterate: x2 = RN(x - q), q = RN(num/D),
// with x > 0, 1 <= D < 2^100 (bits D) and |q| within about one spacing of x. x2 is x or one of its
// neighbours (bits x - 1 or x + 1): x when |q| is below half the spacing
// on q's side, the neighbour when |q| lies between a half and 1.2 spacings
// (the next spacing beyond a power of two at least halves, which 1.2 keeps
// clear of). qe is an FP32 estimate of |num/D| within 2^-18 relative (plus
// an absolute error far below the spacing: x >= 2^-23 and D < 2^100); q's
// own rounding is below 2^-52 relative. With a margin of 2^-16 around the
// half-spacing threshold the estimate decides like the exact quotient;
// nearer the threshold, or for x or D out of range, false is returned and
// the caller computes q exactly. On true, *step is -1, 0 or +1 and
// x2 = x + *step as bits. `ulp` returns the spacing above x as FP32.
FS_BITS_FN bool newton_step_in_spacing(uint64_t num, uint64_t D, uint64_t x, float qe,
                                       int *step, float *ulp) {
  const int ex = (int)(x >> 52);  // x > 0: no sign bit
  if (ex < 1000 || ex > 1160 || (D >> 52) >= 1123) return false;
  *ulp = float_from_bits((uint32_t)(ex - 948) << 23);             // 2^(ex-1075)
  const bool down = (num >> 63) == 0;                              // q > 0: below x
  const bool half = down && (x << 12) == 0;                        // x a power of 2
  const float inv = float_from_bits((uint32_t)(1202 - ex + (half ? 1 : 0)) << 23);
  const float r = qe * inv;  // |q| in spacings on its side (a power-of-2 scaling)
  if (r < 0.5f * (1.f - 0x1p-16f)) {
    *step = 0;
    return true;
  }
  if (r > 0.5f * (1.f + 0x1p-16f) && r < 1.2f) {
    *step = down ? -1 : 1;
    return true;
  }
  return false;
}

}  // namespace fs
