// fs_kernels.cu -- sm_103a kernels of the FastScape timestep, over a batch
// of realizations (a single model is a batch of one).
//
// One timestep = six launches on the stream:
//   1. k_receivers_filter  D8 steepest descent over the interior
//      + k_receivers_fixup (fastscape_RB.cpp:160-182): FP32 proof of the
//                          receiver, FP64 reference formula for the cells
//                          the proof cannot settle
//   2. k_donors_level0     donor masks (pull form of fastscape_RB.cpp:188-203)
//                          and the level-0 frontier (fastscape_RB.cpp:221-227)
//   3. k_order             persistent cooperative kernel: level-by-level
//                          ordering (:229-251)
//   4. k_accum             persistent cooperative kernel: flow accumulation
//                          back down the levels (:262-279); uplifts the pits
//   5. k_erode             persistent cooperative kernel: uplift (:285-296)
//                          and the implicit erosion solved upward from base
//                          level (:306-328, in the level order of
//                          fastscape_RB+P.cpp:319-350).
//   In the three walk kernels all realizations walk their levels in lock
//   step, so one grid barrier per level serves the whole batch.
//
// Floating point follows the reference's operation order exactly; the whole
// file is compiled with -fmad=false so no multiply-add is contracted, every
// FP64 division is correctly rounded, and the additions and subtractions
// done in integer arithmetic (fs_bits.h) give the bits of the FP64 ones.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "fastscape_gb300.h"
#include "fs_bits.h"
#include "fs_internal.h"

namespace fs {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWalkThreads = 512;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kPer = 8;   // entries per thread per expansion chunk (measured best of 4..16)
constexpr int kLevelCache = 2048;  // level offsets a single grid's walk keeps in shared memory
constexpr int kChunk = kPer * kWalkThreads;
constexpr int kNewtonMaxIt = 1000;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_i32(const int *p) {
  return *reinterpret_cast<const volatile int *>(p);
}

__device__ __forceinline__ void raise_err(Ctl *ctl, int code, int phase) {
  if (atomicCAS(&ctl->err, 0, code) == 0) ctl->err_detail = phase;
}

__device__ __forceinline__ bool stopped(const Ctl *ctl) {
  return (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) != 0;
}

__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch. The arrival counter only grows
// during a launch (reset by the host before it), so barrier number `epoch`
// completes when bar reaches epoch*gridDim.x. Arrival: the block barrier
// orders the block's writes before thread 0's release reduction; wait:
// thread 0's acquire loads see every block's release, and the closing block
// barrier orders the rest of the block after them (the release/acquire
// pattern of the CUTLASS grid barrier). Every wait is bounded by
// `timeout_ns` of wall time; on timeout, or when another block has raised
// an error (the error word is polled every 16 spins), it returns false and
// the caller leaves the kernel.
__device__ bool grid_barrier(Ctl *ctl, unsigned *bar, unsigned &epoch,
                             unsigned long long timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ++epoch;
    const unsigned target = epoch * gridDim.x;
    red_release_add_u32(bar, 1u);
    int ok = 1;
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    while (ld_acquire_u32(bar) < target) {
      ++spins;
      if ((spins & 15u) == 0 && ld_volatile_i32(&ctl->err) != 0) { ok = 0; break; }
      if ((spins & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
        raise_err(ctl, FS_ERR_TIMEOUT, kPhaseBarrier);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// nshift[k] (fastscape_RB.cpp:137) for a run-time k without a local array:
// dx+1 and dy+1 of the 8 directions packed two bits per direction
// (W, NW, N, NE, E, SE, S, SW).
__device__ __forceinline__ int nbr_off(int k, int W) {
  const int dx = ((0x1A90 >> (2 * k)) & 3) - 1;
  const int dy = ((0xA901 >> (2 * k)) & 3) - 1;
  return dy * W + dx;
}

// Exclusive block scan of one int per thread; t is the thread's linear index
// in the block and nthreads the block size (a multiple of 32, at most 1024).
// Returns the prefix and the block total.
__device__ __forceinline__ int block_excl_scan(int v, int &total, int t, int nthreads) {
  __shared__ int s_w[32];
  const int lane = t & 31, wid = t >> 5;
  const int nw = nthreads >> 5;
  int incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int x = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += x;
  }
  if (lane == 31) s_w[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? s_w[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int x = __shfl_up_sync(kFull, w, d);
      if (lane >= d) w += x;
    }
    if (lane < nw) s_w[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  total = s_w[nw - 1];
  const int before = wid ? s_w[wid - 1] : 0;
  __syncthreads();  // s_w may be reused by the caller's next scan
  return before + incl - v;
}

// Exclusive prefix over realizations of count(r) into s_pre[0..n]; the walk
// kernel's block-wide view of how a level's work splits across the batch.
template <class F>
__device__ __forceinline__ int block_prefix(int n, F count, int *s_pre) {
  const int per = (n + kWalkThreads - 1) / kWalkThreads;
  const int r0 = threadIdx.x * per;
  int sum = 0;
  for (int r = r0; r < r0 + per && r < n; r++) sum += count(r);
  int total;
  int run = block_excl_scan(sum, total, threadIdx.x, kWalkThreads);
  for (int r = r0; r < r0 + per && r < n; r++) {
    s_pre[r] = run;
    run += count(r);
  }
  if (threadIdx.x == 0) s_pre[n] = total;
  __syncthreads();
  return total;
}

// Realization of global work item g: the r with s_pre[r] <= g < s_pre[r+1]
// (g < s_pre[n]); empty realizations are skipped because the largest such
// r is taken.
__device__ __forceinline__ int find_real(const int *s_pre, int n, int g) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (s_pre[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ long long abs_bits(double x) {
  return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll;
}

// FP64 add / multiply of bit patterns held in integer registers. Keeping
// elevations as integers between the FP64 instructions avoids the FP64
// moves the compiler otherwise emits for merges, selects and negations of
// doubles (each an instruction on this part's narrow FP64 pipe).
__device__ __forceinline__ uint64_t fadd_bits(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("{\n\t.reg .f64 x, y;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\t"
      "add.rn.f64 x, x, y;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

__device__ __forceinline__ uint64_t fmul_bits(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("{\n\t.reg .f64 x, y;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\t"
      "mul.rn.f64 x, x, y;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

constexpr uint64_t kSignBit = 0x8000000000000000ull;

// FP64 addition in a branch taken by few cells: volatile, so that the
// compiler does not execute it speculatively for the others.
__device__ __forceinline__ uint64_t fadd_bits_volatile(uint64_t a, uint64_t b) {
  uint64_t r;
  asm volatile(
      "{\n\t.reg .f64 x, y;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\t"
      "add.rn.f64 x, x, y;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

// The erosion's FP64 pipe is its bottleneck while its integer pipes idle, so
// some of its additions run in integer arithmetic (fs_bits.h, each
// bit-identical to the hardware's RN operation on the operands it accepts;
// the rest take the FP64 addition).
//
// The uplift h + U*dt of an eroded cell: two positive normal operands (every
// cell of a landscape above base level). Off the cell's critical path (it
// does not wait for the receiver's elevation), so always worth it.
__device__ __forceinline__ uint64_t uplift_bits(uint64_t h, uint64_t udt) {
  if (add_pos_operand(h) && add_pos_operand(udt)) return add_pos_rn_bits(h, udt);
  return fadd_bits_volatile(h, udt);
}

// RN(x - y) of a cell's and its receiver's elevation: the exact integer
// difference when y >= x/2 (sub_near_bits), else in FP64.
__device__ __forceinline__ uint64_t sub_near(uint64_t x, uint64_t y) {
  if (add_pos_operand(x) && add_pos_operand(y) && x > y) {
    const uint64_t r = sub_near_bits(x, y);
    if (r) return r;
  }
  return fadd_bits_volatile(x, y ^ kSignBit);
}

// RN(x - y) of an elevation and its erosion: in integer arithmetic when y's
// exponent is at least 2 below x's (sub_far_bits), else in FP64.
__device__ __forceinline__ uint64_t sub_far(uint64_t x, uint64_t y) {
  if (add_pos_operand(x) && add_pos_operand(y)) {
    const uint64_t r = sub_far_bits(x, y);
    if (r) return r;
  }
  return fadd_bits_volatile(x, y ^ kSignBit);
}

// RN(x - y) for any two elevations: the exact integer difference when both
// are positive normal and within a factor 2 of each other (Sterbenz), else
// in FP64.
__device__ __forceinline__ uint64_t sub_sterbenz(uint64_t x, uint64_t y) {
  if (add_pos_operand(x) && add_pos_operand(y) && x != y) {
    const bool gt = x > y;
    const uint64_t r = sub_near_bits(gt ? x : y, gt ? y : x);
    if (r) return gt ? r : (r ^ kSignBit);
  }
  return fadd_bits_volatile(x, y ^ kSignBit);
}

// -RN(num/D) on bit patterns, given Rn = -R, R = RN(1/D), in one FP64
// operation. q0n = RN(num*Rn) = -RN(num*R) (RN is symmetric), within
// 2^-52 (1 + 2^-52) of num/D relatively when num, q0, D and 1/D are normal.
// The residual |num| - |q0|*|D| is then exact in integer arithmetic, in
// units of ulp(q0)*ulp(D): r = mn*2^k - mq*mD with mn, mq, mD the
// significands (implicit bit set) and k = en - eq - eD + 1075 from the
// biased exponents; |r| < 2.01 mD < 2^55, so the difference taken modulo
// 2^64 (the low halves of the 106-bit products) is r itself. In magnitude
// num/D = q0 + (r/mD) ulp(q0), so the correctly rounded quotient is q0 when
// 2|r| < mD and q0 one ulp further from or nearer to 0 when mD < 2|r| < 3mD
// (q0 not a power of two, so the spacing is ulp(q0) on both sides; a
// quotient is never a rounding midpoint, and the equalities fall back).
// tests/native/division_check.cpp replays this on the host against the
// IEEE division, near rounding midpoints included. It replaces Markstein's
// correction q1 = RN(q0 + r0*R) with r0 = num - q0*D by a fused
// multiply-add (P. Markstein, IBM J. Res. Dev. 34(1), 1990), which cost two
// more FP64 operations on the erosion's FP64 pipe. Anything else takes the
// IEEE division, volatile PTX in a branch; the numerator and result stay in
// integer registers.
__device__ __forceinline__ uint64_t neg_div_rn_bits(uint64_t numb, double D, double Rn) {
  constexpr uint64_t kMant = (1ull << 52) - 1, kHidden = 1ull << 52;
  const uint64_t q0b = (uint64_t)__double_as_longlong(__longlong_as_double(numb) * Rn);
  const uint64_t Db = (uint64_t)__double_as_longlong(D);
  const int eq = (int)((q0b << 1) >> 53);
  const int en = (int)((numb << 1) >> 53);
  const int ed = (int)((Db << 1) >> 53);
  const int k = en - eq - ed + 1075;
  if ((unsigned)(eq - 64) <= 1980u - 64u && (unsigned)(en - 1) <= 2045u &&
      (unsigned)(ed - 1) <= 2043u && (unsigned)(k - 48) <= 12u && (q0b << 12) != 0) {
    const uint64_t mq = (q0b & kMant) | kHidden, mn = (numb & kMant) | kHidden,
                   md = (Db & kMant) | kHidden;
    const long long r = (long long)((mn << k) - mq * md);
    const uint64_t a2 = (uint64_t)(r < 0 ? -r : r) << 1;
    if (a2 < md) return q0b;
    if (a2 > md && a2 < 3 * md) return r > 0 ? q0b + 1 : q0b - 1;
  }
  uint64_t r;
  asm volatile(
      "{\n\t.reg .f64 x, y;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\t"
      "div.rn.f64 x, x, y;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(numb), "l"(Db));
  return r ^ kSignBit;
}

// ---------------------------------------------------------------------------
// 1. Receivers: fastscape_RB.cpp:160-182. slope = (h[c]-h[n])/dr[n], strict
// '>' against a running maximum that starts at 0, so the first maximum in
// neighbour order wins and a cell with no strictly lower neighbour keeps
// NO_FLOW. k_receivers_exact is that formula verbatim in FP64 (kept to test
// the fast path against); k_receivers_filter + k_receivers_fixup is the fast
// path.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int receiver_fp64(const double *h, int c, int W, double dr_orth,
                                             double dr_diag) {
  const double hc = h[c];
  double max_slope = 0;
  int max_n = FS_NO_FLOW;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const double slope = (hc - h[c + nbr_off(n, W)]) / ((n & 1) ? dr_diag : dr_orth);
    if (slope > max_slope) {
      max_slope = slope;
      max_n = n;
    }
  }
  return max_n == FS_NO_FLOW ? kPit : max_n;
}

// The same formula for the cells the FP32 filter leaves open -- mostly
// flat ground, where neighbours are equal or differ by less than the
// filter's bound. Only a strictly lower neighbour can have a slope above the
// running maximum (which starts at 0), so the others are skipped by an
// integer comparison of order-preserving keys of the bit patterns: a flat
// cell costs no FP64 operation. (Keys order -0 below +0 where FP64 calls
// them equal; that lets through a slope of +0, which never wins. A NaN
// neighbour is skipped or yields a NaN slope, which never wins either.)
__device__ __forceinline__ uint64_t order_key(uint64_t x) {
  return (x >> 63) ? ~x : (x | 0x8000000000000000ull);
}

__device__ __forceinline__ int receiver_fp64_lower(const double *h, int c, const RealDesc &d) {
  const unsigned long long *hb = reinterpret_cast<const unsigned long long *>(h);
  const uint64_t hcb = hb[c];
  if ((hcb & ~kSignBit) > 0x7FF0000000000000ull) return kPit;  // NaN: every slope NaN
  const uint64_t kc = order_key(hcb);
  uint64_t max_slope = 0;  // bits of +0; slopes compared as non-negative bit patterns
  int max_n = FS_NO_FLOW;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const uint64_t hnb = hb[c + nbr_off(n, d.W)];
    if (order_key(hnb) >= kc || (hnb & ~kSignBit) > 0x7FF0000000000000ull) continue;
    const uint64_t db = sub_sterbenz(hcb, hnb);  // RN(hc - hn) > 0 (or +0)
    const double dr = (n & 1) ? d.dr_diag : d.dr_orth;
    const double rn = (n & 1) ? d.rdr_diag_n : d.rdr_orth_n;
    uint64_t slope;
    if (__double_as_longlong(rn) != 0) {
      slope = neg_div_rn_bits(db, dr, rn) ^ kSignBit;  // RN(d / dr)
    } else {
      slope = (uint64_t)__double_as_longlong(__longlong_as_double(db) / dr);
    }
    if (slope > max_slope) {
      max_slope = slope;
      max_n = n;
    }
  }
  return max_n == FS_NO_FLOW ? kPit : max_n;
}

__global__ void __launch_bounds__(256) k_receivers_exact(StepArgs a) {
  if (stopped(a.ctl)) return;
  const Tile t = a.rtiles[blockIdx.x];
  const RealDesc &d = a.desc[t.r];
  const double *h = a.h + d.off;
  int8_t *rec = a.rec + d.off;
  const int x = t.x0 + threadIdx.x;
#pragma unroll 1
  for (int y = t.y0 + threadIdx.y; y < t.y0 + kRyTile; y += 8) {
    if (x < d.W - 2 && y < d.H - 2) {
      const int c = y * d.W + x;
      rec[c] = (int8_t)receiver_fp64(h, c, d.W, d.dr_orth, d.dr_diag);
    }
  }
}

// GB300 runs FP64 at ~1.6 lanes/clock/SM against ~113 for FP32, so the eight
// FP64 divides per cell of the reference formula would dominate the
// timestep. The filter decides the receiver from FP32 approximations with a
// rigorous error bound and queues the rare cells it cannot prove for the
// FP64 formula. The result is identical to k_receivers_exact for every input.
//
// Bound: f = h truncated to FP32 (|f-h| <= 2^-23|h| + 2^-126),
// a_n = fl(fl(f_c - f_n) * g_n) with g_n = fl(1/dr_n); then for the exact
// reference slope q_n = RN(RN(h_c-h_n)/dr_n):
//   |a_n - q_n| <= 2^-20 * gmax * (M + 2^-100) =: E/2,
// M >= max |f| over the 3x3 window (the kernel takes the maximum over the
// whole staged tile, which only widens the bound), gmax = max g_n. So
//   best - second > 2E  and best > E  => q_best is the unique maximum > 0;
//   best < -E                         => every q_n < 0 (NO_FLOW);
// otherwise (near-ties, zero slopes, NaN, |h| >= 2^128) the cell is queued.
//
// High ground: the bound grows with the elevations themselves, so a tile
// whose largest |h| reaches 2^(kRelEmin-1023) is staged a second time,
// relative to its first cell: X = fixed_in_binade(h, et) (fs_bits.h; et the
// tile's largest biased exponent, unit u = 2^(et-1084), truncation error
// below u), f = RN32(X - X_ref) * u. Then
// |f - (h - X_ref*u)| <= 2^-24 |h - X_ref*u| + 1.01 u, a common offset that
// cancels in every difference h_c - h_n, so the same bound holds with M the
// largest |f| of the relative values plus 2^22 u for the truncation:
//   E/2 = 2^-20 * gmax * (M + 2^22 u),
// and M is taken per cell over its own 3x3 window (the proof needs no
// more), so a jump inside the tile -- base level beside high ground --
// widens the bound only next to it. Tiles below 2^(kRelEmax-1022) qualify
// (f and u stay normal FP32); others, and tiles below 2^(kRelEmin-1023),
// where truncation is already tight, keep the truncated values and the
// tile's M. tests/native/filter_bound_check.cpp restates these decisions on
// the host and checks them against the FP64 formula.

// trunc_bits_to_float (fs_bits.h): truncation of a double to FP32 with
// integer operations only (no FP64 pipe).
constexpr int kRelEmin = 1030;  // |h| >= 128
constexpr int kRelEmax = 1123;  // |h| < 2^101

// TMA staging of a single grid's tile (TMA variant): one box of FP64 values,
// columns x0-2 .. x0+33 (the box's x must be even: 16-byte aligned) and rows
// y0-1 .. y0+96, into shared memory; the staging then reads the values from
// there (column offset 1) instead of loading them from global memory.
constexpr int kRtW = kRxTile + 4, kRtH = kRyTile + 2;

__device__ __forceinline__ uint32_t rf_smem(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Loads the box into dst with the transaction counted on bar (thread 0).
__device__ __forceinline__ void rf_tma_tile(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(rf_smem(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(rf_smem(bar)),
               "r"(static_cast<uint32_t>(kRtW * kRtH * 8))
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(rf_smem(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(rf_smem(bar)), "r"(x), "r"(y)
      : "memory");
}

// Waits for the box (phase 0 of bar); false after limit_ns.
__device__ __forceinline__ bool rf_wait(uint64_t *bar, unsigned long long limit_ns) {
  const unsigned long long t0 = globaltimer_ns();
  for (int it = 0;; it++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(rf_smem(bar))
        : "memory");
    if (ok) return true;
    if ((it & 15) == 15 && globaltimer_ns() - t0 > limit_ns) return false;
  }
}

template <bool TMA>
__global__ void __launch_bounds__(256)
    k_receivers_filter(const __grid_constant__ CUtensorMap hmap, StepArgs a) {
  if (stopped(a.ctl)) return;
  __shared__ float s[kRyTile + 2][kRxTile + 3];
  __shared__ alignas(128) unsigned long long s64[TMA ? kRtH : 1][TMA ? kRtW : 1];
  __shared__ uint64_t s_bar;
  __shared__ unsigned s_wmax[8];
  const Tile t = a.rtiles[blockIdx.x];
  const RealDesc &d = a.desc[t.r];
  const int W = d.W, H = d.H;
  const double *h = a.h + d.off;
  int8_t *rec = a.rec + d.off;
  const int x0 = t.x0 - 1, y0 = t.y0 - 1;  // grid coordinates of s[0][0]
  // Stage the tile and its halo; M = max |f| and whether any value is NaN
  // (|h| >= 2^128, Inf, NaN) are taken over the whole tile.
  float m = 0.f;
  bool bad = false;
  constexpr int kSw = kRxTile + 2, kSn = (kRyTile + 2) * kSw;
  constexpr int kSPer = (kSn + 255) / 256;  // staged values per thread
  // all of a thread's loads in flight before the first is used
  const int t0 = threadIdx.y * 32 + threadIdx.x;
  if (TMA) {
    if (t0 == 0) rf_tma_tile(&s64[0][0], &hmap, &s_bar, x0 - 1, y0);
    __syncthreads();  // the barrier is initialised
    if (!rf_wait(&s_bar, a.timeout_ns)) {
      raise_err(a.ctl, FS_ERR_TIMEOUT, kPhaseNone);
      return;
    }
  }
  auto load_value = [&](int tb, int k) -> unsigned long long {  // staged value tb + 256k
    const int i = tb + 256 * k;
    const int ly = i / kSw, lx = i - ly * kSw;
    if (TMA) return i < kSn ? s64[ly][lx + 1] : 0ull;  // zero-filled outside the grid
    const int gx = x0 + lx, gy = y0 + ly;
    if (i < kSn && gx < W && gy < H)
      return __ldg(reinterpret_cast<const unsigned long long *>(h) + (gy * W + gx));
    return 0;  // bits of +0.0
  };
  // Truncated values first, with the tile's largest biased exponent, which
  // decides whether the tile is staged again relative to its first cell.
  __shared__ int s_wexp[8];
  int ew = 0;
  {
    unsigned long long hv[kSPer];
#pragma unroll
    for (int k = 0; k < kSPer; k++) hv[k] = load_value(t0, k);
#pragma unroll
    for (int k = 0; k < kSPer; k++) {
      const int i = t0 + 256 * k;
      if (i < kSn) {
        const int ly = i / kSw, lx = i - ly * kSw;
        const float f = trunc_bits_to_float(hv[k]);
        s[ly][lx] = f;
        m = fmaxf(m, fabsf(f));
        bad |= !(f == f);
        ew = max(ew, (int)(hv[k] >> 52) & 0x7FF);
      }
    }
  }
  const unsigned wm = __reduce_max_sync(kFull, __float_as_uint(m));  // m >= 0: bits order
  ew = __reduce_max_sync(kFull, ew);
  if (threadIdx.x == 0) {
    s_wmax[threadIdx.y] = wm;
    s_wexp[threadIdx.y] = ew;
  }
  const bool tile_bad = __syncthreads_or(bad) != 0;
  float M = 0.f;
  int et = 0;
#pragma unroll
  for (int w = 0; w < 8; w++) {
    M = fmaxf(M, __uint_as_float(s_wmax[w]));
    et = max(et, s_wexp[w]);
  }
  float absterm = 0x1p-100f;
  const bool rel = et >= kRelEmin && et <= kRelEmax;  // block-uniform; no NaN then
  if (rel) {
    // Staged again relative to the tile's first cell (interior: tiles start
    // at x, y >= 2), from a second read of the tile (cached). No thread
    // reads s before the barrier below.
    const long long xr = fixed_in_binade(
        __ldg(reinterpret_cast<const unsigned long long *>(h) + (t.y0 * W + t.x0)), et);
    const float unit = float_from_bits((uint32_t)(et - 1084 + 127) << 23);  // u
    absterm = float_from_bits((uint32_t)(et - 1062 + 127) << 23);           // 2^22 u
    // an opaque copy of t0: the indices are recomputed here instead of
    // being kept in registers across the first pass
    int tb;
    asm volatile("mov.u32 %0, %1;" : "=r"(tb) : "r"(t0));
    // two batches of loads in flight (one loop body: fewer registers)
    constexpr int kHalf = (kSPer + 1) / 2;
#pragma unroll 1
    for (int k0 = 0; k0 < kSPer; k0 += kHalf) {
      unsigned long long hv[kHalf];
#pragma unroll
      for (int k = 0; k < kHalf; k++) hv[k] = k0 + k < kSPer ? load_value(tb, k0 + k) : 0;
#pragma unroll
      for (int k = 0; k < kHalf; k++) {
        const int i = tb + 256 * (k0 + k);
        if (k0 + k < kSPer && i < kSn) {
          const int ly = i / kSw, lx = i - ly * kSw;
          s[ly][lx] = (float)(fixed_in_binade(hv[k], et) - xr) * unit;
        }
      }
    }
    __syncthreads();
  }
  const float g_orth = d.g_orth, g_diag = d.g_diag;
  const float cE = 0x1p-19f * d.gmax;
  const int lx = threadIdx.x + 1;
  const int gx = x0 + lx;
  unsigned qbits = 0;  // bit r: the cell of row lyb + r is queued
  // Each thread takes kRows consecutive rows of its column, sliding a 3x3
  // window down: 3 new shared loads per row. LOCAL (relative tiles): M is
  // the largest |f| of each cell's own window instead of the tile's, so a
  // jump inside the tile (base level next to high ground) widens the bound
  // only where it is.
  constexpr int kRows = kRyTile / 8;
  const int lyb = kRows * threadIdx.y + 1;
  auto rows = [&](auto local) {
    constexpr bool LOCAL = decltype(local)::value;
    float u0 = s[lyb - 1][lx - 1], u1 = s[lyb - 1][lx], u2 = s[lyb - 1][lx + 1];
    float m0 = s[lyb][lx - 1], m1 = s[lyb][lx], m2 = s[lyb][lx + 1];
    float E = cE * (M + absterm);
    float cu = 0.f, cm = 0.f;  // LOCAL: largest |f| of the window's upper and middle rows
    if (LOCAL) {
      cu = fmaxf(fabsf(u0), fmaxf(fabsf(u1), fabsf(u2)));
      cm = fmaxf(fabsf(m0), fmaxf(fabsf(m1), fabsf(m2)));
    }
#pragma unroll
    for (int r = 0; r < kRows; r++) {
      const int ly = lyb + r;
      const float d0 = s[ly + 1][lx - 1], d1 = s[ly + 1][lx], d2 = s[ly + 1][lx + 1];
      if (LOCAL) {
        const float cd = fmaxf(fabsf(d0), fmaxf(fabsf(d1), fabsf(d2)));
        E = cE * (fmaxf(cu, fmaxf(cm, cd)) + absterm);
        cu = cm;
        cm = cd;
      }
      const int gy = y0 + ly;
      if (gx < W - 2 && gy < H - 2) {
        const float fc = m1;
        // Largest and second largest approximate slope. Within a direction
        // class (orthogonal W N E S = codes 0 2 4 6, diagonal NW NE SE SW =
        // 1 3 5 7) a_n = fl(fl(fc - f_n) * g) does not increase with f_n
        // (rounding is monotone), so the class's largest and second largest
        // slopes are those of its smallest and second smallest f -- the same
        // values as over all eight slopes. bn is the direction of the
        // largest; it is used only when the largest exceeds every other
        // slope, when its f is the unique minimum of its class (a tie leaves
        // best == second, which queues the cell). Without NaN in the tile no
        // slope is NaN (an overflowing difference is +-Inf, and Inf - Inf
        // below only queues).
        const float lo1 = fminf(m0, m2), hi1 = fmaxf(m0, m2);  // W, E
        const float lo2 = fminf(u1, d1), hi2 = fmaxf(u1, d1);  // N, S
        const float lo3 = fminf(u0, u2), hi3 = fmaxf(u0, u2);  // NW, NE
        const float lo4 = fminf(d2, d0), hi4 = fmaxf(d2, d0);  // SE, SW
        const float omin = fminf(lo1, lo2), osec = fminf(fmaxf(lo1, lo2), fminf(hi1, hi2));
        const float dmin = fminf(lo3, lo4), dsec = fminf(fmaxf(lo3, lo4), fminf(hi3, hi4));
        const int oi = lo2 < lo1 ? (d1 < u1 ? 6 : 2) : (m2 < m0 ? 4 : 0);
        const int di = lo4 < lo3 ? (d0 < d2 ? 7 : 5) : (u2 < u0 ? 3 : 1);
        const float bo = (fc - omin) * g_orth, so = (fc - osec) * g_orth;
        const float bd = (fc - dmin) * g_diag, sd = (fc - dsec) * g_diag;
        const float best = fmaxf(bo, bd);
        const float second = fmaxf(fminf(bo, bd), fmaxf(so, sd));
        const int bn = bo > bd ? oi : di;
        int code = -1;
        if (!tile_bad) {
          if (best - second > 2.f * E && best > E) code = bn;
          else if (best < -E) code = kPit;
        }
        if (code != -1) rec[gy * W + gx] = (int8_t)code;
        else qbits |= 1u << r;
      }
      u0 = m0; u1 = m1; u2 = m2;
      m0 = d0; m1 = d1; m2 = d2;
    }
  };
  if (rel) rows(std::true_type{});
  else rows(std::false_type{});
  // The queued cells of the tile, placed with one atomic per tile (a
  // counter shared by the whole grid would serialise on one address).
  int total;
  const int tt = threadIdx.y * 32 + threadIdx.x;
  const int excl = block_excl_scan(__popc(qbits), total, tt, 256);
  if (total == 0) return;
  __shared__ int s_qbase;
  if (tt == 0) s_qbase = atomicAdd(&a.ctl->amb, total);
  __syncthreads();
  int q = s_qbase + excl;
#pragma unroll 1
  for (int r = 0; r < kRyTile / 8; r++) {
    if (qbits >> r & 1u) {
      const int gy = y0 + kRows * threadIdx.y + r + 1;
      a.amb[q] = d.off + gy * W + gx;
      a.amb_r[q] = t.r;
      ++q;
    }
  }
}

// The queued cells of k_receivers_filter, with the reference formula in FP64.
__global__ void __launch_bounds__(256) k_receivers_fixup(StepArgs a) {
  if (stopped(a.ctl)) return;
  const int n_amb = ld_volatile_i32(&a.ctl->amb);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_amb; i += gridDim.x * blockDim.x) {
    const RealDesc &d = a.desc[a.amb_r[i]];
    const int c = a.amb[i] - d.off;
    a.rec[d.off + c] = (int8_t)receiver_fp64_lower(a.h + d.off, c, d);
  }
}

// ---------------------------------------------------------------------------
// 2. Donor masks + level 0.
// Bit k of mask[c] is set when neighbour c+nshift[k] has receiver code
// (k+4)%8, i.e. drains into c (the pull form of fastscape_RB+GPU.cpp:155-182).
// Level 0 = every cell without a receiver (fastscape_RB.cpp:221-227): the
// two outer rings, which never change and sit at ent[0, nring) of their
// realization from creation on, and the interior pits, appended here with
// one atomic per tile.
//
// Four cells per thread, as bytes of one 32-bit word: a tile's rows are
// staged as aligned words of rec, each thread extracts the words of its
// cells' left, centre and right neighbours with funnel shifts, and a
// byte-wise equality test against the direction code gives the eight mask
// bits of four cells at once.
// ---------------------------------------------------------------------------

// 0x80 in every byte of x equal to the byte t, 0 in the others (no carry
// crosses a byte: (y & 0x7F) + 0x7F <= 0xFE).
__device__ __forceinline__ unsigned bytes_eq(unsigned x, unsigned t) {
  const unsigned y = x ^ (t * 0x01010101u);
  return ~(((y & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | y) & 0x80808080u;
}

constexpr int kDRows = kDyTile / 8;       // consecutive rows per thread
constexpr int kDWords = kDxTile / 4 + 4;  // staged words per row

__global__ void __launch_bounds__(256) k_donors_level0(StepArgs a) {
  if (stopped(a.ctl)) return;
  __shared__ unsigned S[kDyTile + 2][kDWords];
  __shared__ int s_sh[kDyTile + 2];
  __shared__ int s_base;
  const Tile t = a.dtiles[blockIdx.x];
  const RealDesc &d = a.desc[t.r];
  const int W = d.W, H = d.H;
  const int8_t *rec = a.rec + d.off;
  const int tt = threadIdx.y * 32 + threadIdx.x;
  // Staged row ly = grid row y0-1+ly (clamped to the grid: rows past it only
  // feed cells that are not written), as the aligned words from the one
  // holding byte x0-4 on; s_sh = position of byte x0-4 in the first word.
  // The reads stay within kRecPad bytes of the realization.
  // (all of a thread's loads in flight before the first is stored)
  constexpr int kSRows = (kDyTile + 2 + 7) / 8;
  static_assert(kDWords > 32 && kDWords <= 64, "two words per lane and row");
  unsigned wv[kSRows][2];
  int shv[kSRows];
#pragma unroll
  for (int k = 0; k < kSRows; k++) {
    const int ly = threadIdx.y + 8 * k;
    wv[k][0] = wv[k][1] = 0;
    shv[k] = 0;
    if (ly < kDyTile + 2) {
      const int gy = min(t.y0 - 1 + ly, H - 1);
      const uintptr_t first = reinterpret_cast<uintptr_t>(rec + (size_t)gy * W + t.x0) - 4;
      const unsigned *src = reinterpret_cast<const unsigned *>(first & ~(uintptr_t)3);
      wv[k][0] = __ldg(src + threadIdx.x);
      if (threadIdx.x + 32 < kDWords) wv[k][1] = __ldg(src + 32 + threadIdx.x);
      shv[k] = (int)(first & 3);
    }
  }
#pragma unroll
  for (int k = 0; k < kSRows; k++) {
    const int ly = threadIdx.y + 8 * k;
    if (ly < kDyTile + 2) {
      S[ly][threadIdx.x] = wv[k][0];
      if (threadIdx.x + 32 < kDWords) S[ly][32 + threadIdx.x] = wv[k][1];
      if (threadIdx.x == 0) s_sh[ly] = shv[k];
    }
  }
  __syncthreads();
  const int gx0 = t.x0 + 4 * threadIdx.x;   // the thread's first cell
  const int ly0 = 1 + kDRows * threadIdx.y;  // its first staged row
  // left / centre / right neighbour words of the four cells in staged row ly
  auto words = [&](int ly, unsigned &L, unsigned &C, unsigned &R) {
    const int p = 3 + s_sh[ly] + 4 * threadIdx.x;  // byte of the first left neighbour
    const int sh = (p & 3) * 8;
    const unsigned *w = &S[ly][p >> 2];
    const unsigned w0 = w[0], w1 = w[1], w2 = w[2];
    L = __funnelshift_r(w0, w1, sh);
    C = __funnelshift_rc(w0, w1, sh + 8);
    R = sh <= 16 ? __funnelshift_rc(w0, w1, sh + 16) : __funnelshift_r(w1, w2, sh - 16);
  };
  unsigned vx = 0;  // 0xFF in the bytes of cells with 1 <= x <= W-2
#pragma unroll
  for (int j = 0; j < 4; j++)
    if (gx0 + j >= 1 && gx0 + j <= W - 2) vx |= 0xFFu << (8 * j);
  unsigned UL, UC, UR, ML, MC, MR, DL, DC, DR;
  words(ly0 - 1, UL, UC, UR);
  words(ly0, ML, MC, MR);
  uint8_t *mask = a.mask + d.off;
  unsigned pits[kDRows];
  int npit = 0;
#pragma unroll
  for (int i = 0; i < kDRows; i++) {
    const int gy = t.y0 + kDRows * threadIdx.y + i;
    words(ly0 + i + 1, DL, DC, DR);
    const unsigned m = (bytes_eq(ML, 4) >> 7) | (bytes_eq(UL, 5) >> 6) |   // W, NW
                       (bytes_eq(UC, 6) >> 5) | (bytes_eq(UR, 7) >> 4) |   // N, NE
                       (bytes_eq(MR, 0) >> 3) | (bytes_eq(DR, 1) >> 2) |   // E, SE
                       (bytes_eq(DC, 2) >> 1) | bytes_eq(DL, 3);           // S, SW
    const unsigned v = gy <= H - 2 ? vx : 0u;
    pits[i] = bytes_eq(MC, (unsigned)(uint8_t)kPit) & v;
    npit += __popc(pits[i]);
    if (v) {
      uint8_t *row = mask + (size_t)gy * W + gx0;
      if (v == 0xFFFFFFFFu && (reinterpret_cast<uintptr_t>(row) & 3) == 0) {
        *reinterpret_cast<unsigned *>(row) = m;
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
          if ((v >> (8 * j)) & 1u) row[j] = (uint8_t)(m >> (8 * j));
      }
    }
    UL = ML; UC = MC; UR = MR;
    ML = DL; MC = DC; MR = DR;
  }
  int total;
  const int excl = block_excl_scan(npit, total, tt, 256);
  if (total == 0) return;
  if (tt == 0) s_base = d.off + d.nring + atomicAdd(&a.rctl[t.r].top, total);
  __syncthreads();
  int pos = s_base + excl;
#pragma unroll
  for (int i = 0; i < kDRows; i++) {
    const int gy = t.y0 + kDRows * threadIdx.y + i;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if ((pits[i] >> (8 * j + 7)) & 1u) a.ent[pos++] = gy * W + gx0 + j;
  }
}

// ---------------------------------------------------------------------------
// 3. Erosion of one cell and the division it needs.
// ---------------------------------------------------------------------------

// Correctly rounded num/D for D > 0 given R = RN(1/D), without the FP64
// divide routine: Markstein's correction q1 = q0 + (num - q0*D)*R with
// fused multiply-adds (P. Markstein, IBM J. Res. Dev. 34(1), 1990), then an
// exact check of the remainder r1 = num - q1*D: q1 is accepted only if
// |r1| < D*ulp(q1)/2 (then |num/D - q1| < ulp(q1)/2, so q1 = RN(num/D)),
// q1 is not a power of two (where the spacing below halves) and its
// exponent is far from the subnormal/overflow range. Anything else -- zero
// numerators included -- takes the IEEE division. 4 FP64 operations against
// ~7.5 for the divide routine on this part.
__device__ __forceinline__ double div_rn(double num, double D, double R) {
  const double q0 = num * R;
  const double r0 = fma(-q0, D, num);
  const double q1 = fma(r0, R, q0);
  const double r1 = fma(-q1, D, num);
  const long long qb = abs_bits(q1);
  const int e = (int)(qb >> 52);
  if (e >= 64 && e <= 1980 && (qb & 0x000FFFFFFFFFFFFFll) != 0) {
    const long long thr = __double_as_longlong(D) + ((long long)(e - 1076) << 52);
    if (abs_bits(r1) < thr) return q1;
  }
  return num / D;
}

// pow(x, n) and pow(x, n-1) for the Newton update of fastscape_RB.cpp:322.
template <int NMODE>
__device__ __forceinline__ void powers(double x, double neq, double &pn, double &pn1) {
  if (NMODE == kNOne) {
    pn = x;
    pn1 = 1.0;
  } else if (NMODE == kNTwo) {
    pn = x * x;
    pn1 = x;
  } else {
    pn = pow(x, neq);
    pn1 = pow(x, neq - 1.0);
  }
}

// The fields of a table record the n = 1 erosion reads up front.
struct TabN1 {
  uint64_t fact, D, Rn;
};

__device__ __forceinline__ TabN1 load_tab_n1(const unsigned long long *Tb) {
  return TabN1{__ldg(Tb + 0), __ldg(Tb + 1), __ldg(Tb + 3)};
}

// True when |RN(x - y)| <= tol is proven for x = RN(y - q), y the previous
// iterate and qn = -q: |RN(x - y)| <= (|q| + 2^-51(|y|+|q|))(1+2^-53), and
// an FP32 test on truncated magnitudes (each within 2^-23 relative, flushed
// below 2^-126) with 2^-21 of slack proves it for almost every cell without
// the subtraction.
__device__ __forceinline__ bool step_below_tol(uint64_t qn, uint64_t y, const RealDesc &d) {
  const float qf = fabsf(trunc_bits_to_float(qn));
  const float yf = fabsf(trunc_bits_to_float(y));
  return qf * (1.f + 0x1p-21f) + yf * 0x1p-48f <= d.tol_lo_f;
}

// RN(x + y), y = -q with |q| far below x > 0 (a Newton correction): in
// integer arithmetic when the operands allow, else in FP64.
__device__ __forceinline__ uint64_t add_correction(uint64_t x, uint64_t y) {
  return (y & kSignBit) ? sub_far(x, y ^ kSignBit) : uplift_bits(x, y);
}

// RN(x / y) of bit patterns on the FP64 pipe.
// IEEE division in a branch taken by few cells (volatile: not executed
// speculatively for the others).
__device__ __forceinline__ uint64_t fdiv_bits_volatile(uint64_t a, uint64_t b) {
  uint64_t r;
  asm volatile(
      "{\n\t.reg .f64 x, y;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\t"
      "div.rn.f64 x, x, y;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

__device__ __forceinline__ uint64_t ffma_bits(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("{\n\t.reg .f64 x, y, z;\n\tmov.b64 x, %1;\n\tmov.b64 y, %2;\n\tmov.b64 z, %3;\n\t"
      "fma.rn.f64 x, x, y, z;\n\tmov.b64 %0, x;\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b), "l"(c));
  return r;
}

// RN(num/den) on bit patterns for a denominator with no tabled reciprocal
// (the n = 2 erosion's), in three FP64 operations: the IEEE FP32 reciprocal
// of |den| truncated to FP32 (within 1.5*2^-23 of 1/|den|), one Newton step
// r1 = r0 + r0*(1 - |den|*r0) by fused multiply-adds (within ~2^-44.8),
// q0 = RN(|num|*r1) (within ~2^8.2 ulp of the quotient), and the rounding
// from the exact integer residual (round_quotient_bits, fs_bits.h). Newton's
// iteration for the reciprocal and the residual check are the published
// methods (e.g. P. Markstein, IBM J. Res. Dev. 34(1), 1990);
// tests/native/division_check.cpp replays the sequence on the host against
// the IEEE division. Operands outside [2^-99, 2^102) and the rare cases the
// rounding leaves open take the IEEE division.
__device__ __forceinline__ uint64_t fdiv_rn_bits(uint64_t nb, uint64_t db) {
  const uint64_t an = nb & ~kSignBit, ad = db & ~kSignBit;
  if ((unsigned)((int)(an >> 52) - 924) <= 200u && (unsigned)((int)(ad >> 52) - 924) <= 200u) {
    const uint32_t rb = __float_as_uint(__frcp_rn(trunc_bits_to_float(ad)));
    // widen the positive normal FP32 reciprocal to FP64 bits
    const uint64_t r0 = ((uint64_t)((rb >> 23) + 896) << 52) | ((uint64_t)(rb & 0x7FFFFFu) << 29);
    const uint64_t e = ffma_bits(ad ^ kSignBit, r0, 0x3FF0000000000000ull);  // 1 - |den| r0
    const uint64_t r1 = ffma_bits(r0, e, r0);
    const uint64_t q = round_quotient_bits(an, ad, fmul_bits(an, r1));
    if (q) return q | ((nb ^ db) & kSignBit);
  }
  return fdiv_bits_volatile(nb, db);
}

// RN(x - y) for any operands: in integer arithmetic when both are positive
// normal (sub_near_bits within a factor 2, sub_far_bits from an exponent gap
// of 2) or x is positive and y negative (add_pos_rn_bits), else in FP64.
__device__ __forceinline__ uint64_t sub_gen(uint64_t x, uint64_t y) {
  if (add_pos_operand(x)) {
    if (add_pos_operand(y)) {
      if (x != y) {
        const bool gt = x > y;
        const uint64_t hi = gt ? x : y, lo = gt ? y : x;
        const uint64_t r = ((int)(hi >> 52) - (int)(lo >> 52) >= 2) ? sub_far_bits(hi, lo)
                                                                     : sub_near_bits(hi, lo);
        if (r) return gt ? r : (r ^ kSignBit);
      }
    } else if (add_pos_operand(y ^ kSignBit)) {
      return add_pos_rn_bits(x, y ^ kSignBit);
    }
  }
  return fadd_bits_volatile(x, y ^ kSignBit);
}

// Erosion of one cell for n = 2 (fastscape_RB.cpp:315-326; pow(x,2) as x*x,
// pow(x,1) = x) on bit patterns, iterate by iterate in the reference's
// operation order: x' = RN(x - RN(num/den)) with
//   num = RN(RN(x - h0) + RN(fact*RN(RN(x-hn)^2))),
//   den = RN(1 + RN(RN(fact*n)*RN(x-hn))),
// RN(fact*n) hoisted (the reference's grouping), the first iterate's
// x - h0 = +0 dropped, and |x' - x| <= tol proven in FP32 for most
// iterates without the subtraction. With ISUB the subtractions run in
// integer arithmetic.
template <bool ISUB>
__device__ __forceinline__ uint64_t erode_cell_n2(const RealDesc &d, double neq, Ctl *ctl,
                                                  uint64_t factb, uint64_t h0, uint64_t hn) {
  auto sub = [](uint64_t x, uint64_t y) { return ISUB ? sub_gen(x, y) : fadd_bits(x, y ^ kSignBit); };
  constexpr uint64_t kOne = 0x3FF0000000000000ull;
  const uint64_t fact2 = fmul_bits(factb, (uint64_t)__double_as_longlong(neq));
  uint64_t x = h0;
  for (int it = 1;; ++it) {
    const uint64_t dx = sub(x, hn);
    const uint64_t fpn = fmul_bits(factb, fmul_bits(dx, dx));
    uint64_t num;
    if (it == 1) {
      num = (fpn << 1) == 0 ? 0 : fpn;  // RN(+0 + fpn)
    } else {
      const uint64_t a = sub(x, h0);
      num = ISUB ? sub_gen(fpn, a ^ kSignBit) : fadd_bits(a, fpn);
    }
    const uint64_t den = fadd_bits(kOne, fmul_bits(fact2, dx));
    const uint64_t q = fdiv_rn_bits(num, den);
    const uint64_t xn = sub(x, q);
    if (step_below_tol(q ^ kSignBit, x, d)) return xn;
    const uint64_t df = sub(xn, x);
    x = xn;
    // fabs(diff) > tol as an integer compare (a NaN diff stops the loop)
    const long long m = (long long)(df & ~kSignBit);
    if (!(m > d.tol_bits && m <= 0x7FF0000000000000ll)) return x;
    if (it >= kNewtonMaxIt) {
      raise_err(ctl, FS_ERR_NEWTON, kPhaseErode);
      return x;
    }
  }
}

// Erosion of one cell for n = 1 (fastscape_RB.cpp:315-326) on bit
// patterns: h0 the uplifted elevation, hn the receiver's final elevation,
// t the table record of the cell's drainage count and direction class
// (fact, D = 1 + fact, -1/D; Tb the record itself for 1/D).
//
// The reference's loop for n = 1 (pow(x,1) = x, pow(x,0) = 1):
//   x' = RN(x - RN(RN(RN(x - h0) + RN(fact*RN(x - hn))) / D)),
//   stop when |RN(x' - x)| <= tol.
// First iterate (x = h0): RN(h0 - h0) = +0, so x1 = RN(h0 - RN(RN(fact*
// RN(h0-hn)) / D)). Cells whose erosion exceeds tol take a second iterate,
// unrolled here too; its residual num2 is often exactly 0 (then x2 = x1).
// Rarer third iterates follow the generic loop. With ISUB the subtractions
// of elevations run in integer arithmetic: that relieves the FP64 pipe but
// lengthens the cell's dependency chain after the receiver's elevation
// arrives, which pays where the pipe, not latency, limits the erosion (the
// autotuner decides per workload).
template <bool ISUB>
__device__ __forceinline__ uint64_t erode_cell_n1(const RealDesc &d, Ctl *ctl,
                                                  const unsigned long long *Tb, TabN1 t,
                                                  uint64_t h0, uint64_t hn) {
  const uint64_t factb = t.fact;
  const double D = __longlong_as_double(t.D), Rn = __longlong_as_double(t.Rn);
  const uint64_t dh = ISUB ? sub_near(h0, hn) : fadd_bits(h0, hn ^ kSignBit);
  const uint64_t num = fmul_bits(factb, dh);
  const uint64_t qn = neg_div_rn_bits(num, D, Rn);  // -q
  const uint64_t x1 = ISUB ? sub_far(h0, qn ^ kSignBit) : fadd_bits(h0, qn);
  if (step_below_tol(qn, h0, d)) return x1;
  // diff = RN(x1 - h0); |diff| > tol as an integer compare of the
  // magnitudes' bits (a NaN diff stops the loop, as fabs(NaN) > tol is false)
  const uint64_t a = ISUB ? sub_sterbenz(x1, h0) : fadd_bits(x1, h0 ^ kSignBit);
  auto more = [&](uint64_t df) {
    const long long m = (long long)(df & ~kSignBit);
    return m > d.tol_bits && m <= 0x7FF0000000000000ll;
  };
  if (!more(a)) return x1;
  // second iterate: num2 = RN(a + RN(fact * RN(x1 - hn)))
  const uint64_t b = ISUB ? sub_sterbenz(x1, hn) : fadd_bits(x1, hn ^ kSignBit);
  const uint64_t c = fmul_bits(factb, b);
  const uint64_t num2 = ISUB ? sub_sterbenz(c, a ^ kSignBit) : fadd_bits(a, c);
  if ((num2 << 1) == 0) return x1;  // RN(0/D) = +0 and x1 - 0 = x1: diff = 0
  // The correction is a residual of x1's rounding: x2 is x1 or a neighbour,
  // decided from an FP32 estimate of the quotient (newton_step_in_spacing),
  // and a step of at most one spacing <= tol ends the loop.
  if (add_pos_operand(x1)) {
    const float qe = __fdividef(fabsf(trunc_bits_to_float(num2)), trunc_bits_to_float(t.D));
    int step;
    float ulp;
    if (newton_step_in_spacing(num2, t.D, x1, qe, &step, &ulp) && ulp <= d.tol_lo_f)
      return x1 + (uint64_t)(int64_t)step;
  }
  const uint64_t q2n = neg_div_rn_bits(num2, D, Rn);
  const uint64_t x2 = ISUB ? add_correction(x1, q2n) : fadd_bits(x1, q2n);
  if (step_below_tol(q2n, x1, d)) return x2;
  // third and later iterates: the reference's loop in FP64
  const double R = __longlong_as_double(__ldg(Tb + 2));
  const double fact = __longlong_as_double(factb), h0d = __longlong_as_double(h0),
               hnd = __longlong_as_double(hn);
  double x = __longlong_as_double(x2);
  double diff = x - __longlong_as_double(x1), hp = x;
  int it = 2;
  while (more((uint64_t)__double_as_longlong(diff))) {
    const double n3 = (x - h0d) + fact * (x - hnd);
    x -= div_rn(n3, D, R);
    diff = x - hp;
    hp = x;
    if (++it >= kNewtonMaxIt) {
      raise_err(ctl, FS_ERR_NEWTON, kPhaseErode);
      break;
    }
  }
  return (uint64_t)__double_as_longlong(x);
}

// Erosion of one cell for n != 1: fastscape_RB.cpp:315-326 with h0 the
// uplifted elevation, hn the receiver's final elevation and T the table
// record of the cell's drainage count and direction class (T[0] = fact).
template <int NMODE>
__device__ __forceinline__ double erode_cell(const RealDesc &d, double neq, Ctl *ctl,
                                             const double *T, double h0, double hn) {
  const double fact = T[0];
  double hnew, hp, diff;
  int it;
  hnew = h0;
  hp = h0;
  diff = 2 * d.tol;
  it = 0;
  while (fabs(diff) > d.tol) {
    double pn, pn1;
    powers<NMODE>(hnew - hn, neq, pn, pn1);
    hnew -= (hnew - h0 + fact * pn) / (1. + fact * neq * pn1);
    diff = hnew - hp;
    hp = hnew;
    if (++it >= kNewtonMaxIt) {
      raise_err(ctl, FS_ERR_NEWTON, kPhaseErode);
      break;
    }
  }
  return hnew;
}

// ---------------------------------------------------------------------------
// 4. Persistent level walker (cooperative launch).
//
// The ordering is kept as arrays indexed by position in the level order
// (fs_internal.h): accumulation and erosion read them by position --
// coalesced -- instead of gathering receivers, masks and counts by cell.
// Per level, every block keeps each realization's range [lo, hi) in shared
// memory and maps global work items (expansion chunks, 32-entry groups) to
// realizations through a prefix over the batch.
// ---------------------------------------------------------------------------
template <bool SINGLE, int MINB>
__global__ void __launch_bounds__(kWalkThreads, MINB) k_order(StepArgs a) {
  extern __shared__ int smem[];
  const int nreal = a.nreal;
  int *s_lo = smem;               // per realization: current range start
  int *s_hi = s_lo + nreal;       // and end (local positions)
  int *s_nlev = s_hi + nreal;     // levels found so far
  int *s_pre = s_nlev + nreal;    // prefix over the batch, nreal+1
  __shared__ int s_cw[2][kWalkWarps];  // warp totals / prefixes of a chunk
  __shared__ int s_cbase[2];           // the chunk's first position
  int cbuf = 0;
  __shared__ uint8_t s_own[kWalkWarps][32 * 8];  // (lane, direction) per donor slot of a pass
  unsigned epoch = 0;
  Ctl *ctl = a.ctl;
  if (stopped(ctl)) return;
  // A batch of one keeps its descriptor in registers and skips the
  // realization lookups.
  RealDesc d0;
  if (SINGLE) d0 = a.desc[0];
  auto desc = [&](int r) -> const RealDesc & { return SINGLE ? d0 : a.desc[r]; };
  auto real_of = [&](int g) -> int { return SINGLE ? 0 : find_real(s_pre, nreal, g); };
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool stamp = a.stamp && tid == 0;
  unsigned long long t_prev = stamp ? globaltimer_ns() : 0;
  auto lap = [&](int slot) {
    if (stamp) {
      const unsigned long long t = globaltimer_ns();
      atomicAdd(&ctl->walk_ns[slot], t - t_prev);
      t_prev = t;
    }
  };

  // ---- ordering: fastscape_RB.cpp:229-251 -------------------------------
  // Level k+1 = the donors of level k. A block expands a chunk of kChunk
  // consecutive entries of one realization; warp w covers 32*kPer of them
  // in kPer coalesced passes (entry wbase+32q+lane). Warp scans give each
  // entry's first-donor offset in entry order, one block scan over the
  // warps and one atomic place the chunk, and the donors are written
  // cooperatively (lane r writes the r-th donor of the pass), so the next
  // level keeps this level's order. Each realization's append counter
  // rotates over three words so a block that reads the size of level k after
  // the barrier never races with the reset for level k+2.
  // s_tot[L & 1]: entries of level L over the batch (double-buffered: the
  // next level's count is summed while this one's may still be read)
  __shared__ int s_tot[2];
  if (threadIdx.x == 0) s_tot[0] = s_tot[1] = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
    const RealDesc &d = desc(r);
    s_lo[r] = 0;
    s_hi[r] = d.nring + ld_volatile_i32(&a.rctl[r].top);
    s_nlev[r] = 1;
    atomicAdd(&s_tot[0], s_hi[r]);
    if (blockIdx.x == 0) {
      a.lvl_off[d.lvl_base + 0] = 0;
      a.lvl_off[d.lvl_base + 1] = s_hi[r];
    }
  }
  __syncthreads();
  int L = 0;  // level being expanded
  for (;;) {
    const int j = L % 3;
    if (blockIdx.x == 0)
      for (int r = threadIdx.x; r < nreal; r += kWalkThreads) a.rctl[r].lvlcnt[(L + 1) % 3] = 0;
    // Passes per warp in this level's chunks: kPer, or one for a level that
    // fits one round of one-pass chunks over the grid, so that its chunks
    // spread over more blocks (two compiled forms: a run-time pass count
    // slows the big levels' expansion).
    const bool one_pass = s_tot[L & 1] <= (int)gridDim.x * kWalkThreads;
    if (threadIdx.x == 0) s_tot[(L + 1) & 1] = 0;  // summed after this level's barrier
    const int chunk = (one_pass ? 1 : kPer) * kWalkThreads;
    const int nchunks = block_prefix(
        nreal, [&](int r) { return (s_hi[r] - s_lo[r] + chunk - 1) / chunk; }, s_pre);
    auto expand = [&](auto passes, int g) {
      constexpr int NP = decltype(passes)::value;
      const int r = real_of(g);
      const RealDesc &d = desc(r);
      const int hi = s_hi[r];
      const int base = s_lo[r] + (g - s_pre[r]) * (NP * kWalkThreads);
      const int wbase = base + wid * (32 * NP);
      int32_t *ent = a.ent + d.off;
      const uint8_t *mask = a.mask + d.off;
      const int offk = nbr_off(lane & 7, d.W);  // lane k < 8: offset of direction k
      // Per pass q: the entry's cell, and its donor mask with the warp's
      // inclusive donor prefix (relative to the warp's first donor, below
      // 32 * 8 * kPer) packed as (prefix << 8) | mask, to keep the chunk's
      // state in registers across its barriers.
      int cs[NP];
      unsigned mi[NP];
#pragma unroll
      for (int q = 0; q < NP; q++) {
        const int i = wbase + 32 * q + lane;
        cs[q] = 0;
        mi[q] = 0;
        if (i < hi) {
          cs[q] = __ldcg(&ent[i]);
          mi[q] = mask[cs[q]];
        }
      }
      int wtot = 0;
#pragma unroll
      for (int q = 0; q < NP; q++) {
        int v = __popc(mi[q]);
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
          const int x = __shfl_up_sync(kFull, v, dd);
          if (lane >= dd) v += x;
        }
        mi[q] |= (unsigned)(wtot + v) << 8;  // inclusive prefix
        wtot += __shfl_sync(kFull, v, 31);
      }
      // Place the chunk: prefix of the warp totals and one atomic, with two
      // barriers; the shared words alternate between two buffers so the next
      // chunk can fill one while this chunk's readers finish with the other.
      if (lane == 0) s_cw[cbuf][wid] = wtot;
      __syncthreads();
      if (wid == 0) {
        int w = lane < kWalkWarps ? s_cw[cbuf][lane] : 0;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
          const int x = __shfl_up_sync(kFull, w, dd);
          if (lane >= dd) w += x;
        }
        if (lane < kWalkWarps) s_cw[cbuf][lane] = w;  // inclusive prefix over warps
        const int total = __shfl_sync(kFull, w, kWalkWarps - 1);
        if (lane == 0) s_cbase[cbuf] = total ? atomicAdd(&a.rctl[r].lvlcnt[j], total) : 0;
      }
      __syncthreads();
      // position of the warp's first donor
      const int cbase = hi + s_cbase[cbuf] + (wid ? s_cw[cbuf][wid - 1] : 0);
      cbuf ^= 1;
#pragma unroll
      for (int q = 0; q < NP; q++) {
        const int i = wbase + 32 * q + lane;
        const unsigned msk = mi[q] & 0xFFu;
        const int incl = (int)(mi[q] >> 8);
        const int n_d = __popc(msk);
        if (i < hi) {
          a.acc[d.off + i] = 1u;  // the cell itself; donors add theirs below
        }
        // The pass's donors go to positions cbase + [q_lo, q_lo + q_n) in
        // entry order. Each lane records (its lane, direction) for the slots
        // of its donors in the warp's shared bytes; then lane t writes slot t
        // of every 32, coalesced.
        const int q_lo = __shfl_sync(kFull, incl - n_d, 0);
        const int q_n = __shfl_sync(kFull, incl, 31) - q_lo;  // <= 32 * 8
        {
          int slot = incl - n_d - q_lo;
          // every direction, predicated: no divergence across the warp (a
          // loop over the set bits runs as long as the lane with most donors)
#pragma unroll
          for (int k = 0; k < 8; k++) {
            if (msk >> k & 1u) s_own[wid][slot++] = (uint8_t)((lane << 3) | k);
          }
        }
        __syncwarp();
        for (int r0 = 0; r0 < q_n; r0 += 32) {
          const int rr = r0 + lane;
          const unsigned pk = rr < q_n ? s_own[wid][rr] : 0u;
          const int k = pk & 7;
          const int oc = __shfl_sync(kFull, cs[q], pk >> 3);
          const int ok = __shfl_sync(kFull, offk, k);
          if (rr < q_n) {
            const int pos = cbase + q_lo + rr;
            if (pos < d.size) {
              ent[pos] = oc + ok;
              a.pdir[d.off + pos] = (uint8_t)((k + 4) & 7);
              a.par[d.off + pos] = wbase + 32 * q + (int)(pk >> 3);  // receiver's position
            } else {
              raise_err(ctl, FS_ERR_LEVEL_OVERFLOW, kPhaseOrder);
            }
          }
        }
        __syncwarp();  // s_own is refilled by the next pass
      }
        };
    for (int g = blockIdx.x; g < nchunks; g += gridDim.x) {
      if (one_pass) expand(std::integral_constant<int, 1>{}, g);
      else expand(std::integral_constant<int, kPer>{}, g);
    }
    if (!grid_barrier(ctl, &ctl->bar, epoch, a.timeout_ns)) return;
    // Thread r alone reads realization r's size (one load per block, not a
    // load of one word by every thread). Every block sees the same sizes:
    // an overflow ends the walk in all of them; other errors reach them at
    // the next barrier's spin.
    int any = 0, ovf = 0;
    for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
      const int added = ld_volatile_i32(&a.rctl[r].lvlcnt[j]);
      s_lo[r] = s_hi[r];
      if (added) {
        atomicAdd(&s_tot[(L + 1) & 1], added);
        s_hi[r] += added;
        s_nlev[r] = L + 2;
        any = 1;
        if (s_hi[r] > desc(r).size) {
          if (blockIdx.x == 0) raise_err(ctl, FS_ERR_LEVEL_OVERFLOW, kPhaseOrder);
          ovf = 1;
        } else if (blockIdx.x == 0) {
          a.lvl_off[desc(r).lvl_base + L + 2] = s_hi[r];
        }
      }
    }
    if (__syncthreads_or(ovf)) return;
    if (!__syncthreads_or(any)) break;
    ++L;
  }
  // s_hi[r] is the realization's total; anything short of its size means
  // cells that never reached base level: the receivers contain a cycle.
  {
    int bad = 0;
    for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
      if (blockIdx.x == 0) {
        a.rctl[r].nlevels = s_nlev[r];
        a.rctl[r].total = s_hi[r];
      }
      bad |= s_hi[r] != desc(r).size;
    }
    if (__syncthreads_or(bad)) {
      if (tid == 0) raise_err(ctl, FS_ERR_ORDER, kPhaseOrder);
      return;
    }
  }
  lap(0);
}

// Accumulation (fastscape_RB.cpp:262-279) level by level back down to base
// level, then the pits' uplift, after k_order has placed the levels. A
// kernel of its own: its little per-thread state lets it run 4 blocks of
// 512 threads per SM, hiding more of the latency of its loads.
template <bool SINGLE>
__global__ void __launch_bounds__(kWalkThreads, 4) k_accum(StepArgs a) {
  extern __shared__ int smem[];
  const int nreal = a.nreal;
  int *s_lo = smem;
  int *s_hi = s_lo + nreal;
  int *s_nlev = s_hi + nreal;
  int *s_pre = s_nlev + nreal;
  __shared__ int s_maxlev;
  unsigned epoch = 0;
  Ctl *ctl = a.ctl;
  if (stopped(ctl)) return;
  RealDesc d0;
  if (SINGLE) d0 = a.desc[0];
  auto desc = [&](int r) -> const RealDesc & { return SINGLE ? d0 : a.desc[r]; };
  auto real_of = [&](int g) -> int { return SINGLE ? 0 : find_real(s_pre, nreal, g); };
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const int warp_global = tid >> 5, nwarps = nthreads >> 5;
  const bool stamp = a.stamp && tid == 0;
  const unsigned long long t_start = stamp ? globaltimer_ns() : 0;
  if (threadIdx.x == 0) s_maxlev = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
    s_nlev[r] = __ldcg(&a.rctl[r].nlevels);
    atomicMax(&s_maxlev, s_nlev[r]);
  }
  __syncthreads();
  const int maxlev = s_maxlev;

  // Level Lv of every realization as [lo_of(r), hi_of(r)) (empty past its
  // depth), and the prefix of its 32-entry groups over the batch. A batch
  // of one copies its level table into shared memory once (one load per
  // entry and block) and takes each level's range from there into
  // registers: no block barrier, scan or global load per level.
  __shared__ int s_off[kLevelCache + 1];
  if (SINGLE) {
    const int n = min(maxlev, kLevelCache) + 1;
    for (int k = threadIdx.x; k < n; k += kWalkThreads) s_off[k] = __ldcg(&a.lvl_off[d0.lvl_base + k]);
    __syncthreads();
  }
  int lv_lo = 0, lv_hi = 0;
  auto lo_of = [&](int r) -> int { return SINGLE ? lv_lo : s_lo[r]; };
  auto hi_of = [&](int r) -> int { return SINGLE ? lv_hi : s_hi[r]; };
  auto pre_of = [&](int r) -> int { return SINGLE ? 0 : s_pre[r]; };
  auto level_groups = [&](int Lv) -> int {
    if (SINGLE) {
      if (Lv < kLevelCache) {
        lv_lo = s_off[Lv];
        lv_hi = s_off[Lv + 1];
      } else {  // deeper than the cache: one load per block
        __syncthreads();
        if (threadIdx.x == 0) {
          s_lo[0] = __ldcg(&a.lvl_off[d0.lvl_base + Lv]);
          s_hi[0] = __ldcg(&a.lvl_off[d0.lvl_base + Lv + 1]);
        }
        __syncthreads();
        lv_lo = s_lo[0];
        lv_hi = s_hi[0];
      }
      return (lv_hi - lv_lo + 31) >> 5;
    }
    __syncthreads();  // every warp is done with the previous ranges
    for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
      if (Lv < s_nlev[r]) {
        const int b = desc(r).lvl_base;
        s_lo[r] = __ldcg(&a.lvl_off[b + Lv]);
        s_hi[r] = __ldcg(&a.lvl_off[b + Lv + 1]);
      } else {
        s_lo[r] = s_hi[r] = 0;
      }
    }
    __syncthreads();
    return block_prefix(nreal, [&](int r) { return (s_hi[r] - s_lo[r] + 31) >> 5; }, s_pre);
  };

  // ---- accumulation: fastscape_RB.cpp:262-279, pushed level by level ----
  // acc[i] = 1 + the counts of i's donors (the reference's accum is
  // acc*cell_area, exact: integer multiples of cell_area). The ordering set
  // every acc to 1; from the deepest level up, each entry -- whose count is
  // final, its donors having pushed before the last barrier -- adds its
  // count to its receiver's (position par[i]) with a fire-and-forget
  // reduction. Integer sums are exact in any order. A count at level >= 1
  // beyond its realization's erosion table stops the timestep before any
  // elevation changes; the host grows the table and repeats it.
  // Each level's ranges come from the finished level table, so the next
  // level's are set up before this level's barrier.
  int ngroups = maxlev > 1 ? level_groups(maxlev - 1) : 0;
  for (int Lv = maxlev - 1; Lv >= 1; --Lv) {
    // 32-entry groups per warp per iteration. A single grid sums runs of
    // donors in the warp (more work per group) and loads the next groups
    // before reducing these; a batch reduces per donor and keeps more groups'
    // loads in flight instead (each measured faster for its case).
    constexpr int kAccU = SINGLE ? 2 : 4;
    struct Group {
      uint32_t v[kAccU];
      int p[kAccU], r[kAccU];
      bool ok[kAccU];
    };
    auto load_group = [&](int g0) -> Group {
      Group G;
#pragma unroll
      for (int u = 0; u < kAccU; u++) {  // all loads in flight first
        const int g = g0 + u;
        G.ok[u] = false;
        G.v[u] = 0;
        G.p[u] = 0;
        G.r[u] = 0;
        if (g < ngroups) {
          const int r = real_of(g);
          const int i = lo_of(r) + 32 * (g - pre_of(r)) + lane;
          G.r[u] = r;
          if (i < hi_of(r)) {
            const int off = desc(r).off;
            G.ok[u] = true;
            G.v[u] = __ldcg(&a.acc[off + i]);
            G.p[u] = __ldcg(&a.par[off + i]);
          }
        }
      }
      return G;
    };
    Group nxt;
    if (SINGLE) nxt = load_group(warp_global * kAccU);
    for (int g0 = warp_global * kAccU; g0 < ngroups; g0 += nwarps * kAccU) {
      Group G;
      if (SINGLE) {
        G = nxt;
        nxt = load_group(g0 + nwarps * kAccU);
      } else {
        G = load_group(g0);
      }
      const uint32_t *v = G.v;
      const int *pp = G.p, *rr = G.r;
      const bool *ok = G.ok;
#pragma unroll
      for (int u = 0; u < kAccU; u++) {
        if (!SINGLE) {  // batches: one reduction per donor (measured faster there)
          if (ok[u]) {
            const RealDesc &d = desc(rr[u]);
            atomicAdd(&a.acc[d.off + pp[u]], v[u]);
            if (a.do_erode && v[u] >= (uint32_t)d.tab_cap) {
              if (atomicMax(&ctl->abort_k, (int)v[u]) < (int)v[u]) ctl->abort_r = rr[u];
            }
          }
          continue;
        }
        // Donors of one receiver are consecutive: sum each run of equal
        // receiver positions in the group (a warp scan minus its value
        // before the run) and let the run's last lane reduce it into the
        // receiver -- one reduction per receiver and group instead of one
        // per donor. Lanes past the level keep runs of their own.
        const int p = ok[u] ? pp[u] : -1 - lane;
        const int pu = __shfl_up_sync(kFull, p, 1), pd = __shfl_down_sync(kFull, p, 1);
        const bool head = lane == 0 || pu != p, tail = lane == 31 || pd != p;
        const unsigned heads = __ballot_sync(kFull, head) & (0xFFFFFFFFu >> (31 - lane));
        const int hl = 31 - __clz(heads);  // first lane of this lane's run
        uint32_t S = v[u];
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
          const uint32_t x = __shfl_up_sync(kFull, S, dd);
          if (lane >= dd) S += x;
        }
        const uint32_t before = __shfl_sync(kFull, S, (hl + 31) & 31);
        const uint32_t run = S - (hl > 0 ? before : 0u);
        if (ok[u]) {
          const RealDesc &d = desc(rr[u]);
          if (tail) atomicAdd(&a.acc[d.off + p], run);
          if (a.do_erode && v[u] >= (uint32_t)d.tab_cap) {
            if (atomicMax(&ctl->abort_k, (int)v[u]) < (int)v[u]) ctl->abort_r = rr[u];
          }
        }
      }
    }
    if (Lv > 1) ngroups = level_groups(Lv - 1);
    if (!grid_barrier(ctl, &ctl->bar3, epoch, a.timeout_ns)) return;
  }
  // Level 0: counts final. With no table exceeded, uplift the pits (level 0
  // past the rings; fastscape_RB.cpp:291-295) -- the erosion kernel reads
  // them after the kernel boundary.
  if (a.do_erode && ld_volatile_i32(&ctl->abort_k) == 0) {
    __syncthreads();  // every warp is done with the last level's ranges
    for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
      s_lo[r] = desc(r).nring;
      s_hi[r] = __ldcg(&a.lvl_off[desc(r).lvl_base + 1]);
    }
    __syncthreads();
    const int np = block_prefix(nreal, [&](int r) { return s_hi[r] - s_lo[r]; }, s_pre);
    for (int g = tid; g < np; g += nthreads) {
      const int r = real_of(g);
      const RealDesc &d = desc(r);
      unsigned long long *hh = reinterpret_cast<unsigned long long *>(a.h + d.off);
      const int c = __ldcg(&a.ent[d.off + s_lo[r] + (g - s_pre[r])]);
      hh[c] = fadd_bits(__ldcg(&hh[c]), (uint64_t)__double_as_longlong(d.u_dt));
    }
  }
  if (stamp) atomicAdd(&ctl->walk_ns[1], globaltimer_ns() - t_start);
}

// Uplift and erosion (fastscape_RB.cpp:285-296, :306-328) level by level
// from base level, after k_order has placed the levels and the drainage
// counts (and uplifted the pits). A kernel of its own: the ordering and
// accumulation run with more resident threads than the register-hungry FP64
// erosion allows.
// VAR 0: subtractions of elevations on the FP64 pipe; 1: in integer
// arithmetic (n = 1, 2); 2: the reference's Newton loop literally, for every
// n (a test of the fast paths).
template <int NMODE, bool SINGLE, int VAR>
__global__ void __launch_bounds__(kWalkThreads, 2) k_erode(StepArgs a) {
  constexpr bool ISUB = VAR == 1, GENERIC = VAR == 2;
  extern __shared__ int smem[];
  const int nreal = a.nreal;
  int *s_lo = smem;
  int *s_hi = s_lo + nreal;
  int *s_nlev = s_hi + nreal;
  int *s_pre = s_nlev + nreal;
  __shared__ int s_maxlev;
  unsigned epoch = 0;
  Ctl *ctl = a.ctl;
  if (stopped(ctl)) return;
  RealDesc d0;
  if (SINGLE) d0 = a.desc[0];
  auto desc = [&](int r) -> const RealDesc & { return SINGLE ? d0 : a.desc[r]; };
  auto real_of = [&](int g) -> int { return SINGLE ? 0 : find_real(s_pre, nreal, g); };
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int offk0 = SINGLE ? nbr_off(lane & 7, d0.W) : 0;
  const int warp_global = tid >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool stamp = a.stamp && tid == 0;
  const unsigned long long t_start = stamp ? globaltimer_ns() : 0;
  if (threadIdx.x == 0) s_maxlev = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
    s_nlev[r] = __ldcg(&a.rctl[r].nlevels);
    atomicMax(&s_maxlev, s_nlev[r]);
  }
  __syncthreads();
  const int maxlev = s_maxlev;

  // Level Lv of every realization as [lo_of(r), hi_of(r)) (empty past its
  // depth), and the prefix of its 32-entry groups over the batch. A batch
  // of one copies its level table into shared memory once (one load per
  // entry and block) and takes each level's range from there into
  // registers: no block barrier, scan or global load per level.
  __shared__ int s_off[kLevelCache + 1];
  if (SINGLE) {
    const int n = min(maxlev, kLevelCache) + 1;
    for (int k = threadIdx.x; k < n; k += kWalkThreads) s_off[k] = __ldcg(&a.lvl_off[d0.lvl_base + k]);
    __syncthreads();
  }
  int lv_lo = 0, lv_hi = 0;
  auto lo_of = [&](int r) -> int { return SINGLE ? lv_lo : s_lo[r]; };
  auto hi_of = [&](int r) -> int { return SINGLE ? lv_hi : s_hi[r]; };
  auto pre_of = [&](int r) -> int { return SINGLE ? 0 : s_pre[r]; };
  auto level_groups = [&](int Lv) -> int {
    if (SINGLE) {
      if (Lv < kLevelCache) {
        lv_lo = s_off[Lv];
        lv_hi = s_off[Lv + 1];
      } else {  // deeper than the cache: one load per block
        __syncthreads();
        if (threadIdx.x == 0) {
          s_lo[0] = __ldcg(&a.lvl_off[d0.lvl_base + Lv]);
          s_hi[0] = __ldcg(&a.lvl_off[d0.lvl_base + Lv + 1]);
        }
        __syncthreads();
        lv_lo = s_lo[0];
        lv_hi = s_hi[0];
      }
      return (lv_hi - lv_lo + 31) >> 5;
    }
    __syncthreads();  // every warp is done with the previous ranges
    for (int r = threadIdx.x; r < nreal; r += kWalkThreads) {
      if (Lv < s_nlev[r]) {
        const int b = desc(r).lvl_base;
        s_lo[r] = __ldcg(&a.lvl_off[b + Lv]);
        s_hi[r] = __ldcg(&a.lvl_off[b + Lv + 1]);
      } else {
        s_lo[r] = s_hi[r] = 0;
      }
    }
    __syncthreads();
    return block_prefix(nreal, [&](int r) { return (s_hi[r] - s_lo[r] + 31) >> 5; }, s_pre);
  };

  // ---- uplift + erosion: fastscape_RB.cpp:285-296 and :306-328 in the
  // level order of fastscape_RB+P.cpp:319-350. Eroded cells are uplifted on
  // their first read (uplift of every interior cell precedes erosion in the
  // reference; a cell's h is read first by its own erosion, its receiver's
  // h is final).
  // A warp erodes one 32-entry group per iteration, in a software pipeline:
  // the entries (cell, receiver direction, drainage count) of the group two
  // iterations ahead and the elevations of the next group are loaded before
  // this group's erosion, so the chain entry -> elevation -> erosion of one
  // group overlaps the erosion of the groups before it. The next level's
  // ranges and first groups -- entries and the cells' own elevations, which
  // this level does not change -- are loaded before the level's barrier;
  // after it only the receivers' elevations remain to be gathered.
  int ngroups = 0;  // groups of the level being eroded
  struct Entry {
    int c, dir, r;
    uint32_t k;
    bool ok;
  };
  struct Heights {
    uint64_t hc, hn;  // bit patterns in integer registers (see fadd_bits)
  };
  auto load_entry = [&](int g) -> Entry {
    Entry e{0, 0, 0, 0u, false};
    if (g < ngroups) {
      const int r = real_of(g);
      const int i = lo_of(r) + 32 * (g - pre_of(r)) + lane;
      e.r = r;
      if (i < hi_of(r)) {
        const int off = desc(r).off;
        e.ok = true;
        e.c = __ldcg(&a.ent[off + i]);
        e.dir = __ldcg(&a.pdir[off + i]);
        e.k = __ldcg(&a.acc[off + i]);
      }
    }
    return e;
  };
  auto gather_hc = [&](const Entry &e) -> uint64_t {
    return e.ok ? __ldcg(reinterpret_cast<const unsigned long long *>(a.h + desc(e.r).off) + e.c)
                : 0ull;
  };
  auto gather_hn = [&](const Entry &e) -> uint64_t {
    // a group lies in one realization: lane k < 8 holds direction k's offset
    const int offk = SINGLE ? offk0 : nbr_off(lane & 7, desc(e.r).W);
    const int ro = __shfl_sync(kFull, offk, e.dir & 7);
    return e.ok ? __ldcg(reinterpret_cast<const unsigned long long *>(a.h + desc(e.r).off) +
                         e.c + ro)
                : 0ull;
  };
  const int gstride = nwarps;
  Entry e1{}, e2{};
  Heights h1{0, 0};
  bool ahead = false;  // e1, e2 and h1.hc already hold this level's first groups
  for (int Lv = 1; Lv < maxlev; ++Lv) {
    if (!ahead) {
      ngroups = level_groups(Lv);
      e1 = load_entry(warp_global);
      e2 = load_entry(warp_global + gstride);
      h1.hc = gather_hc(e1);
    }
    h1.hn = gather_hn(e1);
    for (int g = warp_global; g < ngroups; g += gstride) {
      const Entry e = e1;
      const Heights hg = h1;
      e1 = e2;
      e2 = load_entry(g + 2 * gstride);
      h1.hc = gather_hc(e1);
      h1.hn = gather_hn(e1);
      if (e.ok) {
        const RealDesc &d = desc(e.r);
        const size_t rec_at = (size_t)e.k * kTabStride + 4 * (e.dir & 1);
        const uint64_t udt = (uint64_t)__double_as_longlong(d.u_dt);
        const uint64_t h0 = uplift_bits(hg.hc, udt);
        uint64_t hnew;
        if (NMODE == kNOne && !GENERIC) {
          const unsigned long long *Tb = reinterpret_cast<const unsigned long long *>(d.tab) + rec_at;
          hnew = erode_cell_n1<ISUB>(d, ctl, Tb, load_tab_n1(Tb), h0, hg.hn);
        } else if (NMODE == kNTwo && !GENERIC) {
          hnew = erode_cell_n2<ISUB>(d, a.neq, ctl,
                                     __ldg(reinterpret_cast<const unsigned long long *>(d.tab) + rec_at),
                                     h0, hg.hn);
        } else {
          hnew = (uint64_t)__double_as_longlong(
              erode_cell<NMODE>(d, a.neq, ctl, d.tab + rec_at, __longlong_as_double(h0),
                                __longlong_as_double(hg.hn)));
        }
        if (((hnew >> 52) & 0x7FF) == 0x7FF)  // Inf or NaN
          raise_err(ctl, FS_ERR_NONFINITE, kPhaseErode);
        reinterpret_cast<unsigned long long *>(a.h + d.off)[e.c] = hnew;
      }
    }
    ahead = Lv + 1 < maxlev;
    if (ahead) {
      ngroups = level_groups(Lv + 1);  // reads only the finished level table
      e1 = load_entry(warp_global);
      e2 = load_entry(warp_global + gstride);
      h1.hc = gather_hc(e1);
    }
    if (Lv + 1 < maxlev && !grid_barrier(ctl, &ctl->bar2, epoch, a.timeout_ns)) return;  }
  if (stamp) atomicAdd(&ctl->walk_ns[2], globaltimer_ns() - t_start);
  if (tid == 0) atomicAdd(&ctl->steps_done, 1);
}

// ---------------------------------------------------------------------------
// Per-realization level walk for batches of many small realizations. The
// grid-wide walk above pays a grid barrier per level for the whole batch,
// and long runs grow hundreds of levels of a few thousand cells each; here
// one CTA walks one realization's levels with block barriers only (several
// realizations per SM), with the same arrays, the same per-cell arithmetic
// and the same level ids, counts and elevations bit for bit (the order of
// entries within a level may differ from the grid walk's, which its atomics
// leave free as well).
//   k_cta_order_accum: level ordering (fastscape_RB.cpp:213-254: level k+1 =
//     the donors of level k, each entry's donors contiguous in direction
//     order) and the accumulation back down the levels (fastscape_RB.cpp:
//     262-279, counts pushed into the receivers' positions); a count beyond
//     the realization's erosion table raises the batch-wide abort, so the
//     next kernel leaves every elevation unchanged and the timestep is redone.
//   k_cta_erode: uplift of the pits, then uplift + erosion level by level
//     (fastscape_RB.cpp:285-328 in the level order of fastscape_RB+P.cpp:
//     319-350), exactly as k_accum's tail and k_erode do.
// ---------------------------------------------------------------------------
constexpr int kCtaThreads = 256;       // ordering CTAs (32 registers: 8 per SM)
constexpr int kCtaErodeThreads = 128;  // erosion CTAs (at most 72 registers: 7 per SM)

__global__ void __launch_bounds__(kCtaThreads, 8) k_cta_order_accum(StepArgs a) {
  Ctl *ctl = a.ctl;
  if (stopped(ctl)) return;
  const int t = threadIdx.x;
  __shared__ int s_lvl[kLevelCache + 1];
  for (int r = blockIdx.x; r < a.nreal; r += gridDim.x) {
    const RealDesc d = a.desc[r];
    int32_t *ent = a.ent + d.off;
    uint8_t *pdir = a.pdir + d.off;
    uint32_t *acc = a.acc + d.off;
    int32_t *par = a.par + d.off;
    const uint8_t *mask = a.mask + d.off;
    int *lvl = a.lvl_off + d.lvl_base;
    int lo = 0, hi = d.nring + ld_volatile_i32(&a.rctl[r].top);
    if (t == 0) {
      lvl[0] = 0;
      lvl[1] = hi;
      s_lvl[0] = 0;
      s_lvl[1] = hi;
    }
    int nlev = 1;
    bool ovf = false;
    for (;;) {
      int next = hi;
      for (int cs = lo; cs < hi; cs += kCtaThreads) {
        const int i = cs + t;
        int cell = 0;
        unsigned m = 0;
        if (i < hi) {
          cell = __ldcg(&ent[i]);
          m = mask[cell];
          acc[i] = 1u;  // the cell itself; donors add theirs below
        }
        int total;
        const int excl = block_excl_scan(__popc(m), total, t, kCtaThreads);
        if (next + total > d.size) {  // block-uniform
          ovf = true;
          break;
        }
        int pos = next + excl;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          if (m >> k & 1u) {
            ent[pos] = cell + nbr_off(k, d.W);
            pdir[pos] = (uint8_t)((k + 4) & 7);
            par[pos] = i;  // the receiver's position
            ++pos;
          }
        }
        next += total;
      }
      __syncthreads();  // the next level's entries are written
      if (ovf || next == hi) break;
      lo = hi;
      hi = next;
      ++nlev;
      if (t == 0) {
        lvl[nlev] = hi;
        if (nlev <= kLevelCache) s_lvl[nlev] = hi;
      }
    }
    if (t == 0) {
      a.rctl[r].nlevels = nlev;
      a.rctl[r].total = hi;
      if (ovf) raise_err(ctl, FS_ERR_LEVEL_OVERFLOW, kPhaseOrder);
      else if (hi != d.size) raise_err(ctl, FS_ERR_ORDER, kPhaseOrder);  // a cycle
    }
    __syncthreads();
    if (ovf || hi != d.size) continue;
    for (int Lv = nlev - 1; Lv >= 1; --Lv) {
      const int l0 = Lv <= kLevelCache ? s_lvl[Lv] : __ldcg(&lvl[Lv]);
      const int l1 = Lv + 1 <= kLevelCache ? s_lvl[Lv + 1] : __ldcg(&lvl[Lv + 1]);
      // two entries per thread load before their pushes (which go one level
      // down, so they cannot change the counts read here)
      for (int i = l0 + t; i < l1; i += 2 * kCtaThreads) {
        const int i2 = i + kCtaThreads;
        const uint32_t v = __ldcg(&acc[i]);
        const int q = __ldcg(&par[i]);
        const uint32_t v2 = i2 < l1 ? __ldcg(&acc[i2]) : 0u;
        const int q2 = i2 < l1 ? __ldcg(&par[i2]) : 0;
        atomicAdd(&acc[q], v);
        if (i2 < l1) atomicAdd(&acc[q2], v2);
        const uint32_t vm = v > v2 ? v : v2;
        if (a.do_erode && vm >= (uint32_t)d.tab_cap) {
          if (atomicMax(&ctl->abort_k, (int)vm) < (int)vm) ctl->abort_r = r;
        }
      }
      __syncthreads();  // this level's counts are final before the next reads them
    }
  }
}

// The erosion walk keeps two entries per thread in flight (as k_erode does):
// the entry after next is loaded and the next one's own elevation gathered
// while a cell erodes; only the receiver's elevation waits for the level
// below, and the next level's first entries are loaded before the barrier
// (a cell's own elevation is written only in its own level). Its CTAs are
// small so that a batch's realizations walk at once (7 per SM, 1064 on 152
// SMs): the walk is bound by the latency of each level, hidden across
// realizations.
template <int NMODE, int VAR>
__global__ void __launch_bounds__(kCtaErodeThreads, 7) k_cta_erode(StepArgs a) {
  constexpr bool ISUB = VAR == 1, GENERIC = VAR == 2;
  Ctl *ctl = a.ctl;
  if (stopped(ctl)) return;  // an error, or a count beyond a table: nothing changes
  const int t = threadIdx.x;
  struct Entry {
    int c, dir;
    uint32_t k;
    bool ok;
  };
  for (int r = blockIdx.x; r < a.nreal; r += gridDim.x) {
    const RealDesc d = a.desc[r];
    const int nlev = __ldcg(&a.rctl[r].nlevels);
    const int *lvl = a.lvl_off + d.lvl_base;
    unsigned long long *hh = reinterpret_cast<unsigned long long *>(a.h + d.off);
    const int32_t *ent = a.ent + d.off;
    const uint8_t *pdir = a.pdir + d.off;
    const uint32_t *acc = a.acc + d.off;
    const uint64_t udt = (uint64_t)__double_as_longlong(d.u_dt);
    // the pits (level 0 after the rings) are uplifted, not eroded
    const int p1 = __ldcg(&lvl[1]);
    for (int i = d.nring + t; i < p1; i += kCtaErodeThreads) {
      const int c = __ldcg(&ent[i]);
      hh[c] = fadd_bits(__ldcg(&hh[c]), udt);
    }
    auto load_entry = [&](int i, int hi) -> Entry {
      Entry e{0, 0, 0u, false};
      if (i < hi) {
        e.ok = true;
        e.c = __ldcg(&ent[i]);
        e.dir = __ldcg(&pdir[i]);
        e.k = __ldcg(&acc[i]);
      }
      return e;
    };
    auto gather_hc = [&](const Entry &e) -> uint64_t { return e.ok ? __ldcg(&hh[e.c]) : 0ull; };
    auto gather_hn = [&](const Entry &e) -> uint64_t {
      return e.ok ? __ldcg(&hh[e.c + nbr_off(e.dir & 7, d.W)]) : 0ull;
    };
    int lo = p1, hi = nlev > 1 ? __ldcg(&lvl[2]) : p1;
    Entry e1 = load_entry(lo + t, hi), e2 = load_entry(lo + t + kCtaErodeThreads, hi);
    uint64_t hc1 = gather_hc(e1);
    __syncthreads();  // the pits are uplifted
    for (int Lv = 1; Lv < nlev; ++Lv) {
      uint64_t hn1 = gather_hn(e1);
      for (int i = lo + t; i < hi; i += kCtaErodeThreads) {
        const Entry e = e1;
        const uint64_t hc = hc1, hn = hn1;
        e1 = e2;
        e2 = load_entry(i + 2 * kCtaErodeThreads, hi);
        hc1 = gather_hc(e1);
        hn1 = gather_hn(e1);
        const uint64_t h0 = uplift_bits(hc, udt);
        const size_t rec_at = (size_t)e.k * kTabStride + 4 * (e.dir & 1);
        uint64_t hnew;
        if (NMODE == kNOne && !GENERIC) {
          const unsigned long long *Tb = reinterpret_cast<const unsigned long long *>(d.tab) + rec_at;
          hnew = erode_cell_n1<ISUB>(d, ctl, Tb, load_tab_n1(Tb), h0, hn);
        } else if (NMODE == kNTwo && !GENERIC) {
          hnew = erode_cell_n2<ISUB>(d, a.neq, ctl,
                                     __ldg(reinterpret_cast<const unsigned long long *>(d.tab) + rec_at),
                                     h0, hn);
        } else {
          hnew = (uint64_t)__double_as_longlong(erode_cell<NMODE>(
              d, a.neq, ctl, d.tab + rec_at, __longlong_as_double(h0), __longlong_as_double(hn)));
        }
        if (((hnew >> 52) & 0x7FF) == 0x7FF)  // Inf or NaN
          raise_err(ctl, FS_ERR_NONFINITE, kPhaseErode);
        hh[e.c] = hnew;
      }
      if (Lv + 1 < nlev) {  // the next level's first entries
        lo = hi;
        hi = __ldcg(&lvl[Lv + 2]);
        e1 = load_entry(lo + t, hi);
        e2 = load_entry(lo + t + kCtaErodeThreads, hi);
        hc1 = gather_hc(e1);
      }
      __syncthreads();  // this level's elevations are final before the next reads them
    }
  }
  if (blockIdx.x == 0 && t == 0) atomicAdd(&ctl->steps_done, 1);
}

__global__ void k_check_finite(const double *__restrict__ h, long long n, Ctl *ctl) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  bool bad = false;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    bad |= !isfinite(h[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) raise_err(ctl, FS_ERR_NONFINITE, kPhaseNone);
}

// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11), counter = cell index,
// key = seed. Two 32-bit outputs give one U[0,1) double with 53 random bits.
__device__ __forceinline__ void philox4x32_10(uint32_t ctr[4], uint32_t key[2]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t k0 = key[0], k1 = key[1];
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(M0, ctr[0]), lo0 = M0 * ctr[0];
    const uint32_t hi1 = __umulhi(M1, ctr[2]), lo1 = M1 * ctr[2];
    const uint32_t n0 = hi1 ^ ctr[1] ^ k0;
    const uint32_t n1 = lo1;
    const uint32_t n2 = hi0 ^ ctr[3] ^ k1;
    const uint32_t n3 = lo0;
    ctr[0] = n0; ctr[1] = n1; ctr[2] = n2; ctr[3] = n3;
    k0 += W0;
    k1 += W1;
  }
}

__global__ void k_philox_field(double *__restrict__ h, int W, int H, uint32_t key0,
                               uint32_t key1) {
  const long long size = (long long)W * H;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < size; c += stride) {
    uint32_t ctr[4] = {(uint32_t)c, (uint32_t)((unsigned long long)c >> 32), 0u, 0u};
    uint32_t key[2] = {key0, key1};
    philox4x32_10(ctr, key);
    const unsigned long long bits =
        ((unsigned long long)(ctr[0] >> 5) << 26) | (unsigned long long)(ctr[1] >> 6);
    double v = (double)bits * (1.0 / 9007199254740992.0);
    const int y = (int)(c / W);
    const int x = (int)(c - (long long)y * W);
    if (x <= 1 || y <= 1 || x >= W - 2 || y >= H - 2) v = 0.0;
    h[c] = v;
  }
}

// ent[0, nring) = the cells of rings 0 and 1 in ascending order: rows 0 and
// 1, then x = 0, 1, W-2, W-1 of rows 2..H-3, then rows H-2 and H-1.
__global__ void k_place_rings(int32_t *ent, int W, int H) {
  const int mid_rows = H > 4 ? H - 4 : 0;
  const int top = 2 * W;
  const int nring = W * H - (W > 4 ? W - 4 : 0) * mid_rows;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nring; i += gridDim.x * blockDim.x) {
    int c;
    if (H <= 4 || W <= 4) {
      c = i;  // no interior: every cell is a ring cell
    } else if (i < top) {
      c = i;
    } else if (i < top + 4 * mid_rows) {
      const int jj = i - top, row = 2 + jj / 4, q = jj % 4;
      const int x = q < 2 ? q : W - 4 + q;
      c = row * W + x;
    } else {
      c = (H - 2) * W + (i - top - 4 * mid_rows);
    }
    ent[i] = c;
  }
}

// A wait on a count that no block ever completes; the bounded wait must give
// up after timeout_ns and report FS_ERR_TIMEOUT. Used by the tests of the
// failure path only.
__global__ void k_test_wait(Ctl *ctl, unsigned long long timeout_ns) {
  if (threadIdx.x == 0) {
    const unsigned target = gridDim.x + 1;  // never reached
    atomicAdd(&ctl->bar, 1u);
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    while (ld_acquire_u32(&ctl->bar) < target) {
      if (ld_volatile_i32(&ctl->err) != 0) break;
      if ((++spins & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
        raise_err(ctl, FS_ERR_TIMEOUT, kPhaseTest);
        break;
      }
      __nanosleep(64);
    }
  }
}

// ---------------------------------------------------------------------------
// 5. The Braun-Willett order (fastscape_BW.cpp:201-221) of the last
// timestep's receiver forest, from the level-walk arrays: a depth-first
// preorder with roots (NO_FLOW cells) in ascending index and each cell's
// donors in ascending index. A cell's preorder position is its parent's
// position + 1 + the subtree sizes (drainage counts) of the siblings before
// it; a root's is the total subtree size of the roots before it. Computed
// level by level, top down, then scattered.
// ---------------------------------------------------------------------------

// cellacc[ent[i]] = acc[i] over one realization.
__global__ void k_scatter_counts(const int32_t *__restrict__ ent, const uint32_t *__restrict__ acc,
                                 int n, int32_t *__restrict__ cellacc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    cellacc[ent[i]] = (int32_t)acc[i];
}

// v[c] = subtree size of c if c is a root, else 0; then an exclusive scan in
// three launches (block sums, one block over the sums, block scans + offsets).
constexpr int kScanBlock = 1024;
__global__ void k_root_sizes_blocksum(const int8_t *__restrict__ rec,
                                      const int32_t *__restrict__ cellacc, int n,
                                      int32_t *__restrict__ v, int32_t *__restrict__ bsum) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int x = (i < n && rec[i] < 0) ? cellacc[i] : 0;
  if (i < n) v[i] = x;
  int total;
  block_excl_scan(x, total, threadIdx.x, kScanBlock);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t *bsum, int nb) {
  // one block: each thread scans a contiguous slice, then the slices
  const int per = (nb + kScanBlock - 1) / kScanBlock;
  const int b0 = threadIdx.x * per;
  int s = 0;
  for (int b = b0; b < b0 + per && b < nb; b++) s += bsum[b];
  int total;
  int run = block_excl_scan(s, total, threadIdx.x, kScanBlock);
  for (int b = b0; b < b0 + per && b < nb; b++) {
    const int x = bsum[b];
    bsum[b] = run;
    run += x;
  }
}

__global__ void k_scan_apply(int32_t *__restrict__ v, const int32_t *__restrict__ bsum, int n) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int x = i < n ? v[i] : 0;
  int total;
  const int e = block_excl_scan(x, total, threadIdx.x, kScanBlock);
  if (i < n) v[i] = bsum[blockIdx.x] + e;
}

// Level 0: dpos[i] = rootpos[ent[i]].
__global__ void k_dfs_level0(const int32_t *__restrict__ ent, const int32_t *__restrict__ rootpos,
                             int n0, int32_t *__restrict__ dpos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n0; i += gridDim.x * blockDim.x)
    dpos[i] = rootpos[ent[i]];
}

// Donors of the entries [b, e): positions after their parent in ascending
// cell-index order (the donor-list order of fastscape_BW.cpp:188-198).
// First and one-past-last donor position of every receiver, from the
// donors' receiver positions (a receiver's donors are contiguous, so they
// start where par changes): kid / kend for positions of levels >= 1.
__global__ void k_dfs_links(const int32_t *__restrict__ par, int b1, int n,
                            int32_t *__restrict__ kid, int32_t *__restrict__ kend) {
  for (int j = b1 + blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int p = par[j];
    if (j == b1 || par[j - 1] != p) kid[p] = j;
    if (j == n - 1 || par[j + 1] != p) kend[p] = j + 1;
  }
}

__global__ void k_dfs_level(const int32_t *__restrict__ kid, const int32_t *__restrict__ kend,
                            const uint8_t *__restrict__ pdir, const uint32_t *__restrict__ acc,
                            int b, int e, int W, int32_t *__restrict__ dpos) {
  for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
    const int k0 = kid[i], n = kend[i] - k0;
    if (n <= 0) continue;
    const int p = dpos[i];
    for (int q = 0; q < n; q++) {
      // the donor's offset from its receiver is minus its receiver offset
      const int oq = -nbr_off(pdir[k0 + q] & 7, W);
      int pos = p + 1;
      for (int s = 0; s < n; s++)
        if (-nbr_off(pdir[k0 + s] & 7, W) < oq) pos += (int)acc[k0 + s];
      dpos[k0 + q] = pos;
    }
  }
}

__global__ void k_dfs_scatter(const int32_t *__restrict__ ent, const int32_t *__restrict__ dpos,
                              int n, int32_t *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[dpos[i]] = ent[i];
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

size_t walk_smem_bytes(int nreal) { return sizeof(int) * (4 * (size_t)nreal + 1); }

int walk_threads() { return kWalkThreads; }

template <int NMODE, bool SINGLE>
const void *erode_ptr(int var) {
  if (var == 1) return reinterpret_cast<const void *>(&k_erode<NMODE, SINGLE, 1>);
  if (var == 2) return reinterpret_cast<const void *>(&k_erode<NMODE, SINGLE, 2>);
  return reinterpret_cast<const void *>(&k_erode<NMODE, SINGLE, 0>);
}

const void *walk_kernel_ptr(int nmode, bool single, int var) {
  if (nmode == kNGeneral) var = var == 2 ? 2 : 0;  // no integer variant
  if (single) {
    if (nmode == kNOne) return erode_ptr<kNOne, true>(var);
    if (nmode == kNTwo) return erode_ptr<kNTwo, true>(var);
    return erode_ptr<kNGeneral, true>(var);
  }
  if (nmode == kNOne) return erode_ptr<kNOne, false>(var);
  if (nmode == kNTwo) return erode_ptr<kNTwo, false>(var);
  return erode_ptr<kNGeneral, false>(var);
}

const void *order_kernel_ptr(bool single, int bps) {
  if (bps >= 3)
    return single ? reinterpret_cast<const void *>(&k_order<true, 3>)
                  : reinterpret_cast<const void *>(&k_order<false, 3>);
  return single ? reinterpret_cast<const void *>(&k_order<true, 2>)
                : reinterpret_cast<const void *>(&k_order<false, 2>);
}

const void *accum_kernel_ptr(bool single) {
  return single ? reinterpret_cast<const void *>(&k_accum<true>)
                : reinterpret_cast<const void *>(&k_accum<false>);
}

cudaError_t prepare_walk_kernels() {
  const int bytes = (int)walk_smem_bytes(kMaxReal);
  for (int single = 0; single < 2; single++) {
    for (int nm = 0; nm < 3; nm++) {
      for (int var = 0; var < 3; var++) {
        cudaError_t e = cudaFuncSetAttribute(walk_kernel_ptr(nm, single != 0, var),
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
      }
    }
    for (int bps = 2; bps <= 3; bps++) {
      cudaError_t e = cudaFuncSetAttribute(order_kernel_ptr(single != 0, bps),
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaFuncSetAttribute(accum_kernel_ptr(single != 0),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

double neg_recip_dr(double dr) {
  return dr >= 1.0 && dr <= 0x1p60 ? -(1.0 / dr) : 0.0;
}

float tol_lower_float(double tol) {
  const double t = tol * (1.0 - 0x1p-20);
  float f = (float)t;
  while ((double)f > t) f = nextafterf(f, 0.f);
  return f;
}

int ring_cells(int W, int H) {
  return W * H - (W > 4 ? W - 4 : 0) * (H > 4 ? H - 4 : 0);
}

int append_tiles(int kind, int r, int W, int H, Tile *out, int cap) {
  // receivers: interior x, y in [2, W-3]; donors: x, y in [1, W-2]
  // (donor tiles start at x = 0 and cover x in [0, W-2]; x = 0 is skipped)
  const int lo = kind == 0 ? 2 : 1;
  const int xlo = kind == 0 ? 2 : 0;
  const int iw = W - 2 * lo, ih = H - 2 * lo;
  if (iw <= 0 || ih <= 0) return 0;
  const int tx = kind == 0 ? kRxTile : kDxTile, ty = kind == 0 ? kRyTile : kDyTile;
  const int xw = W - lo - xlo;  // columns [xlo, W-1-lo]
  const int nx = (xw + tx - 1) / tx, ny = (ih + ty - 1) / ty;
  if ((long long)nx * ny > cap) return -1;
  int n = 0;
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) out[n++] = Tile{r, xlo + x * tx, lo + y * ty, 0};
  return n;
}

void fill_table_range(double keq, double neq, double meq, double dt, double dr_orth,
                      double dr_diag, double cell_area, long long k0, long long k1,
                      double *rec) {
  const double kd = keq * dt;
  const double pl[2] = {std::pow(dr_orth, neq), std::pow(dr_diag, neq)};
  for (long long k = k0; k < k1; k++) {
    const double A = static_cast<double>(k) * cell_area;
    const double pa = std::pow(A, meq);
    double *r = rec + (k - k0) * kTabStride;
    for (int cls = 0; cls < 2; cls++) {
      const double F = kd * pa / pl[cls];
      const double D = 1. + F;
      r[4 * cls + 0] = F;
      r[4 * cls + 1] = D;
      r[4 * cls + 2] = 1. / D;
      r[4 * cls + 3] = -(1. / D);
    }
  }
}

cudaError_t launch_receivers_exact(const StepArgs &a, cudaStream_t s) {
  if (a.nrtiles == 0) return cudaSuccess;
  k_receivers_exact<<<a.nrtiles, dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_receivers_fast(const StepArgs &a, cudaStream_t s, const CUtensorMap *hmap) {
  if (a.nrtiles == 0) return cudaSuccess;
  if (hmap) {
    k_receivers_filter<true><<<a.nrtiles, dim3(32, 8), 0, s>>>(*hmap, a);
  } else {
    CUtensorMap none;
    std::memset(&none, 0, sizeof(none));
    k_receivers_filter<false><<<a.nrtiles, dim3(32, 8), 0, s>>>(none, a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_receivers_fixup<<<8 * sm_count(), 256, 0, s>>>(a);
  return cudaGetLastError();
}

bool make_receiver_map(CUtensorMap *m, const double *h, int W, int H) {
  typedef CUresult (*Encode)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                             const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                             const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                             CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode enc = nullptr;
  if (!enc) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return false;
    enc = reinterpret_cast<Encode>(fn);
  }
  // row stride a multiple of 16 bytes; the tiles' boxes start at even x
  if (W % 2 || W < kRxTile + 4 || H < 5) return false;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(W), static_cast<cuuint64_t>(H)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(W) * 8};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kRtW), static_cast<cuuint32_t>(kRtH)};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<double *>(h), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_donors_level0(const StepArgs &a, cudaStream_t s) {
  if (a.ndtiles == 0) return cudaSuccess;
  k_donors_level0<<<a.ndtiles, dim3(32, 8), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_order(const StepArgs &a, int sms, int bps, cudaStream_t s) {
  StepArgs args = a;
  void *params[] = {&args};
  return cudaLaunchCooperativeKernel(order_kernel_ptr(a.nreal == 1, bps), dim3(sms * bps),
                                     dim3(kWalkThreads), params, walk_smem_bytes(a.nreal), s);
}

cudaError_t launch_erode(const StepArgs &a, int sms, int bps, cudaStream_t s) {
  StepArgs args = a;
  void *params[] = {&args};
  return cudaLaunchCooperativeKernel(walk_kernel_ptr(a.nmode, a.nreal == 1,
                                                     a.erode_generic ? 2 : a.erode_isub ? 1 : 0),
                                     dim3(sms * bps),
                                     dim3(kWalkThreads), params, walk_smem_bytes(a.nreal), s);
}

cudaError_t launch_accum(const StepArgs &a, int sms, int bps, cudaStream_t s) {
  StepArgs args = a;
  void *params[] = {&args};
  return cudaLaunchCooperativeKernel(accum_kernel_ptr(a.nreal == 1), dim3(sms * bps),
                                     dim3(kWalkThreads), params, walk_smem_bytes(a.nreal), s);
}

const void *cta_erode_ptr(int nmode, int var) {
  switch (nmode) {
    case kNOne:
      return var == 2 ? reinterpret_cast<const void *>(&k_cta_erode<kNOne, 2>)
             : var == 1 ? reinterpret_cast<const void *>(&k_cta_erode<kNOne, 1>)
                        : reinterpret_cast<const void *>(&k_cta_erode<kNOne, 0>);
    case kNTwo:
      return var == 2 ? reinterpret_cast<const void *>(&k_cta_erode<kNTwo, 2>)
             : var == 1 ? reinterpret_cast<const void *>(&k_cta_erode<kNTwo, 1>)
                        : reinterpret_cast<const void *>(&k_cta_erode<kNTwo, 0>);
    default:
      return reinterpret_cast<const void *>(&k_cta_erode<kNGeneral, 2>);
  }
}

int cta_threads(bool erode) { return erode ? kCtaErodeThreads : kCtaThreads; }

const void *cta_order_ptr() { return reinterpret_cast<const void *>(&k_cta_order_accum); }

cudaError_t launch_cta_order(const StepArgs &a, int blocks, cudaStream_t s) {
  k_cta_order_accum<<<blocks, kCtaThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cta_erode(const StepArgs &a, int blocks, cudaStream_t s) {
  StepArgs args = a;
  void *params[] = {&args};
  const int var = a.erode_generic ? 2 : a.erode_isub ? 1 : 0;
  return cudaLaunchKernel(cta_erode_ptr(a.nmode, var), dim3(blocks), dim3(kCtaErodeThreads), params, 0,
                          s);
}

cudaError_t launch_walk(const StepArgs &a, int sms, int order_bps, int accum_bps,
                        int erode_bps, cudaStream_t s) {
  cudaError_t e = launch_order(a, sms, order_bps, s);
  if (e == cudaSuccess) e = launch_accum(a, sms, accum_bps, s);
  if (e != cudaSuccess || !a.do_erode) return e;
  return launch_erode(a, sms, erode_bps, s);
}

cudaError_t launch_check_finite(const double *h, long long n, Ctl *ctl, cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  k_check_finite<<<(int)blocks, 256, 0, s>>>(h, n, ctl);
  return cudaGetLastError();
}

cudaError_t launch_philox_field(double *h, int W, int H, uint64_t seed, cudaStream_t s) {
  long long blocks = ((long long)W * H + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  if (blocks < 1) blocks = 1;
  k_philox_field<<<(int)blocks, 256, 0, s>>>(h, W, H, (uint32_t)seed, (uint32_t)(seed >> 32));
  return cudaGetLastError();
}

cudaError_t launch_place_rings(int32_t *ent, int W, int H, cudaStream_t s) {
  k_place_rings<<<64, 256, 0, s>>>(ent, W, H);
  return cudaGetLastError();
}

cudaError_t launch_test_wait(Ctl *ctl, int blocks, unsigned long long timeout_ns,
                             cudaStream_t s) {
  k_test_wait<<<blocks, 32, 0, s>>>(ctl, timeout_ns);
  return cudaGetLastError();
}

size_t dfs_scratch_ints(int size) {
  return 5 * (size_t)size + (size_t)(size + kScanBlock - 1) / kScanBlock + 1;
}

cudaError_t launch_dfs_order(const DfsArgs &d, const int32_t *lvl_host, int nlev,
                             int32_t *scratch, int32_t *out, cudaStream_t s) {
  const int n = d.size;
  int32_t *cellacc = scratch, *v = scratch + n, *dpos = scratch + 2 * (size_t)n;
  int32_t *kid = scratch + 3 * (size_t)n, *kend = scratch + 4 * (size_t)n;
  int32_t *bsum = scratch + 5 * (size_t)n;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  const int g = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  cudaError_t e = cudaMemsetAsync(kid, 0, 2 * (size_t)n * sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  if (nlev > 1 && lvl_host[1] < n) k_dfs_links<<<g, 256, 0, s>>>(d.par, lvl_host[1], n, kid, kend);
  k_scatter_counts<<<g, 256, 0, s>>>(d.ent, d.acc, n, cellacc);
  k_root_sizes_blocksum<<<nb, kScanBlock, 0, s>>>(d.rec, cellacc, n, v, bsum);
  k_scan_sums<<<1, kScanBlock, 0, s>>>(bsum, nb);
  k_scan_apply<<<nb, kScanBlock, 0, s>>>(v, bsum, n);
  k_dfs_level0<<<g, 256, 0, s>>>(d.ent, v, lvl_host[1], dpos);
  for (int L = 0; L + 1 < nlev; L++) {
    const int b = lvl_host[L], e2 = lvl_host[L + 1];
    const int gl = (e2 - b + 255) / 256 < 4096 ? (e2 - b + 255) / 256 : 4096;
    if (gl > 0) k_dfs_level<<<gl, 256, 0, s>>>(kid, kend, d.pdir, d.acc, b, e2, d.W, dpos);
  }
  k_dfs_scatter<<<g, 256, 0, s>>>(d.ent, dpos, n, out);
  return cudaGetLastError();
}

}  // namespace fs
