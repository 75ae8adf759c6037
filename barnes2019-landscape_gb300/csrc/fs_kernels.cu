// fs_kernels.cu -- sm_103a kernels of the FastScape timestep.
//
// One timestep = four launches on the model's stream:
//   1. k_receivers_filter  D8 steepest descent over the interior
//      + k_receivers_fixup (fastscape_RB.cpp:160-182): FP32 proof of the
//                          receiver, FP64 reference formula for the cells
//                          the proof cannot settle
//   2. k_donors_level0     donor masks (pull form of fastscape_RB.cpp:188-203)
//                          and the level-0 frontier (fastscape_RB.cpp:221-227)
//   3. k_walk              persistent cooperative kernel: level-by-level
//                          ordering (:229-251), flow accumulation back down
//                          the levels (:262-279), uplift (:285-296) and the
//                          implicit erosion solved upward from base level
//                          (:306-328, in the level order of
//                          fastscape_RB+P.cpp:319-350).
//
// Floating point follows the reference's operation order exactly; the whole
// file is compiled with -fmad=false so no multiply-add is contracted, and
// every FP64 division is correctly rounded.
#include <cuda_runtime.h>

#include <cstdint>

#include "fastscape_gb300.h"
#include "fs_internal.h"

namespace fs {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWalkThreads = 512;
constexpr int kPer = 8;  // frontier cells per thread per expansion chunk
constexpr int kAccU = 4;  // 32-entry groups per warp per accumulation pass
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

// Grid-wide barrier for a cooperative launch. Arrival counter only grows
// during a launch (reset by the host before it), so barrier number `epoch`
// completes when bar reaches epoch*gridDim.x. Every wait is bounded by
// `timeout_ns` of wall time; on timeout, or when another block has already
// raised an error, it returns false and the caller leaves the kernel.
__device__ bool grid_barrier(Ctl *ctl, unsigned &epoch,
                             unsigned long long timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ++epoch;
    const unsigned target = epoch * gridDim.x;
    __threadfence();
    atomicAdd(&ctl->bar, 1u);
    int ok = 1;
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    while (ld_acquire_u32(&ctl->bar) < target) {
      if (ld_volatile_i32(&ctl->err) != 0) { ok = 0; break; }
      if ((++spins & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
        raise_err(ctl, FS_ERR_TIMEOUT, kPhaseBarrier);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ void nshift8(int W, int o[8]) {
  o[0] = -1; o[1] = -W - 1; o[2] = -W; o[3] = -W + 1;
  o[4] = 1;  o[5] = W + 1;  o[6] = W;  o[7] = W - 1;
}

// nshift[k] (fastscape_RB.cpp:137) for a run-time k without a local array:
// dx+1 and dy+1 of the 8 directions packed two bits per direction.
__device__ __forceinline__ int nbr_off(int k, int W) {
  const int dx = ((0x1A90 >> (2 * k)) & 3) - 1;
  const int dy = ((0xA901 >> (2 * k)) & 3) - 1;
  return dy * W + dx;
}

// ---------------------------------------------------------------------------
// 1. Receivers: fastscape_RB.cpp:160-182. slope = (h[c]-h[n])/dr[n], strict
// '>' against a running maximum that starts at 0, so the first maximum in
// neighbour order wins and a cell with no strictly lower neighbour keeps
// NO_FLOW.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_receivers(const double *__restrict__ h, int8_t *__restrict__ rec, int W,
            int H, double dr_orth, double dr_diag, const Ctl *ctl) {
  if (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (x >= W - 2 || y >= H - 2) return;
  const long long c = (long long)y * W + x;
  int o[8];
  nshift8(W, o);
  const double hc = h[c];
  double max_slope = 0;
  int max_n = FS_NO_FLOW;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const double slope = (hc - h[c + o[n]]) / ((n & 1) ? dr_diag : dr_orth);
    if (slope > max_slope) {
      max_slope = slope;
      max_n = n;
    }
  }
  rec[c] = (int8_t)(max_n == FS_NO_FLOW ? kPit : max_n);
}

// ---------------------------------------------------------------------------
// 1b. Receivers, fast path. GB300 runs FP64 at ~1.6 lanes/clock/SM against
// ~113 for FP32, so the eight FP64 divides per cell of the reference formula
// would dominate the timestep. This kernel decides the receiver from FP32
// approximations with a rigorous error bound and hands the rare cells it
// cannot prove to k_receivers_fixup, which evaluates the reference formula in
// FP64. The result is identical to k_receivers for every input.
//
// Bound: f = h truncated to FP32 (|f-h| <= 2^-23|h| + 2^-126),
// a_n = fl(fl(f_c - f_n) * g_n) with g_n = fl(1/dr_n); then for the exact
// reference slope q_n = RN(RN(h_c-h_n)/dr_n):
//   |a_n - q_n| <= 2^-20 * gmax * (M + 2^-100) =: E/2,
// M = max |f| over the 3x3 window, gmax = max g_n. So
//   best - second > 2E  and best > E  => q_best is the unique maximum > 0;
//   best < -E                         => every q_n < 0 (NO_FLOW);
// otherwise (near-ties, zero slopes, NaN, |h| >= 2^128) the cell is queued.
// ---------------------------------------------------------------------------
constexpr int kRxTile = 32;  // interior cells per tile in x
constexpr int kRyTile = 32;  // interior cells per tile in y

// Truncation of a double to FP32 with integer operations only (no FP64
// pipe): rebias the exponent, keep the top 23 fraction bits. Values below
// 2^-126 flush to signed zero; |x| >= 2^128, Inf and NaN give NaN, which
// sends the cell to the exact path.
__device__ __forceinline__ float trunc_to_float(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  const unsigned frac = (unsigned)(b >> 29) & 0x7FFFFFu;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(0x7FC00000u);
  return __uint_as_float(sign | ((unsigned)e << 23) | frac);
}

__global__ void __launch_bounds__(256)
k_receivers_filter(const double *__restrict__ h, int8_t *__restrict__ rec,
                   int32_t *__restrict__ amb, Ctl *ctl, int W, int H,
                   float g_orth, float g_diag, float gmax) {
  if (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) return;
  __shared__ float s[kRyTile + 2][kRxTile + 3];
  const int x0 = blockIdx.x * kRxTile + 1;  // grid x of s[.][0]
  const int y0 = blockIdx.y * kRyTile + 1;  // grid y of s[0][.]
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int idx = t; idx < (kRyTile + 2) * (kRxTile + 2); idx += 256) {
    const int ly = idx / (kRxTile + 2);
    const int lx = idx - ly * (kRxTile + 2);
    const int gx = x0 + lx, gy = y0 + ly;
    float v = 0.f;
    if (gx < W && gy < H) v = trunc_to_float(h[(size_t)gy * W + gx]);
    s[ly][lx] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x;
  const int lx = threadIdx.x + 1;
  const int gx = x0 + lx;
#pragma unroll 1
  for (int r = 0; r < kRyTile / 8; r++) {
    const int ly = threadIdx.y + 8 * r + 1;
    const int gy = y0 + ly;
    const bool valid = gx < W - 2 && gy < H - 2;
    bool queue = false;
    if (valid) {
      const float fc = s[ly][lx];
      const float f[8] = {s[ly][lx - 1], s[ly - 1][lx - 1], s[ly - 1][lx],
                          s[ly - 1][lx + 1], s[ly][lx + 1], s[ly + 1][lx + 1],
                          s[ly + 1][lx], s[ly + 1][lx - 1]};
      float best = -INFINITY, second = -INFINITY;
      int bn = 0;
      float M = fabsf(fc);
      bool bad = !(fc == fc);
#pragma unroll
      for (int n = 0; n < 8; n++) {
        const float a = (fc - f[n]) * ((n & 1) ? g_diag : g_orth);
        M = fmaxf(M, fabsf(f[n]));
        bad |= !(a == a);
        if (a > best) {
          second = best;
          best = a;
          bn = n;
        } else if (a > second) {
          second = a;
        }
      }
      const float E = 0x1p-19f * gmax * (M + 0x1p-100f);
      int code = 0;
      queue = true;
      if (!bad) {
        if (best - second > 2.f * E && best > E) {
          code = bn;
          queue = false;
        } else if (best < -E) {
          code = kPit;
          queue = false;
        }
      }
      if (!queue) rec[(size_t)gy * W + gx] = (int8_t)code;
    }
    const unsigned bq = __ballot_sync(kFull, queue);
    if (bq) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&ctl->amb, __popc(bq));
      base = __shfl_sync(kFull, base, 0);
      if (queue) amb[base + __popc(bq & ((1u << lane) - 1u))] = gy * W + gx;
    }
  }
}

// The queued cells of k_receivers_filter, with the reference formula in FP64.
__global__ void __launch_bounds__(256)
k_receivers_fixup(const double *__restrict__ h, int8_t *__restrict__ rec,
                  const int32_t *__restrict__ amb, const Ctl *ctl, int W,
                  double dr_orth, double dr_diag) {
  if (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) return;
  const int n_amb = ld_volatile_i32(&ctl->amb);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_amb; i += gridDim.x * blockDim.x) {
    const int c = amb[i];
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
    rec[c] = (int8_t)(max_n == FS_NO_FLOW ? kPit : max_n);
  }
}

// ---------------------------------------------------------------------------
// 2. Donor masks + level 0.
// Bit k of mask[c] is set when neighbour c+nshift[k] has receiver code
// (k+4)%8, i.e. drains into c (the pull form of fastscape_RB+GPU.cpp:155-182).
// Level 0 = every cell without a receiver (fastscape_RB.cpp:221-227): the
// two outer rings, which never change and sit at stack[0, nring) from model
// creation on, and the interior pits, appended here with one atomic per
// 32x64 tile (block scan of the per-thread pit counts).
// ---------------------------------------------------------------------------
constexpr int kDxTile = 32;  // tile of cells over [1, W-2] x [1, H-2]
constexpr int kDyTile = 64;
constexpr int kDRows = kDyTile / 8;

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
    const int t = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) s_w[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? s_w[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(kFull, w, d);
      if (lane >= d) w += t;
    }
    if (lane < nw) s_w[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  total = s_w[nw - 1];
  const int before = wid ? s_w[wid - 1] : 0;
  __syncthreads();  // s_w may be reused by the caller's next scan
  return before + incl - v;
}

__global__ void __launch_bounds__(256)
k_donors_level0(const int8_t *__restrict__ rec, uint8_t *__restrict__ mask,
                int32_t *__restrict__ ent, Ctl *ctl, int W, int H, int nring) {
  if (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) return;
  __shared__ int8_t sr[kDyTile + 2][kDxTile + 4];
  __shared__ int s_base;
  const int x0 = blockIdx.x * kDxTile;  // grid x of sr[.][0]
  const int y0 = blockIdx.y * kDyTile;  // grid y of sr[0][.]
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int ly = threadIdx.y; ly < kDyTile + 2; ly += 8) {
    const int gy = y0 + ly;
    for (int lx = threadIdx.x; lx < kDxTile + 2; lx += 32) {
      const int gx = x0 + lx;
      sr[ly][lx] = (gx < W && gy < H) ? rec[(size_t)gy * W + gx] : (int8_t)FS_NO_FLOW;
    }
  }
  __syncthreads();
  const int lx = threadIdx.x + 1;
  const int gx = x0 + lx;
  unsigned pit_bits = 0;
#pragma unroll
  for (int r = 0; r < kDRows; r++) {
    const int ly = threadIdx.y + 8 * r + 1;
    const int gy = y0 + ly;
    if (gx <= W - 2 && gy <= H - 2) {
      unsigned m = 0;
      m |= (sr[ly][lx - 1] == 4) ? 1u : 0u;         // W  neighbour drains E
      m |= (sr[ly - 1][lx - 1] == 5) ? 2u : 0u;     // NW drains SE
      m |= (sr[ly - 1][lx] == 6) ? 4u : 0u;         // N  drains S
      m |= (sr[ly - 1][lx + 1] == 7) ? 8u : 0u;     // NE drains SW
      m |= (sr[ly][lx + 1] == 0) ? 16u : 0u;        // E  drains W
      m |= (sr[ly + 1][lx + 1] == 1) ? 32u : 0u;    // SE drains NW
      m |= (sr[ly + 1][lx] == 2) ? 64u : 0u;        // S  drains N
      m |= (sr[ly + 1][lx - 1] == 3) ? 128u : 0u;   // SW drains NE
      mask[(size_t)gy * W + gx] = (uint8_t)m;
      if (sr[ly][lx] == kPit) pit_bits |= 1u << r;
    }
  }
  int total;
  const int excl = block_excl_scan(__popc(pit_bits), total, t, 256);
  if (total == 0) return;
  if (t == 0) s_base = nring + atomicAdd(&ctl->top, total);
  __syncthreads();
  int pos = s_base + excl;
#pragma unroll
  for (int r = 0; r < kDRows; r++)
    if (pit_bits >> r & 1u) ent[pos++] = (y0 + threadIdx.y + 8 * r + 1) * W + gx;
}

__device__ __forceinline__ long long abs_bits(double x) {
  return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll;
}

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

// Erosion of one cell: fastscape_RB.cpp:315-326 with h0 the uplifted
// elevation, hn the receiver's final elevation and T the table record of the
// cell's drainage count and direction class (T[0] = fact).
template <int NMODE>
__device__ __forceinline__ double erode_cell(const WalkArgs &a, const double *T,
                                             double h0, double hn) {
  const double fact = T[0];
  double hnew, hp, diff;
  int it;
  if (NMODE == kNOne) {
    // First iterate: hnew - h0 = +0, pow(x,1) = x and pow(x,0) = 1, so
    // hnew = RN(h0 - RN(RN(fact*RN(h0-hn)) / D)) with D = RN(1+fact).
    const double D = T[1], R = T[2];
    const double num = fact * (h0 - hn);
    const double q = div_rn(num, D, R);
    hnew = h0 - q;
    // The loop stops after this iterate iff |RN(hnew - h0)| <= tol. Since
    // |RN(hnew-h0)| <= |q| + 2^-51(|h0|+|q|), an FP32 test on truncated
    // magnitudes with 2^-21 of slack proves it for almost every cell without
    // spending the FP64 subtraction (see the bound in fs_kernels.cu's
    // header); the rest evaluate diff exactly and follow the reference loop.
    const float qf = fabsf(trunc_to_float(q));
    const float hf = fabsf(trunc_to_float(h0));
    if (qf * (1.f + 0x1p-21f) + hf * 0x1p-48f <= a.tol_lo_f) return hnew;
    diff = hnew - h0;
    hp = hnew;
    it = 1;
    // fabs(diff) > tol as an integer compare of the magnitudes' bits (both
    // non-negative; a NaN diff stops the loop, as fabs(NaN) > tol is false)
    while (abs_bits(diff) > a.tol_bits && abs_bits(diff) <= 0x7FF0000000000000ll) {
      const double num2 = (hnew - h0) + fact * (hnew - hn);
      hnew -= div_rn(num2, D, R);
      diff = hnew - hp;
      hp = hnew;
      if (++it >= kNewtonMaxIt) {
        raise_err(a.ctl, FS_ERR_NEWTON, kPhaseErode);
        break;
      }
    }
    return hnew;
  }
  hnew = h0;
  hp = h0;
  diff = 2 * a.tol;
  it = 0;
  while (fabs(diff) > a.tol) {
    double pn, pn1;
    powers<NMODE>(hnew - hn, a.neq, pn, pn1);
    hnew -= (hnew - h0 + fact * pn) / (1. + fact * a.neq * pn1);
    diff = hnew - hp;
    hp = hnew;
    if (++it >= kNewtonMaxIt) {
      raise_err(a.ctl, FS_ERR_NEWTON, kPhaseErode);
      break;
    }
  }
  return hnew;
}

// Uplift of the interior level-0 cells (pits), fastscape_RB.cpp:291-295.
__device__ __forceinline__ void uplift_pits(const WalkArgs &a, int lvl0_end, int tid,
                                            int nthreads) {
  for (int i = a.nring + tid; i < lvl0_end; i += nthreads) {
    const int c = __ldcg(&a.ent[i]);
    a.h[c] = __ldcg(&a.h[c]) + a.u_dt;
  }
}

// ---------------------------------------------------------------------------
// 3. Persistent level walker (cooperative launch, one grid barrier per level
// per sweep).
//
// The ordering is kept as arrays indexed by position in the level order
// ("stack" in the reference): ent[i] the cell, pdir[i] its receiver
// direction (bit 3: the receiver is a pit), nd[i] and kid[i] the number of
// donors and the position of the first one in the next level (the donors of
// one entry are contiguous), acc[i] the drainage count. Accumulation and
// erosion then read these by position -- coalesced -- instead of gathering
// receivers, masks and counts by cell index.
// ---------------------------------------------------------------------------
template <int NMODE>
__global__ void __launch_bounds__(kWalkThreads)
k_walk(WalkArgs a) {
  unsigned epoch = 0;
  Ctl *ctl = a.ctl;
  if (ld_volatile_i32(&ctl->err) | ld_volatile_i32(&ctl->abort_k)) return;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
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
  // Level k+1 = the donors of level k. Each block expands chunks of
  // kPer*blockDim.x consecutive frontier entries (kPer consecutive per
  // thread, so the next level keeps the frontier's spatial order) with one
  // block scan and one atomic per chunk. The append counter rotates over
  // three words so a block that reads the size of level k after the barrier
  // never races with the reset for level k+2.
  int lo = 0;
  int hi = a.nring + ld_volatile_i32(&ctl->top);
  const int lvl0_end = hi;
  if (tid == 0) {
    a.lvl_off[0] = 0;
    a.lvl_off[1] = hi;
  }
  int nlev = 1;
  __shared__ int s_base;
  for (;;) {
    const int j = (nlev - 1) % 3;  // counter of this expansion
    if (tid == 0) ctl->lvlcnt[nlev % 3] = 0;  // counter of the next one
    // A block expands a chunk of kPer*blockDim.x consecutive entries; warp w
    // covers 32*kPer of them in kPer coalesced passes (entry wbase+32q+lane).
    // Warp scans give each entry's first-donor offset in entry order, one
    // block scan over the warps and one atomic place the chunk, and the
    // donors are written cooperatively (lane r writes the r-th donor of the
    // pass), so every store of the expansion is coalesced and the next level
    // keeps this level's order.
    const int chunk = kPer * kWalkThreads;
    const int wid = threadIdx.x >> 5;
    for (int base = lo + blockIdx.x * chunk; base < hi; base += gridDim.x * chunk) {
      const int wbase = base + wid * (32 * kPer);
      int cs[kPer];
      unsigned ms[kPer];
      int incl[kPer];
#pragma unroll
      for (int q = 0; q < kPer; q++) {
        const int i = wbase + 32 * q + lane;
        cs[q] = 0;
        ms[q] = 0;
        if (i < hi) {
          cs[q] = __ldcg(&a.ent[i]);
          ms[q] = a.mask[cs[q]];
        }
      }
      int wtot = 0;
#pragma unroll
      for (int q = 0; q < kPer; q++) {
        int v = __popc(ms[q]);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int t = __shfl_up_sync(kFull, v, d);
          if (lane >= d) v += t;
        }
        incl[q] = wtot + v;  // inclusive, relative to the warp's first donor
        wtot += __shfl_sync(kFull, v, 31);
      }
      int total;
      const int wexcl = block_excl_scan(lane == 0 ? wtot : 0, total, threadIdx.x, kWalkThreads);
      const int wstart = __shfl_sync(kFull, wexcl, 0);
      if (threadIdx.x == 0) s_base = total ? atomicAdd(&ctl->lvlcnt[j], total) : 0;
      __syncthreads();
      const int cbase = hi + s_base + wstart;  // position of the warp's first donor
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kPer; q++) {
        const int i = wbase + 32 * q + lane;
        const int nd = __popc(ms[q]);
        if (i < hi) {
          a.kid[i] = cbase + incl[q] - nd;
          a.nd[i] = (uint8_t)nd;
        }
        const int q_lo = __shfl_sync(kFull, incl[q] - nd, 0);
        const int q_hi = __shfl_sync(kFull, incl[q], 31);
        for (int r0 = q_lo; r0 < q_hi; r0 += 32) {
          const int r = r0 + lane;
          // owner = number of lanes whose inclusive count is <= r
          int o = 0;
#pragma unroll
          for (int step = 16; step >= 1; step >>= 1) {
            const int v = __shfl_sync(kFull, incl[q], o + step - 1);
            if (v <= r) o += step;
          }
          const int oc = __shfl_sync(kFull, cs[q], o);
          unsigned om = __shfl_sync(kFull, ms[q], o);
          const int ofirst = __shfl_sync(kFull, incl[q] - __popc(ms[q]), o);
          if (r < q_hi) {
            for (int skip = r - ofirst; skip > 0; --skip) om &= om - 1;
            const int k = __ffs(om) - 1;
            // level-1 entries remember whether their receiver is a pit
            // (a level-0 entry past the rings)
            const unsigned pit = (nlev == 1 && wbase + 32 * q + o >= a.nring) ? 8u : 0u;
            const int pos = cbase + r;
            if (pos < a.size) {
              a.ent[pos] = oc + nbr_off(k, a.W);
              a.pdir[pos] = (uint8_t)(((k + 4) & 7) | pit);
            } else {
              raise_err(ctl, FS_ERR_LEVEL_OVERFLOW, kPhaseOrder);
            }
          }
        }
      }
    }
    if (!grid_barrier(ctl, epoch, a.timeout_ns)) return;
    const int added = ld_volatile_i32(&ctl->lvlcnt[j]);
    if (added == 0) break;
    lo = hi;
    hi = hi + added;
    ++nlev;
    if (hi > a.size) {
      if (tid == 0) raise_err(ctl, FS_ERR_LEVEL_OVERFLOW, kPhaseOrder);
      return;
    }
    if (tid == 0) a.lvl_off[nlev] = hi;
  }
  if (tid == 0) {
    ctl->nlevels = nlev;
    ctl->total = hi;
  }
  if (hi != a.size) {
    // Some cells never reached base level: the receivers contain a cycle.
    if (tid == 0) raise_err(ctl, FS_ERR_ORDER, kPhaseOrder);
    return;
  }
  lap(0);

  // ---- accumulation: fastscape_RB.cpp:262-279, pulled level by level ----
  // acc[i] = 1 + sum of the donors' counts, read from the contiguous run
  // [kid[i], kid[i] + nd[i]) of the next level; the reference's accum is
  // acc*cell_area (exact: integer multiples of cell_area). A count at level
  // >= 1 beyond the erosion table stops the timestep before any elevation
  // changes; the host grows the table and repeats it.
  for (int L = nlev - 1; L >= 0; --L) {
    if (L == 0 && ld_volatile_i32(&ctl->abort_k) != 0) return;
    const int b = __ldcg(&a.lvl_off[L]);
    const int e = __ldcg(&a.lvl_off[L + 1]);
    // Warp-cooperative: a warp takes kAccU groups of 32 consecutive entries
    // (each group lies inside one expansion chunk, so its donors form one
    // contiguous run starting at kid of its first entry), loads the runs
    // coalesced -- all groups' first 32 donors in flight together -- and
    // each lane sums its own donors out of the run with shuffles.
    for (int g0 = b + (tid & ~31); g0 < e; g0 += kAccU * nthreads) {
      int n[kAccU], incl[kAccU], run[kAccU], tot[kAccU];
      uint32_t v0[kAccU];
#pragma unroll
      for (int u = 0; u < kAccU; u++) {
        const int i = g0 + u * nthreads + lane;
        int k = 0;
        n[u] = 0;
        if (i < e) {
          n[u] = __ldcg(&a.nd[i]);
          k = __ldcg(&a.kid[i]);
        }
        int v = n[u];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int t = __shfl_up_sync(kFull, v, d);
          if (lane >= d) v += t;
        }
        incl[u] = v;
        tot[u] = __shfl_sync(kFull, v, 31);
        run[u] = __shfl_sync(kFull, k, 0);
      }
#pragma unroll
      for (int u = 0; u < kAccU; u++)
        v0[u] = lane < tot[u] ? __ldcg(&a.acc[run[u] + lane]) : 0u;
#pragma unroll
      for (int u = 0; u < kAccU; u++) {
        const int first = incl[u] - n[u];
        uint32_t s = 1;
        for (int r0 = 0; r0 < tot[u]; r0 += 32) {
          uint32_t v = v0[u];
          if (r0 > 0) v = r0 + lane < tot[u] ? __ldcg(&a.acc[run[u] + r0 + lane]) : 0u;
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const int r = first + q - r0;
            const uint32_t x = __shfl_sync(kFull, v, r & 31);
            if (q < n[u] && r >= 0 && r < 32) s += x;
          }
        }
        const int i = g0 + u * nthreads + lane;
        if (i < e) {
          a.acc[i] = s;
          if (a.do_erode && L > 0 && s >= (uint32_t)a.tab_cap) atomicMax(&ctl->abort_k, (int)s);
        }
      }
    }
    if (L > 0 && !grid_barrier(ctl, epoch, a.timeout_ns)) return;
  }
  lap(1);
  if (!a.do_erode) return;

  // ---- uplift + erosion: fastscape_RB.cpp:285-296 and :306-328 in the
  // level order of fastscape_RB+P.cpp:319-350. Eroded cells are uplifted on
  // their first read; level-1 cells add the uplift of a pit receiver on
  // read, and the pits themselves are uplifted once no level-1 cell can read
  // them any more (during level 2, or after a barrier when level 1 is the
  // last). No barrier is needed before level 1: it reads counts complete
  // since the barrier after accumulation level 1 and never-written h.
  // Two entries per thread per pass, their loads issued together.
  for (int L = 1; L < nlev; ++L) {
    const int b = __ldcg(&a.lvl_off[L]);
    const int e = __ldcg(&a.lvl_off[L + 1]);
    for (int i = b + tid; i < e; i += 2 * nthreads) {
      const int i2 = i + nthreads;
      const bool two = i2 < e;
      const int c1 = __ldcg(&a.ent[i]);
      const int d1 = __ldcg(&a.pdir[i]);
      const uint32_t k1 = __ldcg(&a.acc[i]);
      int c2 = c1, d2 = d1;
      uint32_t k2 = k1;
      if (two) {
        c2 = __ldcg(&a.ent[i2]);
        d2 = __ldcg(&a.pdir[i2]);
        k2 = __ldcg(&a.acc[i2]);
      }
      const int n1 = c1 + nbr_off(d1 & 7, a.W);
      const int n2 = c2 + nbr_off(d2 & 7, a.W);
      const double *T1 = a.tab + (size_t)k1 * kTabStride + 4 * (d1 & 1);
      const double *T2 = a.tab + (size_t)k2 * kTabStride + 4 * (d2 & 1);
      const double hc1 = __ldcg(&a.h[c1]);
      double hn1 = __ldcg(&a.h[n1]);
      const double hc2 = __ldcg(&a.h[c2]);
      double hn2 = __ldcg(&a.h[n2]);
      if (d1 & 8) hn1 = hn1 + a.u_dt;
      if (d2 & 8) hn2 = hn2 + a.u_dt;
      const double r1 = erode_cell<NMODE>(a, T1, hc1 + a.u_dt, hn1);
      if (!isfinite(r1)) raise_err(ctl, FS_ERR_NONFINITE, kPhaseErode);
      a.h[c1] = r1;
      if (two) {
        const double r2 = erode_cell<NMODE>(a, T2, hc2 + a.u_dt, hn2);
        if (!isfinite(r2)) raise_err(ctl, FS_ERR_NONFINITE, kPhaseErode);
        a.h[c2] = r2;
      }
    }
    if (L == 2) uplift_pits(a, lvl0_end, tid, nthreads);
    if (L + 1 < nlev && !grid_barrier(ctl, epoch, a.timeout_ns)) return;
  }
  if (nlev <= 2) {
    if (nlev == 2 && !grid_barrier(ctl, epoch, a.timeout_ns)) return;
    uplift_pits(a, lvl0_end, tid, nthreads);
  }
  lap(2);
  if (tid == 0) atomicAdd(&ctl->steps_done, 1);
}

__global__ void k_check_finite(const double *__restrict__ h, int size, Ctl *ctl) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  bool bad = false;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += stride)
    bad |= !isfinite(h[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0)
    raise_err(ctl, FS_ERR_NONFINITE, kPhaseNone);
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

__global__ void k_philox_field(double *__restrict__ h, int W, int H, int size,
                               uint32_t key0, uint32_t key1) {
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

// A wait on a count that no block ever completes; the bounded barrier must
// give up after timeout_ns and report FS_ERR_TIMEOUT. Used by the tests of
// the failure path only.
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

}  // namespace

int walk_threads() { return kWalkThreads; }

float tol_lower_float(double tol) {
  const double t = tol * (1.0 - 0x1p-20);
  float f = (float)t;
  while ((double)f > t) f = nextafterf(f, 0.f);
  return f;
}

cudaError_t launch_receivers(const double *h, int8_t *rec, const Ctl *ctl, StepGeom g,
                             double dr_orth, double dr_diag, cudaStream_t s) {
  const int iw = g.W - 4, ih = g.H - 4;
  if (iw <= 0 || ih <= 0) return cudaSuccess;
  dim3 block(32, 8);
  dim3 grid((iw + 31) / 32, (ih + 7) / 8);
  k_receivers<<<grid, block, 0, s>>>(h, rec, g.W, g.H, dr_orth, dr_diag, ctl);
  return cudaGetLastError();
}

cudaError_t launch_receivers_fast(const double *h, int8_t *rec, int32_t *amb,
                                  Ctl *ctl, StepGeom g, double dr_orth,
                                  double dr_diag, cudaStream_t s) {
  const int iw = g.W - 4, ih = g.H - 4;
  if (iw <= 0 || ih <= 0) return cudaSuccess;
  const float g_orth = (float)(1.0 / dr_orth), g_diag = (float)(1.0 / dr_diag);
  const float gmax = g_orth > g_diag ? g_orth : g_diag;
  dim3 block(32, 8);
  dim3 grid((iw + kRxTile - 1) / kRxTile, (ih + kRyTile - 1) / kRyTile);
  k_receivers_filter<<<grid, block, 0, s>>>(h, rec, amb, ctl, g.W, g.H, g_orth, g_diag, gmax);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_receivers_fixup<<<sms, 256, 0, s>>>(h, rec, amb, ctl, g.W, dr_orth, dr_diag);
  return cudaGetLastError();
}

cudaError_t launch_donors_level0(const int8_t *rec, uint8_t *mask,
                                 int32_t *ent, Ctl *ctl, StepGeom g, int nring,
                                 cudaStream_t s) {
  const int iw = g.W - 2, ih = g.H - 2;
  if (iw <= 0 || ih <= 0) return cudaSuccess;
  dim3 block(32, 8);
  dim3 grid((iw + kDxTile - 1) / kDxTile, (ih + kDyTile - 1) / kDyTile);
  k_donors_level0<<<grid, block, 0, s>>>(rec, mask, ent, ctl, g.W, g.H, nring);
  return cudaGetLastError();
}

const void *walk_kernel_ptr(int nmode) {
  if (nmode == kNOne) return reinterpret_cast<const void *>(&k_walk<kNOne>);
  if (nmode == kNTwo) return reinterpret_cast<const void *>(&k_walk<kNTwo>);
  return reinterpret_cast<const void *>(&k_walk<kNGeneral>);
}

cudaError_t launch_walk(const WalkArgs &a, int blocks, cudaStream_t s) {
  WalkArgs args = a;
  void *params[] = {&args};
  return cudaLaunchCooperativeKernel(walk_kernel_ptr(a.nmode), dim3(blocks),
                                     dim3(kWalkThreads), params, 0, s);
}

cudaError_t launch_check_finite(const double *h, int size, Ctl *ctl,
                                cudaStream_t s) {
  int blocks = (size + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  k_check_finite<<<blocks, 256, 0, s>>>(h, size, ctl);
  return cudaGetLastError();
}

cudaError_t launch_philox_field(double *h, StepGeom g, uint64_t seed,
                                cudaStream_t s) {
  int blocks = (g.size + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  if (blocks < 1) blocks = 1;
  k_philox_field<<<blocks, 256, 0, s>>>(h, g.W, g.H, g.size, (uint32_t)seed,
                                       (uint32_t)(seed >> 32));
  return cudaGetLastError();
}

cudaError_t launch_test_wait(Ctl *ctl, int blocks,
                             unsigned long long timeout_ns, cudaStream_t s) {
  k_test_wait<<<blocks, 32, 0, s>>>(ctl, timeout_ns);
  return cudaGetLastError();
}

}  // namespace fs
