// sg_conv.cu -- the surrogate's dense contraction: 3x3 (and 1x1)
// convolutions over plane-major BF16 tensors ([B][C/8][H][W][8], 16 bytes
// per pixel per plane) as implicit GEMMs on the 5th-generation
// tensor cores (tcgen05.mma kind::f16, BF16 x BF16 -> FP32), operands staged
// in shared memory by TMA (cp.async.bulk.tensor), accumulators in tensor
// memory (TMEM), read back with tcgen05.ld for a fused epilogue. No library
// GEMM, no cluster multicast: every tensor map covers this GPU's own memory.
//
// Forward / data gradient (k_conv): D[p][n] = sum over taps and input
// channels of A[p + off(tap)][ci] * Bw[n][tap*cin + ci].
//   M = 128 pixels of one image (BW x BH, BW = min(W,128)), N = output
//   channels of the tile (<= 256), K = taps * cin in blocks of cb channels.
//   A block is one TMA load of cb/8 planes of the BW x BH pixels at the
//   tap's offset: coordinates outside the image read zeros, which is the
//   convolution's zero padding. The tensor maps view a plane row as 2*W
//   64-bit elements, so one box row is a whole 128-pixel row of a plane
//   (2048 bytes: the TMA engine issues requests per box row, and rows of a
//   plane of 8 channels alone would be 16 bytes each). A is K-major without
//   swizzle (8 pixels of a plane = one 128-byte core matrix, planes = K
//   chunks), the weights K-major with the box's swizzle (32-, 64- or
//   128-byte rows). The data gradient is the same kernel on the output
//   gradient with flipped, transposed weights (launch_flip_weights).
// Forward, channels on M (k_conv_t): see there.
// Weight gradient, K = pixels (128 per step, or 64), both operands MN-major
//   without swizzle (8 channels of 8 pixels = one core matrix, planes one
//   step's pixels apart); the pixel range is split across CTAs, each adding
//   its FP32 partial sums into dW with reductions.
//   k_wgrad_taps (up to 128 output and 256 input channels):
//     dW[co][tap][ci] = sum over q of dY[q - off(tap)][co] * X[q][ci], M =
//     (tap, co) -- each tap's dY planes fetched at its shifted coordinates --
//     and N = ci.
//   k_wgrad (the rest): dW^T[(tap,ci)][co] = sum over p of X[p + off(tap)][ci]
//     * dY[p][co], M = chunks of (tap, channel block) stacked plane after
//     plane, N = co.
//
// Warp roles: warp 0 issues the TMA loads into a ring of stages
// (full/empty mbarriers), warp 1 issues the MMAs and frees each stage with
// tcgen05.commit -- both run their loops with every lane and issue through
// elect.sync -- and the epilogue warps that follow read the accumulator
// back, warp w from TMEM lanes 32*(w%4)..+31 (its pixels, or its rows):
// for the forward / data-gradient kernels NG groups of four warps that take
// every NG-th tile (NG = 2, or 1 when three CTAs share an SM), four for the
// weight gradient. CTAs are persistent; one, two or three share an SM
// (ConvPlan::cps), their pipelines hiding each other's waits.
// Every mbarrier wait is bounded (1 s of the global timer): on expiry the
// CTA sets the error word, stops issuing, waits (again bounded) for its own
// copies and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "sg_internal.h"

namespace sg {
namespace {

constexpr int kThreads = 128;
constexpr int kM = 128;                             // rows of every MMA tile
constexpr int kKPix = 128;                          // pixels per weight-gradient step
constexpr int kMaxStages = 16;
constexpr int kMaxBias = 512;                       // biased outputs of a forward conv
constexpr size_t kSmemBudget = 200 * 1024;          // stage ring (plus 1 KB alignment slack)
constexpr size_t kPlanarSmem = 222 * 1024;          // planar form: weights + ring + guard (+ static)
constexpr size_t kPairSmem = 104 * 1024;            // one of two CTAs per SM
constexpr size_t kTripleSmem = 70 * 1024;           // one of three CTAs per SM (one epilogue group)
constexpr unsigned long long kWaitNs = 1000000000ull;

// ---------------------------------------------------------------- PTX ----

__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of `parity` to complete; false after kWaitNs, or as
// soon as *abort is set when watch_abort.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort,
                                          bool watch_abort) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (int it = 1;; it++) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 15) == 0) {
      if (watch_abort && *abort) return false;
      if (gtimer() - t0 > kWaitNs) return false;
    }
  }
}

// mbar_wait for a whole warp: true only if every lane saw the phase.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *bar, uint32_t parity, volatile int *abort,
                                               bool watch_abort) {
  return __all_sync(0xffffffffu, mbar_wait(bar, parity, abort, watch_abort));
}

__device__ __forceinline__ void tma_prefetch(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   su32(slot)),
               "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// The producer and MMA warps run their loops with every lane (the same,
// warp-uniform coordinates and descriptors); one lane, chosen by elect.sync
// inside the same statement, issues each TMA copy, MMA and commit.
// umma_bf16_el: D[tmem] (+)= A[smem] * B[smem]^T, BF16 inputs, FP32
// accumulation; umma_commit_el: the mbarrier receives one arrival once every
// MMA issued before has completed.
__device__ __forceinline__ void mbar_expect_tx_el(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\t"
      "@p mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n\t}" ::"r"(su32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d_el(void *dst, const CUtensorMap *map, uint64_t *bar,
                                               int c0, int c1, int c2, int c3) {
  asm volatile(
      "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\t"
      "@p cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];\n\t}" ::"r"(su32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(su32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

__device__ __forceinline__ void tma_load_2d_el(void *dst, const CUtensorMap *map, uint64_t *bar,
                                               int c0, int c1) {
  asm volatile(
      "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\t"
      "@p cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];\n\t}" ::"r"(su32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(su32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void umma_bf16_el(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                             uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "elect.sync _|p, 0xffffffff;\n\t"
      "setp.ne.b32 q, %4, 0;\n\t"
      "@p tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit_el(uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\t"
      "@p tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}" ::"r"(
          su32(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void red_add_f32(float *p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// Swizzle-mode code of the shared-memory descriptor for rows of `row_bytes`
// (the TMA box's swizzle span): 128 B -> 2, 64 B -> 4, 32 B -> 6.
__host__ __device__ constexpr uint64_t swizzle_code(int row_bytes) {
  return row_bytes == 128 ? 2 : row_bytes == 64 ? 4 : 6;
}

// Shared-memory matrix descriptor (tcgen05): start address, leading and
// stride byte offsets (16-byte units), descriptor version 1, swizzle mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo,
                                              uint64_t swz) {
  uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFF) >> 4);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= swz << 61;
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B,
// A/B K-major (0) or MN-major (1), N = n, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int n, int a_mn, int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(a_mn) << 15) |
         (static_cast<uint32_t>(b_mn) << 16) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(kM >> 4) << 24);
}

__device__ __forceinline__ void sg_raise(int *err, volatile int *abort, int code) {
  *abort = 1;
  atomicCAS(err, 0, code);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&v);
}

struct ConvArgs {
  int H, W, BW, BH, tiles_x, tiles_y;
  int cin, taps, bn, stages;
  int mtiles, ntiles;  // tiles of 128 pixels, and of bn output channels
  const float *bias;
  int relu;
  const bf16 *mask;   // ntot channels, plane-major like out
  bf16 *out;
  int oplanes;        // planes per image of out and mask (ntot / 8, or more)
  int up;             // 1: out is 2H x 2W, each pixel stored into its 2x2 block
  int nbuf;           // TMEM accumulator buffers (k_conv, k_conv_planar)
  int *err;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

constexpr int kConvThreads = 320;   // producer warp, MMA warp, 8 epilogue warps (k_conv_t)
constexpr int kMaxAccBufs = 4;      // accumulator buffers of a forward / data-gradient CTA

// Accumulator columns of an N tile and the buffers TMEM's 512 columns hold:
// the MMAs of the next tiles run while the epilogue drains earlier ones.
__host__ __device__ constexpr uint32_t acc_cols(int bn) {
  return bn <= 32 ? 32 : bn <= 64 ? 64 : bn <= 128 ? 128 : 256;
}
__host__ __device__ constexpr uint32_t pow2_cols(uint32_t n) {
  return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}
__host__ __device__ constexpr int acc_bufs(int bn) {
  return static_cast<int>(512 / acc_cols(bn)) < kMaxAccBufs ? static_cast<int>(512 / acc_cols(bn))
                                                            : kMaxAccBufs;
}
constexpr int kWgradThreads = 192;  // producer warp, MMA warp, 4 epilogue warps

// Stores of an output upsampled 2x when the warp's 32 lanes hold 32
// consecutive pixels of one row: the row's 64 slots from the warp's first
// pixel (lane 0's out minus 16 lane elements) as two fully used 512-byte
// stores, slot s holding pixel s/2 (values moved by shuffles), in both rows.
__device__ __forceinline__ void store_up_rows(uint4 o, bf16 *out, long long rowd) {
  const int lane = threadIdx.x & 31;
  uint4 a, b;
  a.x = __shfl_sync(0xffffffffu, o.x, lane >> 1);
  a.y = __shfl_sync(0xffffffffu, o.y, lane >> 1);
  a.z = __shfl_sync(0xffffffffu, o.z, lane >> 1);
  a.w = __shfl_sync(0xffffffffu, o.w, lane >> 1);
  b.x = __shfl_sync(0xffffffffu, o.x, 16 + (lane >> 1));
  b.y = __shfl_sync(0xffffffffu, o.y, 16 + (lane >> 1));
  b.z = __shfl_sync(0xffffffffu, o.z, 16 + (lane >> 1));
  b.w = __shfl_sync(0xffffffffu, o.w, 16 + (lane >> 1));
  bf16 *base = out - 8 * lane;  // slot `lane` of the warp's row run
  *reinterpret_cast<uint4 *>(base) = a;
  *reinterpret_cast<uint4 *>(base + 256) = b;
  *reinterpret_cast<uint4 *>(base + rowd) = a;
  *reinterpret_cast<uint4 *>(base + rowd + 256) = b;
}

// One 16-column chunk of a tile row: + bias (shared memory), ReLU, zeroed
// where the mask is not positive, rounded to BF16, stored as 16 bytes in
// each of two planes (ps elements apart); with rowd > 0 (an output upsampled
// 2x, rows rowd elements apart) into the pixel's 2x2 block of each plane
// (rowd < 0: the same, the warp holding 32 consecutive pixels of one row).
__device__ __forceinline__ void epi16(const uint32_t (&v)[16], const float *sb, int relu,
                                      const bf16 *msk, bf16 *out, long long ps,
                                      long long rowd) {
  float f[16];
#pragma unroll
  for (int j = 0; j < 16; j++) f[j] = __uint_as_float(v[j]);
  if (sb) {
#pragma unroll
    for (int j = 0; j < 16; j++) f[j] += sb[j];
  }
  if (relu) {
#pragma unroll
    for (int j = 0; j < 16; j++) f[j] = fmaxf(f[j], 0.0f);
  }
  if (msk) {
    const uint4 m0 = *reinterpret_cast<const uint4 *>(msk);
    const uint4 m1 = *reinterpret_cast<const uint4 *>(msk + ps);
    const bf16 *mb0 = reinterpret_cast<const bf16 *>(&m0);
    const bf16 *mb1 = reinterpret_cast<const bf16 *>(&m1);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (!(__bfloat162float(mb0[j]) > 0.0f)) f[j] = 0.0f;
      if (!(__bfloat162float(mb1[j]) > 0.0f)) f[8 + j] = 0.0f;
    }
  }
  uint4 o0, o1;
  o0.x = pack_bf16(f[0], f[1]);
  o0.y = pack_bf16(f[2], f[3]);
  o0.z = pack_bf16(f[4], f[5]);
  o0.w = pack_bf16(f[6], f[7]);
  o1.x = pack_bf16(f[8], f[9]);
  o1.y = pack_bf16(f[10], f[11]);
  o1.z = pack_bf16(f[12], f[13]);
  o1.w = pack_bf16(f[14], f[15]);
  if (rowd < 0) {
    store_up_rows(o0, out, -rowd);
    store_up_rows(o1, out + ps, -rowd);
    return;
  }
  *reinterpret_cast<uint4 *>(out) = o0;
  *reinterpret_cast<uint4 *>(out + ps) = o1;
  if (rowd) {
    *reinterpret_cast<uint4 *>(out + 8) = o0;
    *reinterpret_cast<uint4 *>(out + ps + 8) = o1;
    *reinterpret_cast<uint4 *>(out + rowd) = o0;
    *reinterpret_cast<uint4 *>(out + rowd + 8) = o0;
    *reinterpret_cast<uint4 *>(out + ps + rowd) = o1;
    *reinterpret_cast<uint4 *>(out + ps + rowd + 8) = o1;
  }
}

// Columns [c_lo, c_hi) of this warp's 32 TMEM lanes (d: lane quarter and
// accumulator base), two 16-column loads in flight per wait; out and msk
// point at this lane's pixel in the plane of column 0, planes ps elements
// apart (rowd: as in epi16).
__device__ __forceinline__ void epi_columns(uint32_t d, int c_lo, int c_hi, const float *sb,
                                            int relu, const bf16 *msk, bf16 *out, long long ps,
                                            long long rowd) {
  int c = c_lo;
  for (; c + 32 <= c_hi; c += 32) {
    uint32_t v0[16], v1[16];
    tmem_ld16(d + c, v0);
    tmem_ld16(d + c + 16, v1);
    tmem_ld_wait();
    const long long o0 = (c / 8) * ps, o1 = ((c + 16) / 8) * ps;
    epi16(v0, sb ? sb + c : nullptr, relu, msk ? msk + o0 : nullptr, out + o0, ps, rowd);
    epi16(v1, sb ? sb + c + 16 : nullptr, relu, msk ? msk + o1 : nullptr, out + o1, ps, rowd);
  }
  if (c < c_hi) {
    uint32_t v0[16];
    tmem_ld16(d + c, v0);
    tmem_ld_wait();
    const long long o0 = (c / 8) * ps;
    epi16(v0, sb ? sb + c : nullptr, relu, msk ? msk + o0 : nullptr, out + o0, ps, rowd);
  }
}

// ------------------------------------------------------ forward / dgrad ----
// Persistent: CTA b takes tiles b, b + gridDim.x, ... (pixel tile major, N
// tile minor). The stage ring runs on across tiles; the accumulator has up
// to four buffers in TMEM (acc_full: MMAs of a tile done; acc_empty: its
// epilogue has read it), and the epilogue warps form two groups of four
// that drain alternate tiles, so the epilogues of two tiles overlap each
// other and the MMAs of the next ones.
template <int CB, int NG>
__global__ void __launch_bounds__(64 + 128 * NG, NG == 1 ? 3 : 2)
    k_conv(const __grid_constant__ CUtensorMap tma, const __grid_constant__ CUtensorMap tmb,
           const ConvArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full[kMaxAccBufs],
      acc_empty[kMaxAccBufs], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float s_bias[kMaxBias];
  if (a.bias)
    for (int i = threadIdx.x; i < a.bn * a.ntiles; i += blockDim.x) s_bias[i] = a.bias[i];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kRow = CB * 2;      // bytes per weight row (the swizzle span)
  constexpr int kAPlane = kM * 16;  // one plane of the A tile: 128 pixels x 8 channels
  const int a_bytes = kM * kRow;
  const int b_bytes = a.bn * kRow;
  const int stage_bytes = (a_bytes + b_bytes + 1023) & ~1023;
  const int S = a.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t cols = acc_cols(a.bn);
  const int nbuf = a.nbuf;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int i = 0; i < nbuf; i++) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);  // one epilogue group of four warps
    }
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tma_prefetch(&tma);
    tma_prefetch(&tmb);
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, nbuf * cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  const int tiles_img = a.tiles_x * a.tiles_y;
  const int kch = a.cin / CB;
  const int nkb = a.taps * kch;
  const int ntot_tiles = a.mtiles * a.ntiles;

  if (warp == 0) {
    // producer (the whole warp; one lane issues)
    int kbg = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x) {
      const int mt = t / a.ntiles, nt = t - mt * a.ntiles;
      const int b = mt / tiles_img;
      const int tt = mt - b * tiles_img;
      const int y0 = (tt / a.tiles_x) * a.BH, x0 = (tt % a.tiles_x) * a.BW;
      const int n0 = nt * a.bn;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int s = kbg % S;
        if (!mbar_wait_warp(&empty[s], ((kbg / S) & 1) ^ 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        const int tap = kb / kch, cc = kb - tap * kch;
        const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
        unsigned char *sa = smem + s * stage_bytes;
        mbar_expect_tx_el(&full[s], a_bytes + b_bytes);
        tma_load_4d_el(sa, &tma, &full[s], 2 * (x0 + dx), y0 + dy, cc * (CB / 8), b);
        tma_load_2d_el(sa + a_bytes, &tmb, &full[s], tap * a.cin + cc * CB, n0);
      }
    }
    // leave no copy in flight into this CTA's shared memory
    for (int k = kbg > S ? kbg - S : 0; k < kbg; k++)
      if (!mbar_wait_warp(&full[k % S], (k / S) & 1, &abort_flag, false)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
  } else if (warp == 1) {
    // MMA issuer (the whole warp; one lane issues)
    const uint32_t idesc = idesc_bf16(a.bn, 0, 0);
    int kbg = 0, it = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x, it++) {
      const int buf = it % nbuf;
      if (!mbar_wait_warp(&acc_empty[buf], ((it / nbuf) & 1) ^ 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + buf * cols;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int s = kbg % S;
        if (!mbar_wait_warp(&full[s], (kbg / S) & 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        tc_fence_after();
        const uint32_t sa = su32(smem + s * stage_bytes);
        // A: K-major, no swizzle: K chunks (planes) kAPlane apart, 8-row
        // groups 128 bytes apart; B: K-major, swizzled rows of kRow bytes
        const uint64_t da = smem_desc(sa, kAPlane, 128, 0);
        const uint64_t db = smem_desc(sa + a_bytes, 16, 8 * kRow, swizzle_code(kRow));
#pragma unroll
        for (int k = 0; k < CB / 16; k++)  // K = 16 per MMA: two planes of A, 32 bytes of B
          umma_bf16_el(d, da + ((2 * k * kAPlane) >> 4), db + 2 * k, idesc, (kb | k) != 0);
        umma_commit_el(&empty[s]);
      }
      if (!stop) umma_commit_el(&acc_full[buf]);
    }
    // every MMA this warp issued has completed before the teardown
    umma_commit_el(&done);
    if (!mbar_wait_warp(&done, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (one pixel each);
    // group (w-2)/4 takes every other tile of this CTA
    const int q = warp & 3;
    const int grp = (warp - 2) >> 2;
    const int r = q * 32 + lane;
    for (int t = blockIdx.x + grp * gridDim.x, it = grp; t < ntot_tiles;
         t += NG * gridDim.x, it += NG) {
      const int buf = it % nbuf;
      if (!mbar_wait(&acc_full[buf], (it / nbuf) & 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const int mt = t / a.ntiles, nt = t - mt * a.ntiles;
      const int b = mt / tiles_img;
      const int tt = mt - b * tiles_img;
      const int y0 = (tt / a.tiles_x) * a.BH, x0 = (tt % a.tiles_x) * a.BW;
      const int n0 = nt * a.bn;
      const int py = y0 + r / a.BW, px = x0 + r % a.BW;
      const long long hw = static_cast<long long>(a.H) * a.W << (2 * a.up);
      const long long at =
          plane_at(b, n0 / 8, (static_cast<long long>(py) * a.W << (2 * a.up)) + (px << a.up),
                   a.oplanes, hw);
      const uint32_t d = tmem + buf * cols + (static_cast<uint32_t>(q * 32) << 16);
      // a warp's 32 pixels lie in one row when the tile is a multiple of 32 wide
      const long long rowd = !a.up ? 0 : a.BW % 32 == 0 ? -16ll * a.W : 16ll * a.W;
      epi_columns(d, 0, a.bn, a.bias ? s_bias + n0 : nullptr, a.relu,
                  a.mask ? a.mask + at : nullptr, a.out + at, hw * 8, rowd);
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, nbuf * cols);
  }
}

// ------------------------------------------- forward / dgrad, planar A ----
// For images at least 128 pixels wide with 3x3 taps and weights that fit in
// shared memory (the narrow layers): each K-block is one image row (dy) of
// cb channels, staged once by one TMA box as cb/8 planes of 130 pixels x 8
// channels (16 bytes per pixel, no swizzle: the K-major core-matrix layout
// with 8-row groups 128 bytes apart and K chunks one plane apart), and the
// three taps dx of that row are the same planes read from byte offset
// 16*dx -- a third of the A traffic of one load per tap. The weights of
// every tap are loaded into shared memory once per CTA and stay there.
constexpr int kPlanePix = 130;                              // x0-1 .. x0+128
constexpr int kPlaneBytes = kPlanePix * 16;                 // one staged plane row: 2080 bytes
constexpr int kPlaneStride = (kPlaneBytes + 127) & ~127;    // 128-byte aligned TMA targets
// A staged plane row is two TMA boxes: pixels x0-1 .. x0+126 (256 64-bit
// elements, 2048 bytes) and the tail x0+127, x0+128 (4 elements).
constexpr int kGuardBytes = 4 * 1024;  // slack after the ring (the MMAs read inside each stage)

template <int CB, int NG>
__global__ void __launch_bounds__(64 + 128 * NG, NG == 1 ? 3 : 2)
    k_conv_planar(const __grid_constant__ CUtensorMap tmp, const __grid_constant__ CUtensorMap tmt,
                  const __grid_constant__ CUtensorMap tmb,
                  const ConvArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full[kMaxAccBufs],
      acc_empty[kMaxAccBufs], done, wfull;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float s_bias[kMaxBias];
  if (a.bias)
    for (int i = threadIdx.x; i < a.bn; i += blockDim.x) s_bias[i] = a.bias[i];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kRow = CB * 2;
  constexpr int kPlanes = CB / 8;
  constexpr int kStageA = (kPlanes * kPlaneStride + 1023) & ~1023;
  const int kch = a.cin / CB;
  const int wbox = a.bn * kRow;  // one (tap, channel block) box of weights
  const int wbytes = 9 * kch * wbox;
  unsigned char *ring = smem + ((wbytes + 1023) & ~1023);
  const int S = a.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t cols = acc_cols(a.bn);
  const int nbuf = a.nbuf;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int i = 0; i < nbuf; i++) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);  // one epilogue group of four warps
    }
    mbar_init(&done, 1);
    mbar_init(&wfull, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tma_prefetch(&tmp);
    tma_prefetch(&tmt);
    tma_prefetch(&tmb);
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, nbuf * cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int tiles_img = a.tiles_x * a.tiles_y;
  const int nkb = 3 * kch;  // (dy, channel block)
  const int ntot_tiles = a.mtiles;

  if (warp == 0) {
    // producer (the whole warp; one lane issues)
    // weights once: box (tap, cc) at smem + (tap*kch + cc)*wbox
    mbar_expect_tx_el(&wfull, wbytes);
    for (int tap = 0; tap < 9; tap++)
      for (int cc = 0; cc < kch; cc++)
        tma_load_2d_el(smem + (tap * kch + cc) * wbox, &tmb, &wfull, tap * a.cin + cc * CB, 0);
    int kbg = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x) {
      const int b = t / tiles_img;
      const int tt = t - b * tiles_img;
      const int y0 = tt / a.tiles_x, x0 = (tt % a.tiles_x) * 128;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int s = kbg % S;
        if (!mbar_wait_warp(&empty[s], ((kbg / S) & 1) ^ 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        const int dy = kb / kch, cc = kb - dy * kch;
        unsigned char *sa = ring + s * kStageA;
        mbar_expect_tx_el(&full[s], kPlanes * kPlaneBytes);
#pragma unroll
        for (int pl = 0; pl < kPlanes; pl++) {
          tma_load_4d_el(sa + pl * kPlaneStride, &tmp, &full[s], 2 * (x0 - 1), y0 + dy - 1,
                         cc * kPlanes + pl, b);
          tma_load_4d_el(sa + pl * kPlaneStride + 2048, &tmt, &full[s], 2 * (x0 + 127),
                         y0 + dy - 1, cc * kPlanes + pl, b);
        }
      }
    }
    for (int k = kbg > S ? kbg - S : 0; k < kbg; k++)
      if (!mbar_wait_warp(&full[k % S], (k / S) & 1, &abort_flag, false)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
    if (!mbar_wait_warp(&wfull, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else if (warp == 1) {
    // MMA issuer (the whole warp; one lane issues)
    const uint32_t idesc = idesc_bf16(a.bn, 0, 0);
    bool stop = !mbar_wait_warp(&wfull, 0, &abort_flag, true);
    if (stop) sg_raise(a.err, &abort_flag, kSgTimeout);
    tc_fence_after();
    const uint32_t wbase = su32(smem);
    int kbg = 0, it = 0;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x, it++) {
      const int buf = it % nbuf;
      if (!mbar_wait_warp(&acc_empty[buf], ((it / nbuf) & 1) ^ 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + buf * cols;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int s = kbg % S;
        if (!mbar_wait_warp(&full[s], (kbg / S) & 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        tc_fence_after();
        const int dy = kb / kch, cc = kb - dy * kch;
        const uint32_t sa = su32(ring + s * kStageA);
#pragma unroll
        for (int dx = 0; dx < 3; dx++) {
          const uint32_t wb = wbase + ((3 * dy + dx) * kch + cc) * wbox;
          const uint64_t db = smem_desc(wb, 16, 8 * kRow, swizzle_code(kRow));
#pragma unroll
          for (int k = 0; k < CB / 16; k++) {
            // K-major, no swizzle: K chunks (planes) kPlaneStride apart, 8-row
            // groups 128 bytes apart; 16 channels = two planes per MMA
            const uint64_t da = smem_desc(sa + 16 * dx + 2 * k * kPlaneStride, kPlaneStride, 128, 0);
            umma_bf16_el(d, da, db + 2 * k, idesc, (kb | dx | k) != 0);
          }
        }
        umma_commit_el(&empty[s]);
      }
      if (!stop) umma_commit_el(&acc_full[buf]);
    }
    umma_commit_el(&done);
    if (!mbar_wait_warp(&done, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else {
    const int q = warp & 3;
    const int grp = (warp - 2) >> 2;
    const int r = q * 32 + lane;
    for (int t = blockIdx.x + grp * gridDim.x, it = grp; t < ntot_tiles;
         t += NG * gridDim.x, it += NG) {
      const int buf = it % nbuf;
      if (!mbar_wait(&acc_full[buf], (it / nbuf) & 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const int b = t / tiles_img;
      const int tt = t - b * tiles_img;
      const int py = tt / a.tiles_x, px = (tt % a.tiles_x) * 128 + r;
      const long long hw = static_cast<long long>(a.H) * a.W << (2 * a.up);
      const long long at =
          plane_at(b, 0, (static_cast<long long>(py) * a.W << (2 * a.up)) + (px << a.up),
                   a.oplanes, hw);
      const uint32_t d = tmem + buf * cols + (static_cast<uint32_t>(q * 32) << 16);
      epi_columns(d, 0, a.bn, a.bias ? s_bias : nullptr, a.relu,
                  a.mask ? a.mask + at : nullptr, a.out + at, hw * 8, a.up ? -16ll * a.W : 0);
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, nbuf * cols);
  }
}

struct WgradArgs {
  int H, W, BW, BH, tiles_x, tiles_y;
  int cin, cout, taps, nchunk, stages, ksteps, kper;
  float *dw;
  int *err;
};

// ---------------------------------- forward / dgrad, channels on M ----
// For images whose rows are multiples of 256 pixels, 3x3 taps and at most
// 128 output channels: D[co][p] = sum over (dy, dx, ci) of W[co][tap][ci] *
// X[y + dy - 1][p + dx - 1][ci]. M = output channels: the resident weight
// tiles are the K-major A operand (their rows beyond the output channels
// read whatever follows them in shared memory and are discarded); N = 256
// pixels of one row: each K-block stages a row (dy) of cb channels as cb/8
// planes of 258 pixels, and the taps dx read them from byte offset 16*dx
// (K-major, no swizzle). The MMAs then run at N = 256 whatever the channel
// count (with N = the channel count they cost about the same per
// instruction at a fraction of the work). One TMEM lane holds one channel,
// so the epilogue transposes each warp's 32 channels x 16 pixels through
// shared memory into 8-channel planes before the stores. No mask: the plan
// sends data gradients to k_conv_planar.
//
// Used for forward convolutions (no mask) of at least 64 input channels
// whose weights leave no room for two planar CTAs per SM (64 -> 64 channels
// at 256^2: 0.20 against 0.24 ms at batch 32); where two planar CTAs fit,
// they are as fast (96 -> 32 at 512^2: both ~0.97 ms, against 1.63 ms for
// one planar CTA). With fewer input channels one CTA of each is even; with
// the data gradient's mask it is about 2x slower (the epilogue's mask loads
// stall it; TMEM reads of more lanes to spread the work slow the MMAs).
constexpr int kTN = 256;                                     // pixels per tile
constexpr int kTPix = kTN + 2;                               // x0-1 .. x0+256
constexpr int kTSlot = (kTPix * 16 + 127) & ~127;            // 4224: a staged plane row
constexpr size_t kTSmem = 208 * 1024;                        // dynamic shared memory

template <int CB>
__global__ void __launch_bounds__(kConvThreads, 1)
    k_conv_t(const __grid_constant__ CUtensorMap tmp, const __grid_constant__ CUtensorMap tmt,
             const __grid_constant__ CUtensorMap tmb, const ConvArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full[2], acc_empty[2], done, wfull;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float s_bias[kM];
  __shared__ uint32_t s_tr[8][32][8];  // per epilogue warp: 32 channels x 16 pixels (bf16 pairs)
  if (a.bias)
    for (int i = threadIdx.x; i < a.bn; i += blockDim.x) s_bias[i] = a.bias[i];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kRow = CB * 2;
  constexpr int kPlanes = CB / 8;
  constexpr int kStageB = (kPlanes * kTSlot + 1023) & ~1023;
  const int kch = a.cin / CB;
  const int wbox = a.bn * kRow;  // one (tap, channel block) box of weights
  const int wbytes = 9 * kch * wbox;
  unsigned char *ring = smem + ((wbytes + 1023) & ~1023);
  const int S = a.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t cols = kTN;

  if (threadIdx.x == 0) {
    for (int st = 0; st < S; st++) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);  // one epilogue group of four warps
    }
    mbar_init(&done, 1);
    mbar_init(&wfull, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tma_prefetch(&tmp);
    tma_prefetch(&tmt);
    tma_prefetch(&tmb);
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, 2 * cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int tiles_row = a.W / kTN;
  const int tiles_img = tiles_row * a.H;
  const int nkb = 3 * kch;  // (dy, channel block)
  const int ntot_tiles = a.mtiles;

  if (warp == 0) {
    // producer (the whole warp; one lane issues)
    mbar_expect_tx_el(&wfull, wbytes);
    for (int tap = 0; tap < 9; tap++)
      for (int cc = 0; cc < kch; cc++)
        tma_load_2d_el(smem + (tap * kch + cc) * wbox, &tmb, &wfull, tap * a.cin + cc * CB, 0);
    int kbg = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x) {
      const int b = t / tiles_img;
      const int tt = t - b * tiles_img;
      const int y0 = tt / tiles_row, x0 = (tt % tiles_row) * kTN;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int st = kbg % S;
        if (!mbar_wait_warp(&empty[st], ((kbg / S) & 1) ^ 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        const int dy = kb / kch, cc = kb - dy * kch;
        unsigned char *sb = ring + st * kStageB;
        mbar_expect_tx_el(&full[st], kPlanes * kTPix * 16);
#pragma unroll
        for (int pl = 0; pl < kPlanes; pl++) {
          unsigned char *d = sb + pl * kTSlot;
          const int yy = y0 + dy - 1, pp = cc * kPlanes + pl;
          tma_load_4d_el(d, &tmp, &full[st], 2 * (x0 - 1), yy, pp, b);
          tma_load_4d_el(d + 2048, &tmp, &full[st], 2 * (x0 + 127), yy, pp, b);
          tma_load_4d_el(d + 4096, &tmt, &full[st], 2 * (x0 + 255), yy, pp, b);
        }
      }
    }
    for (int k = kbg > S ? kbg - S : 0; k < kbg; k++)
      if (!mbar_wait_warp(&full[k % S], (k / S) & 1, &abort_flag, false)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
    if (!mbar_wait_warp(&wfull, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else if (warp == 1) {
    // MMA issuer (the whole warp; one lane issues)
    const uint32_t idesc = idesc_bf16(kTN, 0, 0);
    bool stop = !mbar_wait_warp(&wfull, 0, &abort_flag, true);
    if (stop) sg_raise(a.err, &abort_flag, kSgTimeout);
    tc_fence_after();
    const uint32_t wbase = su32(smem);
    int kbg = 0, it = 0;
    for (int t = blockIdx.x; t < ntot_tiles && !stop; t += gridDim.x, it++) {
      const int buf = it & 1;
      if (!mbar_wait_warp(&acc_empty[buf], ((it >> 1) & 1) ^ 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + buf * cols;
      for (int kb = 0; kb < nkb; kb++, kbg++) {
        const int st = kbg % S;
        if (!mbar_wait_warp(&full[st], (kbg / S) & 1, &abort_flag, true)) {
          sg_raise(a.err, &abort_flag, kSgTimeout);
          stop = true;
          break;
        }
        tc_fence_after();
        const int dy = kb / kch, cc = kb - dy * kch;
        const uint32_t sb = su32(ring + st * kStageB);
#pragma unroll
        for (int dx = 0; dx < 3; dx++) {
          // A: the weight tile (K-major, swizzled rows of kRow bytes)
          const uint32_t wa = wbase + ((3 * dy + dx) * kch + cc) * wbox;
          const uint64_t da = smem_desc(wa, 16, 8 * kRow, swizzle_code(kRow));
#pragma unroll
          for (int k = 0; k < CB / 16; k++) {
            // B: K-major, no swizzle: K chunks (planes) kTSlot apart, 8-pixel
            // groups 128 bytes apart; 16 channels = two planes per MMA
            const uint64_t db = smem_desc(sb + 16 * dx + 2 * k * kTSlot, kTSlot, 128, 0);
            umma_bf16_el(d, da + 2 * k, db, idesc, (kb | dx | k) != 0);
          }
        }
        umma_commit_el(&empty[st]);
      }
      if (!stop) umma_commit_el(&acc_full[buf]);
    }
    umma_commit_el(&done);
    if (!mbar_wait_warp(&done, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4)..+31 = channels; group
    // (w-2)/4 takes every other tile of this CTA
    const int q = warp & 3;
    const int grp = (warp - 2) >> 2;
    const int co = q * 32 + lane;
    const int g = lane >> 3, kk = lane & 7;  // after the transpose: plane 4q+g, pixels 2kk, 2kk+1
    const int cg = 4 * q + g;
    const bool active = q * 32 < a.bn;
    const bool writer = 8 * cg < a.bn;
    uint32_t(*tr)[8] = s_tr[warp - 2];
    const float bias = a.bias && co < a.bn ? s_bias[co] : 0.0f;
    const long long hw = static_cast<long long>(a.H) * a.W << (2 * a.up);
    for (int t = blockIdx.x + grp * gridDim.x, it = grp; t < ntot_tiles;
         t += 2 * gridDim.x, it += 2) {
      const int buf = it & 1;
      const int b = t / tiles_img;
      const int tt = t - b * tiles_img;
      const int y0 = tt / tiles_row, x0 = (tt % tiles_row) * kTN;
      const long long at =
          plane_at(b, writer ? cg : 0,
                   (static_cast<long long>(y0) * a.W << (2 * a.up)) + ((x0 + 2 * kk) << a.up),
                   a.oplanes, hw);
      if (!mbar_wait(&acc_full[buf], (it >> 1) & 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      if (active) {
        const uint32_t d = tmem + buf * cols + (static_cast<uint32_t>(q * 32) << 16);
        for (int c = 0; c < kTN; c += 16) {
          uint32_t v[16];
          tmem_ld16(d + c, v);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; j += 2) {
            float f0 = __uint_as_float(v[j]) + bias, f1 = __uint_as_float(v[j + 1]) + bias;
            if (a.relu) {
              f0 = fmaxf(f0, 0.0f);
              f1 = fmaxf(f1, 0.0f);
            }
            tr[lane][j / 2] = pack_bf16(f0, f1);  // pixels c+j, c+j+1 of channel co
          }
          __syncwarp();
          // pixels c+2kk and c+2kk+1, channels 8g .. 8g+7 of this quarter
          uint32_t w[8];
#pragma unroll
          for (int ch = 0; ch < 8; ch++) w[ch] = tr[8 * g + ch][kk];
          __syncwarp();
          uint4 o0, o1;
          o0.x = __byte_perm(w[0], w[1], 0x5410);
          o0.y = __byte_perm(w[2], w[3], 0x5410);
          o0.z = __byte_perm(w[4], w[5], 0x5410);
          o0.w = __byte_perm(w[6], w[7], 0x5410);
          o1.x = __byte_perm(w[0], w[1], 0x7632);
          o1.y = __byte_perm(w[2], w[3], 0x7632);
          o1.z = __byte_perm(w[4], w[5], 0x7632);
          o1.w = __byte_perm(w[6], w[7], 0x7632);
          if (writer && !a.up) {
            const long long o = at + 8ll * c;
            *reinterpret_cast<uint4 *>(a.out + o) = o0;
            *reinterpret_cast<uint4 *>(a.out + o + 8) = o1;
          } else if (writer) {
            // pixels 2p .. 2p+3 of rows 2y0 and 2y0+1 of the 2x output
            uint4 *o = reinterpret_cast<uint4 *>(a.out + at + 16ll * c);
            uint4 *o2 = o + 2 * a.W;
            o[0] = o0;
            o[1] = o0;
            o[2] = o1;
            o[3] = o1;
            o2[0] = o0;
            o2[1] = o0;
            o2[2] = o1;
            o2[3] = o1;
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * cols);
  }
}

// --------------------------------------------------------- weight grad ----
// CWA: channels per chunk of X (M side), CWB: per chunk of dY (N side).
template <int CWA, int CWB>
__global__ void __launch_bounds__(kThreads, 1)
    k_wgrad(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmy,
            const WgradArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], accf;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kRowA = CWA * 2, kRowB = CWB * 2;
  constexpr int kChunkA = kKPix * kRowA;  // one (tap, channel block) chunk: CWA/8 planes
  constexpr int kChunkB = kKPix * kRowB;
  constexpr int kPix16 = kKPix * 16;      // one plane of 128 pixels
  constexpr int kPerTile = kM / CWA;      // chunks stacked in one M tile
  const int a_bytes = kPerTile * kChunkA;  // = 128 * 256 bytes
  const int b_bytes = (a.cout / CWB) * kChunkB;
  const int stage_bytes = a_bytes + b_bytes;  // multiples of 1024
  const int S = a.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = a.cout <= 32 ? 32 : a.cout <= 64 ? 64 : a.cout <= 128 ? 128 : 256;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accf, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tma_prefetch(&tmx);
    tma_prefetch(&tmy);
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, ncols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  const int q0 = blockIdx.x * kPerTile;  // first chunk of this M tile
  const int nq = min(kPerTile, a.nchunk - q0);
  const int kchx = a.cin / CWA;
  const int k_lo = blockIdx.y * a.kper;
  const int k_hi = min(a.ksteps, k_lo + a.kper);
  const int nk = k_hi - k_lo;
  const int tiles_img = a.tiles_x * a.tiles_y;

  if (warp == 0) {
    // producer (the whole warp; one lane issues)
    int issued = 0;
    const uint32_t tx = nq * kChunkA + b_bytes;
    for (int i = 0; i < nk; i++) {
      const int s = i % S;
      if (!mbar_wait_warp(&empty[s], ((i / S) & 1) ^ 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      const int kt = k_lo + i;
      const int b = kt / tiles_img, t = kt - b * tiles_img;
      const int y0 = (t / a.tiles_x) * a.BH, x0 = (t % a.tiles_x) * a.BW;
      unsigned char *sa = smem + s * stage_bytes;
      unsigned char *sb = sa + a_bytes;
      mbar_expect_tx_el(&full[s], tx);
      for (int j = 0; j < nq; j++) {
        const int q = q0 + j;
        const int tap = q / kchx, cc = q - tap * kchx;
        const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
        tma_load_4d_el(sa + j * kChunkA, &tmx, &full[s], 2 * (x0 + dx), y0 + dy, cc * (CWA / 8),
                       b);
      }
      tma_load_4d_el(sb, &tmy, &full[s], 2 * x0, y0, 0, b);  // every plane of dY
      issued = i + 1;
    }
    for (int i = issued > S ? issued - S : 0; i < issued; i++)
      if (!mbar_wait_warp(&full[i % S], (i / S) & 1, &abort_flag, false)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
  } else if (warp == 1) {
    // MMA issuer (the whole warp; one lane issues)
    const uint32_t idesc = idesc_bf16(a.cout, 1, 1);
    for (int i = 0; i < nk; i++) {
      const int s = i % S;
      if (!mbar_wait_warp(&full[s], (i / S) & 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const uint32_t sa = su32(smem + s * stage_bytes);
      // MN-major, no swizzle: MN chunks (planes) kPix16 apart, 8-pixel K
      // groups 128 bytes apart; 16 pixels (256 bytes of every plane) per MMA
      const uint64_t da = smem_desc(sa, 128, kPix16, 0);
      const uint64_t db = smem_desc(sa + a_bytes, 128, kPix16, 0);
#pragma unroll
      for (int k = 0; k < kKPix / 16; k++)
        umma_bf16_el(tmem, da + 16 * k, db + 16 * k, idesc, (i | k) != 0);
      umma_commit_el(&empty[s]);
    }
    umma_commit_el(&accf);
  }
  __syncwarp();

  const bool ok = mbar_wait(&accf, 0, &abort_flag, false);
  if (!ok) sg_raise(a.err, &abort_flag, kSgTimeout);
  tc_fence_after();
  if (ok && !abort_flag && nk > 0) {
    const int r = warp * 32 + lane;
    const int j = r / CWA;
    const bool valid = j < nq;
    const int q = q0 + j;
    const int tap = q / kchx;
    const int ci = (q - tap * kchx) * CWA + (r % CWA);
    const long long kdim = static_cast<long long>(a.taps) * a.cin;
    float *dst = a.dw + tap * a.cin + ci;
    for (int c = 0; c < a.cout; c += 16) {
      uint32_t v[16];
      tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c, v);
      tmem_ld_wait();
      if (valid) {
#pragma unroll
        for (int jj = 0; jj < 16; jj++) red_add_f32(dst + (c + jj) * kdim, __uint_as_float(v[jj]));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

__device__ __forceinline__ void red_add_v4(float *p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

// -------------------------------------------- weight grad, taps on M ----
// dW[co][tap][ci] = sum over pixels q of dY[q - off(tap)][co] * X[q][ci]:
// M = (tap of the CTA's tap group, co) (ntap*cout <= 128 rows), N = ci,
// K = 128 pixels per step. Each tap's dY operand is its own TMA box taken at
// the shifted coordinates (outside the image it reads zeros, where the
// forward convolution's padding was), so the taps' planes stack at one
// stride; X's planes are loaded once per step for every tap of the group.
// Both operands MN-major without swizzle. Rows of M beyond the group's taps
// hold whatever the stage held and are never read back. With db, N has 16
// more columns whose X planes hold ones (written once, never loaded): for
// the centre tap (offset 0) they are the bias gradient sum over q of
// dY[q][co].
struct WgradTapsArgs {
  int H, W, BW, BH, tiles_x, tiles_y, cin, cout, taps, per, stages, ksteps, kper;
  int kpix;   // pixels per K step (128, or 64 where that lets two CTAs share an SM)
  float *dw;
  float *db;  // or null
  int *err;
};

__global__ void __launch_bounds__(kWgradThreads, 1)
    k_wgrad_taps(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmy,
                 const WgradTapsArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full, done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int kPlane = a.kpix * 16;     // one plane of a K step's pixels
  const int yp = a.cout / 8, xp = a.cin / 8;
  // M's planes: the group's taps' dY planes; the MMA reads 16 planes (128
  // rows) from the stage's start, the rows beyond the taps reading the X
  // planes that follow (discarded), so the region is at least 16 planes
  // less X's
  const int a_planes = max(a.per * yp, 16 - xp - (a.db ? 2 : 0));
  const int a_bytes = a_planes * kPlane;
  const int stage_bytes = a_bytes + (xp + (a.db ? 2 : 0)) * kPlane;
  const int S = a.stages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nb = a.cin + (a.db ? 16 : 0);  // N: input channels (+ the ones)
  const uint32_t cols = pow2_cols(static_cast<uint32_t>(nb));
  const int tap0 = blockIdx.x * a.per;
  const int ntap = min(a.per, a.taps - tap0);
  const int centre = a.taps == 9 ? 4 : 0;
  if (a.db) {
    // the ones planes of X (bf16 1.0 = 0x3F80) in every stage, made visible
    // to the tensor cores by the proxy fence below
    for (int st = 0; st < S; st++) {
      uint4 *o = reinterpret_cast<uint4 *>(smem + st * stage_bytes + a_bytes + xp * kPlane);
      for (int i = threadIdx.x; i < 2 * kPlane / 16; i += blockDim.x)
        o[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    }
  }

  if (threadIdx.x == 0) {
    for (int st = 0; st < S; st++) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tma_prefetch(&tmx);
    tma_prefetch(&tmy);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    tmem_alloc(&tmem_slot, cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int tiles_img = a.tiles_x * a.tiles_y;
  const int k_lo = blockIdx.y * a.kper;
  const int k_hi = min(a.ksteps, k_lo + a.kper);
  const int nk = k_hi - k_lo;

  if (warp == 0) {
    // producer (the whole warp; one lane issues)
    int issued = 0;
    const uint32_t tx = static_cast<uint32_t>((ntap * yp + xp) * kPlane);
    for (int i = 0; i < nk; i++) {
      const int st = i % S;
      if (!mbar_wait_warp(&empty[st], ((i / S) & 1) ^ 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      const int kt = k_lo + i;
      const int b = kt / tiles_img, t = kt - b * tiles_img;
      const int y0 = (t / a.tiles_x) * a.BH, x0 = (t % a.tiles_x) * a.BW;
      unsigned char *sa = smem + st * stage_bytes;
      mbar_expect_tx_el(&full[st], tx);
      for (int j = 0; j < ntap; j++) {
        const int tap = tap0 + j;
        const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
        tma_load_4d_el(sa + j * yp * kPlane, &tmy, &full[st], 2 * (x0 - dx), y0 - dy, 0, b);
      }
      tma_load_4d_el(sa + a_bytes, &tmx, &full[st], 2 * x0, y0, 0, b);
      issued = i + 1;
    }
    for (int i = issued > S ? issued - S : 0; i < issued; i++)
      if (!mbar_wait_warp(&full[i % S], (i / S) & 1, &abort_flag, false)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
  } else if (warp == 1) {
    // MMA issuer (the whole warp; one lane issues)
    const uint32_t idesc = idesc_bf16(nb, 1, 1);
    for (int i = 0; i < nk; i++) {
      const int st = i % S;
      if (!mbar_wait_warp(&full[st], (i / S) & 1, &abort_flag, true)) {
        sg_raise(a.err, &abort_flag, kSgTimeout);
        break;
      }
      tc_fence_after();
      const uint32_t sa = su32(smem + st * stage_bytes);
      // MN-major, no swizzle: MN chunks (planes) kPlane apart, 8-pixel K
      // groups 128 bytes apart; 16 pixels per MMA
      const uint64_t da = smem_desc(sa, 128, kPlane, 0);
      const uint64_t db = smem_desc(sa + a_bytes, 128, kPlane, 0);
      for (int k = 0; k < a.kpix / 16; k++)
        umma_bf16_el(tmem, da + 16 * k, db + 16 * k, idesc, (i | k) != 0);
      umma_commit_el(&empty[st]);
    }
    umma_commit_el(&acc_full);
    umma_commit_el(&done);
    if (!mbar_wait_warp(&done, 0, &abort_flag, false)) sg_raise(a.err, &abort_flag, kSgTimeout);
  } else if (nk > 0) {
    const int q = warp & 3;
    const int m = q * 32 + lane;
    const int j = m / a.cout, co = m - j * a.cout;
    const bool ok = mbar_wait(&acc_full, 0, &abort_flag, true);
    if (!ok) sg_raise(a.err, &abort_flag, kSgTimeout);
    tc_fence_after();
    if (ok && !abort_flag) {
      float *dst = a.dw + (static_cast<long long>(co) * a.taps + tap0 + j) * a.cin;
      for (int c = 0; c < a.cin; c += 16) {
        uint32_t v[16];
        tmem_ld16(tmem + (static_cast<uint32_t>(q * 32) << 16) + c, v);
        tmem_ld_wait();
        if (j < ntap) {
#pragma unroll
          for (int u = 0; u < 16; u += 4)
            red_add_v4(dst + c + u, __uint_as_float(v[u]), __uint_as_float(v[u + 1]),
                       __uint_as_float(v[u + 2]), __uint_as_float(v[u + 3]));
        }
      }
      if (a.db && tap0 <= centre && centre < tap0 + ntap) {
        uint32_t v[16];
        tmem_ld16(tmem + (static_cast<uint32_t>(q * 32) << 16) + a.cin, v);
        tmem_ld_wait();
        if (j == centre - tap0) red_add_f32(a.db + co, __uint_as_float(v[0]));
      }
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, cols);
  }
}

__global__ void k_flip_weights(const bf16 *__restrict__ w, bf16 *__restrict__ wd, int cout,
                               int cin, int taps) {
  const long long n = static_cast<long long>(cout) * taps * cin;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int ci = static_cast<int>(i % cin);
    const int tap = static_cast<int>((i / cin) % taps);
    const int co = static_cast<int>(i / (static_cast<long long>(cin) * taps));
    wd[(static_cast<long long>(ci) * taps + (taps - 1 - tap)) * cout + co] = w[i];
  }
}

// ------------------------------------------------------------- host ----

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

CUtensorMapSwizzle swizzle_of(int row_bytes) {
  return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
         : row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                           : CU_TENSOR_MAP_SWIZZLE_32B;
}

// Boxes of a plane-major tensor viewed as 64-bit elements (2 per pixel of a
// plane row), without swizzle: dims {2W, H, C/8, B}; box {e0, bh, np, 1} =
// e0/2 pixels of bh rows of np planes, stored in shared memory plane after
// plane (a box row of e0 elements is one run of e0*8 bytes).
cudaError_t map_act(CUtensorMap *m, const Act &t, int e0, int bh, int np) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[4] = {2 * static_cast<cuuint64_t>(t.W), static_cast<cuuint64_t>(t.H),
                              static_cast<cuuint64_t>(t.C / 8), static_cast<cuuint64_t>(t.B)};
  const cuuint64_t hw16 = static_cast<cuuint64_t>(t.W) * t.H * 16;
  // byte strides of dims 1..3: a row, a plane, an image
  const cuuint64_t strides[3] = {static_cast<cuuint64_t>(t.W) * 16, hw16,
                                 hw16 * static_cast<cuuint64_t>(t.C / 8)};
  const cuuint32_t box[4] = {static_cast<cuuint32_t>(e0), static_cast<cuuint32_t>(bh),
                             static_cast<cuuint32_t>(np), 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, t.p, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// {cb, bn} boxes of a [rows][cols] BF16 matrix.
cudaError_t map_mat(CUtensorMap *m, const bf16 *p, int rows, int cols, int cb, int bn) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(cols) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(cb), static_cast<cuuint32_t>(bn)};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(p), dims,
                         strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(cb * 2),
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

PixTile pixel_tile(int H, int W) {
  PixTile pt;
  if (W <= 0 || H <= 0) return pt;
  if (W >= kM) {
    if (W % kM) return pt;
    pt.BW = kM;
    pt.BH = 1;
  } else {
    if (kM % W) return pt;
    pt.BW = W;
    pt.BH = kM / W;
    if (H % pt.BH) return pt;
  }
  pt.tiles_x = W / pt.BW;
  pt.tiles_y = H / pt.BH;
  pt.ok = true;
  return pt;
}

cudaError_t plan_conv(ConvPlan &p, const Act &src, const bf16 *w, int taps, int ntot,
                      const float *bias, int relu, const bf16 *mask, bf16 *out,
                      const char **why, int out_planes, int out_up) {
  const char *dummy;
  if (!why) why = &dummy;
  p = ConvPlan{};
  if (out_planes && (out_planes < ntot / 8 || mask))
    return *why = "an output inside a wider tensor needs room for ntot channels and no mask",
           cudaErrorInvalidValue;
  if (out_up && mask) return *why = "an upsampled output takes no mask", cudaErrorInvalidValue;
  p.up = out_up ? 1 : 0;
  p.pt = pixel_tile(src.H, src.W);
  if (!p.pt.ok) return *why = "image width must divide or be a multiple of 128", cudaErrorInvalidValue;
  if (src.C % 16 || src.C <= 0) return *why = "source channels must be a multiple of 16", cudaErrorInvalidValue;
  if (taps != 1 && taps != 9) return *why = "taps must be 1 or 9", cudaErrorInvalidValue;
  if (ntot % 16 || ntot <= 0) return *why = "output channels must be a multiple of 16", cudaErrorInvalidValue;
  if (bias && ntot > kMaxBias) return *why = "at most 512 biased output channels", cudaErrorInvalidValue;
  if (!aligned16(src.p) || !aligned16(w) || !aligned16(out) || (mask && !aligned16(mask)))
    return *why = "tensors must be 16-byte aligned", cudaErrorInvalidValue;
  // N tile: the whole output up to 128 channels or at exactly 256 (MMAs of
  // N = 256 run at the tensor cores' full rate), else the largest divisor
  // <= 128 that is a multiple of 16 (an N tile of at most 128 columns lets
  // two CTAs per SM double-buffer their accumulators in half the TMEM: the
  // data gradients to 192 and 384 channels run 25% faster split so)
  int bn = ntot;
  if (bn > 128 && bn != 256) {
    bn = 0;
    for (int c = 128; c >= 16; c -= 16)
      if (ntot % c == 0) {
        bn = c;
        break;
      }
  }
  p.oplanes = out_planes ? out_planes : ntot / 8;
  p.B = src.B;
  p.H = src.H;
  p.W = src.W;
  p.cin = src.C;
  p.taps = taps;
  p.ntot = ntot;
  p.bn = bn;
  p.cb = channel_block(src.C);
  const size_t stage = (static_cast<size_t>(kM) * p.cb * 2 + static_cast<size_t>(bn) * p.cb * 2 + 1023) &
                       ~static_cast<size_t>(1023);
  int S = static_cast<int>(kSmemBudget / stage);
  if (S > kMaxStages) S = kMaxStages;
  const int nkb = taps * (src.C / p.cb);
  if (S > nkb) S = nkb < 2 ? 2 : nkb;
  if (S < 2) return *why = "stage does not fit shared memory", cudaErrorInvalidValue;
  p.stages = S;
  p.smem = S * stage + 1024;
  p.cps = 1;
  p.nbuf = acc_bufs(bn);
  // Two CTAs per SM (two pipelines interleaving their waits) where each fits
  // half the shared memory with a ring of at least three stages and half the
  // TMEM with at least two accumulator buffers.
  {
    const int nb2 = static_cast<int>(256 / acc_cols(bn)) < kMaxAccBufs
                        ? static_cast<int>(256 / acc_cols(bn)) : kMaxAccBufs;
    int S2 = static_cast<int>((kPairSmem - 1024) / stage);
    if (S2 > kMaxStages) S2 = kMaxStages;
    if (S2 > nkb) S2 = nkb;
    if (nb2 >= 2 && S2 >= 3) {
      p.cps = 2;
      p.nbuf = nb2;
      p.stages = S2;
      p.smem = S2 * stage + 1024;
    }
    const int nb3 = static_cast<int>(128 / acc_cols(bn)) < kMaxAccBufs
                        ? static_cast<int>(128 / acc_cols(bn)) : kMaxAccBufs;
    int S3 = static_cast<int>((kTripleSmem - 1024) / stage);
    if (S3 > kMaxStages) S3 = kMaxStages;
    if (S3 > nkb) S3 = nkb;
    if (nb3 >= 2 && S3 >= 3) {
      p.cps = 3;
      p.nbuf = nb3;
      p.stages = S3;
      p.smem = S3 * stage + 1024;
    }
  }
  // the planar form: wide images, 3x3 taps, one N tile whose weights fit
  // beside a ring of at least two stages and the guard
  {
    const size_t wbytes = (static_cast<size_t>(9) * src.C * bn * 2 + 1023) & ~static_cast<size_t>(1023);
    const size_t stage_a = (static_cast<size_t>(p.cb / 8) * kPlaneStride + 1023) & ~static_cast<size_t>(1023);
    const size_t room = kPlanarSmem - 1024 - kGuardBytes;
    const size_t stage_t = (static_cast<size_t>(p.cb / 8) * kTSlot + 1023) & ~static_cast<size_t>(1023);
    const size_t room_t = kTSmem - 1024 - 16 * 1024;  // slack: the weight tiles' extra rows read into it
    // the planar form with two CTAs per SM where it fits, else channels on M
    // (k_conv_t) where it applies, else the planar form with one CTA per SM
    const int nb2 = static_cast<int>(256 / acc_cols(bn)) < kMaxAccBufs
                        ? static_cast<int>(256 / acc_cols(bn)) : kMaxAccBufs;
    const size_t room2 = kPairSmem - 1024 - kGuardBytes;
    const bool planar_ok = taps == 9 && src.W >= kM && bn == ntot && wbytes + 2 * stage_a <= room;
    const bool planar_pair = planar_ok && nb2 >= 2 && wbytes + 3 * stage_a <= room2;
    if (!planar_pair && taps == 9 && src.W % kTN == 0 && bn == ntot && ntot <= kM && !mask &&
        src.C >= 64 && wbytes + 2 * stage_t <= room_t) {
      int St = static_cast<int>((room_t - wbytes) / stage_t);
      if (St > kMaxStages) St = kMaxStages;
      p.planar = 2;
      p.stages = St;
      p.smem = kTSmem;
      p.cps = 1;
    } else if (planar_ok) {
      int Sp = static_cast<int>((room - wbytes) / stage_a);
      if (Sp > kMaxStages) Sp = kMaxStages;
      p.planar = 1;
      p.stages = Sp;
      p.smem = wbytes + Sp * stage_a + kGuardBytes + 1024;
      p.cps = 1;
      p.nbuf = acc_bufs(bn);
      const int nb3 = static_cast<int>(128 / acc_cols(bn)) < kMaxAccBufs
                          ? static_cast<int>(128 / acc_cols(bn)) : kMaxAccBufs;
      const size_t room3 = kTripleSmem - 1024 - kGuardBytes;
      if (nb3 >= 2 && wbytes + 3 * stage_a <= room3) {
        int S3 = static_cast<int>((room3 - wbytes) / stage_a);
        if (S3 > kMaxStages) S3 = kMaxStages;
        p.cps = 3;
        p.nbuf = nb3;
        p.stages = S3;
        p.smem = wbytes + S3 * stage_a + kGuardBytes + 1024;
      } else if (planar_pair) {
        int S2 = static_cast<int>((room2 - wbytes) / stage_a);
        if (S2 > kMaxStages) S2 = kMaxStages;
        p.cps = 2;
        p.nbuf = nb2;
        p.stages = S2;
        p.smem = wbytes + S2 * stage_a + kGuardBytes + 1024;
      }
    }
  }
  p.bias = bias;
  p.relu = relu;
  p.mask = mask;
  p.out = out;
  p.grid_x = static_cast<int>(src.pixels() / kM);
  p.grid_y = ntot / bn;
  int dev = 0;
  cudaGetDevice(&dev);
  p.sms = 1;
  cudaDeviceGetAttribute(&p.sms, cudaDevAttrMultiProcessorCount, dev);
  if (p.sms < 1) p.sms = 1;
  cudaError_t e = p.planar ? map_act(&p.tma, src, 256, 1, 1)
                           : map_act(&p.tma, src, 2 * p.pt.BW, p.pt.BH, p.cb / 8);
  if (e == cudaSuccess && p.planar) e = map_act(&p.tmt, src, 4, 1, 1);
  if (e != cudaSuccess) return *why = "tensor map (source)", e;
  e = map_mat(&p.tmb, w, ntot, taps * src.C, p.cb, bn);
  if (e != cudaSuccess) return *why = "tensor map (weights)", e;
  return cudaSuccess;
}

// Splits `ksteps` pixel steps so that about three CTAs per SM run, each
// over at least 8 steps.
// Pixel splits of a weight gradient over `groups` row tiles with
// `resident` CTAs on the whole GPU at once: the count whose groups x splits
// CTAs fill whole rounds best (at most three rounds; a smaller count unless
// a larger one fills 2% better), each split at least 8 steps. (Three CTAs
// per SM regardless of what fits left 1.5 rounds for the two-per-SM forms
// and a few CTAs in a fourth round for the one-per-SM forms.)
int best_splits(int groups, int ksteps, int resident) {
  const int most = std::max(1, ksteps / 8);
  int best = 1;
  double beff = -1.0;
  for (int sp = 1; sp <= most && groups * sp <= 3 * resident; sp++) {
    const int tot = groups * sp;
    const int rounds = (tot + resident - 1) / resident;
    const double eff = static_cast<double>(tot) / (static_cast<double>(rounds) * resident);
    if (eff > beff + 0.02) {
      beff = eff;
      best = sp;
    }
  }
  return best;
}

void split_pixels(WgradPlan &p, int ksteps, int resident) {
  const int splits = best_splits(p.mtiles, ksteps, resident);
  p.kper = (ksteps + splits - 1) / splits;
  p.splits = (ksteps + p.kper - 1) / p.kper;
}

cudaError_t plan_wgrad(WgradPlan &p, const Act &x, const Act &dy, int taps, float *dw, int sms,
                       const char **why, float *db) {
  const char *dummy;
  if (!why) why = &dummy;
  p = WgradPlan{};
  if (x.B != dy.B || x.H != dy.H || x.W != dy.W)
    return *why = "X and dY must have the same pixel grid", cudaErrorInvalidValue;
  p.pt = pixel_tile(x.H, x.W);
  if (!p.pt.ok) return *why = "image width must divide or be a multiple of 128", cudaErrorInvalidValue;
  if (x.C % 16 || dy.C % 16 || dy.C > 256 || x.C <= 0 || dy.C <= 0)
    return *why = "channels must be multiples of 16, at most 256 output channels", cudaErrorInvalidValue;
  if (taps != 1 && taps != 9) return *why = "taps must be 1 or 9", cudaErrorInvalidValue;
  if (!aligned16(x.p) || !aligned16(dy.p) || !aligned16(dw))
    return *why = "tensors must be 16-byte aligned", cudaErrorInvalidValue;
  p.B = x.B;
  p.H = x.H;
  p.W = x.W;
  p.cin = x.C;
  p.cout = dy.C;
  p.taps = taps;
  p.cwa = channel_block(x.C);
  p.cwb = channel_block(dy.C);
  const size_t a_bytes = static_cast<size_t>(kM) * kKPix * 2;
  const size_t b_bytes = static_cast<size_t>(dy.C) * kKPix * 2;
  int S = static_cast<int>(kSmemBudget / (a_bytes + b_bytes));
  if (S > kMaxStages) S = kMaxStages;
  if (S < 2) return *why = "stage does not fit shared memory", cudaErrorInvalidValue;
  p.stages = S;
  p.smem = S * (a_bytes + b_bytes) + 1024;
  const int nchunk = taps * (x.C / p.cwa);
  p.mtiles = (nchunk + (kM / p.cwa) - 1) / (kM / p.cwa);
  p.ksteps = static_cast<int>(x.pixels() / kKPix);
  p.sms = sms;
  split_pixels(p, p.ksteps, sms);  // one CTA per SM (its shared memory holds no second)
  p.dw = dw;
  // taps on M for up to 128 output and 256 input channels (any pixel tile)
  if (dy.C <= kM && x.C <= 256) {
    const int g = kM / dy.C;                 // taps one 128-row tile holds
    const int ng = (taps + g - 1) / g;
    p.tap_per = (taps + ng - 1) / ng;        // balanced groups
    p.ngroups = (taps + p.tap_per - 1) / p.tap_per;
    const bool ones = db && x.C + 16 <= 256;  // the bias gradient rides along
    const int a_planes = std::max(p.tap_per * dy.C / 8, 16 - x.C / 8 - (ones ? 2 : 0));
    const size_t planes = a_planes + x.C / 8 + (ones ? 2 : 0);  // per stage (>= 16)
    const size_t stage = planes * kKPix * 16;
    int St = static_cast<int>(kSmemBudget / stage);
    if (St > kMaxStages) St = kMaxStages;
    if (St >= 2) {
      p.form = 2;
      p.db = ones ? db : nullptr;
      p.kpix = kKPix;
      p.stages = St;
      p.smem = St * stage + 1024;
      // two CTAs per SM: two stages of 128-pixel steps where they fit, else
      // for one-tap groups 64-pixel steps (planes of half the bytes) with at
      // least three stages (128 -> 128 channels: 0.22 -> 0.17 ms; with three
      // taps a step of four MMAs waits on four copies, 0.77 -> 1.00 ms)
      const size_t half = planes * 64 * 16;
      const uint32_t cols = pow2_cols(static_cast<uint32_t>(x.C + (ones ? 16 : 0)));
      // three CTAs per SM (static shared memory 288 bytes: 74 KB each fit)
      if (2 * stage + 1024 <= 74 * 1024 && cols <= 128) {
        p.stages = 2;
        p.smem = 2 * stage + 1024;
        p.cps = 3;
      } else if (2 * stage + 1024 <= kPairSmem + 6 * 1024) {
        p.stages = 2;
        p.smem = 2 * stage + 1024;
        p.cps = 2;
      } else if (p.tap_per == 1 && 3 * half + 1024 <= kPairSmem && x.W >= 64 && x.W % 64 == 0) {
        int S2 = static_cast<int>((kPairSmem - 1024) / half);
        if (S2 > kMaxStages) S2 = kMaxStages;
        p.kpix = 64;
        p.stages = S2;
        p.smem = S2 * half + 1024;
        p.cps = 2;
      }
      p.tpt = p.pt;
      if (p.kpix == 64) {
        p.tpt.BW = 64;
        p.tpt.BH = 1;
        p.tpt.tiles_x = x.W / 64;
        p.tpt.tiles_y = x.H;
      }
      cudaError_t e = map_act(&p.tmx, x, 2 * p.tpt.BW, p.tpt.BH, x.C / 8);
      if (e != cudaSuccess) return *why = "tensor map (X)", e;
      e = map_act(&p.tmy, dy, 2 * p.tpt.BW, p.tpt.BH, dy.C / 8);
      if (e != cudaSuccess) return *why = "tensor map (dY)", e;
      return cudaSuccess;
    }
  }
  cudaError_t e = map_act(&p.tmx, x, 2 * p.pt.BW, p.pt.BH, p.cwa / 8);
  if (e != cudaSuccess) return *why = "tensor map (X)", e;
  e = map_act(&p.tmy, dy, 2 * p.pt.BW, p.pt.BH, dy.C / 8);
  if (e != cudaSuccess) return *why = "tensor map (dY)", e;
  return cudaSuccess;
}

namespace {

template <int CB>
cudaError_t launch_conv_cb(const ConvPlan &p, int *err, cudaStream_t s, int nimg) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv<CB, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kSmemBudget + 1024));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_conv<CB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kTripleSmem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_conv_planar<CB, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kPlanarSmem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_conv_planar<CB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kTripleSmem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_conv_t<CB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kTSmem));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  ConvArgs a{};
  a.H = p.H;
  a.W = p.W;
  a.BW = p.pt.BW;
  a.BH = p.pt.BH;
  a.tiles_x = p.pt.tiles_x;
  a.tiles_y = p.pt.tiles_y;
  a.cin = p.cin;
  a.taps = p.taps;
  a.bn = p.bn;
  a.stages = p.stages;
  a.bias = p.bias;
  a.relu = p.relu;
  a.mask = p.mask;
  a.out = p.out;
  a.oplanes = p.oplanes;
  a.up = p.up;
  a.nbuf = p.nbuf;
  a.err = err;
  a.mtiles = nimg > 0 ? nimg * p.pt.tiles_x * p.pt.tiles_y : p.grid_x;
  a.ntiles = p.grid_y;
  if (p.planar == 2) a.mtiles = (nimg > 0 ? nimg : p.B) * p.H * (p.W / kTN);
  const int tiles = a.mtiles * a.ntiles;
  const int grid = tiles < p.cps * p.sms ? tiles : p.cps * p.sms;
  if (p.planar == 2)
    k_conv_t<CB><<<grid, kConvThreads, p.smem, s>>>(p.tma, p.tmt, p.tmb, a);
  else if (p.planar && p.cps == 3)
    k_conv_planar<CB, 1><<<grid, 64 + 128, p.smem, s>>>(p.tma, p.tmt, p.tmb, a);
  else if (p.planar)
    k_conv_planar<CB, 2><<<grid, 64 + 256, p.smem, s>>>(p.tma, p.tmt, p.tmb, a);
  else if (p.cps == 3)
    k_conv<CB, 1><<<grid, 64 + 128, p.smem, s>>>(p.tma, p.tmb, a);
  else
    k_conv<CB, 2><<<grid, 64 + 256, p.smem, s>>>(p.tma, p.tmb, a);
  return cudaGetLastError();
}

template <int CWA, int CWB>
cudaError_t launch_wgrad_cw(const WgradPlan &p, int *err, cudaStream_t s, int nimg) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_wgrad<CWA, CWB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kSmemBudget + 1024));
    // the largest shared-memory carveout, which the occupancy calculator
    // then assumes as the launches get it
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_wgrad<CWA, CWB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               static_cast<int>(cudaSharedmemCarveoutMaxShared));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  WgradArgs a{};
  a.H = p.H;
  a.W = p.W;
  a.BW = p.pt.BW;
  a.BH = p.pt.BH;
  a.tiles_x = p.pt.tiles_x;
  a.tiles_y = p.pt.tiles_y;
  a.cin = p.cin;
  a.cout = p.cout;
  a.taps = p.taps;
  a.nchunk = p.taps * (p.cin / p.cwa);
  a.stages = p.stages;
  WgradPlan q = p;
  split_pixels(q, nimg > 0 ? nimg * p.pt.tiles_x * p.pt.tiles_y : p.ksteps, p.cps * p.sms);
  a.ksteps = nimg > 0 ? nimg * p.pt.tiles_x * p.pt.tiles_y : p.ksteps;
  a.kper = q.kper;
  a.dw = p.dw;
  a.err = err;
  k_wgrad<CWA, CWB><<<dim3(p.mtiles, q.splits), kThreads, p.smem, s>>>(p.tmx, p.tmy, a);
  return cudaGetLastError();
}

template <int CWA>
cudaError_t launch_wgrad_a(const WgradPlan &p, int *err, cudaStream_t s, int nimg) {
  switch (p.cwb) {
    case 64: return launch_wgrad_cw<CWA, 64>(p, err, s, nimg);
    case 32: return launch_wgrad_cw<CWA, 32>(p, err, s, nimg);
    default: return launch_wgrad_cw<CWA, 16>(p, err, s, nimg);
  }
}

}  // namespace

cudaError_t launch_conv(const ConvPlan &p, int *err, cudaStream_t s, int nimg) {
  if (p.grid_x <= 0 || nimg < 0 || nimg > p.B) return cudaErrorInvalidValue;
  switch (p.cb) {
    case 64: return launch_conv_cb<64>(p, err, s, nimg);
    case 32: return launch_conv_cb<32>(p, err, s, nimg);
    default: return launch_conv_cb<16>(p, err, s, nimg);
  }
}

cudaError_t launch_wgrad_taps(const WgradPlan &p, int *err, cudaStream_t s, int nimg) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_wgrad_taps, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kSmemBudget + 1024));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_wgrad_taps, cudaFuncAttributePreferredSharedMemoryCarveout,
                               static_cast<int>(cudaSharedmemCarveoutMaxShared));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  WgradTapsArgs a{};
  a.H = p.H;
  a.W = p.W;
  a.BW = p.tpt.BW;
  a.BH = p.tpt.BH;
  a.tiles_x = p.tpt.tiles_x;
  a.tiles_y = p.tpt.tiles_y;
  a.cin = p.cin;
  a.cout = p.cout;
  a.taps = p.taps;
  a.per = p.tap_per;
  a.stages = p.stages;
  a.kpix = p.kpix;
  a.ksteps = (nimg > 0 ? nimg : p.B) * p.tpt.tiles_x * p.tpt.tiles_y;
  // whole rounds of the CTAs the plan sized to share an SM (shared memory,
  // TMEM) over the tap groups, each split over >= 8 steps
  int splits = best_splits(p.ngroups, a.ksteps, p.cps * p.sms);
  a.kper = (a.ksteps + splits - 1) / splits;
  splits = (a.ksteps + a.kper - 1) / a.kper;
  a.dw = p.dw;
  a.db = p.db;
  a.err = err;
  k_wgrad_taps<<<dim3(p.ngroups, splits), kWgradThreads, p.smem, s>>>(p.tmx, p.tmy, a);
  return cudaGetLastError();
}

cudaError_t launch_wgrad(const WgradPlan &p, int *err, cudaStream_t s, int nimg) {
  if (p.mtiles <= 0 || nimg < 0 || nimg > p.B) return cudaErrorInvalidValue;
  if (p.form == 2) return launch_wgrad_taps(p, err, s, nimg);
  switch (p.cwa) {
    case 64: return launch_wgrad_a<64>(p, err, s, nimg);
    case 32: return launch_wgrad_a<32>(p, err, s, nimg);
    default: return launch_wgrad_a<16>(p, err, s, nimg);
  }
}

cudaError_t launch_flip_weights(const bf16 *w, bf16 *wd, int cout, int cin, int taps,
                                cudaStream_t s) {
  const long long n = static_cast<long long>(cout) * taps * cin;
  int blocks = static_cast<int>((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_flip_weights<<<blocks, 256, 0, s>>>(w, wd, cout, cin, taps);
  return cudaGetLastError();
}

}  // namespace sg
