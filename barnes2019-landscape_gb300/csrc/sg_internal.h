// sg_internal.h -- the learned surrogate's device building blocks, shared by
// the convolution kernels (sg_conv.cu), the network (sg_net.cu) and the
// judged ensemble (sg_ensemble.cu). Not part of the public ABI.
//
// Activations are plane-major BF16 tensors [B][C/8][H][W][8]: a plane holds
// 8 channels of one image, 16 bytes per pixel, so a row of a plane is one
// contiguous run that a TMA box reads in full lines, and 8 consecutive
// pixels of a plane are exactly one 128-byte core matrix of the tensor
// cores' no-swizzle operand layouts (C a multiple of 16). Weights of a 3x3
// (or 1x1) convolution are BF16 [cout][tap][cin] with tap = 3*dy + dx (the
// GEMM's K dimension tap*cin + ci contiguous), kept with an FP32 master
// copy; weight gradients are FP32 in the same layout.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace sg {

using bf16 = __nv_bfloat16;

// Error codes written to the device error word (0 = none).
enum SgErr : int {
  kSgOk = 0,
  kSgTimeout = 1,  // an mbarrier wait ran out (producer, MMA or epilogue)
};

// A plane-major activation tensor on the device.
struct Act {
  bf16 *p = nullptr;
  int B = 0, H = 0, W = 0, C = 0;
  long long pixels() const { return static_cast<long long>(B) * H * W; }
  size_t bytes() const { return static_cast<size_t>(pixels()) * C * sizeof(bf16); }
};

// Element offset of channels [8*plane, 8*plane + 8) of pixel pix (y*W + x)
// of image b in a plane-major tensor with `planes` planes per image of hw
// pixels.
__host__ __device__ inline long long plane_at(int b, int plane, long long pix, int planes,
                                              long long hw) {
  return ((static_cast<long long>(b) * planes + plane) * hw + pix) * 8;
}

// Channels one K-block (one TMA box of planes) of a tensor with C channels
// spans: 64 when C is a multiple of 64, else 32, else 16; the weights' box
// of the same K-block has 128-, 64- or 32-byte swizzled rows.
inline int channel_block(int C) { return C % 64 == 0 ? 64 : C % 32 == 0 ? 32 : 16; }

// Pixel tile of 128 pixels of one image: BW x BH with BW = min(W, 128).
struct PixTile {
  int BW = 0, BH = 0, tiles_x = 0, tiles_y = 0;
  bool ok = false;
};
PixTile pixel_tile(int H, int W);

// A forward (or data-gradient) convolution prepared for launches: the tensor
// maps of its source and weights, the tile shape and the epilogue.
struct ConvPlan {
  // source planes viewed as 64-bit elements: box {2*BW, BH, cb/8, 1} (planar:
  // {256, 1, 1, 1}, one plane row from x0-1, with tmt's {4, 1, 1, 1} tail)
  CUtensorMap tma;
  CUtensorMap tmt;
  CUtensorMap tmb;  // weights [ntot][taps*cin], box {cb, bn}
  int B = 0, H = 0, W = 0, cin = 0, taps = 9, ntot = 0, bn = 0, cb = 0, stages = 0;
  PixTile pt;
  const float *bias = nullptr;  // [ntot] or null
  int relu = 0;
  const bf16 *mask = nullptr;   // output zeroed where mask <= 0 (or null; ntot channels)
  bf16 *out = nullptr;          // ntot channels
  int oplanes = 0;              // planes per image of out: ntot / 8, or more when out is
                                // a run of planes inside a wider tensor
  int up = 0;                   // 1: out is 2H x 2W, each output pixel stored into its
                                // 2x2 block (nearest-neighbour upsampling)
  size_t smem = 0;
  int grid_x = 0, grid_y = 0;  // pixel tiles and N tiles
  int sms = 1;                 // SMs of the device
  int cps = 1;                 // persistent CTAs per SM (1, 2, or 3 with one epilogue group)
  int nbuf = 2;                // TMEM accumulator buffers per CTA
  int planar = 0;              // resident weights with row staging: 1 pixels on M (k_conv_planar),
                               // 2 channels on M and 256 pixels on N (k_conv_t)
};

// A weight-gradient convolution prepared for launches: dW[co][tap][ci] +=
// sum over pixels of dY[p][co] * X[p + off(tap)][ci]; the taps-on-M kernel
// (k_wgrad_taps) where it fits, else the (tap, ci)-on-M kernel (k_wgrad).
struct WgradPlan {
  // X and dY planes viewed as 64-bit elements: X box {2*BW, BH, cwa/8, 1}
  // (taps form: {2*BW, BH, cin/8, 1}), dY box {2*BW, BH, cout/8, 1}
  CUtensorMap tmx;
  CUtensorMap tmy;
  int B = 0, H = 0, W = 0, cin = 0, cout = 0, taps = 9, cwa = 0, cwb = 0, stages = 0;
  PixTile pt;
  int mtiles = 0, splits = 0, ksteps = 0, kper = 0, sms = 1;
  float *dw = nullptr;
  size_t smem = 0;
  // taps-on-M form (form 2: at most 128 output and 256 input channels):
  // ngroups groups of tap_per taps, one CTA row of the grid each
  int form = 0, ngroups = 0, tap_per = 0;
  int kpix = 128;  // taps form: pixels per K step, and their tile
  PixTile tpt;
  float *db = nullptr;  // taps form: bias gradient accumulated too (else null)
  int cps = 1;          // CTAs per SM its shared memory and TMEM are sized for
};

// Builds a plan; returns cudaErrorInvalidValue (with a message in *why) for
// shapes the kernels do not take. Source and output tensors must stay
// allocated for the plan's lifetime. out_planes > 0 writes the output into
// ntot/8 planes of a tensor with out_planes planes per image, from `out`
// (which then points at the first of them in image 0); out_up != 0 writes
// it upsampled 2x (nearest) into an output of 2H x 2W pixels. No mask with
// either.
cudaError_t plan_conv(ConvPlan &p, const Act &src, const bf16 *w, int taps, int ntot,
                      const float *bias, int relu, const bf16 *mask, bf16 *out,
                      const char **why, int out_planes = 0, int out_up = 0);
// db (optional): where the bias gradient goes; the plan's db is non-null
// when its launches accumulate it (else the caller sums it separately).
cudaError_t plan_wgrad(WgradPlan &p, const Act &x, const Act &dy, int taps, float *dw, int sms,
                       const char **why, float *db = nullptr);
// nimg > 0 runs the plan over the first nimg images only (the tensor maps
// cover the plan's full batch).
cudaError_t launch_conv(const ConvPlan &p, int *err, cudaStream_t s, int nimg = 0);
cudaError_t launch_wgrad(const WgradPlan &p, int *err, cudaStream_t s, int nimg = 0);

// Flipped, transposed weights for the data gradient:
// wd[ci][8 - tap][co] = w[co][tap][ci] (taps = 9), wd[ci][0][co] = w[co][0][ci] (taps = 1).
cudaError_t launch_flip_weights(const bf16 *w, bf16 *wd, int cout, int cin, int taps,
                                cudaStream_t s);

}  // namespace sg
