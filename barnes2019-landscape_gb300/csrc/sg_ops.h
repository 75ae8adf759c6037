// sg_ops.h -- launchers of the surrogate network's memory-bound kernels
// (sg_ops.cu). Not part of the public ABI.
#pragma once

#include "sg_internal.h"

namespace sg {

// Input planes of the network: 0 h/s, 1 log(s/u)/4, 2..4 K, m, U mapped to
// about [-1, 1], 5 ring mask (1 on the two outer rings), 6 log2(drainage
// count)/16, 7 drop to the D8 receiver / u, 8 and 9 central differences
// along x and y / (2u), 10 (h - mean of the 8 neighbours) / u, 11..15 zero.
// Planes 7..10 are 0 on ring 0 (no full neighbourhood). They are formed in
// FP32 from FP32 heights before the BF16 rounding, so slopes keep their
// precision however high the ground stands (h/s alone would quantise them
// to 2^-8 of s).
constexpr int kInputChannels = 16;

// Per-sample constants of one jump. s = max(max h, u) scales the heights,
// u = jump * U * dt is the jump's uplift (the target is (h_next - h)/u).
struct SampleMeta {
  float s, u, log_su, k_n, m_n, u_n, weight;
  float inv_s, inv_u;  // FP32 reciprocals of s and u
  float pad[3];
};

// The samples of one network pass: sample b reads field src = idx[b] (or b
// when idx is null) from h64[src] (FP64 device fields) or h32 + src*W*H,
// target y + src*W*H (training), constants meta[src].
struct SampleView {
  int n = 0;
  const int *idx = nullptr;
  const SampleMeta *meta = nullptr;
  double *const *h64 = nullptr;
  const float *h32 = nullptr;
  const float *y = nullptr;
  const float *a32 = nullptr;              // dataset: plane 6 per cell
  const uint32_t *const *cnt = nullptr;    // fields: drainage counts
};

cudaError_t launch_input(const SampleView &v, bf16 *in, float *yt, int W, int H, cudaStream_t s);
// out = 2x2 average of out.C channels of in from plane in_off on
cudaError_t launch_avgpool2(const Act &in, int in_off, const Act &out, cudaStream_t s);
cudaError_t launch_sumpool2(const Act &gcat, const Act &gd, cudaStream_t s);
// gs = gcat's channels [cd, cd + gs.C) + the pooling path's gp, masked where
// the skip tensor (those channels of cat) is not positive
cudaError_t launch_skipgrad(const Act &gcat, int cd, const Act &cat, const Act &gp,
                            const Act &gs, cudaStream_t s);
// head = [w_0 .. w_{C-1}, b] (FP32); dhead accumulates the same layout
cudaError_t launch_head_train(const Act &x, const float *head, const float *yt,
                              const SampleView &v, const Act &gx, float *dhead, double *loss,
                              cudaStream_t s);
cudaError_t launch_head_apply(const Act &x, const float *head, const SampleView &v,
                              double *const *hout, cudaStream_t s);
cudaError_t launch_bias_grad(const Act &g, float *db, cudaStream_t s);
// lr_t, eps_t: Adam's bias-corrected step size and epsilon; wf/wd (may be
// null): BF16 copies in the forward and data-gradient layouts
// The weight runs of a parameter vector with BF16 copies: run k is
// elements [off[k], off[k] + cout*taps*cin), weights [cout][tap][cin], whose
// forward copy goes to wf[k] and flipped copy ([cin][8 - tap][cout]) to wd[k].
struct AdamRuns {
  static constexpr int kMax = 16;
  int n = 0;
  long long off[kMax];
  bf16 *wf[kMax], *wd[kMax];
  int cout[kMax], cin[kMax], taps[kMax];
};
// One Adam step over the n elements of p (bias-corrected lr_t, eps_t), and
// the BF16 copies of the weight runs in one launch.
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, long long n, float lr_t,
                        float b1, float b2, float eps_t, const AdamRuns &runs, cudaStream_t s);
cudaError_t launch_to_bf16(const float *p, long long n, bf16 *wf, bf16 *wd, int cout, int cin,
                           int taps, cudaStream_t s);
cudaError_t launch_field_max(double *const *h64, const float *h32, int nfields, long long hw,
                             double *out, cudaStream_t s);
cudaError_t launch_record(double *const *ht, double *const *hn, const int *slot, const float *u,
                          int n, int W, int H, float *dh, float *dy, cudaStream_t s);
// plane 6 of fields k (drainage counts cnt[k]) into da + slot[k]*W*H
cudaError_t launch_count_plane(const uint32_t *const *cnt, const int *slot, int n, long long hw,
                               float *da, cudaStream_t s);
// the training loss of y_pred = 1 (uplift only) and y_pred = 0 (no change),
// added into out[0] and out[1]
cudaError_t launch_baseline_loss(const SampleView &v, int W, int H, double *out, cudaStream_t s);
cudaError_t launch_copy_fields(double *const *src, double *const *dst, int n, long long hw,
                               cudaStream_t s);

}  // namespace sg
