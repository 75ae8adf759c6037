// sg_ops.cu -- the surrogate network's memory-bound kernels: input planes,
// 2x2 pooling and its adjoint, upsample-and-concatenate and its adjoint, the
// 1x1 output head with the loss and its gradient, bias gradients, Adam, and
// the jump that applies a prediction to an FP64 elevation field. All
// plane-major BF16 tensors ([B][C/8][H][W][8]) move one pixel of one plane
// (8 channels, 16 bytes) per access, consecutive threads on consecutive
// pixels of a plane.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sg_ops.h"

namespace sg {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void load8(const bf16 *p, float (&f)[8]) {
  const uint4 v = *reinterpret_cast<const uint4 *>(p);
  const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&v);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float2 t = __bfloat1622float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}

__device__ __forceinline__ void store8(bf16 *p, const float (&f)[8]) {
  uint4 v;
  __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&v);
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  *reinterpret_cast<uint4 *>(p) = v;
}

// Index arithmetic of the network kernels is 32-bit: their launchers refuse
// tensors of 2^31 or more 16-byte groups (a batch of 32 planes of 512^2 has
// 2^23 pixels).
constexpr long long kMaxGroups = 1ll << 31;

bool fits32(long long n) { return n >= 0 && n < kMaxGroups; }

int blocks_for(long long n) {
  long long b = (n + kBlock - 1) / kBlock;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : static_cast<int>(b);
}

// ring cells (the halo and the base-level ring) never change
__device__ __forceinline__ bool interior(int x, int y, int W, int H) {
  return x >= 2 && y >= 2 && x < W - 2 && y < H - 2;
}

__device__ __forceinline__ float field_at(const SampleView &v, int src, long long hw,
                                          long long pix) {
  return v.h64 ? static_cast<float>(v.h64[src][pix]) : v.h32[src * hw + pix];
}

__device__ __forceinline__ float count_plane(uint32_t c) {
  return log2f(static_cast<float>(c > 0u ? c : 1u)) * 0.0625f;
}

// All plane arithmetic is FP32 on FP32 heights (no FP64 on the narrow FP64
// pipe; -fmad=false keeps every operation separately rounded).
__global__ void k_input(const SampleView v, bf16 *__restrict__ in, float *__restrict__ yt, int W,
                        int H) {
  const unsigned hw = static_cast<unsigned>(W) * static_cast<unsigned>(H);
  const unsigned n = hw * static_cast<unsigned>(v.n);
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const int b = static_cast<int>(i / hw);
    const unsigned pix = i - static_cast<unsigned>(b) * hw;
    const int y = static_cast<int>(pix / static_cast<unsigned>(W));
    const int x = static_cast<int>(pix - static_cast<unsigned>(y) * static_cast<unsigned>(W));
    const int src = v.idx ? v.idx[b] : b;
    const SampleMeta m = v.meta[src];
    const float h = field_at(v, src, hw, pix);
    float f[16];
    f[0] = h * m.inv_s;
    f[1] = m.log_su;
    f[2] = m.k_n;
    f[3] = m.m_n;
    f[4] = m.u_n;
    f[5] = interior(x, y, W, H) ? 0.0f : 1.0f;
    f[6] = v.a32 ? v.a32[src * hw + pix] : (v.cnt ? count_plane(v.cnt[b][pix]) : 0.0f);
#pragma unroll
    for (int j = 7; j < 16; j++) f[j] = 0.0f;
    if (x >= 1 && y >= 1 && x < W - 1 && y < H - 1) {
      // neighbours in the reference's order W, NW, N, NE, E, SE, S, SW
      const long long off[8] = {-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1};
      float nb[8];
#pragma unroll
      for (int k = 0; k < 8; k++) nb[k] = field_at(v, src, hw, pix + off[k]);
      float best = 0.0f, drop = 0.0f, sum = 0.0f;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const float d = h - nb[k];
        const float slope = (k & 1) ? d / 1.41421356f : d;
        if (slope > best) {
          best = slope;
          drop = d;
        }
        sum += nb[k];
      }
      f[7] = drop * m.inv_u;
      f[8] = (nb[4] - nb[0]) * 0.5f * m.inv_u;
      f[9] = (nb[6] - nb[2]) * 0.5f * m.inv_u;
      f[10] = (h - 0.125f * sum) * m.inv_u;
    }
    float lo[8], hi[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      lo[j] = f[j];
      hi[j] = f[8 + j];
    }
    store8(in + plane_at(b, 0, pix, 2, hw), lo);
    store8(in + plane_at(b, 1, pix, 2, hw), hi);
    if (yt) yt[i] = v.y ? v.y[static_cast<long long>(src) * hw + pix] : 0.0f;
  }
}

// out = 2x2 average of planes [ioff, ioff + C/8) of in (ip planes per image
// at twice the resolution); i runs over (image, plane) pairs and pixels of out
__global__ void k_avgpool2(const bf16 *__restrict__ in, int ip, int ioff, bf16 *__restrict__ out,
                           int B, int Ho, int Wo, int C) {
  const int po_ = C / 8;
  const unsigned hwo = static_cast<unsigned>(Ho) * static_cast<unsigned>(Wo);
  const long long Wi = 2ll * Wo;
  const unsigned n = static_cast<unsigned>(B) * po_ * hwo;
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const unsigned bp = i / hwo, po = i - bp * hwo;
    const int b = static_cast<int>(bp / static_cast<unsigned>(po_));
    const int pl = static_cast<int>(bp - static_cast<unsigned>(b) * po_);
    const int y = static_cast<int>(po / static_cast<unsigned>(Wo));
    const int x = static_cast<int>(po - static_cast<unsigned>(y) * static_cast<unsigned>(Wo));
    const bf16 *p = in + plane_at(b, ioff + pl, 2ll * y * Wi + 2 * x, ip, 4ll * hwo);
    float a[8], t[8];
    load8(p, a);
    load8(p + 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
    load8(p + Wi * 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
    load8(p + Wi * 8 + 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = 0.25f * (a[j] + t[j]);
    store8(out + static_cast<long long>(i) * 8, a);
  }
}

// gd[b, :, y, x] = sum over the 2x2 block of g[b, 0:Cd, 2y+i, 2x+j] (g has C
// channels at twice the resolution): the adjoint of nearest upsampling
__global__ void k_sumpool2(const bf16 *__restrict__ g, int C, bf16 *__restrict__ gd, int B,
                           int Ho, int Wo, int Cd) {
  const int pd = Cd / 8, pc = C / 8;
  const unsigned hwo = static_cast<unsigned>(Ho) * static_cast<unsigned>(Wo);
  const long long Wi = 2ll * Wo;
  const unsigned n = static_cast<unsigned>(B) * pd * hwo;
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const unsigned bp = i / hwo, po = i - bp * hwo;
    const int b = static_cast<int>(bp / static_cast<unsigned>(pd));
    const int pl = static_cast<int>(bp - static_cast<unsigned>(b) * pd);
    const int y = static_cast<int>(po / static_cast<unsigned>(Wo));
    const int x = static_cast<int>(po - static_cast<unsigned>(y) * static_cast<unsigned>(Wo));
    const bf16 *p = g + plane_at(b, pl, 2ll * y * Wi + 2 * x, pc, 4 * hwo);
    float a[8], t[8];
    load8(p, a);
    load8(p + 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
    load8(p + Wi * 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
    load8(p + Wi * 8 + 8, t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
    store8(gd + static_cast<long long>(i) * 8, a);
  }
}

// gs = gcat[:, Cd:Cd+Cs] + (s > 0) * gp(up) / 4: the skip tensor's gradient
// from the decoder (already masked) plus the pooling path's, masked by ReLU;
// s is read from the concatenation cat (same layout as gcat)
__global__ void k_skipgrad(const bf16 *__restrict__ gcat, int C, int Cd,
                           const bf16 *__restrict__ cat, const bf16 *__restrict__ gp,
                           bf16 *__restrict__ gs, int B, int H, int W, int Cs) {
  const int ps = Cs / 8, pc = C / 8, pd = Cd / 8;
  const unsigned hw = static_cast<unsigned>(H) * static_cast<unsigned>(W);
  const unsigned n = static_cast<unsigned>(B) * ps * hw;
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const unsigned bp = i / hw, pix = i - bp * hw;
    const int b = static_cast<int>(bp / static_cast<unsigned>(ps));
    const int j = static_cast<int>(bp - static_cast<unsigned>(b) * ps);
    const int y = static_cast<int>(pix / static_cast<unsigned>(W));
    const int x = static_cast<int>(pix - static_cast<unsigned>(y) * static_cast<unsigned>(W));
    float a[8], sv[8], pv[8];
    const long long at = plane_at(b, pd + j, pix, pc, hw);
    load8(gcat + at, a);
    load8(cat + at, sv);
    load8(gp + plane_at(b, j, static_cast<long long>(y / 2) * (W / 2) + x / 2, ps, hw / 4), pv);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (sv[k] > 0.0f) a[k] += 0.25f * pv[k];
    store8(gs + static_cast<long long>(i) * 8, a);
  }
}

// 1x1 head on the last decoder activation x (C channels): z = b + w.x;
// training: err = z - y on interior cells, the loss
//   L = (1/n) sum_s wgt_s * mean_interior(err^2),
// dz = dL/dz, gx = dz * w * (x > 0) (the ReLU of x), dw += dz * x, db += dz.
template <int C>
__global__ void __launch_bounds__(kBlock) k_head_train(const bf16 *__restrict__ x,
                                                       const float *__restrict__ hw_,
                                                       const float *__restrict__ yt,
                                                       const SampleView v, int W, int H,
                                                       bf16 *__restrict__ gx,
                                                       float *__restrict__ dwb,
                                                       double *__restrict__ loss) {
  __shared__ float s_w[C + 1];
  __shared__ float s_red[kBlock / 32][C + 2];
  if (threadIdx.x <= C) s_w[threadIdx.x] = hw_[threadIdx.x];
  __syncthreads();
  // 32-bit index arithmetic (a batch's pixels stay below 2^31) and FP32 per
  // pixel: the FP64 pipe is narrow on this part, the loss only a diagnostic
  const unsigned hwn = static_cast<unsigned>(W) * static_cast<unsigned>(H);
  const unsigned n = hwn * static_cast<unsigned>(v.n);
  const float inv_int = static_cast<float>(1.0 / (static_cast<double>(W - 4) * (H - 4) * v.n));
  float acc[C + 1];
#pragma unroll
  for (int j = 0; j <= C; j++) acc[j] = 0.0f;
  float lsum = 0.0f;
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const int b = static_cast<int>(i / hwn);
    const unsigned pix = i - static_cast<unsigned>(b) * hwn;
    const int py = static_cast<int>(pix / static_cast<unsigned>(W));
    const int px = static_cast<int>(pix - static_cast<unsigned>(py) * static_cast<unsigned>(W));
    float xv[C];
#pragma unroll
    for (int j = 0; j < C; j += 8) {
      float t[8];
      load8(x + plane_at(b, j / 8, pix, C / 8, hwn), t);
#pragma unroll
      for (int k = 0; k < 8; k++) xv[j + k] = t[k];
    }
    float z = s_w[C];
#pragma unroll
    for (int j = 0; j < C; j++) z += s_w[j] * xv[j];
    float dz = 0.0f;
    if (interior(px, py, W, H)) {
      const int src = v.idx ? v.idx[b] : b;
      const float wgt = v.meta[src].weight;
      const float err = z - yt[i];
      const float we = wgt * err * inv_int;
      lsum += we * err;
      dz = 2.0f * we;
    }
#pragma unroll
    for (int j = 0; j < C; j += 8) {
      float t[8];
#pragma unroll
      for (int k = 0; k < 8; k++) t[k] = xv[j + k] > 0.0f ? dz * s_w[j + k] : 0.0f;
      store8(gx + plane_at(b, j / 8, pix, C / 8, hwn), t);
    }
#pragma unroll
    for (int j = 0; j < C; j++) acc[j] += dz * xv[j];
    acc[C] += dz;
  }
  // block reduction: warp shuffles, then one row per warp in shared memory
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j <= C; j++) {
    float t = acc[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) s_red[warp][j] = t;
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) s_red[warp][C + 1] = lsum;
  __syncthreads();
  if (threadIdx.x <= C) {
    float t = 0.0f;
    for (int k = 0; k < kBlock / 32; k++) t += s_red[k][threadIdx.x];
    atomicAdd(dwb + threadIdx.x, t);
  }
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kBlock / 32; k++) t += s_red[k][C + 1];
    atomicAdd(loss, t);
  }
}

// inference: h_out = h_in + u * z on interior cells (FP64), rings unchanged
template <int C>
__global__ void __launch_bounds__(kBlock) k_head_apply(const bf16 *__restrict__ x,
                                                       const float *__restrict__ hw_,
                                                       const SampleView v, int W, int H,
                                                       double *const *__restrict__ hout) {
  __shared__ float s_w[C + 1];
  if (threadIdx.x <= C) s_w[threadIdx.x] = hw_[threadIdx.x];
  __syncthreads();
  const unsigned hwn = static_cast<unsigned>(W) * static_cast<unsigned>(H);
  const unsigned n = hwn * static_cast<unsigned>(v.n);
  for (unsigned i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const int b = static_cast<int>(i / hwn);
    const unsigned pix = i - static_cast<unsigned>(b) * hwn;
    const int py = static_cast<int>(pix / static_cast<unsigned>(W));
    const int px = static_cast<int>(pix - static_cast<unsigned>(py) * static_cast<unsigned>(W));
    const int src = v.idx ? v.idx[b] : b;
    const double h = v.h64[src][pix];
    double out = h;
    if (interior(px, py, W, H)) {
      float z = s_w[C];
#pragma unroll
      for (int j = 0; j < C; j += 8) {
        float t[8];
        load8(x + plane_at(b, j / 8, pix, C / 8, hwn), t);
#pragma unroll
        for (int k = 0; k < 8; k++) z += s_w[j + k] * t[k];
      }
      out = h + static_cast<double>(v.meta[src].u) * z;
    }
    hout[b][pix] = out;
  }
}

// db[8*pl + j] += sum over pixels of plane pl (blockIdx.y) of g
__global__ void __launch_bounds__(kBlock) k_bias_grad(const bf16 *__restrict__ g, int B,
                                                      long long hw, int planes,
                                                      float *__restrict__ db) {
  __shared__ float s_acc[kBlock / 32][8];
  const int pl = blockIdx.y;
  const long long n = static_cast<long long>(B) * hw;
  float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int b = static_cast<int>(i / hw);
    float t[8];
    load8(g + plane_at(b, pl, i - b * hw, planes, hw), t);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += t[j];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float t = a[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) s_acc[warp][j] = t;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    float t = 0.0f;
    for (int w = 0; w < kBlock / 32; w++) t += s_acc[w][threadIdx.x];
    atomicAdd(db + pl * 8 + threadIdx.x, t);
  }
}

// Adam (bias-corrected) on FP32 masters; conv weights also refresh their BF16
// copies: forward layout [cout][tap][cin] and the data-gradient layout
// [cin][taps-1-tap][cout]
// Adam over the whole parameter vector; an element inside a weight run
// also writes its BF16 forward and flipped copies
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, long long n, float lr_t, float b1, float b2,
                       float eps_t, const AdamRuns runs) {
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr_t * mi / (sqrtf(vi) + eps_t);
    p[i] = pi;
    for (int k = 0; k < runs.n; k++) {
      const int cin = runs.cin[k], taps = runs.taps[k], cout = runs.cout[k];
      const long long j = i - runs.off[k];
      if (j < 0 || j >= static_cast<long long>(cout) * taps * cin) continue;
      const bf16 q = __float2bfloat16_rn(pi);
      runs.wf[k][j] = q;
      const int ci = static_cast<int>(j % cin);
      const int tap = static_cast<int>((j / cin) % taps);
      const int co = static_cast<int>(j / (static_cast<long long>(cin) * taps));
      runs.wd[k][(static_cast<long long>(ci) * taps + (taps - 1 - tap)) * cout + co] = q;
      break;
    }
  }
}

__global__ void k_to_bf16(const float *__restrict__ p, long long n, bf16 *__restrict__ wf,
                          bf16 *__restrict__ wd, int cout, int cin, int taps) {
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const bf16 q = __float2bfloat16_rn(p[i]);
    wf[i] = q;
    const int ci = static_cast<int>(i % cin);
    const int tap = static_cast<int>((i / cin) % taps);
    const int co = static_cast<int>(i / (static_cast<long long>(cin) * taps));
    wd[(static_cast<long long>(ci) * taps + (taps - 1 - tap)) * cout + co] = q;
  }
}

// per-field maximum (one block per field; every field has hw cells)
__global__ void __launch_bounds__(kBlock) k_field_max(double *const *__restrict__ h64,
                                                      const float *__restrict__ h32,
                                                      long long hw, double *__restrict__ out) {
  const int f = blockIdx.x;
  double mx = -1e300;
  for (long long i = threadIdx.x; i < hw; i += kBlock) {
    const double t = h64 ? h64[f][i] : static_cast<double>(h32[f * hw + i]);
    mx = t > mx ? t : mx;
  }
  __shared__ double s[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    mx = s[0];
    for (int k = 1; k < kBlock / 32; k++) mx = fmax(mx, s[k]);
    out[f] = mx;
  }
}

// dataset record: h_t as FP32 and the target y = (h_next - h_t)/u (0 on the rings)
__global__ void k_record(double *const *__restrict__ ht, double *const *__restrict__ hn,
                         const int *__restrict__ slot, const float *__restrict__ u, int n, int W,
                         int H, float *__restrict__ dh, float *__restrict__ dy) {
  const long long hw = static_cast<long long>(W) * H;
  const long long tot = hw * n;
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < tot;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int k = static_cast<int>(i / hw);
    const long long pix = i - k * hw;
    const int x = static_cast<int>(pix % W), y = static_cast<int>(pix / W);
    const long long o = static_cast<long long>(slot[k]) * hw + pix;
    const double a = ht[k][pix];
    if (dh) dh[o] = static_cast<float>(a);
    if (dy) dy[o] = interior(x, y, W, H) ? static_cast<float>((hn[k][pix] - a) / u[k]) : 0.0f;
  }
}

// losses of the two jumps that need no network, with the training loss's
// weighting: uplift only (y_pred = 1) into out[0], no change (y_pred = 0)
// into out[1]
__global__ void __launch_bounds__(kBlock) k_baseline_loss(const SampleView v, int W, int H,
                                                          double *__restrict__ out) {
  const long long hw = static_cast<long long>(W) * H;
  const long long n = hw * v.n;
  const double inv_int = 1.0 / (static_cast<double>(W - 4) * (H - 4) * v.n);
  double a = 0.0, b = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int k = static_cast<int>(i / hw);
    const long long pix = i - k * hw;
    const int x = static_cast<int>(pix % W), y = static_cast<int>(pix / W);
    if (!interior(x, y, W, H)) continue;
    const int src = v.idx ? v.idx[k] : k;
    const double w = v.meta[src].weight;
    const double t = v.y[static_cast<long long>(src) * hw + pix];
    a += w * (1.0 - t) * (1.0 - t) * inv_int;
    b += w * t * t * inv_int;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, a);
    atomicAdd(out + 1, b);
  }
}

__global__ void k_count_plane(const uint32_t *const *__restrict__ cnt, const int *__restrict__ slot,
                              int n, long long hw, float *__restrict__ da) {
  const long long tot = hw * n;
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < tot;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int k = static_cast<int>(i / hw);
    const long long pix = i - k * hw;
    da[static_cast<long long>(slot[k]) * hw + pix] = count_plane(cnt[k][pix]);
  }
}

// copies FP64 fields (gather by pointer)
__global__ void k_copy_fields(double *const *__restrict__ src, double *const *__restrict__ dst,
                              int n, long long hw) {
  const long long tot = hw * n;
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < tot;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int k = static_cast<int>(i / hw);
    const long long pix = i - k * hw;
    dst[k][pix] = src[k][pix];
  }
}

}  // namespace

cudaError_t launch_input(const SampleView &v, bf16 *in, float *yt, int W, int H, cudaStream_t s) {
  // 16 planes per pixel: the input tensor's groups are the pixels times two
  if (!fits32(2ll * W * H * v.n)) return cudaErrorInvalidValue;
  k_input<<<blocks_for(static_cast<long long>(W) * H * v.n), kBlock, 0, s>>>(v, in, yt, W, H);
  return cudaGetLastError();
}

cudaError_t launch_avgpool2(const Act &in, int in_off, const Act &out, cudaStream_t s) {
  if (!fits32(in.pixels() * in.C / 8) || in_off < 0 || (in_off + out.C / 8) * 8 > in.C ||
      in.B != out.B || in.H != 2 * out.H || in.W != 2 * out.W)
    return cudaErrorInvalidValue;
  k_avgpool2<<<blocks_for(out.pixels() * out.C / 8), kBlock, 0, s>>>(
      in.p, in.C / 8, in_off, out.p, out.B, out.H, out.W, out.C);
  return cudaGetLastError();
}

cudaError_t launch_sumpool2(const Act &gcat, const Act &gd, cudaStream_t s) {
  if (!fits32(gcat.pixels() * gcat.C / 8)) return cudaErrorInvalidValue;
  k_sumpool2<<<blocks_for(gd.pixels() * gd.C / 8), kBlock, 0, s>>>(gcat.p, gcat.C, gd.p, gd.B,
                                                                   gd.H, gd.W, gd.C);
  return cudaGetLastError();
}

cudaError_t launch_skipgrad(const Act &gcat, int cd, const Act &cat, const Act &gp,
                            const Act &gs, cudaStream_t s) {
  if (!fits32(gcat.pixels() * gcat.C / 8) || cat.C != gcat.C || cat.H != gcat.H ||
      cat.W != gcat.W || cd + gs.C > gcat.C)
    return cudaErrorInvalidValue;
  k_skipgrad<<<blocks_for(gs.pixels() * gs.C / 8), kBlock, 0, s>>>(
      gcat.p, gcat.C, cd, cat.p, gp.p, gs.p, gs.B, gs.H, gs.W, gs.C);
  return cudaGetLastError();
}

cudaError_t launch_head_train(const Act &x, const float *head, const float *yt,
                              const SampleView &v, const Act &gx, float *dhead, double *loss,
                              cudaStream_t s) {
  if (!fits32(x.pixels() * x.C / 8)) return cudaErrorInvalidValue;
  const int blocks = blocks_for(x.pixels());
  switch (x.C) {
    case 16:
      k_head_train<16><<<blocks, kBlock, 0, s>>>(x.p, head, yt, v, x.W, x.H, gx.p, dhead, loss);
      break;
    case 32:
      k_head_train<32><<<blocks, kBlock, 0, s>>>(x.p, head, yt, v, x.W, x.H, gx.p, dhead, loss);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_head_apply(const Act &x, const float *head, const SampleView &v,
                              double *const *hout, cudaStream_t s) {
  if (!fits32(x.pixels() * x.C / 8)) return cudaErrorInvalidValue;
  const int blocks = blocks_for(x.pixels());
  switch (x.C) {
    case 16: k_head_apply<16><<<blocks, kBlock, 0, s>>>(x.p, head, v, x.W, x.H, hout); break;
    case 32: k_head_apply<32><<<blocks, kBlock, 0, s>>>(x.p, head, v, x.W, x.H, hout); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_bias_grad(const Act &g, float *db, cudaStream_t s) {
  if (g.C % 8 || g.C > 256) return cudaErrorInvalidValue;
  // per plane, at least 64 pixels per thread, about four blocks per SM in all
  const int planes = g.C / 8;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  long long bx = (g.pixels() + 64ll * kBlock - 1) / (64ll * kBlock);
  const long long cap = (4ll * sms + planes - 1) / planes;
  if (bx > cap) bx = cap;
  if (bx < 1) bx = 1;
  k_bias_grad<<<dim3(static_cast<unsigned>(bx), planes), kBlock, 0, s>>>(
      g.p, g.B, static_cast<long long>(g.H) * g.W, planes, db);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *p, const float *g, float *m, float *v, long long n, float lr_t,
                        float b1, float b2, float eps_t, const AdamRuns &runs, cudaStream_t s) {
  if (runs.n < 0 || runs.n > AdamRuns::kMax) return cudaErrorInvalidValue;
  k_adam<<<blocks_for(n), kBlock, 0, s>>>(p, g, m, v, n, lr_t, b1, b2, eps_t, runs);
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float *p, long long n, bf16 *wf, bf16 *wd, int cout, int cin,
                           int taps, cudaStream_t s) {
  k_to_bf16<<<blocks_for(n), kBlock, 0, s>>>(p, n, wf, wd, cout, cin, taps);
  return cudaGetLastError();
}

cudaError_t launch_field_max(double *const *h64, const float *h32, int nfields, long long hw,
                             double *out, cudaStream_t s) {
  k_field_max<<<nfields, kBlock, 0, s>>>(h64, h32, hw, out);
  return cudaGetLastError();
}

cudaError_t launch_record(double *const *ht, double *const *hn, const int *slot, const float *u,
                          int n, int W, int H, float *dh, float *dy, cudaStream_t s) {
  k_record<<<blocks_for(static_cast<long long>(W) * H * n), kBlock, 0, s>>>(ht, hn, slot, u, n, W,
                                                                            H, dh, dy);
  return cudaGetLastError();
}

cudaError_t launch_baseline_loss(const SampleView &v, int W, int H, double *out, cudaStream_t s) {
  k_baseline_loss<<<blocks_for(static_cast<long long>(W) * H * v.n), kBlock, 0, s>>>(v, W, H, out);
  return cudaGetLastError();
}

cudaError_t launch_count_plane(const uint32_t *const *cnt, const int *slot, int n, long long hw,
                               float *da, cudaStream_t s) {
  k_count_plane<<<blocks_for(hw * n), kBlock, 0, s>>>(cnt, slot, n, hw, da);
  return cudaGetLastError();
}

cudaError_t launch_copy_fields(double *const *src, double *const *dst, int n, long long hw,
                               cudaStream_t s) {
  k_copy_fields<<<blocks_for(hw * n), kBlock, 0, s>>>(src, dst, n, hw);
  return cudaGetLastError();
}

}  // namespace sg
