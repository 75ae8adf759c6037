// sg_net.cu -- the learned surrogate: network, device dataset, training and
// inference (include/fastscape_surrogate.h). The convolutions run on the
// tensor-core kernels of sg_conv.cu, everything else on sg_ops.cu; the host
// side here only plans, wires and launches, all on the network's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "fastscape_gb300.h"
#include "fastscape_surrogate.h"
#include "fs_internal.h"
#include "sg_net.h"

namespace {

int fail(int status, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return fs::record_error(status, buf);
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA, "surrogate: %s: %s",
              what, cudaGetErrorString(e));
}

#define SG_CUDA(x)                                          \
  do {                                                      \
    cudaError_t e_ = (x);                                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);        \
  } while (0)

constexpr double kLog10UMid = -3.1505;   // log10 of sqrt(1e-4 * 5e-3)
constexpr double kLog10UHalf = 0.8495;   // half the range of log10 U

}  // namespace

// ------------------------------------------------------------ helpers ----
namespace sg {

SampleMeta make_meta(const fs_params &p, double hmax, double hmax_next, int jump, double dt) {
  SampleMeta m{};
  const double u = jump * p.ueq * dt;
  const double s = std::max(hmax, u);
  m.s = static_cast<float>(s);
  m.u = static_cast<float>(u);
  m.log_su = static_cast<float>(std::log(s / u) / 4.0);
  m.k_n = static_cast<float>((std::log10(p.keq) + 5.5) / 0.5);
  m.m_n = static_cast<float>((p.meq - 0.45) / 0.15);
  m.u_n = static_cast<float>((std::log10(p.ueq) - kLog10UMid) / kLog10UHalf);
  const double r = std::max(hmax_next, u);
  m.weight = static_cast<float>((u / r) * (u / r));
  m.inv_s = 1.0f / m.s;
  m.inv_u = 1.0f / m.u;
  m.pad[0] = m.pad[1] = m.pad[2] = 0.0f;
  return m;
}

}  // namespace sg

using sg::Act;
using sg::bf16;

struct SgLayer {
  int cin = 0, cout = 0, taps = 9;
  long long w_off = 0, b_off = 0;
  bf16 *wf = nullptr, *wd = nullptr;
  Act *x = nullptr, *y = nullptr, *gy = nullptr, *gx = nullptr;
  Act *dmask = nullptr;  // ReLU output whose mask the data gradient applies
  int y_planes = 0;      // planes per image of the buffer y lies in (0: y's own)
  int y_up = 0;          // 1: y is stored upsampled 2x into that buffer
  sg::ConvPlan fwd, dgr;
  sg::WgradPlan wgr;
};

struct fs_surrogate {
  fs_sg_config cfg{};
  int W = 0, H = 0, c0 = 0, cap = 0;
  int device = 0, sms = 0;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  // parameters
  long long np = 0, head_off = 0;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  long long adam_t = 0;
  SgLayer L[14];
  // activations (forward) and their gradients
  Act in0, e0a, s0, p0, e1a, s1, p1, e2a, s2, p2, b1, b2, cat2, d2a, d2b, cat1, d1a, d1b, cat0,
      d0a, d0b;
  Act g_d0b, g_d0a, g_cat0, g_d1b, g_d1a, g_cat1, g_d2b, g_d2a, g_cat2, g_b2, g_b1, g_p2, g_s2,
      g_e2a, g_p1, g_s1, g_e1a, g_p0, g_s0, g_e0a;
  float *yt = nullptr;
  double *d_loss = nullptr;
  int *d_err = nullptr;
  int *d_idx = nullptr;
  sg::SampleMeta *d_meta = nullptr;  // per-pass constants (inference)
  double **d_hptr = nullptr, **d_optr = nullptr;
  double *d_hmax = nullptr;
  uint32_t *cnt_buf = nullptr;       // drainage counts of one inference pass
  uint32_t **d_cptr = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double train_ms = 0;
  // dataset
  float *data_h = nullptr, *data_y = nullptr, *data_a = nullptr;
  sg::SampleMeta *data_meta = nullptr;
  int ds_cap = 0, ds_n = 0, ds_held = 0;
  std::mt19937_64 rng;
};

namespace {

template <class T>
cudaError_t dalloc(fs_surrogate *s, T **out, size_t count) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(16, count * sizeof(T)));
  if (e == cudaSuccess) s->allocs.push_back(q);
  *out = static_cast<T *>(q);
  return e;
}

cudaError_t act_alloc(fs_surrogate *s, Act &a, int H, int W, int C) {
  a.B = s->cap;
  a.H = H;
  a.W = W;
  a.C = C;
  return dalloc(s, &a.p, static_cast<size_t>(a.pixels()) * C);
}

Act view(const Act &a, int n) {
  Act v = a;
  v.B = n;
  return v;
}

void free_all(fs_surrogate *s) {
  if (!s) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (void *q : s->allocs) cudaFree(q);
  s->allocs.clear();
  if (s->data_h) cudaFree(s->data_h);
  if (s->data_y) cudaFree(s->data_y);
  if (s->data_meta) cudaFree(s->data_meta);
  if (s->data_a) cudaFree(s->data_a);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  cudaSetDevice(prev);
  delete s;
}

struct DeviceGuard {
  int prev = 0;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() { cudaSetDevice(prev); }
};

bool levels_tile(int W, int H) {
  for (int l = 0; l < 4; l++) {
    if (!sg::pixel_tile(H >> l, W >> l).ok) return false;
  }
  return true;
}

int check_err(fs_surrogate *s) {
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  SG_CUDA(cudaStreamSynchronize(s->stream));
  if (herr) return fail(FS_ERR_TIMEOUT, "surrogate: a tensor-core pipeline wait ran out (%d)", herr);
  return FS_OK;
}

// ---- wiring --------------------------------------------------------------

int build(fs_surrogate *s) {
  const int W = s->W, H = s->H, c = s->c0;
  const int W1 = W / 2, H1 = H / 2, W2 = W / 4, H2 = H / 4, W3 = W / 8, H3 = H / 8;
  struct A {
    Act *a;
    int h, w, ch;
  } acts[] = {
      {&s->in0, H, W, sg::kInputChannels}, {&s->e0a, H, W, c},
      {&s->p0, H1, W1, c}, {&s->e1a, H1, W1, 2 * c},
      {&s->p1, H2, W2, 2 * c}, {&s->e2a, H2, W2, 4 * c},
      {&s->p2, H3, W3, 4 * c}, {&s->b1, H3, W3, 8 * c},
      {&s->cat2, H2, W2, 12 * c}, {&s->d2a, H2, W2, 4 * c},
      {&s->cat1, H1, W1, 6 * c}, {&s->d1a, H1, W1, 2 * c},
      {&s->cat0, H, W, 3 * c}, {&s->d0a, H, W, c}, {&s->d0b, H, W, c},
      {&s->g_d0b, H, W, c}, {&s->g_d0a, H, W, c}, {&s->g_cat0, H, W, 3 * c},
      {&s->g_d1b, H1, W1, 2 * c}, {&s->g_d1a, H1, W1, 2 * c}, {&s->g_cat1, H1, W1, 6 * c},
      {&s->g_d2b, H2, W2, 4 * c}, {&s->g_d2a, H2, W2, 4 * c}, {&s->g_cat2, H2, W2, 12 * c},
      {&s->g_b2, H3, W3, 8 * c}, {&s->g_b1, H3, W3, 8 * c}, {&s->g_p2, H3, W3, 4 * c},
      {&s->g_s2, H2, W2, 4 * c}, {&s->g_e2a, H2, W2, 4 * c}, {&s->g_p1, H2, W2, 2 * c},
      {&s->g_s1, H1, W1, 2 * c}, {&s->g_e1a, H1, W1, 2 * c}, {&s->g_p0, H1, W1, c},
      {&s->g_s0, H, W, c}, {&s->g_e0a, H, W, c},
  };
  for (auto &a : acts) SG_CUDA(act_alloc(s, *a.a, a.h, a.w, a.ch));
  // The concatenations are written by the convolutions of both their
  // halves: the decoder output one level down stored upsampled 2x into the
  // first planes, the encoder's skip tensor into the planes after them.
  // Neither exists on its own (the backward takes the ReLU masks from the
  // concatenations).
  auto skip_in = [&](Act &sk, const Act &cat, int cd) {
    sk = cat;
    sk.C = cat.C - cd;
    sk.p = cat.p + static_cast<size_t>(cd / 8) * cat.H * cat.W * 8;
  };
  auto up_in = [&](Act &d, const Act &cat, int cd) {
    d = cat;
    d.C = cd;
    d.H = cat.H / 2;
    d.W = cat.W / 2;
  };
  skip_in(s->s0, s->cat0, 2 * c);
  skip_in(s->s1, s->cat1, 4 * c);
  skip_in(s->s2, s->cat2, 8 * c);
  up_in(s->d1b, s->cat0, 2 * c);
  up_in(s->d2b, s->cat1, 4 * c);
  up_in(s->b2, s->cat2, 8 * c);
  // layers: input, output, output gradient, input gradient, mask
  struct Wire {
    Act *x, *y, *gy, *gx, *mask;
  } wire[14] = {
      {&s->in0, &s->e0a, &s->g_e0a, nullptr, nullptr},
      {&s->e0a, &s->s0, &s->g_s0, &s->g_e0a, &s->e0a},
      {&s->p0, &s->e1a, &s->g_e1a, &s->g_p0, nullptr},
      {&s->e1a, &s->s1, &s->g_s1, &s->g_e1a, &s->e1a},
      {&s->p1, &s->e2a, &s->g_e2a, &s->g_p1, nullptr},
      {&s->e2a, &s->s2, &s->g_s2, &s->g_e2a, &s->e2a},
      {&s->p2, &s->b1, &s->g_b1, &s->g_p2, nullptr},
      {&s->b1, &s->b2, &s->g_b2, &s->g_b1, &s->b1},
      {&s->cat2, &s->d2a, &s->g_d2a, &s->g_cat2, &s->cat2},
      {&s->d2a, &s->d2b, &s->g_d2b, &s->g_d2a, &s->d2a},
      {&s->cat1, &s->d1a, &s->g_d1a, &s->g_cat1, &s->cat1},
      {&s->d1a, &s->d1b, &s->g_d1b, &s->g_d1a, &s->d1a},
      {&s->cat0, &s->d0a, &s->g_d0a, &s->g_cat0, &s->cat0},
      {&s->d0a, &s->d0b, &s->g_d0b, &s->g_d0a, &s->d0a},
  };
  long long off = 0;
  for (int l = 0; l < 14; l++) {
    SgLayer &L = s->L[l];
    L.x = wire[l].x;
    L.y = wire[l].y;
    L.gy = wire[l].gy;
    L.gx = wire[l].gx;
    L.dmask = wire[l].mask;
    if (L.y == &s->s0 || L.y == &s->d1b) L.y_planes = s->cat0.C / 8;
    if (L.y == &s->s1 || L.y == &s->d2b) L.y_planes = s->cat1.C / 8;
    if (L.y == &s->s2 || L.y == &s->b2) L.y_planes = s->cat2.C / 8;
    L.y_up = L.y == &s->d1b || L.y == &s->d2b || L.y == &s->b2;
    L.cin = L.x->C;
    L.cout = L.y->C;
    L.taps = 9;
    L.w_off = off;
    off += static_cast<long long>(L.cout) * L.taps * L.cin;
    L.b_off = off;
    off += L.cout;
  }
  s->head_off = off;
  off += c + 1;
  s->np = (off + 3) & ~3ll;
  SG_CUDA(dalloc(s, &s->p, s->np));
  SG_CUDA(dalloc(s, &s->g, s->np));
  SG_CUDA(dalloc(s, &s->m, s->np));
  SG_CUDA(dalloc(s, &s->v, s->np));
  SG_CUDA(cudaMemsetAsync(s->g, 0, s->np * sizeof(float), s->stream));
  SG_CUDA(cudaMemsetAsync(s->m, 0, s->np * sizeof(float), s->stream));
  SG_CUDA(cudaMemsetAsync(s->v, 0, s->np * sizeof(float), s->stream));
  SG_CUDA(dalloc(s, &s->yt, static_cast<size_t>(s->cap) * W * H));
  SG_CUDA(dalloc(s, &s->d_loss, 1));
  SG_CUDA(dalloc(s, &s->d_err, 1));
  SG_CUDA(dalloc(s, &s->d_idx, s->cap));
  SG_CUDA(dalloc(s, &s->d_meta, s->cap));
  SG_CUDA(dalloc(s, &s->d_hptr, s->cap));
  SG_CUDA(dalloc(s, &s->d_optr, s->cap));
  SG_CUDA(dalloc(s, &s->d_hmax, s->cap));
  SG_CUDA(dalloc(s, &s->cnt_buf, static_cast<size_t>(s->cap) * W * H));
  SG_CUDA(dalloc(s, &s->d_cptr, s->cap));
  SG_CUDA(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream));
  for (int l = 0; l < 14; l++) {
    SgLayer &L = s->L[l];
    const size_t nw = static_cast<size_t>(L.cout) * L.taps * L.cin;
    SG_CUDA(dalloc(s, &L.wf, nw));
    SG_CUDA(dalloc(s, &L.wd, nw));
    const char *why = nullptr;
    cudaError_t e = sg::plan_conv(L.fwd, *L.x, L.wf, L.taps, L.cout, s->p + L.b_off, 1, nullptr,
                                  L.y->p, &why, L.y_planes, L.y_up);
    if (e != cudaSuccess) return fail(FS_ERR_ARG, "surrogate layer %d forward: %s", l, why);
    e = sg::plan_wgrad(L.wgr, *L.x, *L.gy, L.taps, s->g + L.w_off, s->sms, &why, s->g + L.b_off);
    if (e != cudaSuccess) return fail(FS_ERR_ARG, "surrogate layer %d weight gradient: %s", l, why);
    if (L.gx) {
      e = sg::plan_conv(L.dgr, *L.gy, L.wd, L.taps, L.cin, nullptr, 0,
                        L.dmask ? L.dmask->p : nullptr, L.gx->p, &why);
      if (e != cudaSuccess) return fail(FS_ERR_ARG, "surrogate layer %d data gradient: %s", l, why);
    }
  }
  return FS_OK;
}

// He-normal weights (std sqrt(2/fan_in)), zero biases, a small head.
int init_params(fs_surrogate *s) {
  std::vector<float> h(s->np, 0.0f);
  std::mt19937_64 gen(s->cfg.seed * 0x9E3779B97F4A7C15ull + 12345);
  for (int l = 0; l < 14; l++) {
    const SgLayer &L = s->L[l];
    const int fan_in = L.taps * (l == 0 ? 6 : L.cin);  // input planes 6..15 are zero
    std::normal_distribution<double> d(0.0, std::sqrt(2.0 / fan_in));
    for (long long i = 0; i < static_cast<long long>(L.cout) * L.taps * L.cin; i++)
      h[L.w_off + i] = static_cast<float>(d(gen));
  }
  std::normal_distribution<double> dh(0.0, 0.1 / std::sqrt(static_cast<double>(s->c0)));
  for (int j = 0; j < s->c0; j++) h[s->head_off + j] = static_cast<float>(dh(gen));
  SG_CUDA(cudaMemcpyAsync(s->p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice,
                          s->stream));
  SG_CUDA(cudaStreamSynchronize(s->stream));
  return FS_OK;
}

int refresh_bf16(fs_surrogate *s) {
  for (int l = 0; l < 14; l++) {
    const SgLayer &L = s->L[l];
    SG_CUDA(sg::launch_to_bf16(s->p + L.w_off, static_cast<long long>(L.cout) * L.taps * L.cin,
                               L.wf, L.wd, L.cout, L.cin, L.taps, s->stream));
  }
  return FS_OK;
}

// ---- passes ----------------------------------------------------------------

int forward(fs_surrogate *s, const sg::SampleView &v, bool train) {
  const int n = v.n;
  cudaStream_t st = s->stream;
  SG_CUDA(sg::launch_input(v, s->in0.p, train ? s->yt : nullptr, s->W, s->H, st));
  auto conv = [&](int l) -> cudaError_t { return sg::launch_conv(s->L[l].fwd, s->d_err, st, n); };
  SG_CUDA(conv(0));
  SG_CUDA(conv(1));
  SG_CUDA(sg::launch_avgpool2(view(s->cat0, n), 2 * s->c0 / 8, view(s->p0, n), st));
  SG_CUDA(conv(2));
  SG_CUDA(conv(3));
  SG_CUDA(sg::launch_avgpool2(view(s->cat1, n), 4 * s->c0 / 8, view(s->p1, n), st));
  SG_CUDA(conv(4));
  SG_CUDA(conv(5));
  SG_CUDA(sg::launch_avgpool2(view(s->cat2, n), 8 * s->c0 / 8, view(s->p2, n), st));
  SG_CUDA(conv(6));
  SG_CUDA(conv(7));
  SG_CUDA(conv(8));
  SG_CUDA(conv(9));
  SG_CUDA(conv(10));
  SG_CUDA(conv(11));
  SG_CUDA(conv(12));
  SG_CUDA(conv(13));
  return FS_OK;
}

int backward(fs_surrogate *s, const sg::SampleView &v) {
  const int n = v.n;
  cudaStream_t st = s->stream;
  SG_CUDA(cudaMemsetAsync(s->g, 0, s->np * sizeof(float), st));
  SG_CUDA(sg::launch_head_train(view(s->d0b, n), s->p + s->head_off, s->yt, v, view(s->g_d0b, n),
                                s->g + s->head_off, s->d_loss, st));
  auto layer = [&](int l) -> cudaError_t {
    SgLayer &L = s->L[l];
    cudaError_t e = sg::launch_wgrad(L.wgr, s->d_err, st, n);
    if (e == cudaSuccess && !L.wgr.db) e = sg::launch_bias_grad(view(*L.gy, n), s->g + L.b_off, st);
    if (e == cudaSuccess && L.gx) e = sg::launch_conv(L.dgr, s->d_err, st, n);
    return e;
  };
  const int c = s->c0;
  SG_CUDA(layer(13));
  SG_CUDA(layer(12));
  SG_CUDA(sg::launch_sumpool2(view(s->g_cat0, n), view(s->g_d1b, n), st));
  SG_CUDA(layer(11));
  SG_CUDA(layer(10));
  SG_CUDA(sg::launch_sumpool2(view(s->g_cat1, n), view(s->g_d2b, n), st));
  SG_CUDA(layer(9));
  SG_CUDA(layer(8));
  SG_CUDA(sg::launch_sumpool2(view(s->g_cat2, n), view(s->g_b2, n), st));
  SG_CUDA(layer(7));
  SG_CUDA(layer(6));
  SG_CUDA(sg::launch_skipgrad(view(s->g_cat2, n), 8 * c, view(s->cat2, n), view(s->g_p2, n),
                              view(s->g_s2, n), st));
  SG_CUDA(layer(5));
  SG_CUDA(layer(4));
  SG_CUDA(sg::launch_skipgrad(view(s->g_cat1, n), 4 * c, view(s->cat1, n), view(s->g_p1, n),
                              view(s->g_s1, n), st));
  SG_CUDA(layer(3));
  SG_CUDA(layer(2));
  SG_CUDA(sg::launch_skipgrad(view(s->g_cat0, n), 2 * c, view(s->cat0, n), view(s->g_p0, n),
                              view(s->g_s0, n), st));
  SG_CUDA(layer(1));
  SG_CUDA(layer(0));
  return FS_OK;
}

int adam(fs_surrogate *s, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  s->adam_t++;
  const double t = static_cast<double>(s->adam_t);
  const double c1 = 1.0 - std::pow(0.9, t), c2 = 1.0 - std::pow(0.999, t);
  const float lr_t = static_cast<float>(lr * std::sqrt(c2) / c1);
  const float eps_t = static_cast<float>(eps * std::sqrt(c2));
  // every parameter (weights, biases, head) in one launch; the weight runs
  // also refresh their BF16 copies
  sg::AdamRuns runs;
  for (int l = 0; l < 14; l++) {
    const SgLayer &L = s->L[l];
    runs.off[runs.n] = L.w_off;
    runs.wf[runs.n] = L.wf;
    runs.wd[runs.n] = L.wd;
    runs.cout[runs.n] = L.cout;
    runs.cin[runs.n] = L.cin;
    runs.taps[runs.n] = L.taps;
    runs.n++;
  }
  SG_CUDA(sg::launch_adam(s->p, s->g, s->m, s->v, s->head_off + s->c0 + 1, lr_t, b1, b2, eps_t,
                          runs, s->stream));
  return FS_OK;
}

sg::SampleView data_view(const fs_surrogate *s, int n, const int *d_idx) {
  sg::SampleView v;
  v.n = n;
  v.idx = d_idx;
  v.meta = s->data_meta;
  v.h32 = s->data_h;
  v.y = s->data_y;
  v.a32 = s->data_a;
  return v;
}

int ensure_dataset(fs_surrogate *s, int need) {
  if (need <= s->ds_cap) return FS_OK;
  return fail(FS_ERR_ARG, "surrogate dataset holds %d samples (fs_sg_reserve), %d needed",
              s->ds_cap, need);
}

double conv_flops(const fs_surrogate *s, int pass) {
  // pass 0: forward only; 1: forward + data + weight gradients
  double f = 0;
  for (int l = 0; l < 14; l++) {
    const SgLayer &L = s->L[l];
    const double mac = static_cast<double>(L.x->H) * L.x->W * L.taps * L.cin * L.cout;
    f += 2 * mac;                           // forward
    if (pass) f += 2 * mac * (L.gx ? 2 : 1);  // weight (+ data) gradient
  }
  return f;
}

}  // namespace

// ---------------------------------------------------------------- ABI ----

extern "C" {

void fs_sg_config_default(fs_sg_config *c) {
  if (!c) return;
  c->width = 512;
  c->height = 512;
  c->base_channels = 32;
  c->batch = 32;
  c->jump = 50;
  c->dt = 1000.0;
  c->seed = 1;
}

fs_surrogate *fs_sg_create(const fs_sg_config *c, int *status) {
  int dummy = 0;
  if (!status) status = &dummy;
  *status = FS_OK;
  if (!c) {
    *status = fail(FS_ERR_ARG, "surrogate: config is NULL");
    return nullptr;
  }
  if (c->width < 128 || c->height < 128 || c->width > 4096 || c->height > 4096 ||
      c->width % 64 || c->height % 64 || !levels_tile(c->width, c->height)) {
    *status = fail(FS_ERR_ARG, "surrogate: grid %d x %d must be 128..4096, multiples of 64",
                   c->width, c->height);
    return nullptr;
  }
  if (c->base_channels != 16 && c->base_channels != 32) {
    *status = fail(FS_ERR_ARG, "surrogate: base_channels must be 16 or 32");
    return nullptr;
  }
  if (c->batch < 1 || c->batch > 256 || c->jump < 1 || !(c->dt > 0)) {
    *status = fail(FS_ERR_ARG, "surrogate: batch must be 1..256, jump >= 1, dt > 0");
    return nullptr;
  }
  fs_surrogate *s = new (std::nothrow) fs_surrogate();
  if (!s) {
    *status = fail(FS_ERR_NOMEM, "surrogate: host allocation failed");
    return nullptr;
  }
  s->cfg = *c;
  s->W = c->width;
  s->H = c->height;
  s->c0 = c->base_channels;
  s->cap = c->batch;
  s->rng.seed(c->seed);
  cudaGetDevice(&s->device);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
  if (e != cudaSuccess) {
    *status = cuda_fail(e, "stream");
    free_all(s);
    return nullptr;
  }
  int st = build(s);
  if (st == FS_OK) st = init_params(s);
  if (st == FS_OK) st = refresh_bf16(s);
  if (st == FS_OK && cudaStreamSynchronize(s->stream) != cudaSuccess)
    st = cuda_fail(cudaGetLastError(), "init");
  if (st != FS_OK) {
    *status = st;
    free_all(s);
    return nullptr;
  }
  return s;
}

void fs_sg_destroy(fs_surrogate *s) { free_all(s); }

int fs_sg_get_config(const fs_surrogate *s, fs_sg_config *c) {
  if (!s || !c) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  *c = s->cfg;
  return FS_OK;
}

int fs_sg_param_count(const fs_surrogate *s, int64_t *n) {
  if (!s || !n) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  *n = s->head_off + s->c0 + 1;
  return FS_OK;
}

int fs_sg_get_params(const fs_surrogate *s, float *out) {
  if (!s || !out) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  DeviceGuard dg(s->device);
  SG_CUDA(cudaMemcpyAsync(out, s->p, (s->head_off + s->c0 + 1) * sizeof(float),
                          cudaMemcpyDeviceToHost, s->stream));
  SG_CUDA(cudaStreamSynchronize(s->stream));
  return FS_OK;
}

int fs_sg_set_params(fs_surrogate *s, const float *in) {
  if (!s || !in) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  DeviceGuard dg(s->device);
  SG_CUDA(cudaMemcpyAsync(s->p, in, (s->head_off + s->c0 + 1) * sizeof(float),
                          cudaMemcpyHostToDevice, s->stream));
  if (int st = refresh_bf16(s)) return st;
  SG_CUDA(cudaStreamSynchronize(s->stream));
  return FS_OK;
}

int fs_sg_get_grads(const fs_surrogate *s, float *out) {
  if (!s || !out) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  DeviceGuard dg(s->device);
  SG_CUDA(cudaMemcpyAsync(out, s->g, (s->head_off + s->c0 + 1) * sizeof(float),
                          cudaMemcpyDeviceToHost, s->stream));
  SG_CUDA(cudaStreamSynchronize(s->stream));
  return FS_OK;
}

int fs_sg_save(const fs_surrogate *s, const char *path) {
  if (!s || !path) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  const long long n = s->head_off + s->c0 + 1;
  std::vector<float> h(n);
  if (int st = fs_sg_get_params(s, h.data())) return st;
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(FS_ERR_ARG, "surrogate: cannot write %s", path);
  const char magic[8] = {'F', 'S', 'S', 'G', 'N', 'E', 'T', '1'};
  const int32_t hdr[4] = {s->W, s->H, s->c0, s->cfg.jump};
  const int64_t cnt = n;
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
            std::fwrite(&s->cfg.dt, sizeof(double), 1, f) == 1 &&
            std::fwrite(&cnt, sizeof(cnt), 1, f) == 1 &&
            std::fwrite(h.data(), sizeof(float), n, f) == static_cast<size_t>(n);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(FS_ERR_ARG, "surrogate: short write to %s", path);
  return FS_OK;
}

int fs_sg_load(fs_surrogate *s, const char *path) {
  if (!s || !path) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(FS_ERR_ARG, "surrogate: cannot read %s", path);
  char magic[8];
  int32_t hdr[4];
  double dt = 0;
  int64_t cnt = 0;
  const long long n = s->head_off + s->c0 + 1;
  std::vector<float> h(n);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "FSSGNET1", 8) == 0 &&
            std::fread(hdr, sizeof(hdr), 1, f) == 1 && std::fread(&dt, sizeof(dt), 1, f) == 1 &&
            std::fread(&cnt, sizeof(cnt), 1, f) == 1;
  if (ok && (hdr[0] != s->W || hdr[1] != s->H || hdr[2] != s->c0 || hdr[3] != s->cfg.jump ||
             dt != s->cfg.dt || cnt != n)) {
    std::fclose(f);
    return fail(FS_ERR_ARG,
                "surrogate: %s holds a %d x %d, c %d, jump %d network; this one is %d x %d, c %d, "
                "jump %d",
                path, hdr[0], hdr[1], hdr[2], hdr[3], s->W, s->H, s->c0, s->cfg.jump);
  }
  ok = ok && std::fread(h.data(), sizeof(float), n, f) == static_cast<size_t>(n);
  std::fclose(f);
  if (!ok) return fail(FS_ERR_ARG, "surrogate: %s is not a surrogate parameter file", path);
  return fs_sg_set_params(s, h.data());
}

int fs_sg_reserve(fs_surrogate *s, int capacity) {
  if (!s || capacity < 0) return fail(FS_ERR_ARG, "surrogate: bad reserve");
  DeviceGuard dg(s->device);
  SG_CUDA(cudaStreamSynchronize(s->stream));
  cudaFree(s->data_h);
  cudaFree(s->data_y);
  cudaFree(s->data_meta);
  cudaFree(s->data_a);
  s->data_h = s->data_y = s->data_a = nullptr;
  s->data_meta = nullptr;
  s->ds_cap = s->ds_n = s->ds_held = 0;
  if (capacity == 0) return FS_OK;
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  SG_CUDA(cudaMalloc(&s->data_h, hw * capacity * sizeof(float)));
  SG_CUDA(cudaMalloc(&s->data_y, hw * capacity * sizeof(float)));
  SG_CUDA(cudaMalloc(&s->data_meta, capacity * sizeof(sg::SampleMeta)));
  SG_CUDA(cudaMalloc(&s->data_a, hw * capacity * sizeof(float)));
  s->ds_cap = capacity;
  return FS_OK;
}

int fs_sg_add_samples(fs_surrogate *s, int n, const double *h_t, const double *h_next,
                      const fs_params *params) {
  if (!s || n < 0 || (n > 0 && (!h_t || !h_next || !params)))
    return fail(FS_ERR_ARG, "surrogate: bad samples");
  if (n == 0) return FS_OK;
  if (int st = ensure_dataset(s, s->ds_n + n)) return st;
  DeviceGuard dg(s->device);
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  // the drainage counts of every h_t: a temporary batch of these fields,
  // analysed without erosion
  std::vector<int> Wv(n, s->W), Hv(n, s->H);
  int status = FS_OK;
  fs_batch *b = fs_batch_create(n, Wv.data(), Hv.data(), params, FS_INIT_ZERO, nullptr, &status);
  if (!b) return status;
  for (int k = 0; k < n && status == FS_OK; k++) status = fs_batch_set_elevation(b, k, h_t + k * hw);
  if (status == FS_OK) status = fs_batch_analyze(b);
  double *dn = nullptr;
  uint32_t *dc = nullptr;
  double **dp = nullptr;
  uint32_t **dcp = nullptr;
  int *dslot = nullptr;
  float *du = nullptr;
  cudaError_t e = cudaMalloc(&dn, hw * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dc, hw * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&dp, 2 * sizeof(double *));
  if (e == cudaSuccess) e = cudaMalloc(&dcp, sizeof(uint32_t *));
  if (e == cudaSuccess) e = cudaMalloc(&dslot, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&du, sizeof(float));
  for (int k = 0; k < n && e == cudaSuccess && status == FS_OK; k++) {
    const double *a = h_t + k * hw, *nx = h_next + k * hw;
    double hmax = 0, hmax2 = 0;
    for (size_t i = 0; i < hw; i++) {
      hmax = std::max(hmax, a[i]);
      hmax2 = std::max(hmax2, nx[i]);
    }
    const sg::SampleMeta m = sg::make_meta(params[k], hmax, hmax2, s->cfg.jump, s->cfg.dt);
    const int slot = s->ds_n + k;
    double *field = nullptr;
    status = fs_batch_device_elevation(b, k, &field);
    if (status == FS_OK) status = fs_batch_drainage_counts(b, k, dc);
    if (status != FS_OK) break;
    double *ptrs[2] = {field, dn};
    e = cudaMemcpyAsync(dn, nx, hw * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp, ptrs, sizeof(ptrs), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcp, &dc, sizeof(dc), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dslot, &slot, sizeof(int), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(du, &m.u, sizeof(float), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = sg::launch_record(dp, dp + 1, dslot, du, 1, s->W, s->H, s->data_h, s->data_y, s->stream);
    if (e == cudaSuccess) e = sg::launch_count_plane(dcp, dslot, 1, hw, s->data_a, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->data_meta + slot, &m, sizeof(m), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  if (e != cudaSuccess && status == FS_OK) status = cuda_fail(e, "add samples");
  cudaFree(dn);
  cudaFree(dc);
  cudaFree(dp);
  cudaFree(dcp);
  cudaFree(dslot);
  cudaFree(du);
  fs_batch_destroy(b);
  if (status == FS_OK) s->ds_n += n;
  return status;
}

int fs_sg_set_holdout(fs_surrogate *s, int held) {
  if (!s || held < 0 || held > s->ds_n) return fail(FS_ERR_ARG, "surrogate: bad hold-out count");
  s->ds_held = held;
  return FS_OK;
}

int fs_sg_dataset_info(const fs_surrogate *s, int *nsamples, int *held) {
  if (!s) return fail(FS_ERR_ARG, "surrogate is NULL");
  if (nsamples) *nsamples = s->ds_n;
  if (held) *held = s->ds_held;
  return FS_OK;
}

int fs_sg_get_sample(const fs_surrogate *s, int k, float *h_t, float *y) {
  if (!s || k < 0 || k >= s->ds_n) return fail(FS_ERR_ARG, "surrogate: sample out of range");
  DeviceGuard dg(s->device);
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  if (h_t)
    SG_CUDA(cudaMemcpyAsync(h_t, s->data_h + k * hw, hw * sizeof(float), cudaMemcpyDeviceToHost,
                            s->stream));
  if (y)
    SG_CUDA(cudaMemcpyAsync(y, s->data_y + k * hw, hw * sizeof(float), cudaMemcpyDeviceToHost,
                            s->stream));
  SG_CUDA(cudaStreamSynchronize(s->stream));
  return FS_OK;
}

int fs_sg_generate(fs_surrogate *s, int ntraj, int per_traj, int max_spinup, uint64_t seed,
                   int *added) {
  if (!s || ntraj < 1 || per_traj < 1 || max_spinup < 10 * per_traj)
    return fail(FS_ERR_ARG, "surrogate: generate needs ntraj >= 1, per_traj >= 1, "
                            "max_spinup >= 10*per_traj");
  if (added) *added = 0;
  const int gap = (max_spinup / per_traj) / 10 * 10;
  if (gap < s->cfg.jump)
    return fail(FS_ERR_ARG, "surrogate: samples of one realization must lie >= jump apart");
  if (int st = ensure_dataset(s, s->ds_n + ntraj * per_traj)) return st;
  DeviceGuard dg(s->device);
  std::mt19937_64 gen(seed);
  std::uniform_real_distribution<double> U01(0.0, 1.0);
  std::vector<fs_params> P(ntraj);
  std::vector<int> Wv(ntraj, s->W), Hv(ntraj, s->H), off(ntraj);
  std::vector<uint64_t> seeds(ntraj);
  for (int r = 0; r < ntraj; r++) {
    fs_params_workload(&P[r], 100.0);
    P[r].keq = std::pow(10.0, -6.0 + U01(gen));
    P[r].meq = 0.3 + 0.3 * U01(gen);
    P[r].ueq = std::pow(10.0, -4.0 + (std::log10(5e-3) + 4.0) * U01(gen));
    P[r].dt = s->cfg.dt;
    off[r] = 10 * static_cast<int>(U01(gen) * (gap / 10));
    seeds[r] = gen();
  }
  int status = FS_OK;
  fs_batch *b = fs_batch_create(ntraj, Wv.data(), Hv.data(), P.data(), FS_INIT_PHILOX,
                                seeds.data(), &status);
  if (!b) return status;
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  double *snap = nullptr;
  double **d_a = nullptr, **d_b = nullptr;
  int *d_slot = nullptr;
  float *d_u = nullptr;
  double *d_mx = nullptr;
  cudaError_t e = cudaMalloc(&snap, hw * ntraj * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&d_a, ntraj * sizeof(double *));
  if (e == cudaSuccess) e = cudaMalloc(&d_b, ntraj * sizeof(double *));
  if (e == cudaSuccess) e = cudaMalloc(&d_slot, ntraj * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&d_u, ntraj * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&d_mx, ntraj * sizeof(double));
  std::vector<double *> field(ntraj);
  for (int r = 0; r < ntraj && e == cudaSuccess && status == FS_OK; r++)
    status = fs_batch_device_elevation(b, r, &field[r]);
  void *bstream = nullptr;
  if (status == FS_OK) status = fs_batch_stream(b, &bstream);
  std::vector<double> hmax_start(ntraj, 0.0);
  std::vector<int> slot_of(ntraj, -1);
  uint32_t *cnt = nullptr;
  uint32_t **d_c = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&cnt, hw * ntraj * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_c, ntraj * sizeof(uint32_t *));
  const int jump = s->cfg.jump;
  const int tmax = (per_traj - 1) * gap + (gap - 10) + jump;
  int t = 0, count = 0;
  std::vector<double *> pa, pb;
  std::vector<uint32_t *> pc;
  std::vector<int> slots, who;
  std::vector<float> us;
  std::vector<double> mx;
  while (e == cudaSuccess && status == FS_OK) {
    // samples ending now: h_t from the snapshot, target from the field
    pa.clear();
    pb.clear();
    slots.clear();
    us.clear();
    who.clear();
    for (int r = 0; r < ntraj; r++) {
      const int k = (t - jump - off[r]) / gap;
      if (t - jump >= off[r] && (t - jump - off[r]) % gap == 0 && k < per_traj) {
        pa.push_back(snap + r * hw);
        pb.push_back(field[r]);
        slots.push_back(slot_of[r]);
        us.push_back(static_cast<float>(jump * P[r].ueq * s->cfg.dt));
        who.push_back(r);
      }
    }
    if (!who.empty()) {
      const int m = static_cast<int>(who.size());
      mx.assign(m, 0.0);
      e = cudaMemcpy(d_a, pa.data(), m * sizeof(double *), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_b, pb.data(), m * sizeof(double *), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_slot, slots.data(), m * sizeof(int), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_u, us.data(), m * sizeof(float), cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = sg::launch_record(d_a, d_b, d_slot, d_u, m, s->W, s->H, s->data_h, s->data_y, s->stream);
      if (e == cudaSuccess) e = sg::launch_field_max(d_b, nullptr, m, hw, d_mx, s->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(mx.data(), d_mx, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
      for (int i = 0; i < m && e == cudaSuccess; i++) {
        const sg::SampleMeta meta =
            sg::make_meta(P[who[i]], hmax_start[who[i]], mx[i], jump, s->cfg.dt);
        e = cudaMemcpy(s->data_meta + slots[i], &meta, sizeof(meta), cudaMemcpyHostToDevice);
      }
    }
    if (t >= tmax) break;
    // samples starting now: snapshot, maximum, drainage counts of h_t
    pa.clear();
    pb.clear();
    pc.clear();
    slots.clear();
    who.clear();
    for (int r = 0; r < ntraj; r++)
      if (t >= off[r] && (t - off[r]) % gap == 0 && (t - off[r]) / gap < per_traj) {
        slot_of[r] = s->ds_n + count++;
        pa.push_back(field[r]);
        pb.push_back(snap + r * hw);
        pc.push_back(cnt + r * hw);
        slots.push_back(slot_of[r]);
        who.push_back(r);
      }
    if (!who.empty() && e == cudaSuccess) {
      const int m = static_cast<int>(who.size());
      status = fs_batch_set_active(b, m, who.data());
      if (status == FS_OK) status = fs_batch_analyze(b);
      for (int i = 0; i < m && status == FS_OK; i++)
        status = fs_batch_drainage_counts(b, who[i], pc[i]);
      if (status == FS_OK) status = fs_batch_set_active(b, 0, nullptr);
      if (status != FS_OK) break;
      mx.assign(m, 0.0);
      e = cudaMemcpy(d_a, pa.data(), m * sizeof(double *), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_b, pb.data(), m * sizeof(double *), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_c, pc.data(), m * sizeof(uint32_t *), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_slot, slots.data(), m * sizeof(int), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = sg::launch_copy_fields(d_a, d_b, m, hw, s->stream);
      if (e == cudaSuccess) e = sg::launch_count_plane(d_c, d_slot, m, hw, s->data_a, s->stream);
      if (e == cudaSuccess) e = sg::launch_field_max(d_a, nullptr, m, hw, d_mx, s->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(mx.data(), d_mx, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
      for (int i = 0; i < m; i++) hmax_start[who[i]] = mx[i];
    }
    // advance to the next event (every event time is a multiple of 10)
    int next = tmax;
    for (int r = 0; r < ntraj; r++) {
      for (int k = 0; k < per_traj; k++) {
        const int ts = off[r] + k * gap, te = ts + jump;
        if (ts > t && ts < next) next = ts;
        if (te > t && te < next) next = te;
      }
    }
    if (e == cudaSuccess && status == FS_OK) status = fs_batch_step(b, next - t);
    t = next;
  }
  cudaFree(cnt);
  cudaFree(d_c);
  if (e != cudaSuccess && status == FS_OK) status = cuda_fail(e, "generate");
  cudaStreamSynchronize(s->stream);
  cudaFree(snap);
  cudaFree(d_a);
  cudaFree(d_b);
  cudaFree(d_slot);
  cudaFree(d_u);
  cudaFree(d_mx);
  fs_batch_destroy(b);
  if (status == FS_OK) {
    s->ds_n += count;
    if (added) *added = count;
  }
  return status;
}

int fs_sg_grad(fs_surrogate *s, int n, const int *idx, double *loss) {
  if (!s || n < 1 || n > s->cap || !idx) return fail(FS_ERR_ARG, "surrogate: bad batch");
  for (int i = 0; i < n; i++)
    if (idx[i] < 0 || idx[i] >= s->ds_n) return fail(FS_ERR_ARG, "surrogate: sample out of range");
  DeviceGuard dg(s->device);
  SG_CUDA(cudaMemcpyAsync(s->d_idx, idx, n * sizeof(int), cudaMemcpyHostToDevice, s->stream));
  SG_CUDA(cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream));
  const sg::SampleView v = data_view(s, n, s->d_idx);
  if (int st = forward(s, v, true)) return st;
  if (int st = backward(s, v)) return st;
  if (int st = check_err(s)) return st;
  double l = 0;
  SG_CUDA(cudaMemcpy(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost));
  if (loss) *loss = l;  // the head kernel already averages over the samples
  return FS_OK;
}

int fs_sg_train(fs_surrogate *s, int steps, float lr, double *mean_loss) {
  if (!s || steps < 0 || !(lr > 0)) return fail(FS_ERR_ARG, "surrogate: bad training call");
  const int ntrain = s->ds_n - s->ds_held;
  if (ntrain < 1) return fail(FS_ERR_STATE, "surrogate: no training samples");
  DeviceGuard dg(s->device);
  const int n = std::min(s->cap, ntrain);
  std::uniform_int_distribution<int> pick(0, ntrain - 1);
  std::vector<int> idx(static_cast<size_t>(n) * std::max(steps, 1));
  for (int k = 0; k < steps; k++)
    for (int i = 0; i < n; i++) idx[static_cast<size_t>(k) * n + i] = pick(s->rng);
  int *d_all = nullptr;
  SG_CUDA(cudaMalloc(&d_all, idx.size() * sizeof(int)));
  cudaError_t e = cudaMemcpyAsync(d_all, idx.data(), idx.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, s->stream);
  int st = e == cudaSuccess ? FS_OK : cuda_fail(e, "indices");
  if (st == FS_OK) e = cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream);
  if (st == FS_OK) e = cudaEventRecord(s->ev0, s->stream);
  for (int k = 0; k < steps && st == FS_OK && e == cudaSuccess; k++) {
    const sg::SampleView v = data_view(s, n, d_all + static_cast<size_t>(k) * n);
    st = forward(s, v, true);
    if (st == FS_OK) st = backward(s, v);
    if (st == FS_OK) st = adam(s, lr);
  }
  if (st == FS_OK && e == cudaSuccess) e = cudaEventRecord(s->ev1, s->stream);
  if (st == FS_OK && e == cudaSuccess) e = cudaEventSynchronize(s->ev1);
  if (st == FS_OK && e != cudaSuccess) st = cuda_fail(e, "train");
  if (st == FS_OK) st = check_err(s);
  float ms = 0;
  if (st == FS_OK && cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) s->train_ms = ms;
  double l = 0;
  if (st == FS_OK) {
    e = cudaMemcpy(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = cuda_fail(e, "loss");
  }
  cudaFree(d_all);
  if (st == FS_OK && mean_loss) *mean_loss = steps > 0 ? l / steps : 0.0;
  return st;
}

int fs_sg_eval(fs_surrogate *s, double *loss) {
  if (!s) return fail(FS_ERR_ARG, "surrogate is NULL");
  if (s->ds_n < 1) return fail(FS_ERR_STATE, "surrogate: no samples");
  DeviceGuard dg(s->device);
  const int lo = s->ds_held > 0 ? s->ds_n - s->ds_held : 0;
  const int total = s->ds_n - lo;
  // the gradients of the last training step are kept: evaluate into a copy
  float *gsave = nullptr;
  SG_CUDA(cudaMalloc(&gsave, s->np * sizeof(float)));
  cudaError_t e = cudaMemcpyAsync(gsave, s->g, s->np * sizeof(float), cudaMemcpyDeviceToDevice,
                                  s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream);
  int st = e == cudaSuccess ? FS_OK : cuda_fail(e, "eval");
  std::vector<int> idx(s->cap);
  double sum = 0;
  for (int a = lo; a < s->ds_n && st == FS_OK; a += s->cap) {
    const int n = std::min(s->cap, s->ds_n - a);
    for (int i = 0; i < n; i++) idx[i] = a + i;
    e = cudaMemcpyAsync(s->d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) {
      st = cuda_fail(e, "eval");
      break;
    }
    // the pageable copy above is staged before the call returns; idx is
    // rewritten only after the next forward pass is enqueued
    const sg::SampleView v = data_view(s, n, s->d_idx);
    st = forward(s, v, true);
    if (st == FS_OK) {
      e = sg::launch_head_train(view(s->d0b, n), s->p + s->head_off, s->yt, v, view(s->g_d0b, n),
                                s->g + s->head_off, s->d_loss, s->stream);
      if (e != cudaSuccess) st = cuda_fail(e, "eval head");
    }
    // each pass averages over its own n samples: weight it by n
    double chunk = 0;
    if (st == FS_OK) {
      e = cudaMemcpyAsync(&chunk, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
      if (e != cudaSuccess) st = cuda_fail(e, "eval");
    }
    sum += chunk * n;
  }
  if (st == FS_OK) st = check_err(s);
  const double l = sum;
  cudaMemcpyAsync(s->g, gsave, s->np * sizeof(float), cudaMemcpyDeviceToDevice, s->stream);
  cudaStreamSynchronize(s->stream);
  cudaFree(gsave);
  if (st == FS_OK && loss) *loss = l / total;
  return st;
}

int fs_sg_eval_baselines(fs_surrogate *s, double *uplift_only, double *no_change) {
  if (!s) return fail(FS_ERR_ARG, "surrogate is NULL");
  if (s->ds_n < 1) return fail(FS_ERR_STATE, "surrogate: no samples");
  DeviceGuard dg(s->device);
  const int lo = s->ds_held > 0 ? s->ds_n - s->ds_held : 0;
  const int total = s->ds_n - lo;
  std::vector<int> idx(total);
  for (int i = 0; i < total; i++) idx[i] = lo + i;
  int *d = nullptr;
  double *acc = nullptr;
  SG_CUDA(cudaMalloc(&d, total * sizeof(int)));
  cudaError_t e = cudaMalloc(&acc, 2 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, idx.data(), total * sizeof(int), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, 2 * sizeof(double), s->stream);
  if (e == cudaSuccess) e = sg::launch_baseline_loss(data_view(s, total, d), s->W, s->H, acc, s->stream);
  double h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  cudaFree(acc);
  if (e != cudaSuccess) return cuda_fail(e, "baselines");
  // the kernel averages over all `total` samples at once, like fs_sg_eval
  if (uplift_only) *uplift_only = h[0];
  if (no_change) *no_change = h[1];
  return FS_OK;
}

int fs_sg_train_stats(const fs_surrogate *s, double *ms, double *conv_flops_per_step) {
  if (!s) return fail(FS_ERR_ARG, "surrogate is NULL");
  if (ms) *ms = s->train_ms;
  if (conv_flops_per_step) *conv_flops_per_step = conv_flops(s, 1) * s->cap;
  return FS_OK;
}

int fs_sg_time_forward(fs_surrogate *s, int reps, double *ms_per_pass, double *flops_per_pass) {
  if (!s || reps < 1) return fail(FS_ERR_ARG, "surrogate: bad timing call");
  if (s->ds_n < 1) return fail(FS_ERR_STATE, "surrogate: no samples");
  DeviceGuard dg(s->device);
  const int n = std::min(s->cap, s->ds_n);
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  SG_CUDA(cudaMemcpyAsync(s->d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, s->stream));
  const sg::SampleView v = data_view(s, n, s->d_idx);
  if (int st = forward(s, v, false)) return st;  // warm-up
  SG_CUDA(cudaEventRecord(s->ev0, s->stream));
  for (int k = 0; k < reps; k++)
    if (int st = forward(s, v, false)) return st;
  SG_CUDA(cudaEventRecord(s->ev1, s->stream));
  SG_CUDA(cudaEventSynchronize(s->ev1));
  if (int st = check_err(s)) return st;
  float ms = 0;
  SG_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
  if (ms_per_pass) *ms_per_pass = ms / reps;
  if (flops_per_pass) *flops_per_pass = conv_flops(s, 0) * n;
  return FS_OK;
}

int fs_sg_infer_flops(const fs_surrogate *s, double *flops) {
  if (!s || !flops) return fail(FS_ERR_ARG, "surrogate: NULL argument");
  *flops = conv_flops(s, 0);
  return FS_OK;
}

}  // extern "C"

// Jumps n device fields hin[k] (params p[k]) into hout[k] (hout may equal
// hin), in chunks of the network's batch.
int sg_predict_fields(fs_surrogate *s, int n, double *const *hin, double *const *hout,
                      const fs_params *p, uint32_t *const *cnt) {
  DeviceGuard dg(s->device);
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  std::vector<double> mx(s->cap);
  std::vector<sg::SampleMeta> meta(s->cap);
  for (int a = 0; a < n; a += s->cap) {
    const int m = std::min(s->cap, n - a);
    SG_CUDA(cudaMemcpyAsync(s->d_hptr, hin + a, m * sizeof(double *), cudaMemcpyHostToDevice,
                            s->stream));
    SG_CUDA(cudaMemcpyAsync(s->d_optr, hout + a, m * sizeof(double *), cudaMemcpyHostToDevice,
                            s->stream));
    SG_CUDA(cudaMemcpyAsync(s->d_cptr, cnt + a, m * sizeof(uint32_t *), cudaMemcpyHostToDevice,
                            s->stream));
    SG_CUDA(sg::launch_field_max(s->d_hptr, nullptr, m, hw, s->d_hmax, s->stream));
    SG_CUDA(cudaMemcpyAsync(mx.data(), s->d_hmax, m * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
    SG_CUDA(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < m; i++) meta[i] = sg::make_meta(p[a + i], mx[i], mx[i], s->cfg.jump, s->cfg.dt);
    SG_CUDA(cudaMemcpyAsync(s->d_meta, meta.data(), m * sizeof(sg::SampleMeta),
                            cudaMemcpyHostToDevice, s->stream));
    sg::SampleView v;
    v.n = m;
    v.meta = s->d_meta;
    v.h64 = s->d_hptr;
    v.cnt = s->d_cptr;
    if (int st = forward(s, v, false)) return st;
    SG_CUDA(sg::launch_head_apply(view(s->d0b, m), s->p + s->head_off, v, s->d_optr, s->stream));
    SG_CUDA(cudaStreamSynchronize(s->stream));  // the host arrays above are reused
  }
  return check_err(s);
}

extern "C" int fs_sg_predict_batch(fs_surrogate *s, fs_batch *b, int n, const int *idx,
                                   double *const *d_out) {
  if (!s || !b || n < 0 || (n > 0 && !idx)) return fail(FS_ERR_ARG, "surrogate: bad predict call");
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  std::vector<double *> in(n), out(n);
  std::vector<fs_params> p(n);
  for (int k = 0; k < n; k++) {
    int w = 0, h = 0;
    if (int st = fs_batch_get_shape(b, idx[k], &w, &h)) return st;
    if (w != s->W || h != s->H)
      return fail(FS_ERR_ARG, "surrogate: realization %d is %d x %d, the network takes %d x %d",
                  idx[k], w, h, s->W, s->H);
    if (int st = fs_batch_device_elevation(b, idx[k], &in[k])) return st;
    if (int st = fs_batch_get_params(b, idx[k], &p[k])) return st;
    out[k] = d_out ? d_out[k] : in[k];
  }
  std::vector<uint32_t *> cp(s->cap);
  for (int i = 0; i < s->cap; i++) cp[i] = s->cnt_buf + i * hw;
  int st = FS_OK;
  for (int a = 0; a < n && st == FS_OK; a += s->cap) {
    const int m = std::min(s->cap, n - a);
    // drainage counts of the fields about to jump
    st = fs_batch_set_active(b, m, idx + a);
    if (st == FS_OK) st = fs_batch_analyze(b);
    for (int i = 0; i < m && st == FS_OK; i++) st = fs_batch_drainage_counts(b, idx[a + i], cp[i]);
    if (st == FS_OK) st = sg_predict_fields(s, m, in.data() + a, out.data() + a, p.data() + a, cp.data());
  }
  const int st2 = fs_batch_set_active(b, 0, nullptr);
  return st != FS_OK ? st : st2;
}

extern "C" int fs_sg_predict_host(fs_surrogate *s, int n, const double *h_in,
                                  const fs_params *params, double *h_out) {
  if (!s || n < 0 || (n > 0 && (!h_in || !params || !h_out)))
    return fail(FS_ERR_ARG, "surrogate: bad predict call");
  if (n == 0) return FS_OK;
  const size_t hw = static_cast<size_t>(s->W) * s->H;
  std::vector<int> Wv(n, s->W), Hv(n, s->H), idx(n);
  int status = FS_OK;
  fs_batch *b = fs_batch_create(n, Wv.data(), Hv.data(), params, FS_INIT_ZERO, nullptr, &status);
  if (!b) return status;
  for (int k = 0; k < n && status == FS_OK; k++) {
    idx[k] = k;
    status = fs_batch_set_elevation(b, k, h_in + k * hw);
  }
  if (status == FS_OK) status = fs_sg_predict_batch(s, b, n, idx.data(), nullptr);
  for (int k = 0; k < n && status == FS_OK; k++)
    status = fs_batch_get_elevation(b, k, h_out + k * hw);
  fs_batch_destroy(b);
  return status;
}
