// sg_api.cu -- C ABI of the learned surrogate's kernels: the test entry
// point for single convolutions (include/fastscape_gb300_testing.h).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "fastscape_gb300.h"
#include "fastscape_gb300_testing.h"
#include "fs_internal.h"
#include "sg_internal.h"

namespace {

int sg_fail(int status, const char *fmt, const char *what) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), fmt, what ? what : "");
  return fs::record_error(status, buf);
}

int cuda_fail(cudaError_t e, const char *what) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return fs::record_error(FS_ERR_CUDA, buf);
}

// NHWC host tensors <-> the device's plane-major layout [B][C/8][H][W][8].
std::vector<uint16_t> to_planes(const uint16_t *x, long long pix_img, int B, int C) {
  std::vector<uint16_t> o(static_cast<size_t>(pix_img) * B * C);
  for (int b = 0; b < B; b++)
    for (long long p = 0; p < pix_img; p++)
      for (int c = 0; c < C; c++)
        o[static_cast<size_t>(sg::plane_at(b, c / 8, p, C / 8, pix_img) + c % 8)] =
            x[(static_cast<size_t>(b) * pix_img + p) * C + c];
  return o;
}

void from_planes(const uint16_t *x, long long pix_img, int B, int C, uint16_t *o) {
  for (int b = 0; b < B; b++)
    for (long long p = 0; p < pix_img; p++)
      for (int c = 0; c < C; c++)
        o[(static_cast<size_t>(b) * pix_img + p) * C + c] =
            x[static_cast<size_t>(sg::plane_at(b, c / 8, p, C / 8, pix_img) + c % 8)];
}

// Device buffers of one test call, released on every path.
struct Bufs {
  void *p[8] = {};
  int n = 0;
  ~Bufs() {
    for (int i = 0; i < n; i++) cudaFree(p[i]);
  }
  template <class T>
  cudaError_t alloc(T **out, size_t bytes) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes < 16 ? 16 : bytes);
    if (e == cudaSuccess) p[n++] = q;
    *out = static_cast<T *>(q);
    return e;
  }
};

}  // namespace

extern "C" int fs_test_sg_conv(int mode, int B, int H, int W, int cin, int cout, int taps,
                               const uint16_t *x, const uint16_t *w, const float *bias, int relu,
                               const uint16_t *mask, void *out) {
  if (mode < 0 || mode > 4)
    return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: mode must be 0 to 4%s", "");
  if (B < 1 || H < 1 || W < 1 || cin < 16 || cout < 16 || cin % 16 || cout % 16 ||
      (taps != 1 && taps != 9) || !x || !w || !out)
    return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: bad shape or NULL buffer%s", "");
  const long long pix = static_cast<long long>(B) * H * W, hw = static_cast<long long>(H) * W;
  const size_t nw = static_cast<size_t>(cout) * taps * cin;
  Bufs bufs;
  sg::bf16 *dx = nullptr, *dw = nullptr, *dwd = nullptr, *dmask = nullptr, *dout = nullptr;
  float *dbias = nullptr, *dgw = nullptr;
  int *derr = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t e = bufs.alloc(&derr, sizeof(int));
  const char *why = nullptr;
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  // modes 3 and 4: the output's cout channels are planes [kGuard, kGuard +
  // cout/8) of a tensor with kGuard sentinel planes before and after them
  // (at 2H x 2W in mode 4)
  constexpr int kGuard = 2;
  constexpr uint16_t kSentinel = 0x7FC5;
  const int up = mode == 4 ? 1 : 0;
  const long long opix = pix << (2 * up), ohw = hw << (2 * up);
  const int oplanes = cout / 8 + 2 * kGuard;
  if (mode == 0) {
    if (e == cudaSuccess) e = bufs.alloc(&dx, pix * cin * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dw, nw * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dout, pix * cout * 2);
    if (e == cudaSuccess && bias) e = bufs.alloc(&dbias, cout * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMemcpy(dx, to_planes(x, hw, B, cin).data(), pix * cin * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, w, nw * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bias) e = cudaMemcpy(dbias, bias, cout * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: buffers");
    sg::Act src{dx, B, H, W, cin};
    sg::ConvPlan plan;
    e = sg::plan_conv(plan, src, dw, taps, cout, dbias, relu, nullptr, dout, &why);
    if (e != cudaSuccess) return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: %s", why);
    e = sg::launch_conv(plan, derr, s);
  } else if (mode >= 3) {
    const size_t on = static_cast<size_t>(opix) * oplanes * 8;
    if (e == cudaSuccess) e = bufs.alloc(&dx, pix * cin * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dw, nw * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dout, on * 2);
    if (e == cudaSuccess && bias) e = bufs.alloc(&dbias, cout * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMemcpy(dx, to_planes(x, hw, B, cin).data(), pix * cin * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, w, nw * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bias) e = cudaMemcpy(dbias, bias, cout * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      const std::vector<uint16_t> fill(on, kSentinel);
      e = cudaMemcpy(dout, fill.data(), on * 2, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: buffers");
    sg::Act src{dx, B, H, W, cin};
    sg::ConvPlan plan;
    e = sg::plan_conv(plan, src, dw, taps, cout, dbias, relu, nullptr,
                      dout + static_cast<size_t>(kGuard) * ohw * 8, &why, oplanes, up);
    if (e != cudaSuccess) return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: %s", why);
    e = sg::launch_conv(plan, derr, s);
  } else if (mode == 1) {
    if (e == cudaSuccess) e = bufs.alloc(&dx, pix * cout * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dw, nw * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dwd, nw * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dout, pix * cin * 2);
    if (e == cudaSuccess && mask) e = bufs.alloc(&dmask, pix * cin * 2);
    if (e == cudaSuccess)
      e = cudaMemcpy(dx, to_planes(x, hw, B, cout).data(), pix * cout * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, w, nw * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && mask)
      e = cudaMemcpy(dmask, to_planes(mask, hw, B, cin).data(), pix * cin * 2,
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = sg::launch_flip_weights(dw, dwd, cout, cin, taps, s);
    if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: buffers");
    sg::Act src{dx, B, H, W, cout};
    sg::ConvPlan plan;
    e = sg::plan_conv(plan, src, dwd, taps, cin, nullptr, 0, dmask, dout, &why);
    if (e != cudaSuccess) return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: %s", why);
    e = sg::launch_conv(plan, derr, s);
  } else {
    if (e == cudaSuccess) e = bufs.alloc(&dx, pix * cin * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dw, pix * cout * 2);
    if (e == cudaSuccess) e = bufs.alloc(&dgw, nw * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMemcpy(dx, to_planes(x, hw, B, cin).data(), pix * cin * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(dw, to_planes(w, hw, B, cout).data(), pix * cout * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dgw, 0, nw * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: buffers");
    sg::Act xa{dx, B, H, W, cin}, ya{dw, B, H, W, cout};
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    sg::WgradPlan plan;
    e = sg::plan_wgrad(plan, xa, ya, taps, dgw, sms > 0 ? sms : 1, &why);
    if (e != cudaSuccess) return sg_fail(FS_ERR_ARG, "fs_test_sg_conv: %s", why);
    e = sg::launch_wgrad(plan, derr, s);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: launch");
  int herr = 0;
  e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: status");
  if (herr) return sg_fail(FS_ERR_TIMEOUT, "fs_test_sg_conv: a pipeline wait ran out%s", "");
  if (mode == 2) {
    e = cudaMemcpy(out, dgw, nw * sizeof(float), cudaMemcpyDeviceToHost);
  } else if (mode >= 3) {
    // every guard plane must still hold the sentinel; the output's planes
    // come back as [B, H, W, cout] (2H x 2W in mode 4)
    std::vector<uint16_t> t(static_cast<size_t>(opix) * oplanes * 8);
    e = cudaMemcpy(t.data(), dout, t.size() * 2, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: copy back");
    std::vector<uint16_t> o(static_cast<size_t>(opix) * cout);
    for (int b = 0; b < B; b++)
      for (int pl = 0; pl < oplanes; pl++) {
        const uint16_t *src = t.data() + static_cast<size_t>(b * oplanes + pl) * ohw * 8;
        const bool guard = pl < kGuard || pl >= kGuard + cout / 8;
        if (guard) {
          for (long long k = 0; k < ohw * 8; k++)
            if (src[k] != kSentinel) {
              char where[64];
              std::snprintf(where, sizeof(where), "image %d plane %d", b, pl);
              return sg_fail(FS_ERR_CUDA, "fs_test_sg_conv: %s outside the output was written",
                             where);
            }
          continue;
        }
        for (long long q = 0; q < ohw; q++)
          std::memcpy(o.data() + (static_cast<size_t>(b) * ohw + q) * cout + 8 * (pl - kGuard),
                      src + q * 8, 16);
      }
    std::memcpy(out, o.data(), o.size() * 2);
  } else {
    const int co = mode == 0 ? cout : cin;
    std::vector<uint16_t> t(static_cast<size_t>(pix) * co);
    e = cudaMemcpy(t.data(), dout, pix * co * 2, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) from_planes(t.data(), hw, B, co, static_cast<uint16_t *>(out));
  }
  if (e != cudaSuccess) return cuda_fail(e, "fs_test_sg_conv: copy back");
  return FS_OK;
}
