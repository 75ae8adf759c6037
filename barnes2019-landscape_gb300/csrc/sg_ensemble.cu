// sg_ensemble.cu -- the surrogate-accelerated ensemble with its judge and
// fallback (fs_sg_ensemble_run), and the judge's field comparison
// (fs_sg_compare_host).
//
// A cycle: the surrogate jumps every realization still on it by `jump`
// timesteps; a seeded share of those jumps is re-run exactly by the plain
// FP64 method from the same state (the judged realizations' jumps go to side
// fields, their own fields take the exact run), together with the plain
// `jump` timesteps of every realization that fell back; the judge compares
// each judged jump with its exact run; then every realization takes
// `plain_steps` plain timesteps. Realizations not on the surrogate any more
// advance exactly as the plain batched method would.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <random>
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
  return fail(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA, "ensemble: %s: %s",
              what, cudaGetErrorString(e));
}

#define EN_CUDA(x)                                   \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
  } while (0)

// Per compared pair: sum of squared differences over interior cells, the
// exact field's maximum and minimum, interior cells with equal receivers.
struct PairStats {
  double sumsq, hmax, hmin;
  unsigned long long agree;
};

__device__ __forceinline__ void atomic_max_d(double *a, double v) {
  unsigned long long *p = reinterpret_cast<unsigned long long *>(a);
  unsigned long long old = *p;
  while (__longlong_as_double(static_cast<long long>(old)) < v) {
    const unsigned long long got =
        atomicCAS(p, old, static_cast<unsigned long long>(__double_as_longlong(v)));
    if (got == old) break;
    old = got;
  }
}

__device__ __forceinline__ void atomic_min_d(double *a, double v) {
  unsigned long long *p = reinterpret_cast<unsigned long long *>(a);
  unsigned long long old = *p;
  while (__longlong_as_double(static_cast<long long>(old)) > v) {
    const unsigned long long got =
        atomicCAS(p, old, static_cast<unsigned long long>(__double_as_longlong(v)));
    if (got == old) break;
    old = got;
  }
}

// D8 receiver of interior cell c with the reference's neighbour order and
// tie-break (fastscape_RB.cpp:160-182): the first strictly steepest descent
// (h[c] - h[n]) / dr[n] > 0, or -1.
__device__ __forceinline__ int receiver_of(const double *h, int c, int W, double dro, double drd) {
  const int off[8] = {-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1};
  double best = 0.0;
  int r = -1;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const double slope = (h[c] - h[c + off[n]]) / ((n & 1) ? drd : dro);
    if (slope > best) {
      best = slope;
      r = n;
    }
  }
  return r;
}

constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) k_compare(double *const *__restrict__ a,
                                                    double *const *__restrict__ b, int W, int H,
                                                    const double *__restrict__ dr,
                                                    PairStats *__restrict__ out) {
  const int f = blockIdx.y;
  const double *ha = a[f], *hb = b[f];
  const double dro = dr[2 * f], drd = dr[2 * f + 1];
  const long long hw = static_cast<long long>(W) * H;
  double ss = 0.0, mx = -1e300, mn = 1e300;
  unsigned long long ag = 0;
  for (long long i = blockIdx.x * static_cast<long long>(kBlock) + threadIdx.x; i < hw;
       i += static_cast<long long>(gridDim.x) * kBlock) {
    const int c = static_cast<int>(i);
    const int x = c % W, y = c / W;
    const double vb = hb[c];
    mx = fmax(mx, vb);
    mn = fmin(mn, vb);
    if (x >= 2 && y >= 2 && x < W - 2 && y < H - 2) {
      const double d = ha[c] - vb;
      ss += d * d;
      ag += receiver_of(ha, c, W, dro, drd) == receiver_of(hb, c, W, dro, drd) ? 1 : 0;
    }
  }
  __shared__ double s_ss[kBlock / 32], s_mx[kBlock / 32], s_mn[kBlock / 32];
  __shared__ unsigned long long s_ag[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    ag += __shfl_xor_sync(0xffffffffu, ag, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_ss[threadIdx.x >> 5] = ss;
    s_mx[threadIdx.x >> 5] = mx;
    s_mn[threadIdx.x >> 5] = mn;
    s_ag[threadIdx.x >> 5] = ag;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ss = s_ss[0];
    mx = s_mx[0];
    mn = s_mn[0];
    ag = s_ag[0];
    for (int k = 1; k < kBlock / 32; k++) {
      ss += s_ss[k];
      mx = fmax(mx, s_mx[k]);
      mn = fmin(mn, s_mn[k]);
      ag += s_ag[k];
    }
    atomicAdd(&out[f].sumsq, ss);
    atomic_max_d(&out[f].hmax, mx);
    atomic_min_d(&out[f].hmin, mn);
    atomicAdd(&out[f].agree, ag);
  }
}

__global__ void k_init_stats(PairStats *s, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    s[i].sumsq = 0.0;
    s[i].hmax = -1e300;
    s[i].hmin = 1e300;
    s[i].agree = 0;
  }
}

// Compares n device field pairs (a = candidate, b = exact) on `stream`;
// rel[k] = RMS over interior cells of (a - b) / (max b - min b),
// agree[k] = share of interior cells whose receivers match.
int compare_fields(int W, int H, int n, double *const *d_a, double *const *d_b,
                   const double *dr_host, double *rel, double *agree, cudaStream_t stream) {
  if (n == 0) return FS_OK;
  double **pa = nullptr, **pb = nullptr;
  double *ddr = nullptr;
  PairStats *st = nullptr;
  cudaError_t e = cudaMalloc(&pa, n * sizeof(double *));
  if (e == cudaSuccess) e = cudaMalloc(&pb, n * sizeof(double *));
  if (e == cudaSuccess) e = cudaMalloc(&ddr, 2 * n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&st, n * sizeof(PairStats));
  if (e == cudaSuccess) e = cudaMemcpyAsync(pa, d_a, n * sizeof(double *), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pb, d_b, n * sizeof(double *), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ddr, dr_host, 2 * n * sizeof(double), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) {
    k_init_stats<<<(n + 127) / 128, 128, 0, stream>>>(st, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    const long long hw = static_cast<long long>(W) * H;
    int gx = static_cast<int>((hw + kBlock * 8 - 1) / (kBlock * 8));
    gx = std::max(1, std::min(gx, 256));
    k_compare<<<dim3(gx, n), kBlock, 0, stream>>>(pa, pb, W, H, ddr, st);
    e = cudaGetLastError();
  }
  std::vector<PairStats> h(n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), st, n * sizeof(PairStats), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  cudaFree(pa);
  cudaFree(pb);
  cudaFree(ddr);
  cudaFree(st);
  if (e != cudaSuccess) return cuda_fail(e, "compare");
  const double ni = static_cast<double>(W - 4) * (H - 4);
  for (int k = 0; k < n; k++) {
    const double relief = h[k].hmax - h[k].hmin;
    const double rms = std::sqrt(h[k].sumsq / ni);
    rel[k] = relief > 0 ? rms / relief : (rms > 0 ? INFINITY : 0.0);
    agree[k] = static_cast<double>(h[k].agree) / ni;
  }
  return FS_OK;
}

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

}  // namespace

extern "C" {

void fs_sg_ensemble_defaults(fs_sg_ensemble_opts *o) {
  if (!o) return;
  o->nsteps = 2000;
  o->plain_steps = 1;
  o->judge_fraction = 0.05;
  o->max_rel_rms = 0.01;
  o->min_agreement = 0.99;
  o->seed = 2019;
}

int fs_sg_compare_host(int width, int height, const fs_params *params, int n, const double *h_a,
                       const double *h_b, double *rel_rms, double *agreement) {
  if (width < 5 || height < 5 || n < 0 || (n > 0 && (!params || !h_a || !h_b || !rel_rms ||
                                                     !agreement)))
    return fail(FS_ERR_ARG, "compare: bad arguments");
  if (n == 0) return FS_OK;
  const size_t hw = static_cast<size_t>(width) * height;
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, 2 * hw * n * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "compare buffers");
  e = cudaMemcpy(d, h_a, hw * n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + hw * n, h_b, hw * n * sizeof(double), cudaMemcpyHostToDevice);
  int st = e == cudaSuccess ? FS_OK : cuda_fail(e, "compare upload");
  std::vector<double *> pa(n), pb(n);
  std::vector<double> dr(2 * n);
  for (int k = 0; k < n; k++) {
    pa[k] = d + k * hw;
    pb[k] = d + (n + k) * hw;
    dr[2 * k] = params[k].dr_orth;
    dr[2 * k + 1] = params[k].dr_diag;
  }
  if (st == FS_OK)
    st = compare_fields(width, height, n, pa.data(), pb.data(), dr.data(), rel_rms, agreement,
                        nullptr);
  cudaFree(d);
  return st;
}

int fs_sg_ensemble_run(fs_batch *b, fs_surrogate *s, const fs_sg_ensemble_opts *o,
                       fs_sg_ensemble_stats *stats, int *fallen) {
  if (!b || !s || !o) return fail(FS_ERR_ARG, "ensemble: NULL argument");
  if (o->nsteps < 0 || o->plain_steps < 0 || !(o->judge_fraction >= 0) ||
      !(o->judge_fraction <= 1))
    return fail(FS_ERR_ARG, "ensemble: nsteps, plain_steps >= 0, judge_fraction in [0, 1]");
  fs_sg_config cfg;
  if (int st = fs_sg_get_config(s, &cfg)) return st;
  int n = 0;
  int64_t cells = 0;
  if (int st = fs_batch_info(b, &n, &cells)) return st;
  std::vector<fs_params> P(n);
  for (int r = 0; r < n; r++) {
    int w = 0, h = 0;
    if (int st = fs_batch_get_shape(b, r, &w, &h)) return st;
    if (w != cfg.width || h != cfg.height)
      return fail(FS_ERR_ARG, "ensemble: realization %d is %d x %d, the network takes %d x %d", r,
                  w, h, cfg.width, cfg.height);
    if (int st = fs_batch_get_params(b, r, &P[r])) return st;
    if (P[r].dt != cfg.dt)
      return fail(FS_ERR_ARG, "ensemble: realization %d has dt %g, the network was built for %g",
                  r, P[r].dt, cfg.dt);
  }
  void *bs = nullptr;
  if (int st = fs_batch_stream(b, &bs)) return st;
  cudaStream_t stream = static_cast<cudaStream_t>(bs);
  const int jump = cfg.jump;
  const int cycle = jump + o->plain_steps;
  const int ncycles = cycle > 0 ? o->nsteps / cycle : 0;
  const int rest = o->nsteps - ncycles * cycle;
  const size_t hw = static_cast<size_t>(cfg.width) * cfg.height;
  const int jmax = static_cast<int>(std::ceil(o->judge_fraction * n)) + 1;
  // side fields of the judged jumps: their predictions, then the fields
  // before the jump (the no-change reference the judge also measures)
  double *side = nullptr;
  if (jmax > 0 && o->judge_fraction > 0) {
    cudaError_t e = cudaMalloc(&side, 2 * hw * jmax * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "judge fields");
  }
  double pers_rel_sum = 0, pers_agree_sum = 0;
  fs_sg_ensemble_stats S{};
  S.rel_rms_max = 0;
  S.agreement_min = 1;
  std::vector<int> mode(n, 0);  // 0 surrogate, 1 plain
  std::mt19937_64 gen(o->seed);
  std::vector<double *> field(n);
  int st = FS_OK;
  for (int r = 0; r < n && st == FS_OK; r++) st = fs_batch_device_elevation(b, r, &field[r]);
  double rel_sum = 0, agree_sum = 0;
  const auto t_all = Clock::now();
  std::vector<int> sur, judged, free_jump, exact;
  std::vector<double *> outs;
  for (int c = 0; c < ncycles && st == FS_OK; c++) {
    sur.clear();
    for (int r = 0; r < n; r++)
      if (mode[r] == 0) sur.push_back(r);
    // the judged jumps of this cycle: a seeded sample of the surrogate's
    int nj = o->judge_fraction > 0
                 ? static_cast<int>(std::lround(o->judge_fraction * sur.size()))
                 : 0;
    if (o->judge_fraction > 0 && nj == 0 && !sur.empty()) nj = 1;
    nj = std::min(nj, jmax);
    std::shuffle(sur.begin(), sur.end(), gen);
    judged.assign(sur.begin(), sur.begin() + nj);
    free_jump.assign(sur.begin() + nj, sur.end());
    std::sort(judged.begin(), judged.end());
    std::sort(free_jump.begin(), free_jump.end());
    // 1. jumps
    auto t0 = Clock::now();
    if (!free_jump.empty())
      st = fs_sg_predict_batch(s, b, static_cast<int>(free_jump.size()), free_jump.data(), nullptr);
    outs.resize(judged.size());
    std::vector<double *> before(judged.size());
    for (size_t k = 0; k < judged.size(); k++) {
      outs[k] = side + k * hw;
      before[k] = side + (jmax + k) * hw;
      if (st == FS_OK &&
          cudaMemcpyAsync(before[k], field[judged[k]], hw * sizeof(double),
                          cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
        st = cuda_fail(cudaGetLastError(), "judge copy");
    }
    if (st == FS_OK && cudaStreamSynchronize(stream) != cudaSuccess)
      st = cuda_fail(cudaGetLastError(), "judge copy");
    if (st == FS_OK && !judged.empty())
      st = fs_sg_predict_batch(s, b, static_cast<int>(judged.size()), judged.data(), outs.data());
    S.ms_infer += ms_since(t0);
    S.jumps += static_cast<int>(sur.size());
    // 2. exact runs: the judged jumps and the realizations on the plain method
    t0 = Clock::now();
    exact.assign(judged.begin(), judged.end());
    for (int r = 0; r < n; r++)
      if (mode[r] == 1) exact.push_back(r);
    std::sort(exact.begin(), exact.end());
    if (st == FS_OK && !exact.empty()) {
      st = fs_batch_set_active(b, static_cast<int>(exact.size()), exact.data());
      if (st == FS_OK) st = fs_batch_step(b, jump);
    }
    S.ms_exact += ms_since(t0);
    // 3. the judge
    t0 = Clock::now();
    if (st == FS_OK && !judged.empty()) {
      std::vector<double *> ex(judged.size());
      std::vector<double> dr(2 * judged.size()), rel(judged.size()), ag(judged.size());
      for (size_t k = 0; k < judged.size(); k++) {
        ex[k] = field[judged[k]];
        dr[2 * k] = P[judged[k]].dr_orth;
        dr[2 * k + 1] = P[judged[k]].dr_diag;
      }
      st = compare_fields(cfg.width, cfg.height, static_cast<int>(judged.size()), outs.data(),
                          ex.data(), dr.data(), rel.data(), ag.data(), stream);
      std::vector<double> rel_p(judged.size()), ag_p(judged.size());
      if (st == FS_OK)
        st = compare_fields(cfg.width, cfg.height, static_cast<int>(judged.size()),
                            before.data(), ex.data(), dr.data(), rel_p.data(), ag_p.data(),
                            stream);
      for (size_t k = 0; k < judged.size() && st == FS_OK; k++) {
        pers_rel_sum += rel_p[k];
        pers_agree_sum += ag_p[k];
      }
      for (size_t k = 0; k < judged.size() && st == FS_OK; k++) {
        S.judged++;
        rel_sum += rel[k];
        agree_sum += ag[k];
        S.rel_rms_max = std::max(S.rel_rms_max, rel[k]);
        S.agreement_min = std::min(S.agreement_min, ag[k]);
        if (!(rel[k] <= o->max_rel_rms) || !(ag[k] >= o->min_agreement)) {
          mode[judged[k]] = 1;
          S.fallbacks++;
        }
      }
    }
    S.ms_judge += ms_since(t0);
    // 4. plain timesteps for every realization
    t0 = Clock::now();
    if (st == FS_OK && o->plain_steps > 0) {
      st = fs_batch_set_active(b, 0, nullptr);
      if (st == FS_OK) st = fs_batch_step(b, o->plain_steps);
    }
    S.ms_plain += ms_since(t0);
    S.cycles++;
  }
  if (st == FS_OK) st = fs_batch_set_active(b, 0, nullptr);
  if (st == FS_OK && rest > 0) {
    const auto t0 = Clock::now();
    st = fs_batch_step(b, rest);
    S.ms_plain += ms_since(t0);
  }
  S.ms_total = ms_since(t_all);
  if (side) cudaFree(side);
  fs_batch_set_active(b, 0, nullptr);
  if (S.judged > 0) {
    S.rel_rms_mean = rel_sum / S.judged;
    S.agreement_mean = agree_sum / S.judged;
    S.rel_rms_unchanged_mean = pers_rel_sum / S.judged;
    S.agreement_unchanged_mean = pers_agree_sum / S.judged;
  } else {
    S.agreement_min = 0;
  }
  if (stats) *stats = S;
  if (fallen)
    for (int r = 0; r < n; r++) fallen[r] = mode[r];
  return st;
}

}  // extern "C"
