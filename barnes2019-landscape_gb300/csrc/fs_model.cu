// fs_model.cu -- host side of the C ABI declared in include/fastscape_gb300.h.
//
// Every model is a batch of realizations on one CUDA stream (fs_create makes
// a batch of one; fs_batch_create a ragged batch). A batch owns its device
// buffers for its whole life (the reference reallocates and frees its
// scratch on every run(), fastscape_RB.cpp:346-358 and :392-397). Layout in
// HBM, for C = the batch's total cells (realization r at [off_r, off_r+size_r)):
//   h       double[C]           elevation (the only state carried between
//                               timesteps, as in the reference)
//   rec     int8[C]             receiver direction code, -1 rings, -2 pits
//   mask    uint8[C]            donor mask (bit k: neighbour k drains here)
//   ent     int32[C]            cells grouped by level (the reference's stack)
//   pdir    uint8[C]            receiver direction by level position
//   acc     uint32[C]           drainage cell counts by level position
//                               (accum = acc*cell_area)
//   par     int32[C]            receiver's position by level position
//   amb     int32[C], amb_r     cells queued for the FP64 receiver fix-up
//   lvl_off int32[C+2n]         level offsets, size_r+2 per realization
//   tab_r   double[8*cap_r]     erosion table of realization r per drainage
//                               count k < cap_r (fs_internal.h); grows on
//                               demand
//   desc, rctl, ctl, tiles      descriptors, counters, status, stencil tiles
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "fastscape_gb300.h"
#include "fs_internal.h"

namespace {

thread_local std::string g_last_error;

int set_error(int status, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int cuda_error(cudaError_t e, const char *what) {
  return set_error(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA, "%s: %s", what,
                   cudaGetErrorString(e));
}

#define FS_CUDA(call)                                           \
  do {                                                          \
    cudaError_t fs_e_ = (call);                                 \
    if (fs_e_ != cudaSuccess) return cuda_error(fs_e_, #call);  \
  } while (0)

const double kSqrt2 = 1.414213562373095048801688724209698078569671875376948;

const char *status_name(int s) {
  switch (s) {
    case FS_OK: return "ok";
    case FS_ERR_ARG: return "invalid argument";
    case FS_ERR_CUDA: return "CUDA error";
    case FS_ERR_TIMEOUT: return "grid barrier wait timed out";
    case FS_ERR_LEVEL_OVERFLOW: return "level walk overflowed the grid size";
    case FS_ERR_NONFINITE: return "non-finite elevation";
    case FS_ERR_ORDER: return "receivers contain a cycle (cells never reach base level)";
    case FS_ERR_NEWTON: return "Newton iteration did not converge";
    case FS_ERR_NOMEM: return "out of device memory";
    case FS_ERR_STATE: return "no timestep executed yet";
    default: return "unknown status";
  }
}

bool valid_params(const fs_params &p) {
  const double v[9] = {p.keq, p.neq, p.meq, p.ueq, p.dt, p.dr_orth, p.dr_diag, p.tol, p.cell_area};
  for (double x : v)
    if (!std::isfinite(x)) return false;
  return p.dr_orth > 0 && p.dr_diag > 0 && p.cell_area > 0 && p.tol >= 0;
}

int nmode_of(double neq) {
  return neq == 1.0 ? fs::kNOne : neq == 2.0 ? fs::kNTwo : fs::kNGeneral;
}

}  // namespace

int fs::record_error(int status, const char *msg) { return set_error(status, "%s", msg); }

// ---------------------------------------------------------------------------
// Batch: the device state of n realizations and how to step it.
// ---------------------------------------------------------------------------
struct fs_batch {
  int n = 0;
  std::vector<int> W, H, size, off, lvl_base, nring;
  std::vector<fs_params> p;
  long long cells = 0, lvl_total = 0;
  int nmode = fs::kNOne;
  double neq = 1.0;
  int device = 0;
  cudaStream_t stream = nullptr;
  double *h = nullptr;
  int8_t *rec = nullptr;
  int8_t *rec_alloc = nullptr;  // rec - kRecPad
  uint8_t *mask = nullptr, *pdir = nullptr;
  int32_t *ent = nullptr, *par = nullptr, *amb = nullptr, *amb_r = nullptr, *lvl = nullptr;
  uint32_t *acc = nullptr;
  fs::RealDesc *d_desc = nullptr;
  fs::RealCtl *d_rctl = nullptr, *h_rctl = nullptr;
  fs::Ctl *d_ctl = nullptr, *h_ctl = nullptr;
  fs::Tile *d_rtiles = nullptr, *d_dtiles = nullptr;
  int nrtiles = 0, ndtiles = 0;
  std::vector<fs::RealDesc> desc;
  std::vector<double *> tab;
  std::vector<int> tab_cap;
  int walk_occ = 1, walk_sms = 1, walk_bps = 2;  // k_erode blocks per SM: limit, SMs, in use
  int order_max = 2, order_bps = 2;              // k_order blocks per SM: limit (2 or 3), in use
  int accum_bps = 1;                             // k_accum blocks per SM
  int erode_isub = 0;                            // k_erode's integer subtractions (n = 1)
  // per-realization walk (one CTA per realization, block barriers only):
  // used when cta_walk and the launch covers more than one realization;
  // resident CTAs per SM of its ordering and erosion kernels (by variant)
  bool cta_walk = false;
  int cta_occ_order = 1, cta_occ_erode[3] = {1, 1, 1};
  // a single grid's receiver filter may stage its tiles by TMA (rmap_ok:
  // the map exists; rtma: in use; the autotuner decides)
  CUtensorMap rmap;
  bool rmap_ok = false, rtma = false;
  unsigned long long timeout_ns = 2000000000ull;
  long long steps = 0;
  bool have_step = false;
  int timing = 0;          // 0 off, 1 per kernel (direct launches), 2 whole calls
  bool exact_receivers = false;
  bool erode_generic = false;                    // test: the reference's Newton loop literally
  bool use_graph = true;  // the autotuner's choice at every size measured
  cudaGraphExec_t graph = nullptr;
  bool graph_dirty = true;
  std::vector<cudaEvent_t> ev;
  double phase_ms[FS_NUM_TIMERS] = {};  // event timers (indices 0-3, 7, 8)
  // Active subset (fs_batch_set_active): act_n > 0 steps only the
  // realizations act_idx through their own descriptor, counter and tile
  // arrays (the per-cell arrays are shared); act_n == 0 steps all.
  int act_n = 0;
  std::vector<int> act_idx;
  fs::RealDesc *d_desc_act = nullptr;
  fs::RealCtl *d_rctl_act = nullptr;
  int *d_act_idx = nullptr;
  fs::Tile *d_rtiles_act = nullptr, *d_dtiles_act = nullptr;
  int nrt_act = 0, ndt_act = 0, act_cap = 0, act_tiles_cap[2] = {0, 0};
  int act_walk_bps = 0, act_order_bps = 0, act_accum_bps = 0;
};

struct fs_model {
  fs_batch *b = nullptr;
};

namespace {

struct DeviceGuard {
  int prev = 0;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() { cudaSetDevice(prev); }
};

void free_batch(fs_batch *b) {
  if (!b) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  void *bufs[] = {b->h, b->rec_alloc, b->mask, b->pdir, b->ent, b->par, b->amb, b->amb_r,
                  b->lvl, b->acc, b->d_desc, b->d_rctl, b->d_ctl, b->d_rtiles, b->d_dtiles,
                  b->d_desc_act, b->d_rctl_act, b->d_act_idx, b->d_rtiles_act,
                  b->d_dtiles_act};
  for (void *x : bufs) cudaFree(x);
  for (double *t : b->tab) cudaFree(t);
  if (b->h_ctl) cudaFreeHost(b->h_ctl);
  if (b->h_rctl) cudaFreeHost(b->h_rctl);
  for (auto &e : b->ev) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  cudaSetDevice(prev);
  delete b;
}

// Erosion table of realization r for counts [0, cap), cap from doubling
// until it exceeds `need`, at most size_r + 1. Evaluated on the host with
// the C library's pow in the order of fastscape_RB.cpp:315 (the reference's
// accum[c] is k*cell_area exactly: integer multiples summed below 2^53), so
// the device sees the reference's bits. Parallel over host threads.
int grow_table(fs_batch *b, int r, long long need) {
  long long cap = std::max<long long>(b->tab_cap[r], 1);
  while (cap <= need) cap *= 2;
  cap = std::min<long long>(cap, static_cast<long long>(b->size[r]) + 1);
  if (cap <= b->tab_cap[r])
    return set_error(FS_ERR_CUDA, "erosion table of realization %d cannot grow past %d", r,
                     b->tab_cap[r]);
  std::vector<double> host(static_cast<size_t>(cap) * fs::kTabStride);
  const fs_params &p = b->p[r];
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, 64);
  if (cap < 65536 * 2) nt = 1;
  auto work = [&](unsigned t) {
    const long long lo = cap * t / nt, hi = cap * (t + 1) / nt;
    fs::fill_table_range(p.keq, p.neq, p.meq, p.dt, p.dr_orth, p.dr_diag, p.cell_area, lo, hi,
                         host.data() + lo * fs::kTabStride);
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  double *d = nullptr;
  FS_CUDA(cudaMalloc(&d, host.size() * sizeof(double)));
  cudaError_t e =
      cudaMemcpyAsync(d, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_error(e, "upload(erosion table)");
  }
  cudaFree(b->tab[r]);
  b->tab[r] = d;
  b->tab_cap[r] = static_cast<int>(cap);
  b->desc[r].tab = d;
  b->desc[r].tab_cap = static_cast<int>(cap);
  FS_CUDA(cudaMemcpyAsync(b->d_desc + r, &b->desc[r], sizeof(fs::RealDesc), cudaMemcpyHostToDevice,
                          b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  b->graph_dirty = true;
  return FS_OK;
}

// The reference field (fastscape_RB.cpp:111-130 via random.cpp:45-49),
// generated with the same libstdc++ engine and distribution.
void reference_field(double *h, int W, int H, uint32_t engine_seed) {
  std::mt19937 eng(engine_seed);
  std::uniform_real_distribution<double> d(0.0, 1.0);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      double v = d(eng);
      if (x == 0 || y == 0 || x == W - 1 || y == H - 1) v = 0;
      if (x == 1 || y == 1 || x == W - 2 || y == H - 2) v = 0;
      h[static_cast<size_t>(y) * W + x] = v;
    }
}

fs::StepArgs step_args(const fs_batch *b, int do_erode) {
  fs::StepArgs a{};
  a.h = b->h;
  a.rec = b->rec;
  a.mask = b->mask;
  a.ent = b->ent;
  a.pdir = b->pdir;
  a.par = b->par;
  a.acc = b->acc;
  a.amb = b->amb;
  a.amb_r = b->amb_r;
  a.lvl_off = b->lvl;
  a.desc = b->d_desc;
  a.rctl = b->d_rctl;
  a.ctl = b->d_ctl;
  a.nreal = b->n;
  a.rtiles = b->d_rtiles;
  a.nrtiles = b->nrtiles;
  a.dtiles = b->d_dtiles;
  a.ndtiles = b->ndtiles;
  if (b->act_n > 0) {
    a.desc = b->d_desc_act;
    a.rctl = b->d_rctl_act;
    a.nreal = b->act_n;
    a.rtiles = b->d_rtiles_act;
    a.nrtiles = b->nrt_act;
    a.dtiles = b->d_dtiles_act;
    a.ndtiles = b->ndt_act;
  }
  a.nmode = b->nmode;
  a.neq = b->neq;
  a.do_erode = do_erode;
  a.erode_isub = b->erode_isub;
  a.erode_generic = b->erode_generic ? 1 : 0;
  a.stamp = b->timing == 1 ? 1 : 0;
  a.timeout_ns = b->timeout_ns;
  return a;
}

const CUtensorMap *receiver_map(const fs_batch *b) {
  return b->rtma && b->rmap_ok && b->n == 1 ? &b->rmap : nullptr;
}

// The per-realization walk runs when chosen and the launch covers more than
// one realization (a single grid keeps the grid-wide walk).
bool use_cta(const fs_batch *b, const fs::StepArgs &a) { return b->cta_walk && a.nreal > 1; }

// CTAs of a per-realization walk kernel: every realization at once where
// they fit, else as many as are resident (each loops over realizations).
int cta_blocks(const fs_batch *b, const fs::StepArgs &a, bool erode) {
  const int var = a.erode_generic ? 2 : a.erode_isub ? 1 : 0;
  const int occ = erode ? b->cta_occ_erode[var] : b->cta_occ_order;
  const int resident = b->walk_sms * std::max(occ, 1);
  return std::max(1, std::min(a.nreal, resident));
}

// The launches of one timestep (no synchronization).
cudaError_t launch_step(fs_batch *b, const fs::StepArgs &a) {
  cudaError_t e = cudaMemsetAsync(reinterpret_cast<char *>(b->d_ctl) + fs::kCtlResetOffset, 0,
                                  fs::kCtlResetBytes, b->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(a.rctl, 0, sizeof(fs::RealCtl) * a.nreal, b->stream);
  if (e == cudaSuccess)
    e = b->exact_receivers ? fs::launch_receivers_exact(a, b->stream)
                           : fs::launch_receivers_fast(a, b->stream, receiver_map(b));
  if (e == cudaSuccess) e = fs::launch_donors_level0(a, b->stream);
  if (e == cudaSuccess) {
    if (use_cta(b, a)) {
      e = fs::launch_cta_order(a, cta_blocks(b, a, false), b->stream);
      if (e == cudaSuccess && a.do_erode)
        e = fs::launch_cta_erode(a, cta_blocks(b, a, true), b->stream);
    } else if (b->act_n > 0) {
      e = fs::launch_walk(a, b->walk_sms, b->act_order_bps, b->act_accum_bps, b->act_walk_bps,
                          b->stream);
    } else {
      e = fs::launch_walk(a, b->walk_sms, b->order_bps, b->accum_bps, b->walk_bps, b->stream);
    }
  }
  return e;
}

int ensure_events(fs_batch *b, size_t n) {
  while (b->ev.size() < n) {
    cudaEvent_t e;
    FS_CUDA(cudaEventCreate(&e));
    b->ev.push_back(e);
  }
  return FS_OK;
}

// Events per timed timestep: start, after the receivers, after the donors,
// after the ordering, after the accumulation (the next timestep's start, or
// the final event, closes the erosion kernel).
constexpr int kEvPerStep = 5;

// One timestep with the phase events ev[5i..5i+5] around its launches.
int timed_step(fs_batch *b, const fs::StepArgs &a, int i) {
  cudaEvent_t *ev = &b->ev[kEvPerStep * i];
  FS_CUDA(cudaEventRecord(ev[0], b->stream));
  FS_CUDA(cudaMemsetAsync(reinterpret_cast<char *>(b->d_ctl) + fs::kCtlResetOffset, 0,
                          fs::kCtlResetBytes, b->stream));
  FS_CUDA(cudaMemsetAsync(a.rctl, 0, sizeof(fs::RealCtl) * a.nreal, b->stream));
  FS_CUDA(b->exact_receivers ? fs::launch_receivers_exact(a, b->stream)
                             : fs::launch_receivers_fast(a, b->stream, receiver_map(b)));
  FS_CUDA(cudaEventRecord(ev[1], b->stream));
  FS_CUDA(fs::launch_donors_level0(a, b->stream));
  FS_CUDA(cudaEventRecord(ev[2], b->stream));
  const bool act = b->act_n > 0;
  if (use_cta(b, a)) {
    // ordering + accumulation in one kernel (reported as the ordering's),
    // then the erosion
    FS_CUDA(fs::launch_cta_order(a, cta_blocks(b, a, false), b->stream));
    FS_CUDA(cudaEventRecord(ev[3], b->stream));
    FS_CUDA(cudaEventRecord(ev[4], b->stream));
    FS_CUDA(fs::launch_cta_erode(a, cta_blocks(b, a, true), b->stream));
    return FS_OK;
  }
  FS_CUDA(fs::launch_order(a, b->walk_sms, act ? b->act_order_bps : b->order_bps, b->stream));
  FS_CUDA(cudaEventRecord(ev[3], b->stream));
  FS_CUDA(fs::launch_accum(a, b->walk_sms, act ? b->act_accum_bps : b->accum_bps, b->stream));
  FS_CUDA(cudaEventRecord(ev[4], b->stream));
  FS_CUDA(fs::launch_erode(a, b->walk_sms, act ? b->act_walk_bps : b->walk_bps, b->stream));
  return FS_OK;
}

int harvest_events(fs_batch *b, int k) {
  FS_CUDA(cudaEventSynchronize(b->ev[kEvPerStep * k]));
  // receivers, donors, k_order, k_accum, k_erode
  static const int slot[kEvPerStep] = {0, 1, 7, 9, 8};
  for (int i = 0; i < k; i++)
    for (int j = 0; j < kEvPerStep; j++) {
      float ms = 0;
      FS_CUDA(cudaEventElapsedTime(&ms, b->ev[kEvPerStep * i + j], b->ev[kEvPerStep * i + j + 1]));
      b->phase_ms[slot[j]] += ms;
      if (j >= 2) b->phase_ms[2] += ms;  // the level walk: its three kernels
    }
  float tot = 0;
  FS_CUDA(cudaEventElapsedTime(&tot, b->ev[0], b->ev[kEvPerStep * k]));
  b->phase_ms[3] += tot;
  return FS_OK;
}

// Captures one timestep into a CUDA graph (re-captured whenever the
// launch configuration or a descriptor changes). On any capture failure the
// batch falls back to direct launches.
int build_graph(fs_batch *b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  const fs::StepArgs a = step_args(b, 1);
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t le = launch_step(b, a);
    e = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  if (e != cudaSuccess) {
    b->graph = nullptr;
    b->use_graph = false;
  }
  b->graph_dirty = false;
  return FS_OK;
}

int collect_status(fs_batch *b) {
  FS_CUDA(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  const int err = b->h_ctl->err;
  if (err != 0)
    return set_error(err, "timestep failed: %s (phase %d)", status_name(err), b->h_ctl->err_detail);
  return FS_OK;
}

int read_rctl(const fs_batch *b) {
  FS_CUDA(cudaMemcpyAsync(b->h_rctl, b->d_rctl, sizeof(fs::RealCtl) * b->n, cudaMemcpyDeviceToHost,
                          b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  return FS_OK;
}

// Copies the active subset's per-realization counters (levels found,
// cells placed) back to the realizations' own entries.
__global__ void k_scatter_rctl(const fs::RealCtl *__restrict__ src, const int *__restrict__ idx,
                               int n, fs::RealCtl *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[idx[i]] = src[i];
}

cudaError_t launch_scatter_rctl(fs_batch *b) {
  k_scatter_rctl<<<(b->act_n + 127) / 128, 128, 0, b->stream>>>(b->d_rctl_act, b->d_act_idx,
                                                                b->act_n, b->d_rctl);
  return cudaGetLastError();
}

// Per-cell drainage counts of one realization from the walk's
// position-indexed arrays: counts[ent[i]] = acc[i].
__global__ void k_drainage_counts(const int32_t *__restrict__ ent, const uint32_t *__restrict__ acc,
                                  int size, uint32_t *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x)
    out[ent[i]] = acc[i];
}

// Initial erosion tables of every realization (counts below min(65536,
// size+1)), evaluated on host threads in parallel over realizations -- the
// same records grow_table writes -- then uploaded.
int init_tables(fs_batch *b) {
  const int n = b->n;
  std::vector<std::vector<double>> host(n);
  std::vector<long long> cap(n);
  for (int r = 0; r < n; r++) {
    long long c = 1;
    while (c <= std::min<long long>(b->size[r], 65535)) c *= 2;
    cap[r] = std::min<long long>(c, static_cast<long long>(b->size[r]) + 1);
  }
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, 64);
  nt = std::min<unsigned>(nt, static_cast<unsigned>(n));
  auto work = [&](unsigned t) {
    for (int r = static_cast<int>(t); r < n; r += static_cast<int>(nt)) {
      const fs_params &p = b->p[r];
      host[r].resize(static_cast<size_t>(cap[r]) * fs::kTabStride);
      fs::fill_table_range(p.keq, p.neq, p.meq, p.dt, p.dr_orth, p.dr_diag, p.cell_area, 0,
                           cap[r], host[r].data());
    }
  };
  if (nt <= 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  for (int r = 0; r < n; r++) {
    double *d = nullptr;
    FS_CUDA(cudaMalloc(&d, host[r].size() * sizeof(double)));
    b->tab[r] = d;
    b->tab_cap[r] = static_cast<int>(cap[r]);
    b->desc[r].tab = d;
    b->desc[r].tab_cap = static_cast<int>(cap[r]);
    FS_CUDA(cudaMemcpyAsync(d, host[r].data(), host[r].size() * sizeof(double),
                            cudaMemcpyHostToDevice, b->stream));
    FS_CUDA(cudaStreamSynchronize(b->stream));  // host[r] may be released next
    std::vector<double>().swap(host[r]);
  }
  FS_CUDA(cudaMemcpyAsync(b->d_desc, b->desc.data(), n * sizeof(fs::RealDesc),
                          cudaMemcpyHostToDevice, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  b->graph_dirty = true;
  return FS_OK;
}

// Blocks per SM of a cooperative walk kernel: `want`, or fewer when fewer are
// resident with `smem` bytes of shared memory.
int resident_bps(const void *kernel, size_t smem, int want, int *out) {
  int occ = 0;
  FS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, fs::walk_threads(), smem));
  if (occ < 1) return set_error(FS_ERR_CUDA, "walk kernel cannot be resident");
  *out = std::min(occ, want);
  return FS_OK;
}

// Selects the realizations the next timesteps advance (n = 0: all).
int set_active(fs_batch *b, int n, const int *idx) {
  if (n < 0 || n > b->n) return set_error(FS_ERR_ARG, "active count %d out of [0, %d]", n, b->n);
  if (n > 0 && !idx) return set_error(FS_ERR_ARG, "idx is NULL");
  DeviceGuard dg(b->device);
  FS_CUDA(cudaStreamSynchronize(b->stream));
  b->graph_dirty = true;
  if (n == 0) {
    b->act_n = 0;
    b->act_idx.clear();
    return FS_OK;
  }
  std::vector<char> seen(b->n, 0);
  for (int i = 0; i < n; i++) {
    if (idx[i] < 0 || idx[i] >= b->n)
      return set_error(FS_ERR_ARG, "realization %d out of range [0, %d)", idx[i], b->n);
    if (seen[idx[i]]) return set_error(FS_ERR_ARG, "realization %d listed twice", idx[i]);
    seen[idx[i]] = 1;
  }
  std::vector<fs::RealDesc> desc(n);
  std::vector<fs::Tile> rt, dt;
  for (int i = 0; i < n; i++) {
    const int r = idx[i];
    desc[i] = b->desc[r];
    for (int kind = 0; kind < 2; kind++) {
      std::vector<fs::Tile> &v = kind == 0 ? rt : dt;
      const size_t at = v.size();
      v.resize(at + static_cast<size_t>(b->W[r] / 32 + 2) * (b->H[r] / 32 + 2));
      const int got = fs::append_tiles(kind, i, b->W[r], b->H[r], v.data() + at,
                                       static_cast<int>(v.size() - at));
      v.resize(at + std::max(got, 0));
    }
  }
  if (n > b->act_cap) {
    cudaFree(b->d_desc_act);
    cudaFree(b->d_rctl_act);
    cudaFree(b->d_act_idx);
    b->d_desc_act = nullptr;
    b->d_rctl_act = nullptr;
    b->d_act_idx = nullptr;
    b->act_cap = 0;
    FS_CUDA(cudaMalloc(&b->d_desc_act, n * sizeof(fs::RealDesc)));
    FS_CUDA(cudaMalloc(&b->d_rctl_act, n * sizeof(fs::RealCtl)));
    FS_CUDA(cudaMalloc(&b->d_act_idx, n * sizeof(int)));
    b->act_cap = n;
  }
  fs::Tile **tiles[2] = {&b->d_rtiles_act, &b->d_dtiles_act};
  const size_t ntile[2] = {rt.size(), dt.size()};
  for (int k = 0; k < 2; k++)
    if (static_cast<int>(ntile[k]) > b->act_tiles_cap[k]) {
      cudaFree(*tiles[k]);
      *tiles[k] = nullptr;
      b->act_tiles_cap[k] = 0;
      FS_CUDA(cudaMalloc(tiles[k], std::max<size_t>(1, ntile[k]) * sizeof(fs::Tile)));
      b->act_tiles_cap[k] = static_cast<int>(ntile[k]);
    }
  FS_CUDA(cudaMemcpyAsync(b->d_desc_act, desc.data(), n * sizeof(fs::RealDesc),
                          cudaMemcpyHostToDevice, b->stream));
  FS_CUDA(cudaMemcpyAsync(b->d_act_idx, idx, n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if (!rt.empty())
    FS_CUDA(cudaMemcpyAsync(b->d_rtiles_act, rt.data(), rt.size() * sizeof(fs::Tile),
                            cudaMemcpyHostToDevice, b->stream));
  if (!dt.empty())
    FS_CUDA(cudaMemcpyAsync(b->d_dtiles_act, dt.data(), dt.size() * sizeof(fs::Tile),
                            cudaMemcpyHostToDevice, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  // a subset of one runs the single-grid kernels, which may hold fewer
  // blocks per SM than the batch kernels the launch shape was tuned for
  const bool single = n == 1;
  const size_t smem = fs::walk_smem_bytes(n);
  if (int st = resident_bps(fs::walk_kernel_ptr(b->nmode, single, b->erode_isub ? 1 : 0), smem,
                           b->walk_bps, &b->act_walk_bps))
    return st;
  if (int st = resident_bps(fs::order_kernel_ptr(single, b->order_bps), smem, b->order_bps,
                           &b->act_order_bps))
    return st;
  if (b->act_order_bps < b->order_bps) {
    // the 3-block ordering form is compiled for exactly 3 blocks per SM
    if (int st = resident_bps(fs::order_kernel_ptr(single, 2), smem, 2, &b->act_order_bps))
      return st;
  }
  if (int st = resident_bps(fs::accum_kernel_ptr(single), smem, b->accum_bps,
                           &b->act_accum_bps))
    return st;
  b->nrt_act = static_cast<int>(rt.size());
  b->ndt_act = static_cast<int>(dt.size());
  b->act_idx.assign(idx, idx + n);
  b->act_n = n;
  return FS_OK;
}

// k timesteps of every realization; a timestep that outgrew an erosion table
// stopped before changing h and the rest of the batch did nothing: grow the
// table and carry on from there.
int batch_step(fs_batch *b, int k) {
  if (k < 0) return set_error(FS_ERR_ARG, "step count must be >= 0 (got %d)", k);
  if (k == 0) return FS_OK;
  DeviceGuard dg(b->device);
  int done = 0;
  while (done < k) {
    const int batch = k - done;
    const fs::StepArgs a = step_args(b, 1);
    FS_CUDA(cudaMemsetAsync(b->d_ctl, 0, fs::kCtlCallResetBytes, b->stream));
    if (b->timing == 1) {
      if (int st = ensure_events(b, kEvPerStep * static_cast<size_t>(batch) + 1)) return st;
      for (int i = 0; i < batch; i++)
        if (int st = timed_step(b, a, i)) return st;
      FS_CUDA(cudaEventRecord(b->ev[kEvPerStep * batch], b->stream));
      if (int st = harvest_events(b, batch)) return st;
    } else {
      if (b->use_graph && b->graph_dirty)
        if (int st = build_graph(b)) return st;
      if (b->timing == 2) {
        if (int st = ensure_events(b, 2)) return st;
        FS_CUDA(cudaEventRecord(b->ev[0], b->stream));
      }
      for (int i = 0; i < batch; i++) {
        if (b->use_graph && b->graph)
          FS_CUDA(cudaGraphLaunch(b->graph, b->stream));
        else
          FS_CUDA(launch_step(b, a));
      }
      if (b->timing == 2) {
        // the whole call only: the launch path (graph replay or direct) is
        // the one in use, with no event between its kernels
        FS_CUDA(cudaEventRecord(b->ev[1], b->stream));
        FS_CUDA(cudaEventSynchronize(b->ev[1]));
        float tot = 0;
        FS_CUDA(cudaEventElapsedTime(&tot, b->ev[0], b->ev[1]));
        b->phase_ms[3] += tot;
      }
    }
    if (b->act_n > 0) FS_CUDA(launch_scatter_rctl(b));
    if (int st = collect_status(b)) return st;
    const int completed = b->h_ctl->steps_done;
    done += completed;
    b->steps += completed;
    if (completed > 0) b->have_step = true;
    if (b->h_ctl->abort_k > 0) {
      const int ar = b->act_n > 0 ? b->act_idx[b->h_ctl->abort_r] : b->h_ctl->abort_r;
      if (int st = grow_table(b, ar, b->h_ctl->abort_k)) return st;
      if (b->act_n > 0)
        for (int i = 0; i < b->act_n; i++)
          if (b->act_idx[i] == ar)
            FS_CUDA(cudaMemcpyAsync(b->d_desc_act + i, &b->desc[ar], sizeof(fs::RealDesc),
                                    cudaMemcpyHostToDevice, b->stream));
    } else if (completed != batch) {
      return set_error(FS_ERR_CUDA, "%d of %d timesteps completed without a status", completed,
                       batch);
    }
  }
  return FS_OK;
}

fs_batch *batch_create(int n, const int *widths, const int *heights, const fs_params *params,
                       int init_mode, const uint64_t *seeds, int *status) {
  int dummy = 0;
  if (!status) status = &dummy;
  *status = FS_OK;
  if (n < 1 || n > fs::kMaxReal) {
    *status = set_error(FS_ERR_ARG, "batch size must be in [1, %d] (got %d)", fs::kMaxReal, n);
    return nullptr;
  }
  if (!widths || !heights || !params) {
    *status = set_error(FS_ERR_ARG, "widths, heights and params must not be NULL");
    return nullptr;
  }
  if (init_mode < FS_INIT_ZERO || init_mode > FS_INIT_PHILOX) {
    *status = set_error(FS_ERR_ARG, "unknown init_mode %d", init_mode);
    return nullptr;
  }
  long long cells = 0;
  for (int r = 0; r < n; r++) {
    if (widths[r] < 3 || heights[r] < 3) {
      *status = set_error(FS_ERR_ARG, "width and height must be >= 3 (realization %d: %d x %d)", r,
                          widths[r], heights[r]);
      return nullptr;
    }
    cells += static_cast<long long>(widths[r]) * heights[r];
    if (!valid_params(params[r])) {
      *status = set_error(FS_ERR_ARG,
                          "parameters must be finite, dr and cell_area > 0, tol >= 0 (realization %d)", r);
      return nullptr;
    }
    if (params[r].neq != params[0].neq) {
      *status = set_error(FS_ERR_ARG, "all realizations of a batch must share n (neq)");
      return nullptr;
    }
  }
  if (cells + 2ll * n >= (1ll << 31) - 2) {
    *status = set_error(FS_ERR_ARG, "batch of %lld cells exceeds 2^31-2", cells);
    return nullptr;
  }
  fs_batch *b = new (std::nothrow) fs_batch();
  if (!b) {
    *status = set_error(FS_ERR_NOMEM, "host allocation failed");
    return nullptr;
  }
  auto fail = [&](int st) -> fs_batch * {
    *status = st;
    free_batch(b);
    return nullptr;
  };
  auto cu = [&](cudaError_t e, const char *what) -> bool {
    if (e == cudaSuccess) return true;
    *status = cuda_error(e, what);
    return false;
  };
  b->n = n;
  b->cells = cells;
  b->neq = params[0].neq;
  b->nmode = nmode_of(b->neq);
  cudaGetDevice(&b->device);
  long long o = 0, lb = 0;
  for (int r = 0; r < n; r++) {
    b->W.push_back(widths[r]);
    b->H.push_back(heights[r]);
    b->size.push_back(widths[r] * heights[r]);
    b->off.push_back(static_cast<int>(o));
    b->lvl_base.push_back(static_cast<int>(lb));
    b->nring.push_back(fs::ring_cells(widths[r], heights[r]));
    b->p.push_back(params[r]);
    o += b->size.back();
    lb += b->size.back() + 2;
  }
  b->lvl_total = lb;
  b->tab.assign(n, nullptr);
  b->tab_cap.assign(n, 0);
  const size_t C = static_cast<size_t>(cells);
  if (!cu(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cu(cudaMalloc(&b->h, C * sizeof(double)), "cudaMalloc(h)") ||
      !cu(cudaMalloc(&b->rec_alloc, C + 2 * fs::kRecPad), "cudaMalloc(rec)") ||
      !cu(cudaMalloc(&b->mask, C), "cudaMalloc(mask)") ||
      !cu(cudaMalloc(&b->pdir, C), "cudaMalloc(pdir)") ||
      !cu(cudaMalloc(&b->ent, C * sizeof(int32_t)), "cudaMalloc(ent)") ||
      !cu(cudaMalloc(&b->par, C * sizeof(int32_t)), "cudaMalloc(par)") ||
      !cu(cudaMalloc(&b->amb, C * sizeof(int32_t)), "cudaMalloc(amb)") ||
      !cu(cudaMalloc(&b->amb_r, C * sizeof(int32_t)), "cudaMalloc(amb_r)") ||
      !cu(cudaMalloc(&b->acc, C * sizeof(uint32_t)), "cudaMalloc(acc)") ||
      !cu(cudaMalloc(&b->lvl, static_cast<size_t>(lb) * sizeof(int32_t)), "cudaMalloc(lvl)") ||
      !cu(cudaMalloc(&b->d_desc, n * sizeof(fs::RealDesc)), "cudaMalloc(desc)") ||
      !cu(cudaMalloc(&b->d_rctl, n * sizeof(fs::RealCtl)), "cudaMalloc(rctl)") ||
      !cu(cudaMalloc(&b->d_ctl, sizeof(fs::Ctl)), "cudaMalloc(ctl)") ||
      !cu(cudaMallocHost(&b->h_ctl, sizeof(fs::Ctl)), "cudaMallocHost(ctl)") ||
      !cu(cudaMallocHost(&b->h_rctl, n * sizeof(fs::RealCtl)), "cudaMallocHost(rctl)"))
    return fail(*status);
  b->rec = b->rec_alloc + fs::kRecPad;
  // Rings keep NO_FLOW forever (fastscape_RB.cpp:361-362) and ring-0 cells
  // never have donors: receivers and masks are written for the interior only.
  if (!cu(cudaMemsetAsync(b->rec, 0xff, C, b->stream), "memset(rec)") ||
      !cu(cudaMemsetAsync(b->mask, 0, C, b->stream), "memset(mask)") ||
      !cu(cudaMemsetAsync(b->acc, 0, C * sizeof(uint32_t), b->stream), "memset(acc)") ||
      !cu(cudaMemsetAsync(b->lvl, 0, static_cast<size_t>(lb) * sizeof(int32_t), b->stream),
          "memset(lvl)") ||
      !cu(cudaMemsetAsync(b->d_rctl, 0, n * sizeof(fs::RealCtl), b->stream), "memset(rctl)") ||
      !cu(cudaMemsetAsync(b->d_ctl, 0, sizeof(fs::Ctl), b->stream), "memset(ctl)"))
    return fail(*status);
  // Descriptors; the erosion tables start at min(65536, size+1) records.
  b->desc.resize(n);
  for (int r = 0; r < n; r++) {
    fs::RealDesc &d = b->desc[r];
    const fs_params &p = b->p[r];
    d = fs::RealDesc{};
    d.W = b->W[r];
    d.H = b->H[r];
    d.size = b->size[r];
    d.off = b->off[r];
    d.lvl_base = b->lvl_base[r];
    d.nring = b->nring[r];
    d.u_dt = p.ueq * p.dt;
    d.tol = p.tol;
    std::memcpy(&d.tol_bits, &p.tol, sizeof(double));
    d.tol_lo_f = fs::tol_lower_float(p.tol);
    d.g_orth = static_cast<float>(1.0 / p.dr_orth);
    d.g_diag = static_cast<float>(1.0 / p.dr_diag);
    d.gmax = std::max(d.g_orth, d.g_diag);
    d.dr_orth = p.dr_orth;
    d.dr_diag = p.dr_diag;
    d.rdr_orth_n = fs::neg_recip_dr(p.dr_orth);
    d.rdr_diag_n = fs::neg_recip_dr(p.dr_diag);
  }
  if (!cu(cudaMemcpyAsync(b->d_desc, b->desc.data(), n * sizeof(fs::RealDesc),
                          cudaMemcpyHostToDevice, b->stream),
          "upload(desc)"))
    return fail(*status);
  if (int st = init_tables(b)) return fail(st);
  // Stencil tiles of every realization.
  {
    std::vector<fs::Tile> rt, dt;
    for (int r = 0; r < n; r++) {
      for (int kind = 0; kind < 2; kind++) {
        std::vector<fs::Tile> &v = kind == 0 ? rt : dt;
        const size_t at = v.size();
        v.resize(at + static_cast<size_t>(b->W[r] / 32 + 2) * (b->H[r] / 32 + 2));
        const int got = fs::append_tiles(kind, r, b->W[r], b->H[r], v.data() + at,
                                         static_cast<int>(v.size() - at));
        v.resize(at + std::max(got, 0));
      }
    }
    b->nrtiles = static_cast<int>(rt.size());
    b->ndtiles = static_cast<int>(dt.size());
    if (!cu(cudaMalloc(&b->d_rtiles, std::max<size_t>(1, rt.size()) * sizeof(fs::Tile)),
            "cudaMalloc(rtiles)") ||
        !cu(cudaMalloc(&b->d_dtiles, std::max<size_t>(1, dt.size()) * sizeof(fs::Tile)),
            "cudaMalloc(dtiles)") ||
        (!rt.empty() && !cu(cudaMemcpyAsync(b->d_rtiles, rt.data(), rt.size() * sizeof(fs::Tile),
                                            cudaMemcpyHostToDevice, b->stream),
                            "upload(rtiles)")) ||
        (!dt.empty() && !cu(cudaMemcpyAsync(b->d_dtiles, dt.data(), dt.size() * sizeof(fs::Tile),
                                            cudaMemcpyHostToDevice, b->stream),
                            "upload(dtiles)")) ||
        !cu(cudaStreamSynchronize(b->stream), "sync"))
      return fail(*status);
  }
  // Rings 0 and 1 are the head of level 0 in every timestep; initial fields.
  std::vector<double> host;
  for (int r = 0; r < n; r++) {
    if (!cu(fs::launch_place_rings(b->ent + b->off[r], b->W[r], b->H[r], b->stream), "rings"))
      return fail(*status);
    const uint64_t seed = seeds ? seeds[r] : 0;
    double *hr = b->h + b->off[r];
    if (init_mode == FS_INIT_REFERENCE || init_mode == FS_INIT_MT19937) {
      host.resize(b->size[r]);
      const uint32_t es = init_mode == FS_INIT_REFERENCE ? static_cast<uint32_t>(seed * 0u)
                                                         : static_cast<uint32_t>(seed);
      reference_field(host.data(), b->W[r], b->H[r], es);
      if (!cu(cudaMemcpyAsync(hr, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice,
                              b->stream),
              "upload(h)") ||
          !cu(cudaStreamSynchronize(b->stream), "sync"))
        return fail(*status);
    } else if (init_mode == FS_INIT_PHILOX) {
      if (!cu(fs::launch_philox_field(hr, b->W[r], b->H[r], seed, b->stream), "philox"))
        return fail(*status);
    } else if (!cu(cudaMemsetAsync(hr, 0, b->size[r] * sizeof(double), b->stream), "memset(h)")) {
      return fail(*status);
    }
  }
  int occ = 0;
  if (!cu(fs::prepare_walk_kernels(), "walk smem attribute") ||
      !cu(cudaDeviceGetAttribute(&b->walk_sms, cudaDevAttrMultiProcessorCount, b->device), "attr") ||
      !cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::walk_kernel_ptr(b->nmode, n == 1),
                                                        fs::walk_threads(),
                                                        fs::walk_smem_bytes(n)),
          "occupancy"))
    return fail(*status);
  if (occ < 1) return fail(set_error(FS_ERR_CUDA, "walk kernel cannot be resident"));
  b->rmap_ok = n == 1 && fs::make_receiver_map(&b->rmap, b->h, b->W[0], b->H[0]);
  b->walk_occ = occ;
  b->walk_bps = std::min(occ, 2);
  if (!cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b->cta_occ_order, fs::cta_order_ptr(),
                                                        fs::cta_threads(false), 0),
          "occupancy"))
    return fail(*status);
  for (int v = 0; v < 3; v++)
    if (!cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &b->cta_occ_erode[v], fs::cta_erode_ptr(b->nmode, v), fs::cta_threads(true), 0),
            "occupancy"))
      return fail(*status);
  // k_order: the variant with 3 blocks per SM is available where all three
  // fit (a large batch's shared memory may not allow it); the 2-block one is
  // the default, the autotuner's choice on every single grid measured (1000²
  // to 10000², where 3 blocks per SM took ~25% longer: 0.205 against 0.149 ms
  // per ordering at 4000²).
  for (int bps = 3; bps >= 2; bps--) {
    int o = 0;
    if (!cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fs::order_kernel_ptr(n == 1, bps),
                                                          fs::walk_threads(),
                                                          fs::walk_smem_bytes(n)),
            "occupancy"))
      return fail(*status);
    if (o >= bps) {
      b->order_max = bps;
      break;
    }
    if (bps == 2) return fail(set_error(FS_ERR_CUDA, "order kernel cannot be resident"));
  }
  b->order_bps = 2;
  {
    int o = 0;
    if (!cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fs::accum_kernel_ptr(n == 1),
                                                          fs::walk_threads(),
                                                          fs::walk_smem_bytes(n)),
            "occupancy"))
      return fail(*status);
    if (o < 1) return fail(set_error(FS_ERR_CUDA, "accumulation kernel cannot be resident"));
    b->accum_bps = std::min(o, fs::kAccumMaxBps);
  }
  if (!cu(cudaStreamSynchronize(b->stream), "sync")) return fail(*status);
  return b;
}

int check_r(const fs_batch *b, int r) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (r < 0 || r >= b->n) return set_error(FS_ERR_ARG, "realization %d out of range [0, %d)", r, b->n);
  return FS_OK;
}

int get_elevation(const fs_batch *b, int r, double *out) {
  if (int st = check_r(b, r)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemcpyAsync(out, b->h + b->off[r], sizeof(double) * b->size[r], cudaMemcpyDeviceToHost,
                          b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  return FS_OK;
}

int set_elevation(fs_batch *b, int r, const double *in) {
  if (int st = check_r(b, r)) return st;
  if (!in) return set_error(FS_ERR_ARG, "in is NULL");
  DeviceGuard dg(b->device);
  double *hr = b->h + b->off[r];
  FS_CUDA(cudaMemcpyAsync(hr, in, sizeof(double) * b->size[r], cudaMemcpyHostToDevice, b->stream));
  FS_CUDA(cudaMemsetAsync(b->d_ctl, 0, fs::kCtlCallResetBytes, b->stream));
  FS_CUDA(fs::launch_check_finite(hr, b->size[r], b->d_ctl, b->stream));
  const int st = collect_status(b);
  if (st == FS_ERR_NONFINITE)
    return set_error(FS_ERR_NONFINITE, "set_elevation: input holds NaN or Inf");
  return st;
}

int get_accumulation(const fs_batch *b, int r, double *out) {
  if (int st = check_r(b, r)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  const int n = b->size[r];
  std::vector<uint32_t> acc(n);
  std::vector<int32_t> ent(n);
  FS_CUDA(cudaMemcpyAsync(acc.data(), b->acc + b->off[r], sizeof(uint32_t) * n,
                          cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaMemcpyAsync(ent.data(), b->ent + b->off[r], sizeof(int32_t) * n,
                          cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; i++) out[ent[i]] = static_cast<double>(acc[i]) * b->p[r].cell_area;
  return FS_OK;
}

int get_receivers(const fs_batch *b, int r, int32_t *dir) {
  if (int st = check_r(b, r)) return st;
  if (!dir) return set_error(FS_ERR_ARG, "dir is NULL");
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  std::vector<int8_t> v(b->size[r]);
  FS_CUDA(cudaMemcpyAsync(v.data(), b->rec + b->off[r], b->size[r], cudaMemcpyDeviceToHost,
                          b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->size[r]; i++) dir[i] = v[i] < 0 ? FS_NO_FLOW : v[i];
  return FS_OK;
}

int get_levels(const fs_batch *b, int r, int32_t *level_id, int32_t *nlevels) {
  if (int st = check_r(b, r)) return st;
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  if (int st = read_rctl(b)) return st;
  const int nl = b->h_rctl[r].nlevels;
  if (nlevels) *nlevels = nl;
  if (!level_id) return FS_OK;
  const int n = b->size[r];
  std::vector<int32_t> ent(n), off(nl + 1);
  FS_CUDA(cudaMemcpyAsync(ent.data(), b->ent + b->off[r], sizeof(int32_t) * n,
                          cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaMemcpyAsync(off.data(), b->lvl + b->lvl_base[r], sizeof(int32_t) * (nl + 1),
                          cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; i++) level_id[i] = -1;
  for (int L = 0; L < nl; L++)
    for (int s = off[L]; s < off[L + 1]; s++) level_id[ent[s]] = L;
  return FS_OK;
}

// The Braun-Willett order of the last timestep (fastscape_BW.cpp:201-221),
// computed on the device from the level walk; stack_start (may be NULL)
// gets the first position of each root and a final size entry
// (fastscape_BW+P.cpp:223-240).
int get_stack_dfs(const fs_batch *b, int r, int32_t *stack, int32_t *stack_start,
                  int32_t *nroots) {
  if (int st = check_r(b, r)) return st;
  if (!stack) return set_error(FS_ERR_ARG, "stack is NULL");
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  if (int st = read_rctl(b)) return st;
  const int nl = b->h_rctl[r].nlevels;
  const int n = b->size[r];
  std::vector<int32_t> off(nl + 1);
  FS_CUDA(cudaMemcpyAsync(off.data(), b->lvl + b->lvl_base[r], sizeof(int32_t) * (nl + 1),
                          cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  int32_t *scratch = nullptr, *out = nullptr;
  FS_CUDA(cudaMalloc(&scratch, fs::dfs_scratch_ints(n) * sizeof(int32_t)));
  cudaError_t e = cudaMalloc(&out, n * sizeof(int32_t));
  const int o = b->off[r];
  const fs::DfsArgs d{b->rec + o, b->ent + o, b->par + o, b->pdir + o, b->acc + o,
                      b->W[r], n};
  if (e == cudaSuccess) e = fs::launch_dfs_order(d, off.data(), nl, scratch, out, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(stack, out, n * sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream);
  std::vector<int8_t> rec(n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rec.data(), b->rec + o, n, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(scratch);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_error(e, "depth-first order");
  int k = 0;
  for (int p = 0; p < n; p++)
    if (rec[stack[p]] < 0) {
      if (stack_start) stack_start[k] = p;
      k++;
    }
  if (stack_start) stack_start[k] = n;
  if (nroots) *nroots = k;
  return FS_OK;
}

int get_donor_mask(const fs_batch *b, int r, uint8_t *mask) {
  if (int st = check_r(b, r)) return st;
  if (!mask) return set_error(FS_ERR_ARG, "mask is NULL");
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemcpyAsync(mask, b->mask + b->off[r], b->size[r], cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  return FS_OK;
}

int get_phase_times(const fs_batch *b, double *ms, int reset) {
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  if (ms) {
    for (int i = 0; i < FS_NUM_TIMERS; i++) ms[i] = b->phase_ms[i];
    for (int i = 0; i < 3; i++) ms[4 + i] = b->h_ctl->walk_ns[i] * 1e-6;
  }
  if (reset) {
    for (double &x : const_cast<fs_batch *>(b)->phase_ms) x = 0;
    FS_CUDA(cudaMemsetAsync(reinterpret_cast<char *>(b->d_ctl) + offsetof(fs::Ctl, walk_ns), 0,
                            sizeof(b->h_ctl->walk_ns), b->stream));
    FS_CUDA(cudaStreamSynchronize(b->stream));
  }
  return FS_OK;
}

// Autotuner: times each candidate launch configuration -- ordering and
// erosion blocks per SM with and without the captured graph, then for n = 1
// or 2 the fastest of these with the erosion's integer subtractions -- on the
// batch's own state over `probe` timesteps, restoring the elevation after
// every probe, and keeps the fastest; the level walk is chosen by size.
constexpr int kCtaWalkCells = 1 << 19;

int autotune(fs_batch *b, int probe, int *chosen) {
  DeviceGuard dg(b->device);
  double *save = nullptr;
  FS_CUDA(cudaMalloc(&save, b->cells * sizeof(double)));
  auto release = [&]() { cudaFree(save); };
  cudaError_t e = cudaMemcpyAsync(save, b->h, b->cells * sizeof(double), cudaMemcpyDeviceToDevice,
                                  b->stream);
  if (e != cudaSuccess) {
    release();
    return cuda_error(e, "autotune save");
  }
  const int timing = b->timing;
  const long long steps = b->steps;
  b->timing = 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int best_bps = b->walk_bps, best_obps = b->order_bps, best_isub = 0;
  bool best_graph = false;
  int st = FS_OK;
  // One probe: a warm-up timestep (which also builds the graph), then
  // `probe` timed ones; the elevation is restored afterwards.
  auto time_config = [&](int obps, int bps, bool graph, int isub, float *ms) -> int {
    b->order_bps = obps;
    b->walk_bps = bps;
    b->use_graph = graph;
    b->erode_isub = isub;
    b->graph_dirty = true;
    int r = batch_step(b, 1);
    if (r == FS_OK) {
      cudaEventRecord(e0, b->stream);
      r = batch_step(b, probe);
      cudaEventRecord(e1, b->stream);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(ms, e0, e1);
    }
    cudaMemcpyAsync(b->h, save, b->cells * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
    return r;
  };
  for (int obps = 2; obps <= b->order_max && st == FS_OK; obps++) {
    for (int bps = 1; bps <= std::min(b->walk_occ, 2) && st == FS_OK; bps++) {
      for (int gr = 0; gr < 2 && st == FS_OK; gr++) {
        float ms = 0;
        if ((st = time_config(obps, bps, gr == 1, 0, &ms)) != FS_OK) break;
        if (ms < best) {
          best = ms;
          best_bps = bps;
          best_obps = obps;
          best_graph = gr == 1 && b->use_graph;
        }
      }
    }
  }
  if (st == FS_OK && b->nmode != fs::kNGeneral) {
    float ms = 0;
    st = time_config(best_obps, best_bps, best_graph, 1, &ms);
    if (st == FS_OK && ms < best) {
      best = ms;
      best_isub = 1;
    }
  }
  // a single grid: the receiver filter's tiles staged by TMA or by loads
  bool best_rtma = false;
  if (st == FS_OK && b->rmap_ok) {
    float ms = 0;
    b->rtma = true;
    st = time_config(best_obps, best_bps, best_graph, best_isub, &ms);
    if (st == FS_OK && ms < best) {
      best = ms;
      best_rtma = true;
    }
  }
  b->rtma = best_rtma;
  // The per-realization walk is chosen by size, not by the probes: its
  // advantage (a block barrier per level instead of a grid barrier) grows with
  // the number of levels, which the probes, run on the batch's current state,
  // do not see when that state is young. With every realization at most
  // kCtaWalkCells cells it wins at every depth measured (1024 x 512^2: 13.2 vs
  // 19.0 ms per timestep over 2000 timesteps); a larger realization walked by
  // one CTA serialises (a ragged batch up to 2048^2 ran 7x slower). Within the
  // chosen walk the probes pick the graph.
  const bool cta_before = b->cta_walk;
  const bool want_cta = b->n > 1 && *std::max_element(b->size.begin(), b->size.end()) <= kCtaWalkCells;
  if (want_cta && st == FS_OK) {
    b->cta_walk = true;
    best = 1e30f;
    for (int gr = 0; gr < 2 && st == FS_OK; gr++) {
      float ms = 0;
      st = time_config(best_obps, best_bps, gr == 1, best_isub, &ms);
      if (st == FS_OK && ms < best) {
        best = ms;
        best_graph = gr == 1 && b->use_graph;
      }
    }
  }
  b->cta_walk = st == FS_OK ? want_cta : cta_before;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(b->stream);
  release();
  b->timing = timing;
  b->steps = steps;
  b->walk_bps = best_bps;
  b->order_bps = best_obps;
  b->use_graph = best_graph;
  b->erode_isub = best_isub;
  b->graph_dirty = true;
  if (chosen) {
    chosen[0] = best_bps;
    chosen[1] = best_graph ? 1 : 0;
  }
  return st;
}

}  // namespace

extern "C" {

void fs_params_reference(fs_params *out) {
  if (!out) return;
  out->keq = 2e-6;
  out->neq = 2;
  out->meq = 0.8;
  out->ueq = 2e-3;
  out->dt = 1000.;
  out->dr_orth = 1;
  out->dr_diag = kSqrt2;
  out->tol = 1e-3;
  out->cell_area = 40000;
}

void fs_params_workload(fs_params *out, double dx) {
  if (!out) return;
  out->keq = 2e-6;
  out->neq = 1;
  out->meq = 0.4;
  out->ueq = 2e-3;
  out->dt = 1000.;
  out->dr_orth = dx;
  out->dr_diag = dx * kSqrt2;
  out->tol = 1e-3;
  out->cell_area = dx * dx;
}

// ---- single model: a batch of one ----------------------------------------

fs_model *fs_create(int width, int height, const fs_params *params, int init_mode, uint64_t seed,
                    int *status) {
  int dummy = 0;
  if (!status) status = &dummy;
  if (width < 3 || height < 3) {
    *status = set_error(FS_ERR_ARG, "width and height must be >= 3 (got %d x %d)", width, height);
    return nullptr;
  }
  if ((long long)width * height >= (1ll << 31) - 4) {
    *status = set_error(FS_ERR_ARG, "grid of %lld cells exceeds 2^31-4", (long long)width * height);
    return nullptr;
  }
  fs_params p;
  if (params)
    p = *params;
  else
    fs_params_workload(&p, 100.0);
  if (!valid_params(p)) {
    *status = set_error(FS_ERR_ARG, "parameters must be finite, dr and cell_area > 0, tol >= 0");
    return nullptr;
  }
  if (init_mode < FS_INIT_ZERO || init_mode > FS_INIT_PHILOX) {
    *status = set_error(FS_ERR_ARG, "unknown init_mode %d", init_mode);
    return nullptr;
  }
  fs_model *m = new (std::nothrow) fs_model();
  if (!m) {
    *status = set_error(FS_ERR_NOMEM, "host allocation failed");
    return nullptr;
  }
  m->b = batch_create(1, &width, &height, &p, init_mode, &seed, status);
  if (!m->b) {
    delete m;
    return nullptr;
  }
  return m;
}

void fs_destroy(fs_model *m) {
  if (!m) return;
  free_batch(m->b);
  delete m;
}

#define FS_MODEL(m)                                           \
  if (!(m) || !(m)->b) return set_error(FS_ERR_ARG, "model is NULL")

int fs_step(fs_model *m, int k) {
  FS_MODEL(m);
  return batch_step(m->b, k);
}

int fs_run(fs_model *m, int nstep) {
  FS_MODEL(m);
  if (nstep < -1) return set_error(FS_ERR_ARG, "nstep must be >= -1 (got %d)", nstep);
  return batch_step(m->b, nstep + 1);
}

int fs_get_elevation(const fs_model *m, double *out) {
  FS_MODEL(m);
  return get_elevation(m->b, 0, out);
}

int fs_set_elevation(fs_model *m, const double *in) {
  FS_MODEL(m);
  return set_elevation(m->b, 0, in);
}

int fs_get_accumulation(const fs_model *m, double *out) {
  FS_MODEL(m);
  return get_accumulation(m->b, 0, out);
}

int fs_get_receivers(const fs_model *m, int32_t *dir) {
  FS_MODEL(m);
  return get_receivers(m->b, 0, dir);
}

int fs_get_receiver_index(const fs_model *m, int64_t *idx) {
  FS_MODEL(m);
  if (!idx) return set_error(FS_ERR_ARG, "idx is NULL");
  const fs_batch *b = m->b;
  std::vector<int32_t> dir(b->size[0]);
  if (int st = get_receivers(b, 0, dir.data())) return st;
  const long long W = b->W[0];
  const long long off[8] = {-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1};
  for (int i = 0; i < b->size[0]; i++) idx[i] = dir[i] < 0 ? i : i + off[dir[i]];
  return FS_OK;
}

int fs_get_levels(const fs_model *m, int32_t *level_id, int32_t *nlevels) {
  FS_MODEL(m);
  return get_levels(m->b, 0, level_id, nlevels);
}

int fs_get_donor_mask(const fs_model *m, uint8_t *mask) {
  FS_MODEL(m);
  return get_donor_mask(m->b, 0, mask);
}

int fs_get_stack_dfs(const fs_model *m, int32_t *stack, int32_t *stack_start, int32_t *nroots) {
  FS_MODEL(m);
  return get_stack_dfs(m->b, 0, stack, stack_start, nroots);
}

int fs_get_shape(const fs_model *m, int *width, int *height) {
  FS_MODEL(m);
  if (width) *width = m->b->W[0];
  if (height) *height = m->b->H[0];
  return FS_OK;
}

int fs_get_params(const fs_model *m, fs_params *out) {
  FS_MODEL(m);
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  *out = m->b->p[0];
  return FS_OK;
}

int64_t fs_steps_executed(const fs_model *m) { return m && m->b ? m->b->steps : -1; }

int fs_set_timing(fs_model *m, int enable) {
  FS_MODEL(m);
  return fs_batch_set_timing(m->b, enable);
}

int fs_get_phase_times(const fs_model *m, double *ms, int reset) {
  FS_MODEL(m);
  return get_phase_times(m->b, ms, reset);
}

int fs_set_barrier_timeout(fs_model *m, double ms) {
  FS_MODEL(m);
  if (!(ms > 0) || ms > 3.6e6) return set_error(FS_ERR_ARG, "timeout must be in (0, 3.6e6] ms");
  m->b->timeout_ns = static_cast<unsigned long long>(ms * 1e6);
  m->b->graph_dirty = true;
  return FS_OK;
}

int fs_synchronize(const fs_model *m) {
  FS_MODEL(m);
  FS_CUDA(cudaStreamSynchronize(m->b->stream));
  return FS_OK;
}

size_t fs_last_error(char *buf, size_t n) {
  if (buf && n) {
    const size_t k = std::min(n - 1, g_last_error.size());
    std::memcpy(buf, g_last_error.data(), k);
    buf[k] = 0;
  }
  return g_last_error.size();
}

const char *fs_version(void) { return "fastscape-gb300 0.2 (sm_103a)"; }

// ---- batches ------------------------------------------------------------

fs_batch *fs_batch_create(int n, const int *widths, const int *heights, const fs_params *params,
                          int init_mode, const uint64_t *seeds, int *status) {
  return batch_create(n, widths, heights, params, init_mode, seeds, status);
}

void fs_batch_destroy(fs_batch *b) { free_batch(b); }

int fs_batch_step(fs_batch *b, int k) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  return batch_step(b, k);
}

int fs_batch_run(fs_batch *b, int nstep) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (nstep < -1) return set_error(FS_ERR_ARG, "nstep must be >= -1 (got %d)", nstep);
  return batch_step(b, nstep + 1);
}

int fs_batch_get_elevation(const fs_batch *b, int r, double *out) { return get_elevation(b, r, out); }

int fs_batch_set_elevation(fs_batch *b, int r, const double *in) { return set_elevation(b, r, in); }

int fs_batch_get_accumulation(const fs_batch *b, int r, double *out) {
  return get_accumulation(b, r, out);
}

int fs_batch_get_receivers(const fs_batch *b, int r, int32_t *dir) { return get_receivers(b, r, dir); }

int fs_batch_get_levels(const fs_batch *b, int r, int32_t *level_id, int32_t *nlevels) {
  return get_levels(b, r, level_id, nlevels);
}

int fs_batch_get_stack_dfs(const fs_batch *b, int r, int32_t *stack, int32_t *stack_start,
                           int32_t *nroots) {
  return get_stack_dfs(b, r, stack, stack_start, nroots);
}

int fs_batch_info(const fs_batch *b, int *n, int64_t *cells) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (n) *n = b->n;
  if (cells) *cells = b->cells;
  return FS_OK;
}

int fs_batch_set_timing(fs_batch *b, int enable) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (enable < 0 || enable > FS_TIMING_CALL)
    return set_error(FS_ERR_ARG, "timing mode must be 0, 1 or 2 (got %d)", enable);
  if (b->timing != enable) b->graph_dirty = true;  // the walk's clock stamps change
  b->timing = enable;
  return FS_OK;
}

int fs_batch_get_phase_times(const fs_batch *b, double *ms, int reset) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  return get_phase_times(b, ms, reset);
}

int fs_batch_use_graph(fs_batch *b, int enable) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  b->use_graph = enable != 0;
  b->graph_dirty = true;
  return FS_OK;
}

int fs_batch_use_int_sub(fs_batch *b, int enable) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  b->erode_isub = enable != 0 && b->nmode != fs::kNGeneral ? 1 : 0;
  b->graph_dirty = true;
  return FS_OK;
}

int fs_batch_autotune(fs_batch *b, int probe_steps, int *chosen) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (probe_steps < 1 || probe_steps > 100)
    return set_error(FS_ERR_ARG, "probe_steps must be in [1, 100]");
  return autotune(b, probe_steps, chosen);
}

int fs_batch_launch_config(const fs_batch *b, int *order_bps, int *erode_bps, int *graph,
                           int *erode_int_sub) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (order_bps) *order_bps = b->order_bps;
  if (erode_bps) *erode_bps = b->walk_bps;
  if (graph) *graph = b->use_graph ? 1 : 0;
  if (erode_int_sub) *erode_int_sub = b->erode_isub;
  return FS_OK;
}

int fs_autotune(fs_model *m, int probe_steps, int *chosen) {
  FS_MODEL(m);
  return fs_batch_autotune(m->b, probe_steps, chosen);
}

int fs_use_int_sub(fs_model *m, int enable) {
  FS_MODEL(m);
  return fs_batch_use_int_sub(m->b, enable);
}

int fs_launch_config(const fs_model *m, int *order_bps, int *erode_bps, int *graph,
                     int *erode_int_sub) {
  FS_MODEL(m);
  return fs_batch_launch_config(m->b, order_bps, erode_bps, graph, erode_int_sub);
}

int fs_batch_use_cta_walk(fs_batch *b, int enable) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  b->cta_walk = enable != 0;
  b->graph_dirty = true;
  return FS_OK;
}

int fs_batch_walk_mode(const fs_batch *b, int *cta) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (cta) *cta = b->cta_walk ? 1 : 0;
  return FS_OK;
}

int fs_batch_use_tma_staging(fs_batch *b, int enable) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (enable && !b->rmap_ok)
    return set_error(FS_ERR_ARG, "TMA staging of the receiver filter needs a single grid of "
                                 "even width");
  b->rtma = enable != 0;
  b->graph_dirty = true;
  return FS_OK;
}

int fs_batch_tma_staging(const fs_batch *b, int *on) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (on) *on = b->rtma ? 1 : 0;
  return FS_OK;
}

int fs_use_tma_staging(fs_model *m, int enable) {
  FS_MODEL(m);
  return fs_batch_use_tma_staging(m->b, enable);
}

int fs_tma_staging(const fs_model *m, int *on) {
  FS_MODEL(m);
  return fs_batch_tma_staging(m->b, on);
}

int fs_batch_set_active(fs_batch *b, int n, const int *idx) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  return set_active(b, n, idx);
}

int fs_batch_analyze(fs_batch *b) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  DeviceGuard dg(b->device);
  const fs::StepArgs a = step_args(b, 0);
  FS_CUDA(cudaMemsetAsync(b->d_ctl, 0, fs::kCtlCallResetBytes, b->stream));
  FS_CUDA(launch_step(b, a));
  if (b->act_n > 0) FS_CUDA(launch_scatter_rctl(b));
  if (int st = collect_status(b)) return st;
  b->have_step = true;
  return FS_OK;
}

int fs_batch_drainage_counts(const fs_batch *b, int r, uint32_t *d_counts) {
  if (int st = check_r(b, r)) return st;
  if (!d_counts) return set_error(FS_ERR_ARG, "d_counts is NULL");
  if (!b->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(b->device);
  const int n = b->size[r];
  k_drainage_counts<<<std::min((n + 255) / 256, 1024), 256, 0, b->stream>>>(
      b->ent + b->off[r], b->acc + b->off[r], n, d_counts);
  FS_CUDA(cudaGetLastError());
  FS_CUDA(cudaStreamSynchronize(b->stream));
  return FS_OK;
}

int fs_batch_device_elevation(const fs_batch *b, int r, double **d_h) {
  if (int st = check_r(b, r)) return st;
  if (!d_h) return set_error(FS_ERR_ARG, "d_h is NULL");
  *d_h = b->h + b->off[r];
  return FS_OK;
}

int fs_batch_get_params(const fs_batch *b, int r, fs_params *out) {
  if (int st = check_r(b, r)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  *out = b->p[r];
  return FS_OK;
}

int fs_batch_get_shape(const fs_batch *b, int r, int *width, int *height) {
  if (int st = check_r(b, r)) return st;
  if (width) *width = b->W[r];
  if (height) *height = b->H[r];
  return FS_OK;
}

int fs_batch_stream(const fs_batch *b, void **stream) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  if (!stream) return set_error(FS_ERR_ARG, "stream is NULL");
  *stream = b->stream;
  return FS_OK;
}

int fs_batch_synchronize(const fs_batch *b) {
  if (!b) return set_error(FS_ERR_ARG, "batch is NULL");
  FS_CUDA(cudaStreamSynchronize(b->stream));
  return FS_OK;
}

// ---- testing hooks (declared in include/fastscape_gb300_testing.h) -------

// Replaces the receivers with `dir` (interior cells only; rings must be -1)
// and runs donors, ordering and accumulation without erosion or uplift. Used
// to check the ordering's cycle detection with receivers that the receiver
// kernel itself can never produce.
int fs_test_order_from_receivers(fs_model *m, const int32_t *dir) {
  FS_MODEL(m);
  if (!dir) return set_error(FS_ERR_ARG, "dir is NULL");
  fs_batch *b = m->b;
  const int W = b->W[0], H = b->H[0], n = b->size[0];
  std::vector<int8_t> v(n);
  for (int i = 0; i < n; i++) {
    const int y = i / W, x = i % W;
    const bool interior = x >= 2 && x < W - 2 && y >= 2 && y < H - 2;
    if (dir[i] < -1 || dir[i] > 7 || (!interior && dir[i] != -1))
      return set_error(FS_ERR_ARG, "invalid receiver code %d at cell %d", dir[i], i);
    v[i] = static_cast<int8_t>(interior && dir[i] == FS_NO_FLOW ? fs::kPit : dir[i]);
  }
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemcpyAsync(b->rec, v.data(), n, cudaMemcpyHostToDevice, b->stream));
  FS_CUDA(cudaMemsetAsync(b->d_ctl, 0, sizeof(fs::Ctl), b->stream));
  FS_CUDA(cudaMemsetAsync(b->d_rctl, 0, sizeof(fs::RealCtl) * b->n, b->stream));
  const fs::StepArgs a = step_args(b, 0);
  FS_CUDA(fs::launch_donors_level0(a, b->stream));
  FS_CUDA(fs::launch_walk(a, b->walk_sms, b->order_bps, b->accum_bps, b->walk_bps, b->stream));
  b->have_step = true;
  return collect_status(b);
}

// Selects the receiver kernel: 1 = the FP64 reference formula for every
// cell, 0 = the FP32 filter with FP64 fix-up (default). Both give identical
// receivers; the switch exists to test that.
int fs_test_set_receiver_path(fs_model *m, int exact) {
  FS_MODEL(m);
  m->b->exact_receivers = exact != 0;
  m->b->graph_dirty = true;
  return FS_OK;
}

int fs_test_set_erosion_path(fs_model *m, int generic) {
  FS_MODEL(m);
  m->b->erode_generic = generic != 0;
  m->b->graph_dirty = true;
  return FS_OK;
}

// Number of cells the receiver filter queued for the FP64 fix-up in the last
// timestep.
int fs_test_receiver_fixups(const fs_model *m, int32_t *count) {
  FS_MODEL(m);
  if (!count) return set_error(FS_ERR_ARG, "count is NULL");
  const fs_batch *b = m->b;
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, b->stream));
  FS_CUDA(cudaStreamSynchronize(b->stream));
  *count = b->h_ctl->amb;
  return FS_OK;
}

// Current capacity of the erosion table (drainage counts below it are
// covered).
int fs_test_table_capacity(const fs_model *m, int32_t *cap) {
  FS_MODEL(m);
  if (!cap) return set_error(FS_ERR_ARG, "cap is NULL");
  *cap = m->b->tab_cap[0];
  return FS_OK;
}

// Runs a bounded wait on a count that is never reached and returns its
// status (FS_ERR_TIMEOUT when the limit works). The GPU stays usable.
int fs_test_barrier_timeout(fs_model *m, double ms) {
  FS_MODEL(m);
  if (!(ms > 0) || ms > 10000) return set_error(FS_ERR_ARG, "ms must be in (0, 10000]");
  fs_batch *b = m->b;
  DeviceGuard dg(b->device);
  FS_CUDA(cudaMemsetAsync(b->d_ctl, 0, sizeof(fs::Ctl), b->stream));
  FS_CUDA(fs::launch_test_wait(b->d_ctl, 4, static_cast<unsigned long long>(ms * 1e6), b->stream));
  return collect_status(b);
}

}  // extern "C"
