// fs_model.cu -- host side of the C ABI declared in include/fastscape_gb300.h.
//
// A model owns its device buffers for its whole life (the reference
// reallocates and frees its scratch on every run(), fastscape_RB.cpp:346-358
// and :392-397) and one CUDA stream. Layout in HBM, for size = W*H cells:
//   h       double[size]        elevation (the only state carried between
//                               timesteps, as in the reference)
//   rec     int8[size]          receiver direction code, -1 = NO_FLOW
//   mask    uint8[size]         donor mask (bit k: neighbour k drains here)
//   ent     int32[size]         cells grouped by level (the reference's stack)
//   pdir    uint8[size]         receiver direction by level position
//   nd      uint8[size]         donor count by level position
//   kid     int32[size]         first donor's position by level position
//   lvl_off int32[size+2]       level offsets into stack
//   acc     uint32[size]        drainage cell counts by level position
//                               (accum = acc*cell_area)
//   amb     int32[size]         cells queued for the FP64 receiver fix-up
//   tab     double[8*tab_cap]   erosion table per drainage count k < tab_cap
//                               (see fs_internal.h); grows on demand
//   ctl     fs::Ctl             status word, counters, barrier
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
  return set_error(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA,
                   "%s: %s", what, cudaGetErrorString(e));
}

#define FS_CUDA(call)                                      \
  do {                                                     \
    cudaError_t fs_e_ = (call);                            \
    if (fs_e_ != cudaSuccess) return cuda_error(fs_e_, #call); \
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

bool finite_params(const fs_params &p) {
  const double v[9] = {p.keq, p.neq, p.meq, p.ueq, p.dt, p.dr_orth, p.dr_diag, p.tol, p.cell_area};
  for (double x : v)
    if (!std::isfinite(x)) return false;
  return p.dr_orth > 0 && p.dr_diag > 0 && p.cell_area > 0 && p.tol >= 0;
}

}  // namespace

int fs::record_error(int status, const char *msg) { return set_error(status, "%s", msg); }

struct fs_model {
  int W = 0, H = 0, size = 0;
  fs_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  double *d_h = nullptr;
  int8_t *d_rec = nullptr;
  uint8_t *d_mask = nullptr;
  int32_t *d_ent = nullptr;
  uint8_t *d_pdir = nullptr;
  uint8_t *d_nd = nullptr;
  int32_t *d_kid = nullptr;
  int32_t *d_amb = nullptr;   // cells the receiver filter could not decide
  int32_t *d_lvl = nullptr;
  uint32_t *d_acc = nullptr;
  double *d_tab = nullptr;
  int tab_cap = 0;
  fs::Ctl *d_ctl = nullptr;
  fs::Ctl *h_ctl = nullptr;  // pinned mirror for status reads
  int walk_blocks = 0;
  int nring = 0;             // cells of rings 0 and 1 (always level 0)
  int nmode = fs::kNGeneral;
  double u_dt = 0;
  unsigned long long timeout_ns = 2000000000ull;
  long long steps = 0;
  bool have_step = false;
  bool timing = false;
  bool exact_receivers = false;  // testing: FP64 reference formula for every cell
  std::vector<cudaEvent_t> ev;  // timing mode: 3 per timestep + 1
  double phase_ms[4] = {0, 0, 0, 0};
};

namespace {

void free_model(fs_model *m) {
  if (!m) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->d_h);
  cudaFree(m->d_rec);
  cudaFree(m->d_mask);
  cudaFree(m->d_ent);
  cudaFree(m->d_pdir);
  cudaFree(m->d_nd);
  cudaFree(m->d_kid);
  cudaFree(m->d_amb);
  cudaFree(m->d_lvl);
  cudaFree(m->d_acc);
  cudaFree(m->d_tab);
  cudaFree(m->d_ctl);
  if (m->h_ctl) cudaFreeHost(m->h_ctl);
  for (auto &e : m->ev) cudaEventDestroy(e);
  if (m->stream) cudaStreamDestroy(m->stream);
  cudaSetDevice(prev);
  delete m;
}

// Erosion table records for counts k in [k0, k1): for each direction class
// F = keq*dt*pow(k*cell_area, meq)/pow(dr_cls, neq) evaluated in exactly the
// order of fastscape_RB.cpp:315 with the C library's pow (the reference's
// accum[c] is k*cell_area exactly: integer multiples summed below 2^53), then
// D = 1 + F and R = 1/D, both correctly rounded. Host arithmetic is IEEE
// double without contraction, so the device sees the reference's bits.
void fill_table(const fs_params &p, long long k0, long long k1, double *rec) {
  const double kd = p.keq * p.dt;
  const double pl[2] = {std::pow(p.dr_orth, p.neq), std::pow(p.dr_diag, p.neq)};
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, 64);
  if (k1 - k0 < 65536) nt = 1;
  auto work = [&](unsigned t) {
    const long long lo = k0 + (k1 - k0) * t / nt;
    const long long hi = k0 + (k1 - k0) * (t + 1) / nt;
    for (long long k = lo; k < hi; k++) {
      const double A = static_cast<double>(k) * p.cell_area;
      const double pa = std::pow(A, p.meq);
      double *r = rec + (k - k0) * fs::kTabStride;
      for (int cls = 0; cls < 2; cls++) {
        const double F = kd * pa / pl[cls];
        const double D = 1. + F;
        r[4 * cls + 0] = F;
        r[4 * cls + 1] = D;
        r[4 * cls + 2] = 1. / D;
        r[4 * cls + 3] = 0.;
      }
    }
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
}

// The reference field (fastscape_RB.cpp:111-130 via random.cpp:45-49),
// generated with the same libstdc++ engine and distribution.
void reference_field(std::vector<double> &h, int W, int H, uint32_t engine_seed) {
  std::mt19937 eng(engine_seed);
  std::uniform_real_distribution<double> d(0.0, 1.0);
  h.resize(static_cast<size_t>(W) * H);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const size_t c = static_cast<size_t>(y) * W + x;
      double v = d(eng);
      if (x == 0 || y == 0 || x == W - 1 || y == H - 1) v = 0;
      if (x == 1 || y == 1 || x == W - 2 || y == H - 2) v = 0;
      h[c] = v;
    }
}

struct DeviceGuard {
  int prev = 0;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() { cudaSetDevice(prev); }
};

int check_model(const fs_model *m) {
  if (!m) return set_error(FS_ERR_ARG, "model is NULL");
  return FS_OK;
}

// Reads the device status word and converts it to an ABI status.
int collect_status(fs_model *m) {
  FS_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  const int err = m->h_ctl->err;
  if (err != 0)
    return set_error(err, "timestep failed: %s (phase %d)", status_name(err), m->h_ctl->err_detail);
  return FS_OK;
}

fs::WalkArgs walk_args(const fs_model *m, int do_erode) {
  fs::WalkArgs a{};
  a.h = m->d_h;
  a.mask = m->d_mask;
  a.ent = m->d_ent;
  a.pdir = m->d_pdir;
  a.nd = m->d_nd;
  a.kid = m->d_kid;
  a.acc = m->d_acc;
  a.lvl_off = m->d_lvl;
  a.tab = m->d_tab;
  a.tab_cap = m->tab_cap;
  a.ctl = m->d_ctl;
  a.W = m->W;
  a.size = m->size;
  a.u_dt = do_erode ? m->u_dt : 0.0;
  a.neq = m->p.neq;
  a.tol = m->p.tol;
  std::memcpy(&a.tol_bits, &m->p.tol, 8);
  a.tol_lo_f = fs::tol_lower_float(m->p.tol);
  a.nring = m->nring;
  a.nmode = m->nmode;
  a.do_erode = do_erode;
  a.stamp = m->timing ? 1 : 0;
  a.timeout_ns = m->timeout_ns;
  return a;
}

// One timestep: receivers -> donors/level 0 -> level walk. With timing on,
// events ev[3i..3i+3] bracket the three launches of timestep i.
int one_step(fs_model *m, int i) {
  const fs::StepGeom g{m->W, m->H, m->size};
  if (m->timing) FS_CUDA(cudaEventRecord(m->ev[3 * i], m->stream));
  FS_CUDA(cudaMemsetAsync(reinterpret_cast<char *>(m->d_ctl) + fs::kCtlResetOffset, 0,
                          fs::kCtlResetBytes, m->stream));
  if (m->exact_receivers)
    FS_CUDA(fs::launch_receivers(m->d_h, m->d_rec, m->d_ctl, g, m->p.dr_orth, m->p.dr_diag,
                                 m->stream));
  else
    FS_CUDA(fs::launch_receivers_fast(m->d_h, m->d_rec, m->d_amb, m->d_ctl, g, m->p.dr_orth,
                                      m->p.dr_diag, m->stream));
  if (m->timing) FS_CUDA(cudaEventRecord(m->ev[3 * i + 1], m->stream));
  FS_CUDA(fs::launch_donors_level0(m->d_rec, m->d_mask, m->d_ent, m->d_ctl, g, m->nring,
                                   m->stream));
  if (m->timing) FS_CUDA(cudaEventRecord(m->ev[3 * i + 2], m->stream));
  FS_CUDA(fs::launch_walk(walk_args(m, 1), m->walk_blocks, m->stream));
  return FS_OK;
}

int ensure_events(fs_model *m, size_t n) {
  while (m->ev.size() < n) {
    cudaEvent_t e;
    FS_CUDA(cudaEventCreate(&e));
    m->ev.push_back(e);
  }
  return FS_OK;
}

int harvest_events(fs_model *m, int k) {
  FS_CUDA(cudaEventSynchronize(m->ev[3 * k]));
  for (int i = 0; i < k; i++) {
    for (int j = 0; j < 3; j++) {
      float ms = 0;
      FS_CUDA(cudaEventElapsedTime(&ms, m->ev[3 * i + j], m->ev[3 * i + j + 1]));
      m->phase_ms[j] += ms;
    }
  }
  float tot = 0;
  FS_CUDA(cudaEventElapsedTime(&tot, m->ev[0], m->ev[3 * k]));
  m->phase_ms[3] += tot;
  return FS_OK;
}

// Makes the erosion table cover every drainage count below `need`+1
// (doubling, capped at the grid size + 1).
int grow_table(fs_model *m, long long need) {
  long long cap = std::max<long long>(m->tab_cap, 1);
  while (cap <= need) cap *= 2;
  cap = std::min<long long>(cap, static_cast<long long>(m->size) + 1);
  if (cap <= m->tab_cap) return set_error(FS_ERR_CUDA, "erosion table cannot grow past %d", m->tab_cap);
  std::vector<double> host(static_cast<size_t>(cap) * fs::kTabStride);
  fill_table(m->p, 0, cap, host.data());
  double *d = nullptr;
  FS_CUDA(cudaMalloc(&d, host.size() * sizeof(double)));
  cudaError_t e = cudaMemcpyAsync(d, host.data(), host.size() * sizeof(double),
                                  cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_error(e, "upload(erosion table)");
  }
  cudaFree(m->d_tab);
  m->d_tab = d;
  m->tab_cap = static_cast<int>(cap);
  return FS_OK;
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

fs_model *fs_create(int width, int height, const fs_params *params, int init_mode,
                    uint64_t seed, int *status) {
  int dummy = 0;
  if (!status) status = &dummy;
  *status = FS_OK;
  if (width < 3 || height < 3) {
    *status = set_error(FS_ERR_ARG, "width and height must be >= 3 (got %d x %d)", width, height);
    return nullptr;
  }
  if ((long long)width * height >= (1ll << 31) - 2) {
    *status = set_error(FS_ERR_ARG, "grid of %lld cells exceeds 2^31-2", (long long)width * height);
    return nullptr;
  }
  fs_params p;
  if (params)
    p = *params;
  else
    fs_params_workload(&p, 100.0);
  if (!finite_params(p)) {
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
  m->W = width;
  m->H = height;
  m->size = width * height;
  m->p = p;
  m->u_dt = p.ueq * p.dt;
  m->nmode = (p.neq == 1.0) ? fs::kNOne : (p.neq == 2.0) ? fs::kNTwo : fs::kNGeneral;
  cudaGetDevice(&m->device);
  auto fail = [&](int st) -> fs_model * {
    *status = st;
    free_model(m);
    return nullptr;
  };
  auto cu = [&](cudaError_t e, const char *what) -> bool {
    if (e == cudaSuccess) return true;
    *status = cuda_error(e, what);
    return false;
  };
  const size_t n = static_cast<size_t>(m->size);
  if (!cu(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cu(cudaMalloc(&m->d_h, n * sizeof(double)), "cudaMalloc(h)") ||
      !cu(cudaMalloc(&m->d_rec, n), "cudaMalloc(rec)") ||
      !cu(cudaMalloc(&m->d_mask, n), "cudaMalloc(mask)") ||
      !cu(cudaMalloc(&m->d_ent, n * sizeof(int32_t)), "cudaMalloc(ent)") ||
      !cu(cudaMalloc(&m->d_pdir, n), "cudaMalloc(pdir)") ||
      !cu(cudaMalloc(&m->d_nd, n), "cudaMalloc(nd)") ||
      !cu(cudaMalloc(&m->d_kid, n * sizeof(int32_t)), "cudaMalloc(kid)") ||
      !cu(cudaMalloc(&m->d_amb, n * sizeof(int32_t)), "cudaMalloc(amb)") ||
      !cu(cudaMalloc(&m->d_lvl, (n + 2) * sizeof(int32_t)), "cudaMalloc(lvl)") ||
      !cu(cudaMalloc(&m->d_acc, n * sizeof(uint32_t)), "cudaMalloc(acc)") ||
      !cu(cudaMalloc(&m->d_ctl, sizeof(fs::Ctl)), "cudaMalloc(ctl)") ||
      !cu(cudaMallocHost(&m->h_ctl, sizeof(fs::Ctl)), "cudaMallocHost(ctl)"))
    return fail(*status);
  // Rings keep NO_FLOW forever (fastscape_RB.cpp:361-362): receivers are
  // only ever written for interior cells.
  if (!cu(cudaMemsetAsync(m->d_rec, 0xff, n, m->stream), "memset(rec)") ||
      !cu(cudaMemsetAsync(m->d_mask, 0, n, m->stream), "memset(mask)") ||
      !cu(cudaMemsetAsync(m->d_acc, 0, n * sizeof(uint32_t), m->stream), "memset(acc)") ||
      !cu(cudaMemsetAsync(m->d_lvl, 0, (n + 2) * sizeof(int32_t), m->stream), "memset(lvl)") ||
      !cu(cudaMemsetAsync(m->d_ctl, 0, sizeof(fs::Ctl), m->stream), "memset(ctl)"))
    return fail(*status);

  if (int st = grow_table(m, std::min<long long>(m->size, 65535))) return fail(st);
  {
    // Rings 0 and 1 never get a receiver: they are the head of level 0 in
    // every timestep, in ascending order, written once here.
    std::vector<int32_t> ring;
    for (int y = 0; y < m->H; y++)
      for (int x = 0; x < m->W; x++)
        if (x <= 1 || y <= 1 || x >= m->W - 2 || y >= m->H - 2) ring.push_back(y * m->W + x);
    m->nring = static_cast<int>(ring.size());
    if (!cu(cudaMemcpyAsync(m->d_ent, ring.data(), ring.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice, m->stream), "upload(ring)") ||
        !cu(cudaStreamSynchronize(m->stream), "sync"))
      return fail(*status);
  }

  const fs::StepGeom g{m->W, m->H, m->size};
  if (init_mode == FS_INIT_REFERENCE || init_mode == FS_INIT_MT19937) {
    std::vector<double> h;
    const uint32_t es = (init_mode == FS_INIT_REFERENCE) ? static_cast<uint32_t>(seed * 0u)
                                                         : static_cast<uint32_t>(seed);
    reference_field(h, m->W, m->H, es);
    if (!cu(cudaMemcpyAsync(m->d_h, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, m->stream),
            "upload(h)") ||
        !cu(cudaStreamSynchronize(m->stream), "sync"))
      return fail(*status);
  } else if (init_mode == FS_INIT_PHILOX) {
    if (!cu(fs::launch_philox_field(m->d_h, g, seed, m->stream), "philox"))
      return fail(*status);
  } else {
    if (!cu(cudaMemsetAsync(m->d_h, 0, n * sizeof(double), m->stream), "memset(h)"))
      return fail(*status);
  }

  int occ = 0, sms = 0;
  if (!cu(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device), "attr") ||
      !cu(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::walk_kernel_ptr(m->nmode),
                                                        fs::walk_threads(), 0),
          "occupancy"))
    return fail(*status);
  if (occ < 1) return fail(set_error(FS_ERR_CUDA, "walk kernel cannot be resident"));
  m->walk_blocks = sms * std::min(occ, 2);
  if (!cu(cudaStreamSynchronize(m->stream), "sync")) return fail(*status);
  return m;
}

void fs_destroy(fs_model *m) { free_model(m); }

int fs_step(fs_model *m, int k) {
  if (int st = check_model(m)) return st;
  if (k < 0) return set_error(FS_ERR_ARG, "step count must be >= 0 (got %d)", k);
  if (k == 0) return FS_OK;
  DeviceGuard dg(m->device);
  int done = 0;
  while (done < k) {
    const int batch = k - done;
    if (m->timing)
      if (int st = ensure_events(m, 3 * static_cast<size_t>(batch) + 1)) return st;
    FS_CUDA(cudaMemsetAsync(m->d_ctl, 0, fs::kCtlCallResetBytes, m->stream));
    for (int i = 0; i < batch; i++) {
      if (int st = one_step(m, i)) return st;
    }
    if (m->timing) {
      FS_CUDA(cudaEventRecord(m->ev[3 * batch], m->stream));
      if (int st = harvest_events(m, batch)) return st;
    }
    if (int st = collect_status(m)) return st;
    const int completed = m->h_ctl->steps_done;
    done += completed;
    m->steps += completed;
    if (completed > 0) m->have_step = true;
    if (m->h_ctl->abort_k > 0) {
      // A drainage count outgrew the erosion table; that timestep stopped
      // before changing h and the remaining ones did nothing. Grow and redo.
      if (int st = grow_table(m, m->h_ctl->abort_k)) return st;
    } else if (completed != batch) {
      return set_error(FS_ERR_CUDA, "%d of %d timesteps completed without a status", completed,
                       batch);
    }
  }
  return FS_OK;
}

int fs_run(fs_model *m, int nstep) {
  if (int st = check_model(m)) return st;
  if (nstep < -1) return set_error(FS_ERR_ARG, "nstep must be >= -1 (got %d)", nstep);
  return fs_step(m, nstep + 1);
}

int fs_get_elevation(const fs_model *m, double *out) {
  if (int st = check_model(m)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(out, m->d_h, sizeof(double) * m->size, cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  return FS_OK;
}

int fs_set_elevation(fs_model *m, const double *in) {
  if (int st = check_model(m)) return st;
  if (!in) return set_error(FS_ERR_ARG, "in is NULL");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(m->d_h, in, sizeof(double) * m->size, cudaMemcpyHostToDevice, m->stream));
  FS_CUDA(cudaMemsetAsync(m->d_ctl, 0, fs::kCtlCallResetBytes, m->stream));
  FS_CUDA(fs::launch_check_finite(m->d_h, m->size, m->d_ctl, m->stream));
  const int st = collect_status(m);
  if (st == FS_ERR_NONFINITE)
    return set_error(FS_ERR_NONFINITE, "fs_set_elevation: input holds NaN or Inf");
  return st;
}

int fs_get_accumulation(const fs_model *m, double *out) {
  if (int st = check_model(m)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  if (!m->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(m->device);
  std::vector<uint32_t> acc(m->size);
  std::vector<int32_t> ent(m->size);
  FS_CUDA(cudaMemcpyAsync(acc.data(), m->d_acc, sizeof(uint32_t) * m->size, cudaMemcpyDeviceToHost,
                          m->stream));
  FS_CUDA(cudaMemcpyAsync(ent.data(), m->d_ent, sizeof(int32_t) * m->size, cudaMemcpyDeviceToHost,
                          m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  for (int i = 0; i < m->size; i++) out[ent[i]] = static_cast<double>(acc[i]) * m->p.cell_area;
  return FS_OK;
}

int fs_get_receivers(const fs_model *m, int32_t *dir) {
  if (int st = check_model(m)) return st;
  if (!dir) return set_error(FS_ERR_ARG, "dir is NULL");
  if (!m->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(m->device);
  std::vector<int8_t> r(m->size);
  FS_CUDA(cudaMemcpyAsync(r.data(), m->d_rec, m->size, cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  for (int i = 0; i < m->size; i++) dir[i] = r[i] < 0 ? FS_NO_FLOW : r[i];
  return FS_OK;
}

int fs_get_receiver_index(const fs_model *m, int64_t *idx) {
  if (int st = check_model(m)) return st;
  if (!idx) return set_error(FS_ERR_ARG, "idx is NULL");
  std::vector<int32_t> dir(m->size);
  if (int st = fs_get_receivers(m, dir.data())) return st;
  const long long W = m->W;
  const long long off[8] = {-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1};
  for (int i = 0; i < m->size; i++) idx[i] = dir[i] < 0 ? i : i + off[dir[i]];
  return FS_OK;
}

int fs_get_levels(const fs_model *m, int32_t *level_id, int32_t *nlevels) {
  if (int st = check_model(m)) return st;
  if (!m->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  const int nl = m->h_ctl->nlevels;
  if (nlevels) *nlevels = nl;
  if (!level_id) return FS_OK;
  std::vector<int32_t> stack(m->size), off(nl + 1);
  FS_CUDA(cudaMemcpyAsync(stack.data(), m->d_ent, sizeof(int32_t) * m->size,
                          cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaMemcpyAsync(off.data(), m->d_lvl, sizeof(int32_t) * (nl + 1), cudaMemcpyDeviceToHost,
                          m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  for (int i = 0; i < m->size; i++) level_id[i] = -1;
  for (int L = 0; L < nl; L++)
    for (int s = off[L]; s < off[L + 1]; s++) level_id[stack[s]] = L;
  return FS_OK;
}

int fs_get_donor_mask(const fs_model *m, uint8_t *mask) {
  if (int st = check_model(m)) return st;
  if (!mask) return set_error(FS_ERR_ARG, "mask is NULL");
  if (!m->have_step) return set_error(FS_ERR_STATE, "no timestep executed yet");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(mask, m->d_mask, m->size, cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  return FS_OK;
}

int fs_get_shape(const fs_model *m, int *width, int *height) {
  if (int st = check_model(m)) return st;
  if (width) *width = m->W;
  if (height) *height = m->H;
  return FS_OK;
}

int fs_get_params(const fs_model *m, fs_params *out) {
  if (int st = check_model(m)) return st;
  if (!out) return set_error(FS_ERR_ARG, "out is NULL");
  *out = m->p;
  return FS_OK;
}

int64_t fs_steps_executed(const fs_model *m) { return m ? m->steps : -1; }

int fs_set_timing(fs_model *m, int enable) {
  if (int st = check_model(m)) return st;
  m->timing = enable != 0;
  return FS_OK;
}

int fs_get_phase_times(const fs_model *m, double *ms, int reset) {
  if (int st = check_model(m)) return st;
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  if (ms) {
    for (int i = 0; i < 4; i++) ms[i] = m->phase_ms[i];
    for (int i = 0; i < 3; i++) ms[4 + i] = m->h_ctl->walk_ns[i] * 1e-6;
  }
  if (reset) {
    for (double &x : const_cast<fs_model *>(m)->phase_ms) x = 0;
    FS_CUDA(cudaMemsetAsync(reinterpret_cast<char *>(m->d_ctl) + offsetof(fs::Ctl, walk_ns), 0,
                            sizeof(m->h_ctl->walk_ns), m->stream));
    FS_CUDA(cudaStreamSynchronize(m->stream));
  }
  return FS_OK;
}

int fs_set_barrier_timeout(fs_model *m, double ms) {
  if (int st = check_model(m)) return st;
  if (!(ms > 0) || ms > 3.6e6) return set_error(FS_ERR_ARG, "timeout must be in (0, 3.6e6] ms");
  m->timeout_ns = static_cast<unsigned long long>(ms * 1e6);
  return FS_OK;
}

int fs_synchronize(const fs_model *m) {
  if (int st = check_model(m)) return st;
  FS_CUDA(cudaStreamSynchronize(m->stream));
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

const char *fs_version(void) { return "fastscape-gb300 0.1 (sm_103a)"; }

// ---- testing hooks (declared in include/fastscape_gb300_testing.h) -------

// Replaces the receivers with `dir` (interior cells only; rings must be -1)
// and runs donors, ordering and accumulation without erosion or uplift. Used
// to check the ordering's cycle detection with receivers that the receiver
// kernel itself can never produce.
int fs_test_order_from_receivers(fs_model *m, const int32_t *dir) {
  if (int st = check_model(m)) return st;
  if (!dir) return set_error(FS_ERR_ARG, "dir is NULL");
  std::vector<int8_t> r(m->size);
  for (int i = 0; i < m->size; i++) {
    const int y = i / m->W, x = i % m->W;
    const bool interior = x >= 2 && x < m->W - 2 && y >= 2 && y < m->H - 2;
    if (dir[i] < -1 || dir[i] > 7 || (!interior && dir[i] != -1))
      return set_error(FS_ERR_ARG, "invalid receiver code %d at cell %d", dir[i], i);
    r[i] = static_cast<int8_t>(interior && dir[i] == FS_NO_FLOW ? fs::kPit : dir[i]);
  }
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(m->d_rec, r.data(), m->size, cudaMemcpyHostToDevice, m->stream));
  FS_CUDA(cudaMemsetAsync(m->d_ctl, 0, sizeof(fs::Ctl), m->stream));
  const fs::StepGeom g{m->W, m->H, m->size};
  FS_CUDA(fs::launch_donors_level0(m->d_rec, m->d_mask, m->d_ent, m->d_ctl, g, m->nring,
                                   m->stream));
  FS_CUDA(fs::launch_walk(walk_args(m, 0), m->walk_blocks, m->stream));
  m->have_step = true;
  return collect_status(m);
}

// Selects the receiver kernel: 1 = the FP64 reference formula for every
// cell, 0 = the FP32 filter with FP64 fix-up (default). Both give identical
// receivers; the switch exists to test that.
int fs_test_set_receiver_path(fs_model *m, int exact) {
  if (int st = check_model(m)) return st;
  m->exact_receivers = exact != 0;
  return FS_OK;
}

// Number of cells the receiver filter queued for the FP64 fix-up in the last
// timestep.
int fs_test_receiver_fixups(const fs_model *m, int32_t *count) {
  if (int st = check_model(m)) return st;
  if (!count) return set_error(FS_ERR_ARG, "count is NULL");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, m->stream));
  FS_CUDA(cudaStreamSynchronize(m->stream));
  *count = m->h_ctl->amb;
  return FS_OK;
}

// Current capacity of the erosion table (drainage counts below it are
// covered).
int fs_test_table_capacity(const fs_model *m, int32_t *cap) {
  if (int st = check_model(m)) return st;
  if (!cap) return set_error(FS_ERR_ARG, "cap is NULL");
  *cap = m->tab_cap;
  return FS_OK;
}

// Runs a bounded wait on a count that is never reached and returns its
// status (FS_ERR_TIMEOUT when the limit works). The GPU stays usable.
int fs_test_barrier_timeout(fs_model *m, double ms) {
  if (int st = check_model(m)) return st;
  if (!(ms > 0) || ms > 10000) return set_error(FS_ERR_ARG, "ms must be in (0, 10000]");
  DeviceGuard dg(m->device);
  FS_CUDA(cudaMemsetAsync(m->d_ctl, 0, sizeof(fs::Ctl), m->stream));
  FS_CUDA(fs::launch_test_wait(m->d_ctl, 4, static_cast<unsigned long long>(ms * 1e6), m->stream));
  return collect_status(m);
}

}  // extern "C"
