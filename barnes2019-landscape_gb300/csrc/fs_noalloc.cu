// fs_noalloc.cu -- fs_step_noalloc: FastScape timesteps on a caller-owned
// device elevation buffer, with every piece of scratch memory in one static
// device array, so the call itself never allocates.
//
// Who needs this: callers that are not allowed to allocate device memory
// once they are running -- a host application that hands the library a
// device pointer from its own memory pool and forbids outside cudaMalloc
// (allocating would bypass its accounting or fragment its arena), code that
// runs on a latency-critical path where a cudaMalloc/cudaFree would
// synchronize the device, and plugins that must keep a fixed memory
// footprint decided at load time. fs_create allocates per model; this entry
// point allocates nothing.
//
// Limits and sharing:
//   * grids of at most FS_NOALLOC_MAX_CELLS cells (width*height); larger
//     grids are rejected with FS_ERR_ARG;
//   * the scratch array (~23 MB: receivers, donor masks, level lists and
//     offsets, drainage counts, the erosion table for every possible count,
//     the control block) lives in the library image, so every GPU that loads
//     the library holds it until the process exits;
//   * every call on a device uses the same array and it keeps the last
//     call's contents; calls that overlap on the GPU (two host threads, or
//     two streams) race on it and must be serialized by the caller;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and the walk kernel's occupancy; make that first
//     call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "fastscape_gb300.h"
#include "fs_internal.h"

namespace {

constexpr size_t kMaxCells = FS_NOALLOC_MAX_CELLS;
constexpr size_t kTabRecords = kMaxCells + 1;  // counts 0..kMaxCells
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Regions of the scratch array, each 256-byte aligned.
constexpr size_t kOffCtl = 0;
constexpr size_t kOffTab = align256(kOffCtl + sizeof(fs::Ctl));
constexpr size_t kOffEnt = align256(kOffTab + kTabRecords * fs::kTabStride * sizeof(double));
constexpr size_t kOffKid = align256(kOffEnt + kMaxCells * sizeof(int32_t));
constexpr size_t kOffAmb = align256(kOffKid + kMaxCells * sizeof(int32_t));
constexpr size_t kOffLvl = align256(kOffAmb + kMaxCells * sizeof(int32_t));
constexpr size_t kOffAcc = align256(kOffLvl + (kMaxCells + 2) * sizeof(int32_t));
constexpr size_t kOffRec = align256(kOffAcc + kMaxCells * sizeof(uint32_t));
constexpr size_t kOffMask = align256(kOffRec + kMaxCells);
constexpr size_t kOffPdir = align256(kOffMask + kMaxCells);
constexpr size_t kOffNd = align256(kOffPdir + kMaxCells);
constexpr size_t kScratchBytes = align256(kOffNd + kMaxCells);

// The scratch. Host code must not use this name as a device address (on the
// host it is only a stand-in); the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host copy of the erosion table for the parameters last uploaded.
static double g_host_tab[kTabRecords * fs::kTabStride];

struct DeviceState {
  bool ready = false;
  unsigned char *base = nullptr;  // device address of g_scratch
  int walk_blocks[3] = {0, 0, 0};
  bool tab_valid = false;
  fs_params tab_params{};
};

DeviceState g_dev[kMaxDevices];
std::mutex g_mutex;

int fail(int status, const char *msg) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "fs_step_noalloc: %s", msg);
  return fs::record_error(status, buf);
}

int cuda_fail(cudaError_t e, const char *what) {
  char buf[200];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return fail(FS_ERR_CUDA, buf);
}

bool same_params(const fs_params &a, const fs_params &b) {
  return std::memcmp(&a, &b, sizeof(fs_params)) == 0;
}

// Erosion table records for counts 0..kMaxCells, single-threaded into the
// static host buffer: F = keq*dt*pow(k*cell_area, meq)/pow(dr_cls, neq) in
// the order of fastscape_RB.cpp:315, D = 1 + F, R = 1/D.
void fill_host_table(const fs_params &p) {
  const double kd = p.keq * p.dt;
  const double pl[2] = {std::pow(p.dr_orth, p.neq), std::pow(p.dr_diag, p.neq)};
  for (size_t k = 0; k < kTabRecords; k++) {
    const double pa = std::pow(static_cast<double>(k) * p.cell_area, p.meq);
    double *r = g_host_tab + k * fs::kTabStride;
    for (int cls = 0; cls < 2; cls++) {
      const double F = kd * pa / pl[cls];
      const double D = 1. + F;
      r[4 * cls + 0] = F;
      r[4 * cls + 1] = D;
      r[4 * cls + 2] = 1. / D;
      r[4 * cls + 3] = 0.;
    }
  }
}

// stack[0, nring) = the cells of rings 0 and 1 in ascending order: rows 0
// and 1, then x = 0, 1, W-2, W-1 of rows 2..H-3, then rows H-2 and H-1.
__global__ void k_place_rings(int32_t *stack, int W, int H) {
  const int mid_rows = H > 4 ? H - 4 : 0;
  const int top = 2 * W;
  const int nring = W * H - (W > 4 ? W - 4 : 0) * mid_rows;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nring; i += gridDim.x * blockDim.x) {
    int c;
    if (H <= 4 || W <= 4) {
      c = i;  // no interior: every cell is a ring cell
    } else if (i < top) {
      c = i;
    } else if (i < top + 4 * mid_rows) {
      const int j = i - top, row = 2 + j / 4, q = j % 4;
      const int x = q < 2 ? q : W - 4 + q;
      c = row * W + x;
    } else {
      c = (H - 2) * W + (i - top - 4 * mid_rows);
    }
    stack[i] = c;
  }
}

int setup_device(int dev, DeviceState &d) {
  if (d.ready) return FS_OK;
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  for (int nm = 0; nm < 3; nm++) {
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::walk_kernel_ptr(nm),
                                                      fs::walk_threads(), 0);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy");
    if (occ < 1) return fail(FS_ERR_CUDA, "walk kernel cannot be resident");
    d.walk_blocks[nm] = sms * (occ < 2 ? occ : 2);
  }
  d.base = static_cast<unsigned char *>(ptr);
  d.ready = true;
  return FS_OK;
}

}  // namespace

extern "C" int fs_step_noalloc(double *d_h, int width, int height, const fs_params *params,
                               int nsteps, void *stream) {
  if (!d_h || !params) return fail(FS_ERR_ARG, "d_h and params must not be NULL");
  if (width < 3 || height < 3) return fail(FS_ERR_ARG, "width and height must be >= 3");
  if (static_cast<long long>(width) * height > static_cast<long long>(kMaxCells)) {
    char buf[160];
    std::snprintf(buf, sizeof(buf),
                  "grid of %lld cells exceeds the static scratch limit of %lld cells "
                  "(FS_NOALLOC_MAX_CELLS); use fs_create for larger grids",
                  static_cast<long long>(width) * height, static_cast<long long>(kMaxCells));
    return fail(FS_ERR_ARG, buf);
  }
  if (nsteps < 0) return fail(FS_ERR_ARG, "nsteps must be >= 0");
  const fs_params &p = *params;
  if (!(p.dr_orth > 0) || !(p.dr_diag > 0) || !(p.cell_area > 0) || !(p.tol >= 0) ||
      !std::isfinite(p.keq) || !std::isfinite(p.neq) || !std::isfinite(p.meq) ||
      !std::isfinite(p.ueq) || !std::isfinite(p.dt))
    return fail(FS_ERR_ARG, "parameters must be finite, dr and cell_area > 0, tol >= 0");

  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(FS_ERR_ARG, "device index out of range");
  DeviceState &d = g_dev[dev];
  if (int st = setup_device(dev, d)) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  fs::Ctl *ctl = reinterpret_cast<fs::Ctl *>(d.base + kOffCtl);
  double *tab = reinterpret_cast<double *>(d.base + kOffTab);
  int32_t *ent = reinterpret_cast<int32_t *>(d.base + kOffEnt);
  int32_t *kid = reinterpret_cast<int32_t *>(d.base + kOffKid);
  int32_t *amb = reinterpret_cast<int32_t *>(d.base + kOffAmb);
  int32_t *lvl = reinterpret_cast<int32_t *>(d.base + kOffLvl);
  uint32_t *acc = reinterpret_cast<uint32_t *>(d.base + kOffAcc);
  int8_t *rec = reinterpret_cast<int8_t *>(d.base + kOffRec);
  uint8_t *mask = reinterpret_cast<uint8_t *>(d.base + kOffMask);
  uint8_t *pdir = reinterpret_cast<uint8_t *>(d.base + kOffPdir);
  uint8_t *nd = reinterpret_cast<uint8_t *>(d.base + kOffNd);

  if (!d.tab_valid || !same_params(d.tab_params, p)) {
    fill_host_table(p);
    e = cudaMemcpyAsync(tab, g_host_tab, sizeof(g_host_tab), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      d.tab_valid = false;
      return cuda_fail(e, "upload(erosion table)");
    }
    d.tab_params = p;
    d.tab_valid = true;
  }

  const int size = width * height;
  const fs::StepGeom g{width, height, size};
  const int nring = size - (width > 4 ? width - 4 : 0) * (height > 4 ? height - 4 : 0);
  // Start state: control block zeroed, rings without receivers, ring-0
  // donor masks zero, rings at the head of level 0.
  e = cudaMemsetAsync(ctl, 0, sizeof(fs::Ctl), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(rec, 0xff, size, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(mask, 0, size, s);
  if (e != cudaSuccess) return cuda_fail(e, "scratch reset");
  k_place_rings<<<64, 256, 0, s>>>(ent, width, height);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "ring placement");

  const int nmode = (p.neq == 1.0) ? fs::kNOne : (p.neq == 2.0) ? fs::kNTwo : fs::kNGeneral;
  fs::WalkArgs a{};
  a.h = d_h;
  a.mask = mask;
  a.ent = ent;
  a.pdir = pdir;
  a.nd = nd;
  a.kid = kid;
  a.acc = acc;
  a.lvl_off = lvl;
  a.tab = tab;
  a.tab_cap = static_cast<int>(kTabRecords);
  a.ctl = ctl;
  a.W = width;
  a.size = size;
  a.nring = nring;
  a.u_dt = p.ueq * p.dt;
  a.neq = p.neq;
  a.tol = p.tol;
  std::memcpy(&a.tol_bits, &p.tol, sizeof(double));
  a.tol_lo_f = fs::tol_lower_float(p.tol);
  a.nmode = nmode;
  a.do_erode = 1;
  a.stamp = 0;
  a.timeout_ns = 2000000000ull;
  for (int i = 0; i < nsteps; i++) {
    e = cudaMemsetAsync(reinterpret_cast<char *>(ctl) + fs::kCtlResetOffset, 0,
                        fs::kCtlResetBytes, s);
    if (e == cudaSuccess)
      e = fs::launch_receivers_fast(d_h, rec, amb, ctl, g, p.dr_orth, p.dr_diag, s);
    if (e == cudaSuccess) e = fs::launch_donors_level0(rec, mask, ent, ctl, g, nring, s);
    if (e == cudaSuccess) e = fs::launch_walk(a, d.walk_blocks[nmode], s);
    if (e != cudaSuccess) return cuda_fail(e, "timestep launch");
  }
  fs::Ctl h_ctl;
  e = cudaMemcpyAsync(&h_ctl, ctl, sizeof(fs::Ctl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "status read-back");
  if (h_ctl.err != 0) return fail(h_ctl.err, "a timestep failed on the device");
  if (h_ctl.steps_done != nsteps) return fail(FS_ERR_CUDA, "not every timestep completed");
  return FS_OK;
}
