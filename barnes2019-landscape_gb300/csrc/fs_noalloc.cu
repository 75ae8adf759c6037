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
//   * the scratch array (~24 MB: receivers, donor masks, level lists and
//     offsets, receiver positions, drainage counts, the erosion table for
//     every possible count,
//     stencil tiles, descriptors and the control block) lives in the library
//     image, so every GPU that loads the library holds it until the process
//     exits;
//   * every call on a device uses the same array and it keeps the last
//     call's contents; calls that overlap on the GPU race on it. The library
//     serializes its own calls (a host mutex, and each call waits for its
//     stream before returning), so two calls of this entry point do not
//     overlap; what the caller must still order against the call's stream is
//     its own work on d_h (kernels or copies in flight on other streams);
//   * the input is checked for NaN/Inf first, as fs_set_elevation does
//     (FS_ERR_NONFINITE, d_h untouched);
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and the walk kernel's occupancy; make that first
//     call before any stream capture. Later calls look the address up again
//     and start over when it moved (after a cudaDeviceReset the module is
//     loaded afresh and the array comes back zeroed).
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
constexpr int kMaxTiles = 4096;                // per stencil kernel
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Regions of the scratch array, each 256-byte aligned.
constexpr size_t kOffCtl = 0;
constexpr size_t kOffRctl = align256(kOffCtl + sizeof(fs::Ctl));
constexpr size_t kOffDesc = align256(kOffRctl + sizeof(fs::RealCtl));
constexpr size_t kOffRtiles = align256(kOffDesc + sizeof(fs::RealDesc));
constexpr size_t kOffDtiles = align256(kOffRtiles + kMaxTiles * sizeof(fs::Tile));
constexpr size_t kOffTab = align256(kOffDtiles + kMaxTiles * sizeof(fs::Tile));
constexpr size_t kOffEnt = align256(kOffTab + kTabRecords * fs::kTabStride * sizeof(double));
constexpr size_t kOffPar = align256(kOffEnt + kMaxCells * sizeof(int32_t));
constexpr size_t kOffAmb = align256(kOffPar + kMaxCells * sizeof(int32_t));
constexpr size_t kOffAmbR = align256(kOffAmb + kMaxCells * sizeof(int32_t));
constexpr size_t kOffLvl = align256(kOffAmbR + kMaxCells * sizeof(int32_t));
constexpr size_t kOffAcc = align256(kOffLvl + (kMaxCells + 2) * sizeof(int32_t));
// rec keeps fs::kRecPad bytes on both sides (read, never written, by the
// donor kernel); acc before it is not written while that kernel runs.
constexpr size_t kOffRec = align256(kOffAcc + kMaxCells * sizeof(uint32_t) + fs::kRecPad);
constexpr size_t kOffMask = align256(kOffRec + kMaxCells + fs::kRecPad);
constexpr size_t kOffPdir = align256(kOffMask + kMaxCells);
constexpr size_t kScratchBytes = align256(kOffPdir + kMaxCells);

// The scratch. Host code must not use this name as a device address (on the
// host it is only a stand-in); the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host copies for the parameters last uploaded: erosion table, tiles.
static double g_host_tab[kTabRecords * fs::kTabStride];
static fs::Tile g_host_tiles[2][kMaxTiles];

struct DeviceState {
  bool ready = false;
  unsigned char *base = nullptr;  // device address of g_scratch
  int sms = 0;
  int erode_bps[3] = {0, 0, 0};  // k_erode blocks per SM for each n mode
  int order_bps = 2;
  int accum_bps = 1;
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

int setup_device(int dev, DeviceState &d) {
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
  if (d.ready && d.base == ptr) return FS_OK;
  // first call on this device, or the module was reloaded (the array is
  // zeroed and may sit elsewhere): nothing cached about it holds any more
  d = DeviceState{};
  e = fs::prepare_walk_kernels();
  if (e != cudaSuccess) return cuda_fail(e, "walk smem attribute");
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  for (int nm = 0; nm < 3; nm++) {
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::walk_kernel_ptr(nm, true),
                                                      fs::walk_threads(), fs::walk_smem_bytes(1));
    if (e != cudaSuccess) return cuda_fail(e, "occupancy");
    if (occ < 1) return fail(FS_ERR_CUDA, "walk kernel cannot be resident");
    d.erode_bps[nm] = occ < 2 ? occ : 2;
  }
  // k_order at 2 blocks per SM: the autotuner's choice on every single grid
  // measured (3 blocks per SM took ~25% longer)
  int occ = 0;
  d.order_bps = 2;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::order_kernel_ptr(true, 2),
                                                    fs::walk_threads(), fs::walk_smem_bytes(1));
  if (e != cudaSuccess) return cuda_fail(e, "occupancy");
  if (occ < 2) return fail(FS_ERR_CUDA, "order kernel cannot be resident");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fs::accum_kernel_ptr(true),
                                                    fs::walk_threads(), fs::walk_smem_bytes(1));
  if (e != cudaSuccess) return cuda_fail(e, "occupancy");
  if (occ < 1) return fail(FS_ERR_CUDA, "accumulation kernel cannot be resident");
  d.accum_bps = occ < fs::kAccumMaxBps ? occ : fs::kAccumMaxBps;
  d.sms = sms;
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
  fs::Tile *rt = g_host_tiles[0], *dt = g_host_tiles[1];

  std::lock_guard<std::mutex> lock(g_mutex);
  const int nrt = fs::append_tiles(0, 0, width, height, rt, kMaxTiles);
  const int ndt = fs::append_tiles(1, 0, width, height, dt, kMaxTiles);
  if (nrt < 0 || ndt < 0) return fail(FS_ERR_ARG, "grid too elongated for the static tile list");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(FS_ERR_ARG, "device index out of range");
  DeviceState &d = g_dev[dev];
  if (int st = setup_device(dev, d)) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  fs::Ctl *ctl = reinterpret_cast<fs::Ctl *>(d.base + kOffCtl);
  fs::RealCtl *rctl = reinterpret_cast<fs::RealCtl *>(d.base + kOffRctl);
  fs::RealDesc *desc = reinterpret_cast<fs::RealDesc *>(d.base + kOffDesc);
  fs::Tile *d_rt = reinterpret_cast<fs::Tile *>(d.base + kOffRtiles);
  fs::Tile *d_dt = reinterpret_cast<fs::Tile *>(d.base + kOffDtiles);
  double *tab = reinterpret_cast<double *>(d.base + kOffTab);

  if (!d.tab_valid || !same_params(d.tab_params, p)) {
    fs::fill_table_range(p.keq, p.neq, p.meq, p.dt, p.dr_orth, p.dr_diag, p.cell_area, 0,
                         static_cast<long long>(kTabRecords), g_host_tab);
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
  fs::RealDesc rd{};
  rd.W = width;
  rd.H = height;
  rd.size = size;
  rd.off = 0;
  rd.lvl_base = 0;
  rd.nring = fs::ring_cells(width, height);
  rd.u_dt = p.ueq * p.dt;
  rd.tol = p.tol;
  std::memcpy(&rd.tol_bits, &p.tol, sizeof(double));
  rd.tol_lo_f = fs::tol_lower_float(p.tol);
  rd.g_orth = static_cast<float>(1.0 / p.dr_orth);
  rd.g_diag = static_cast<float>(1.0 / p.dr_diag);
  rd.gmax = rd.g_orth > rd.g_diag ? rd.g_orth : rd.g_diag;
  rd.dr_orth = p.dr_orth;
  rd.dr_diag = p.dr_diag;
  rd.rdr_orth_n = fs::neg_recip_dr(p.dr_orth);
  rd.rdr_diag_n = fs::neg_recip_dr(p.dr_diag);
  rd.tab = tab;
  rd.tab_cap = static_cast<int>(kTabRecords);

  fs::StepArgs a{};
  a.h = d_h;
  a.rec = reinterpret_cast<int8_t *>(d.base + kOffRec);
  a.mask = reinterpret_cast<uint8_t *>(d.base + kOffMask);
  a.ent = reinterpret_cast<int32_t *>(d.base + kOffEnt);
  a.pdir = reinterpret_cast<uint8_t *>(d.base + kOffPdir);
  a.par = reinterpret_cast<int32_t *>(d.base + kOffPar);
  a.acc = reinterpret_cast<uint32_t *>(d.base + kOffAcc);
  a.amb = reinterpret_cast<int32_t *>(d.base + kOffAmb);
  a.amb_r = reinterpret_cast<int32_t *>(d.base + kOffAmbR);
  a.lvl_off = reinterpret_cast<int32_t *>(d.base + kOffLvl);
  a.desc = desc;
  a.rctl = rctl;
  a.ctl = ctl;
  a.nreal = 1;
  a.rtiles = d_rt;
  a.nrtiles = nrt;
  a.dtiles = d_dt;
  a.ndtiles = ndt;
  a.nmode = (p.neq == 1.0) ? fs::kNOne : (p.neq == 2.0) ? fs::kNTwo : fs::kNGeneral;
  a.neq = p.neq;
  a.do_erode = 1;
  a.stamp = 0;
  a.timeout_ns = 2000000000ull;

  // Start state: descriptors and tiles of this grid, control words zeroed,
  // rings without receivers, ring-0 donor masks zero, rings at the head of
  // level 0.
  e = cudaMemcpyAsync(desc, &rd, sizeof(rd), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && nrt > 0)
    e = cudaMemcpyAsync(d_rt, rt, nrt * sizeof(fs::Tile), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && ndt > 0)
    e = cudaMemcpyAsync(d_dt, dt, ndt * sizeof(fs::Tile), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctl, 0, sizeof(fs::Ctl), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.rec, 0xff, size, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.mask, 0, size, s);
  if (e == cudaSuccess) e = fs::launch_place_rings(a.ent, width, height, s);
  // NaN/Inf in the caller's field is refused before any timestep, like
  // fs_set_elevation refuses it
  if (e == cudaSuccess) e = fs::launch_check_finite(d_h, size, ctl, s);
  int in_err = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&in_err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, s);
  // the host copies above read static buffers this call rewrites next time
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "scratch reset");
  if (in_err == FS_ERR_NONFINITE) return fail(FS_ERR_NONFINITE, "input holds NaN or Inf");
  if (in_err != 0) return fail(in_err, "input check failed on the device");

  for (int i = 0; i < nsteps; i++) {
    e = cudaMemsetAsync(reinterpret_cast<char *>(ctl) + fs::kCtlResetOffset, 0,
                        fs::kCtlResetBytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(rctl, 0, sizeof(fs::RealCtl), s);
    if (e == cudaSuccess) e = fs::launch_receivers_fast(a, s);
    if (e == cudaSuccess) e = fs::launch_donors_level0(a, s);
    if (e == cudaSuccess) e = fs::launch_walk(a, d.sms, d.order_bps, d.accum_bps, d.erode_bps[a.nmode], s);
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
