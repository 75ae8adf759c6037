// fs_internal.h -- shared between the host side (fs_model.cu, fs_noalloc.cu)
// and the kernels (fs_kernels.cu). Not part of the public ABI.
//
// Every timestep runs over a batch of realizations (a single model is a
// batch of one). Realization r owns the cells [off_r, off_r + size_r) of
// every per-cell and per-position array and the level-table entries
// [lvl_base_r, lvl_base_r + size_r + 2); cell indices stored in `ent` are
// local to the realization (c = y*W_r + x).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace fs {

// Batch-wide control block. `err` holds the first error status of the
// current fs_step call; the words from `bar` on are reset before every
// timestep.
struct Ctl {
  int err;                 // FS_OK or first FS_ERR_* seen by any kernel
  int err_detail;          // phase code where err was raised
  int abort_k;             // > 0: a drainage count >= its realization's table
                           // capacity was met; the timestep stopped before
                           // touching h
  int steps_done;          // timesteps completed in the current fs_step call
  int abort_r;             // realization that raised abort_k
  int pad0[3];
  unsigned long long walk_ns[3];  // accumulated walk time: ordering,
                                  // accumulation, erosion (block 0's clock)
  // --- reset before every timestep (from `bar` on) ---
  unsigned int bar;        // grid-barrier arrival counter (k_order)
  int amb;                 // cells queued by the receiver filter
  unsigned int bar2;       // grid-barrier arrival counter (k_erode)
  unsigned int bar3;       // grid-barrier arrival counter (k_accum)
};
constexpr size_t kCtlResetOffset = offsetof(Ctl, bar);
constexpr size_t kCtlResetBytes = sizeof(Ctl) - kCtlResetOffset;
constexpr size_t kCtlCallResetBytes = 5 * sizeof(int);  // err .. abort_r

// Per-realization counters written by the kernels; `top` and `lvlcnt` are
// reset before every timestep.
struct RealCtl {
  int top;                 // pits appended to level 0 (after the rings)
  int lvlcnt[3];           // rotating per-level append counters
  int nlevels;             // levels found by the last walk
  int total;               // cells placed in the ordering by the last walk
  int pad[2];
};
constexpr size_t kRealCtlResetBytes = 4 * sizeof(int);  // top, lvlcnt

// Read-only description of one realization.
struct RealDesc {
  int W, H, size;
  int off;                 // first cell / position of the realization
  int lvl_base;            // first entry of its level table
  int nring;               // ring cells, pre-placed at ent[off, off+nring)
  double u_dt;             // ueq*dt
  double tol;
  long long tol_bits;      // bits of tol (magnitude compares as integers)
  float tol_lo_f;          // an FP32 value <= tol*(1-2^-20)
  float g_orth, g_diag, gmax;  // FP32 1/dr for the receiver filter
  double dr_orth, dr_diag;
  double rdr_orth_n, rdr_diag_n;  // -RN(1/dr) for the tabled receiver
                                  // slope division; 0: divide in IEEE FP64
  const double *tab;       // erosion table, kTabStride doubles per count
  int tab_cap;             // counts k < tab_cap are in the table
  int pad;
};

// A 2-D tile of one realization for the stencil kernels.
struct Tile {
  int r;                   // realization
  int x0, y0;              // grid coordinates of the tile's first cell
  int pad;
};

// Receiver code of an interior cell without a lower neighbour. The ABI
// reports it as FS_NO_FLOW (-1), like the rings; internally it marks the
// level-0 cells that are uplifted (fastscape_RB.cpp:291-295).
constexpr int kPit = -2;

// Erosion table: one 64-byte record per drainage count k (cells), holding
// for each direction class (0 orthogonal, 1 diagonal) at doubles 4*cls+0..3:
//   F = keq*dt*pow(k*cell_area, meq)/pow(dr_cls, neq)  (fastscape_RB.cpp:315)
//   D = 1 + F          (the n = 1 Newton denominator, fastscape_RB.cpp:322)
//   R = RN(1/D)        (reciprocal for the correctly rounded division)
//   -R                 (the same, negated)
constexpr int kTabStride = 8;

// Tiles: receivers over the interior [2, W-3]^2; donors over [1, W-2]^2
// with tiles starting at x = 0, 128, 256, ... (four cells per thread, so a
// row of a realization whose byte offset is a multiple of 4 is stored in
// whole words). Tall tiles (a thread slides down 12 rows of receivers, 8 of
// donors) spread each block's fixed costs -- staging halo, tile-wide bound,
// queue scan and atomic -- over more cells; measured fastest from 1000^2 up
// and within microseconds below.
constexpr int kRxTile = 32, kRyTile = 96;
constexpr int kDxTile = 128, kDyTile = 64;

// The donor kernel reads rec as aligned 32-bit words around each tile row,
// up to 8 bytes before the first and 144 bytes past the last byte of a
// realization: rec buffers keep kRecPad readable bytes on both sides that no
// kernel writes while the donor kernel runs.
constexpr size_t kRecPad = 256;

// Where an error was detected (Ctl::err_detail).
enum ErrPhase : int {
  kPhaseNone = 0,
  kPhaseBarrier = 1,
  kPhaseOrder = 2,
  kPhaseErode = 3,
  kPhaseTest = 4,
};

// How pow(x, n) and pow(x, n-1) are evaluated inside the Newton loop.
enum NMode : int {
  kNGeneral = 0,  // CUDA pow (not bit-identical to glibc)
  kNOne = 1,      // pow(x,1) = x, pow(x,0) = 1: exact
  kNTwo = 2,      // pow(x,2) = x*x, pow(x,1) = x
};

// Arrays indexed by position i in the level order (the reference's stack):
//   ent[i]   cell index (local); level 0 starts with the two rings (fixed)
//            followed by the pits of this timestep; each level lists the
//            donors of the level before it, a receiver's donors contiguous
//   pdir[i]  receiver direction of ent[i] (0..7)
//   acc[i]   drainage cell count of ent[i]
//   par[i]   position of ent[i]'s receiver (levels >= 1)
struct StepArgs {
  double *h;
  int8_t *rec;
  uint8_t *mask;
  int32_t *ent;
  uint8_t *pdir;
  uint32_t *acc;
  int32_t *par;
  int32_t *amb;            // queued cells (global index) of the filter
  int32_t *amb_r;          // and their realization
  int32_t *lvl_off;        // per realization: size+2 local level offsets
  const RealDesc *desc;
  RealCtl *rctl;
  Ctl *ctl;
  int nreal;
  const Tile *rtiles;
  int nrtiles;
  const Tile *dtiles;
  int ndtiles;
  int nmode;
  double neq;
  int do_erode;            // 0: ordering + accumulation only
  int erode_isub;          // 1: the n = 1 / n = 2 erosion subtracts
                           // elevations in integer arithmetic (host-side
                           // launch choice)
  int erode_generic;       // 1: the reference's Newton loop literally, for
                           // every n (a test of the fast paths)
  int stamp;               // 1: accumulate phase times into ctl->walk_ns
  unsigned long long timeout_ns;
};

// Largest batch one walk launch handles.
constexpr int kMaxReal = 4096;
// Shared memory the walk kernel needs for `nreal` realizations.
size_t walk_smem_bytes(int nreal);

// Kernel launchers (fs_kernels.cu). All are asynchronous on `s`.
cudaError_t launch_receivers_exact(const StepArgs &a, cudaStream_t s);
// hmap: a single grid's elevation as a {W, H} map of 64-bit elements with
// {36, 98} boxes (make_receiver_map): the filter stages its tiles by TMA.
cudaError_t launch_receivers_fast(const StepArgs &a, cudaStream_t s,
                                  const CUtensorMap *hmap = nullptr);
bool make_receiver_map(CUtensorMap *m, const double *h, int W, int H);
cudaError_t launch_donors_level0(const StepArgs &a, cudaStream_t s);
// The level walk: k_order with order_bps blocks per SM (2 or 3; each has
// its own register budget), k_accum with accum_bps, then (when a.do_erode)
// k_erode with erode_bps blocks per SM; cooperative launches over `sms` SMs.
cudaError_t launch_walk(const StepArgs &a, int sms, int order_bps, int accum_bps,
                        int erode_bps, cudaStream_t s);
cudaError_t launch_order(const StepArgs &a, int sms, int bps, cudaStream_t s);  // k_order
cudaError_t launch_accum(const StepArgs &a, int sms, int bps, cudaStream_t s);  // k_accum
cudaError_t launch_erode(const StepArgs &a, int sms, int bps, cudaStream_t s);  // k_erode
int walk_threads();
// k_erode: var 0 FP64 subtractions, 1 integer subtractions (n = 1, 2), 2 the
// reference's loop literally
const void *walk_kernel_ptr(int nmode, bool single, int var = 0);
const void *order_kernel_ptr(bool single, int bps);     // k_order for bps 2 or 3
const void *accum_kernel_ptr(bool single);              // k_accum
constexpr int kAccumMaxBps = 4;                         // k_accum's register budget
cudaError_t prepare_walk_kernels();  // dynamic shared memory limit
// The per-realization walk (batches of many small realizations): one CTA of
// cta_threads(erode) threads per realization (blocks CTAs in all, looping over
// the realizations); launch_cta_order orders and accumulates,
// launch_cta_erode uplifts and erodes (skipped on an abort or error).
int cta_threads(bool erode);
const void *cta_order_ptr();
const void *cta_erode_ptr(int nmode, int var);
cudaError_t launch_cta_order(const StepArgs &a, int blocks, cudaStream_t s);
cudaError_t launch_cta_erode(const StepArgs &a, int blocks, cudaStream_t s);
cudaError_t launch_check_finite(const double *h, long long n, Ctl *ctl, cudaStream_t s);
cudaError_t launch_philox_field(double *h, int W, int H, uint64_t seed, cudaStream_t s);
cudaError_t launch_place_rings(int32_t *ent, int W, int H, cudaStream_t s);
cudaError_t launch_test_wait(Ctl *ctl, int blocks, unsigned long long timeout_ns,
                             cudaStream_t s);

// One realization's level-walk arrays, for the Braun-Willett order.
struct DfsArgs {
  const int8_t *rec;
  const int32_t *ent;
  const int32_t *par;
  const uint8_t *pdir;
  const uint32_t *acc;
  int W, size;
};
// Scratch ints launch_dfs_order needs for a realization of `size` cells.
size_t dfs_scratch_ints(int size);
// The Braun-Willett (depth-first) order into out[size], given the level
// offsets on the host.
cudaError_t launch_dfs_order(const DfsArgs &d, const int32_t *lvl_host, int nlev,
                             int32_t *scratch, int32_t *out, cudaStream_t s);

// Host helpers shared by the entry points.
float tol_lower_float(double tol);
// -RN(1/dr) when the tabled division covers dr (1 <= dr <= 2^60), else 0.
double neg_recip_dr(double dr);
int ring_cells(int W, int H);
// Appends the receiver (kind 0) or donor (kind 1) tiles of realization r to
// out (capacity cap); returns the number appended, or -1 if out is full.
int append_tiles(int kind, int r, int W, int H, Tile *out, int cap);
// Erosion-table records for counts [k0, k1) into rec (kTabStride doubles
// each), single-threaded.
void fill_table_range(double keq, double neq, double meq, double dt, double dr_orth,
                      double dr_diag, double cell_area, long long k0, long long k1,
                      double *rec);

// Stores `msg` as this thread's fs_last_error() text; returns status.
int record_error(int status, const char *msg);

}  // namespace fs
