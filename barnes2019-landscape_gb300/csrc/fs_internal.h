// fs_internal.h -- shared between the host model (fs_model.cu) and the
// kernels (fs_kernels.cu). Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fs {

// Per-model device control block. `err` holds the first error status of the
// current fs_step call; the remaining words are reset before every timestep.
struct Ctl {
  int err;                 // FS_OK or first FS_ERR_* seen by any kernel
  int err_detail;          // phase code where err was raised
  int abort_k;             // > 0: a drainage count >= the table capacity was
                           // met; the timestep stopped before touching h
  int steps_done;          // timesteps completed in the current fs_step call
  int nlevels;             // levels found by the last walk
  int total;               // cells placed in the ordering by the last walk
  unsigned long long walk_ns[3];  // accumulated walk time: ordering,
                                  // accumulation, erosion (block 0's clock)
  // --- reset before every timestep (from `top` on) ---
  int top;                 // pits appended to level 0 (after the rings)
  unsigned int bar;        // grid-barrier arrival counter
  int lvlcnt[3];           // rotating per-level append counters (relative)
  int amb;                 // cells queued by the receiver filter
  int pad[2];
};
constexpr size_t kCtlCallResetBytes = 4 * sizeof(int);  // err .. steps_done

// Receiver code of an interior cell without a lower neighbour. The ABI
// reports it as FS_NO_FLOW (-1), like the rings; internally it marks the
// level-0 cells that are uplifted (fastscape_RB.cpp:291-295).
constexpr int kPit = -2;

// Erosion table: one 64-byte record per drainage count k (cells), holding
// for each direction class (0 orthogonal, 1 diagonal) at doubles 4*cls+0..2:
//   F = keq*dt*pow(k*cell_area, meq)/pow(dr_cls, neq)  (fastscape_RB.cpp:315)
//   D = 1 + F          (the n = 1 Newton denominator, fastscape_RB.cpp:322)
//   R = RN(1/D)        (reciprocal for the correctly rounded division)
constexpr int kTabStride = 8;
constexpr size_t kCtlResetOffset = offsetof(Ctl, top);
constexpr size_t kCtlResetBytes = sizeof(Ctl) - kCtlResetOffset;

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

struct StepGeom {
  int W, H;
  int size;  // W*H (< 2^31)
};

// Arrays indexed by position i in the level order (the reference's stack):
//   ent[i]   cell index; level 0 starts with the two rings (fixed) followed
//            by the pits of this timestep
//   pdir[i]  receiver direction of ent[i] (0..7), bit 3 set when that
//            receiver is a pit (levels >= 1 only)
//   nd[i]    number of donors of ent[i]
//   kid[i]   position of its first donor; its donors are contiguous
//   acc[i]   drainage cell count of ent[i]
struct WalkArgs {
  double *h;
  const uint8_t *mask;
  int32_t *ent;
  uint8_t *pdir;
  uint8_t *nd;
  int32_t *kid;
  uint32_t *acc;
  int32_t *lvl_off;        // size+2 entries
  const double *tab;       // erosion table, kTabStride doubles per count
  int tab_cap;             // counts k < tab_cap are in the table
  Ctl *ctl;
  int W, size;
  int nring;               // ring cells, pre-placed at ent[0, nring)
  double u_dt, neq, tol;
  long long tol_bits;      // bits of tol (magnitude compares as integers)
  float tol_lo_f;          // an FP32 value <= tol*(1-2^-20)
  int nmode;
  int do_erode;            // 0: ordering + accumulation only
  int stamp;               // 1: accumulate phase times into ctl->walk_ns
  unsigned long long timeout_ns;
};

// An FP32 number not above tol*(1 - 2^-20), for the one-iterate test.
float tol_lower_float(double tol);

// Kernel launchers (fs_kernels.cu). All are asynchronous on `s`.
cudaError_t launch_receivers(const double *h, int8_t *rec, const Ctl *ctl, StepGeom g,
                             double dr_orth, double dr_diag, cudaStream_t s);
cudaError_t launch_receivers_fast(const double *h, int8_t *rec, int32_t *amb,
                                  Ctl *ctl, StepGeom g, double dr_orth,
                                  double dr_diag, cudaStream_t s);
cudaError_t launch_donors_level0(const int8_t *rec, uint8_t *mask,
                                 int32_t *ent, Ctl *ctl, StepGeom g, int nring,
                                 cudaStream_t s);
cudaError_t launch_walk(const WalkArgs &a, int blocks, cudaStream_t s);
int walk_threads();
const void *walk_kernel_ptr(int nmode);
cudaError_t launch_check_finite(const double *h, int size, Ctl *ctl,
                                cudaStream_t s);
cudaError_t launch_philox_field(double *h, StepGeom g, uint64_t seed,
                                cudaStream_t s);
// Stores `msg` as this thread's fs_last_error() text; returns status.
int record_error(int status, const char *msg);

cudaError_t launch_test_wait(Ctl *ctl, int blocks,
                             unsigned long long timeout_ns, cudaStream_t s);

}  // namespace fs
