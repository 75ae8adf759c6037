/*
 * fastscape_gb300.h -- C ABI of the GB300 FastScape timestep.
 *
 * The reference exposes one C++ model object per variant, e.g.
 *   class FastScape_RBP                      fastscape_RB+P.cpp:46
 *     FastScape_RBP(int width, int height)   fastscape_RB+P.cpp:138-154
 *     void run(int nstep)                    fastscape_RB+P.cpp:363-424
 *     std::vector<double>& getH()            fastscape_RB+P.cpp:429-431
 * with its physical constants hard-coded at fastscape_RB.cpp:58-65. This ABI
 * keeps that object model (create from width/height, run N timesteps, read
 * back elevation) behind plain C types, adds the parameters as a struct, and
 * adds read-backs of the intermediate fields the reference keeps private
 * (accumulation, receivers, levels, donors).
 *
 * Conventions (identical to the reference, fastscape_RB.cpp:69-97):
 *   - grids are row-major, cell c = y*width + x, width*height cells;
 *   - ring 0 (outermost) is a halo and ring 1 is fixed base level; only
 *     cells with 2 <= x < width-2 and 2 <= y < height-2 are computed;
 *   - receiver direction codes: 0..7 = W, NW, N, NE, E, SE, S, SW
 *     (neighbour offsets -1, -W-1, -W, -W+1, +1, +W+1, +W, +W-1), and
 *     FS_NO_FLOW (-1) for a cell with no strictly lower neighbour.
 *
 * Every function returns FS_OK (0) or a negative FS_ERR_* status; the text of
 * the last error on the calling thread is available from fs_last_error().
 * No C++ exception crosses this boundary. A model is not thread-safe: use one
 * model per host thread or lock around calls. Each model owns one CUDA stream
 * on the device that was current when it was created.
 */
#ifndef FASTSCAPE_GB300_H
#define FASTSCAPE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS_NO_FLOW (-1)

/* Status codes. */
#define FS_OK 0
#define FS_ERR_ARG (-1)            /* invalid argument                         */
#define FS_ERR_CUDA (-2)           /* CUDA runtime error (see fs_last_error)   */
#define FS_ERR_TIMEOUT (-3)        /* a grid-wide barrier wait ran out         */
#define FS_ERR_LEVEL_OVERFLOW (-4) /* level walk exceeded width*height levels  */
#define FS_ERR_NONFINITE (-5)      /* NaN/Inf elevation produced or supplied   */
#define FS_ERR_ORDER (-6)          /* receivers do not form a forest (cycle)   */
#define FS_ERR_NEWTON (-7)         /* Newton iteration did not converge        */
#define FS_ERR_NOMEM (-8)          /* device allocation failed                 */
#define FS_ERR_STATE (-9)          /* no timestep has been executed yet        */

/* Initial-field generators for fs_create. */
#define FS_INIT_ZERO 0        /* all zeros; set the field with fs_set_elevation */
#define FS_INIT_REFERENCE 1   /* the reference's field: std::mt19937 seeded with
                                 seed*0 (random.cpp:31 seeds thread t with
                                 seed*t; the field is built on thread 0), so it
                                 is the same for every nonzero seed, drawn with
                                 uniform_real_distribution<double>(0,1) over
                                 all cells row-major, rings 0 and 1 set to 0
                                 (fastscape_RB.cpp:111-130)                     */
#define FS_INIT_MT19937 2     /* same generator seeded with `seed` itself       */
#define FS_INIT_PHILOX 3      /* device Philox4x32-10 keyed by `seed`, U[0,1)
                                 with 53-bit resolution; rings set to 0        */

/* Physical constants of one realization; the reference hard-codes them at
 * fastscape_RB.cpp:58-65 (keq, neq, meq, ueq, dt, dr[8], tol, cell_area). */
typedef struct fs_params {
  double keq;       /* stream-power coefficient K                          */
  double neq;       /* slope exponent n                                    */
  double meq;       /* drainage-area exponent m                            */
  double ueq;       /* uplift rate U (applied to interior cells)           */
  double dt;        /* timestep                                            */
  double dr_orth;   /* distance to the W/N/E/S neighbours (dr[0,2,4,6])    */
  double dr_diag;   /* distance to the diagonal neighbours (dr[1,3,5,7])   */
  double tol;       /* Newton convergence tolerance                        */
  double cell_area; /* area of one cell (accumulation unit)                */
} fs_params;

typedef struct fs_model fs_model;

/* The reference's own constants (fastscape_RB.cpp:58-65): K 2e-6, n 2, m 0.8,
 * U 2e-3, dt 1000, dr {1, SQRT2}, tol 1e-3, cell_area 40000. */
void fs_params_reference(fs_params *out);

/* The 1000^2 / 10000^2 workload: K 2e-6, n 1, m 0.4, U 2e-3, dt 1000,
 * dr {dx, dx*SQRT2}, tol 1e-3, cell_area dx*dx, with dx = 100 m. */
void fs_params_workload(fs_params *out, double dx);

/* Replaces the constructor FastScape_RBP(width, height)
 * (fastscape_RB+P.cpp:138-154; terrain fastscape_RB.cpp:111-130).
 * width, height >= 3. Returns NULL on failure with *status set. */
fs_model *fs_create(int width, int height, const fs_params *params,
                    int init_mode, uint64_t seed, int *status);

/* Frees every device buffer. Safe on NULL. */
void fs_destroy(fs_model *m);

/* Replaces FastScape_RBP::run(nstep) (fastscape_RB+P.cpp:363-424): executes
 * nstep+1 timesteps, exactly as the reference's `step<=nstep` loop does
 * (fastscape_RB.cpp:366). nstep >= -1. */
int fs_run(fs_model *m, int nstep);

/* Executes exactly k timesteps (k >= 0). */
int fs_step(fs_model *m, int k);

/* Replaces getH() (fastscape_RB+P.cpp:429-431): copies width*height
 * elevations into caller-owned host memory. */
int fs_get_elevation(const fs_model *m, double *out);

/* Replaces the field (the reference lets callers alter h between runs,
 * fastscape_RB.cpp:334-340). Rejects NaN/Inf with FS_ERR_NONFINITE. */
int fs_set_elevation(fs_model *m, const double *in);

/* Flow accumulation of the last executed timestep (fastscape_RB.cpp:262-279;
 * private and freed in the reference): width*height doubles. */
int fs_get_accumulation(const fs_model *m, double *out);

/* Receiver direction codes of the last executed timestep
 * (fastscape_RB.cpp:160-182): width*height int32 in {-1, 0..7}. */
int fs_get_receivers(const fs_model *m, int32_t *dir);

/* Receiver cell indices: rec index, or the cell itself for FS_NO_FLOW (the
 * self-receiver convention of FastScapeMin.f90:63). */
int fs_get_receiver_index(const fs_model *m, int64_t *idx);

/* Level of every cell in the last timestep's ordering (fastscape_RB.cpp:
 * 213-254): level 0 = FS_NO_FLOW cells, level k+1 = donors of level k.
 * *nlevels = number of non-empty levels. The reference's `nlevel` is
 * *nlevels + 2: its level table ends with the offset of one empty level
 * plus the duplicate end entry (fastscape_RB.cpp:246-251). */
int fs_get_levels(const fs_model *m, int32_t *level_id, int32_t *nlevels);

/* Donor mask of the last timestep: bit k set when the neighbour in
 * direction k drains into the cell. The reference's donor list of a cell
 * (fastscape_RB.cpp:188-203, ascending cell index) is the set bits taken in
 * the order NW(1), N(2), NE(3), W(0), E(4), SW(7), S(6), SE(5). */
int fs_get_donor_mask(const fs_model *m, uint8_t *mask);

/* The Braun-Willett order of the last timestep's receivers
 * (fastscape_BW.cpp:201-221): a depth-first preorder of the receiver forest,
 * roots (FS_NO_FLOW cells) in ascending index, each cell followed by its
 * donors' subtrees in ascending index -- identical to the reference BW's
 * stack. stack holds width*height entries; stack_start (may be NULL; at
 * least width*height+1 entries) receives each root's first position and a
 * final width*height, the stack_start of fastscape_BW+P.cpp:223-240;
 * *nroots the number of roots. Computed on the device from the level walk. */
int fs_get_stack_dfs(const fs_model *m, int32_t *stack, int32_t *stack_start,
                     int32_t *nroots);

/* Grid geometry and counters. */
int fs_get_shape(const fs_model *m, int *width, int *height);
int fs_get_params(const fs_model *m, fs_params *out);
int64_t fs_steps_executed(const fs_model *m);

/* Device time in milliseconds accumulated over timed fs_step/fs_run calls
 * since the last reset, measured with CUDA events on the model's stream
 * (enabled by fs_set_timing(m, FS_TIMING_KERNELS)). ms[] holds FS_NUM_TIMERS
 * values:
 *   0 receiver kernels, 1 donor/level-0 kernel, 2 level walk (both of
 *   its kernels), 3 whole timed calls (first event to last),
 *   4..6 split of the level walk measured inside it by the GPU clock
 *        (ordering, accumulation, uplift+erosion),
 *   7 ordering kernel, 8 erosion kernel, 9 accumulation kernel (events). */
#define FS_NUM_TIMERS 10
/* Timing modes: FS_TIMING_KERNELS launches each timestep's kernels directly
 * with events between them (fills every timer); FS_TIMING_CALL keeps the
 * launch path in use (CUDA-graph replay when chosen) and records events only
 * around each call's launches (fills timer 3 alone). */
#define FS_TIMING_OFF 0
#define FS_TIMING_KERNELS 1
#define FS_TIMING_CALL 2
int fs_set_timing(fs_model *m, int enable);
int fs_get_phase_times(const fs_model *m, double *ms, int reset);

/* fs_batch_autotune / fs_batch_launch_config for a single model (a batch
 * of one). No reference counterpart: the reference has no launch shapes. */
int fs_autotune(fs_model *m, int probe_steps, int *chosen);
int fs_use_int_sub(fs_model *m, int enable);
int fs_launch_config(const fs_model *m, int *order_bps, int *erode_bps, int *graph,
                     int *erode_int_sub);

/* Limit (milliseconds) on every grid-wide barrier wait; default 2000. */
int fs_set_barrier_timeout(fs_model *m, double ms);

/* Waits for the model's stream. */
int fs_synchronize(const fs_model *m);

/* Copies the last error message of this thread into buf (NUL-terminated);
 * returns the message length. */
size_t fs_last_error(char *buf, size_t n);

/* Library version string. */
const char *fs_version(void);

/* ---- Ragged batches ------------------------------------------------------
 * Many independent realizations, each with its own grid size and constants
 * (all sharing the slope exponent n), advanced together: one launch sequence
 * per timestep for the whole batch, all realizations walking their levels in
 * lock step so one grid barrier per level serves every realization. The
 * reference has no batch; each realization behaves exactly like a model of
 * its own (same results bit for bit). */
typedef struct fs_batch fs_batch;

/* n realizations; widths[r] x heights[r] cells with params[r]; seeds may be
 * NULL (all 0). At most 4096 realizations and 2^31-2 cells in total. */
fs_batch *fs_batch_create(int n, const int *widths, const int *heights,
                          const fs_params *params, int init_mode,
                          const uint64_t *seeds, int *status);
void fs_batch_destroy(fs_batch *b);
/* Exactly k timesteps of every realization. */
int fs_batch_step(fs_batch *b, int k);
/* nstep+1 timesteps of every realization (the reference's run semantics). */
int fs_batch_run(fs_batch *b, int nstep);
int fs_batch_get_elevation(const fs_batch *b, int r, double *out);
int fs_batch_set_elevation(fs_batch *b, int r, const double *in);
int fs_batch_get_accumulation(const fs_batch *b, int r, double *out);
int fs_batch_get_receivers(const fs_batch *b, int r, int32_t *dir);
int fs_batch_get_levels(const fs_batch *b, int r, int32_t *level_id,
                        int32_t *nlevels);
int fs_batch_get_stack_dfs(const fs_batch *b, int r, int32_t *stack,
                           int32_t *stack_start, int32_t *nroots);
/* Number of realizations and total cells. */
int fs_batch_info(const fs_batch *b, int *n, int64_t *cells);
int fs_batch_set_timing(fs_batch *b, int enable);
int fs_batch_get_phase_times(const fs_batch *b, double *ms, int reset);
/* Replays each timestep from a captured CUDA graph (1, default: the
 * autotuner's choice at every grid size and ensemble measured) or launches
 * it directly (0). A capture that fails falls back to direct launches. */
int fs_batch_use_graph(fs_batch *b, int enable);
/* With n = 1 or 2, the erosion subtracts elevations in integer arithmetic
 * (1) or on the FP64 pipe (0, default); identical results, different speed
 * (fs_batch_autotune picks). Ignored for other n. */
int fs_batch_use_int_sub(fs_batch *b, int enable);
/* Times every launch configuration (blocks per SM of the ordering and
 * erosion kernels, graph or direct; for n = 1 or 2 then the best of these with
 * the erosion's elevation subtractions in integer arithmetic) over
 * probe_steps timesteps of the batch's own state, restores the state and
 * keeps the fastest; chosen[0] = erosion kernel blocks per SM, chosen[1] =
 * graph (fs_batch_launch_config reports every choice). The level walk is set
 * by size: per realization (fs_batch_use_cta_walk) when the batch has more
 * than one realization and none has more than 2^19 cells, grid-wide
 * otherwise. Results do not depend on the configuration. */
int fs_batch_autotune(fs_batch *b, int probe_steps, int *chosen);
/* The launch configuration in use: blocks per SM of the ordering kernel and
 * of the erosion kernel, graph replay (0/1), integer subtractions in the
 * erosion (0/1). Any pointer may be NULL. */
int fs_batch_launch_config(const fs_batch *b, int *order_bps, int *erode_bps,
                           int *graph, int *erode_int_sub);
int fs_batch_synchronize(const fs_batch *b);

/* Level walk of a batch: 0 = grid-wide (every realization walks its levels
 * in lock step, one grid barrier per level for the batch), 1 = one CTA per
 * realization (block barriers only; for batches of many small realizations
 * whose hundreds of levels each hold a few thousand cells). Identical
 * results; fs_batch_autotune picks by realization size. A launch that covers a single
 * realization always walks grid-wide. No reference counterpart. */
int fs_batch_use_cta_walk(fs_batch *b, int enable);
int fs_batch_walk_mode(const fs_batch *b, int *cta);

/* Receiver filter staging of a single grid of even width: 1 = each tile's
 * FP64 values arrive in shared memory by one TMA box (cp.async.bulk.tensor),
 * 0 = by loads (default). Identical results; fs_batch_autotune picks by
 * speed. FS_ERR_ARG when enabling it for a batch of more than one
 * realization or an odd width. No reference counterpart. */
int fs_batch_use_tma_staging(fs_batch *b, int enable);
int fs_batch_tma_staging(const fs_batch *b, int *on);
int fs_use_tma_staging(fs_model *m, int enable);
int fs_tma_staging(const fs_model *m, int *on);

/* Restricts the following fs_batch_step / fs_batch_run calls to the n
 * realizations listed in idx (distinct, in [0, number of realizations));
 * n = 0 (idx may be NULL) makes every realization active again. Inactive
 * realizations keep their fields; the active ones advance exactly as in a
 * full-batch timestep (same results bit for bit). Read-backs of receivers,
 * levels and accumulation reflect the last timestep that included the
 * realization. No reference counterpart: it lets a caller advance only some
 * members of an ensemble (the surrogate's judged and fallen-back
 * realizations). */
int fs_batch_set_active(fs_batch *b, int n, const int *idx);

/* Receivers, donor masks, level ordering and flow accumulation of the
 * active realizations' current fields (fastscape_RB.cpp:160-279) without
 * uplift or erosion: the fields do not change, and the read-backs
 * (receivers, levels, accumulation, drainage counts) describe them. */
int fs_batch_analyze(fs_batch *b);
/* Drainage count (accumulation / cell_area, an integer number of cells) of
 * every cell of realization r, from the last timestep or analysis that
 * included it, into caller-owned device memory (width*height uint32);
 * waits for the copy. */
int fs_batch_drainage_counts(const fs_batch *b, int r, uint32_t *d_counts);

/* Device address of realization r's elevation (width*height doubles,
 * row-major), valid until fs_batch_destroy: for callers that process the
 * fields on the GPU without a host round trip. Work on it must be ordered
 * against the batch's stream (fs_batch_stream; every fs_batch_* call that
 * launches work waits for it before returning). */
int fs_batch_device_elevation(const fs_batch *b, int r, double **d_h);
/* The batch's CUDA stream (a cudaStream_t). */
int fs_batch_stream(const fs_batch *b, void **stream);
/* Constants and grid size of realization r. */
int fs_batch_get_params(const fs_batch *b, int r, fs_params *out);
int fs_batch_get_shape(const fs_batch *b, int r, int *width, int *height);

/* Largest grid (width*height cells) fs_step_noalloc accepts. */
#define FS_NOALLOC_MAX_CELLS 262144

/* Advances a caller-owned device elevation buffer d_h (width*height doubles,
 * row-major, the layout of fs_get_elevation) by exactly nsteps timesteps on
 * `stream` (a cudaStream_t; NULL for the default stream), with results
 * identical to fs_create + fs_set_elevation + fs_step, and waits for them.
 * Like fs_set_elevation it refuses a field holding NaN or Inf
 * (FS_ERR_NONFINITE, d_h left as it was).
 * No counterpart in the reference. It allocates nothing: for callers that
 * may not allocate device memory while running (a host application that
 * owns all device memory through its own pool, a latency-critical loop where
 * cudaMalloc/cudaFree would synchronize the device, a plugin with a fixed
 * footprint). All scratch (~24 MB) is one static device array in the
 * library, held on every GPU that loads it until the process exits, shared
 * by all calls and keeping the last call's contents: calls that overlap on
 * the GPU race. The library itself serializes its calls (a lock, and each
 * call waits for its stream), so the caller's part is to order its own
 * other work on d_h against `stream`. Grids larger than
 * FS_NOALLOC_MAX_CELLS return FS_ERR_ARG. The first call on a device looks
 * up the array's device address; make it before any stream capture. */
int fs_step_noalloc(double *d_h, int width, int height, const fs_params *params,
                    int nsteps, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FASTSCAPE_GB300_H */
