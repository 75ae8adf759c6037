/*
 * fastscape_oracle.h -- CPU restatement of the FastScape timestep of
 * fastscape_RB.cpp / fastscape_RB+P.cpp (Barnes 2019), used ONLY as the
 * test oracle and as the timed CPU baseline.
 *
 * TEST INFRASTRUCTURE. Nothing in the product path (the CUDA library, its
 * C ABI, the Python mirror) links, loads or calls this code. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Parity is pinned: tests/test_oracle_pin.py checks every function below
 * against the reference's own C++ compiled from its sources
 * (oracle/build_ref.sh), and tests/test_oracle_golden.py against fixtures
 * that reference build produced (tests/golden/make_golden.py).
 *
 * Array conventions follow the reference (fastscape_RB.cpp:69-97):
 *   row-major, index c = y*W + x, outer ring 0 is a halo, ring 1 is base
 *   level, receivers are direction codes 0..7 (W,NW,N,NE,E,SE,S,SW) or -1
 *   (NO_FLOW), donor lists are 8 slots per cell.
 */
#ifndef FASTSCAPE_ORACLE_H
#define FASTSCAPE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fso_params {
  double keq;       /* stream-power coefficient K        fastscape_RB.cpp:58 */
  double neq;       /* slope exponent n                  fastscape_RB.cpp:59 */
  double meq;       /* area exponent m                   fastscape_RB.cpp:60 */
  double ueq;       /* uplift rate U                     fastscape_RB.cpp:61 */
  double dt;        /* timestep                          fastscape_RB.cpp:62 */
  double dr_orth;   /* distance to W/N/E/S neighbours    fastscape_RB.cpp:63 */
  double dr_diag;   /* distance to diagonal neighbours   fastscape_RB.cpp:63 */
  double tol;       /* Newton tolerance                  fastscape_RB.cpp:64 */
  double cell_area; /* area of one cell                  fastscape_RB.cpp:65 */
} fso_params;

/* Reference field: W*H draws of uniform_real_distribution<double>(0,1) from
 * a std::mt19937 seeded with `engine_seed`, row-major over every cell, then
 * rings 0 and 1 set to 0 (fastscape_RB.cpp:111-130; random.cpp:19-49).
 * The reference seeds thread 0's engine with seed*0, so its field is the
 * engine_seed == 0 field for every nonzero CLI seed. */
void fso_terrain_mt19937(double *h, int W, int H, uint32_t engine_seed);

/* Raw mt19937 stream (first n outputs) -- exposes the generator for tests. */
void fso_mt19937_stream(uint32_t seed, uint32_t *out, int n);

/* fastscape_RB.cpp:160-182. rec must hold W*H; rings 0/1 are set NO_FLOW
 * (fastscape_RB.cpp:361-362), interior cells get the steepest-descent code. */
void fso_receivers(const double *h, int W, int H, const fso_params *p,
                   int32_t *rec);

/* fastscape_RB.cpp:188-203. Push inversion in ascending cell order:
 * donor[8*n + k] lists the donors of n in ascending index. */
void fso_donors(const int32_t *rec, int W, int H, int32_t *ndon,
                int32_t *donor);

/* fastscape_RB.cpp:213-254. stack holds W*H; levels must hold W*H+2.
 * Returns the reference's `nlevel` (number of levels + 1). */
int fso_order(const int32_t *rec, const int32_t *ndon, const int32_t *donor,
              int W, int H, int32_t *stack, int32_t *levels);

/* fastscape_BW.cpp:201-221 (and the stack_start of fastscape_BW+P.cpp:
 * 223-240): the Braun-Willett order, a depth-first preorder of the receiver
 * forest -- roots (NO_FLOW cells) in ascending index, each followed by its
 * donors' subtrees in donor-list order. stack holds W*H; stack_start (may be
 * NULL) receives each root's first position plus a final W*H entry.
 * Iterative (the reference recurses). Returns the number of roots. */
int fso_order_bw(const int32_t *rec, const int32_t *ndon, const int32_t *donor,
                 int W, int H, int32_t *stack, int32_t *stack_start);

/* fastscape_RB.cpp:262-279. */
void fso_flowacc(const int32_t *rec, const int32_t *stack, int W, int H,
                 const fso_params *p, double *accum);

/* fastscape_RB.cpp:285-296. */
void fso_uplift(double *h, int W, int H, const fso_params *p);

/* fastscape_RB.cpp:306-328 (serial, stack order). */
void fso_erode(double *h, const int32_t *rec, const int32_t *stack,
               const double *accum, int W, int H, const fso_params *p);

/* fastscape_RB+P.cpp:313-351: level-parallel erosion (OpenMP). Identical
 * results to fso_erode; used by the timed CPU baseline. */
void fso_erode_levels(double *h, const int32_t *rec, const int32_t *stack,
                      const int32_t *levels, int nlevel, const double *accum,
                      int W, int H, const fso_params *p);

/* Scratch for fso_step / fso_run. */
typedef struct fso_work {
  int W, H;
  int32_t *rec, *ndon, *donor, *stack, *levels;
  double *accum;
  int nlevel;
} fso_work;

int  fso_work_init(fso_work *w, int W, int H);
void fso_work_free(fso_work *w);

/* One timestep in the reference order (fastscape_RB.cpp:366-373).
 * parallel != 0 uses the level-parallel erosion of fastscape_RB+P.
 * Per-phase wall times (seconds) are added to phase_s[0..5] when non-NULL. */
void fso_step(fso_work *w, double *h, const fso_params *p, int parallel,
              double *phase_s);

/* fastscape_RB.cpp:341-398: executes nstep+1 timesteps (step<=nstep). */
void fso_run(double *h, int W, int H, const fso_params *p, int nstep,
             int parallel);

/* Level id (depth in the receiver forest) of every cell from stack/levels. */
void fso_level_ids(const int32_t *stack, const int32_t *levels, int nlevel,
                   int W, int H, int32_t *level_id);

int fso_omp_threads(void);

#ifdef __cplusplus
}
#endif

#endif
