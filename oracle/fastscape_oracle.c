/*
 * fastscape_oracle.c -- CPU restatement of the FastScape timestep
 * (fastscape_RB.cpp, fastscape_RB+P.cpp). TEST INFRASTRUCTURE ONLY: used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU baseline, never by the
 * product path. Build: oracle/build.py (-O3 -ffp-contract=off -fopenmp).
 *
 * Floating-point expressions keep the reference's operation order exactly and
 * are compiled without FMA contraction, so results are bit-identical to the
 * reference built with -ffp-contract=off.
 */
#include "fastscape_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NO_FLOW (-1)

/* ---------------------------------------------------------------------------
 * Mersenne Twister MT19937 (Matsumoto & Nishimura 1998, the published
 * algorithm; the same engine as std::mt19937) and the libstdc++ mapping of
 * std::uniform_real_distribution<double>: generate_canonical<double,53> draws
 * two 32-bit words g1, g2 and returns (g1 + g2*2^32) / 2^64, clamped below 1.
 * Used by random.cpp:45-49 through fastscape_RB.cpp:116.
 * ------------------------------------------------------------------------- */
typedef struct { uint32_t mt[624]; int idx; } mt_state;

static void mt_seed(mt_state *s, uint32_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->idx = 624;
}

static void mt_twist(mt_state *s) {
  for (int i = 0; i < 624; i++) {
    uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
    uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
    if (y & 1u) v ^= 0x9908b0dfu;
    s->mt[i] = v;
  }
  s->idx = 0;
}

static uint32_t mt_next(mt_state *s) {
  if (s->idx >= 624) mt_twist(s);
  uint32_t y = s->mt[s->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

static double mt_canonical(mt_state *s) {
  const double g1 = (double)mt_next(s);
  const double g2 = (double)mt_next(s);
  double sum = 0.0;
  sum += g1 * 1.0;
  sum += g2 * 4294967296.0;
  double r = sum / 18446744073709551616.0;
  if (r >= 1.0) r = nextafter(1.0, 0.0);
  return r;
}

void fso_mt19937_stream(uint32_t seed, uint32_t *out, int n) {
  mt_state s;
  mt_seed(&s, seed);
  for (int i = 0; i < n; i++) out[i] = mt_next(&s);
}

/* fastscape_RB.cpp:111-130 */
void fso_terrain_mt19937(double *h, int W, int H, uint32_t engine_seed) {
  mt_state *s = (mt_state *)malloc(sizeof(mt_state));
  mt_seed(s, engine_seed);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const size_t c = (size_t)y * W + x;
      double v = mt_canonical(s) * (1.0 - 0.0) + 0.0;
      if (x == 0 || y == 0 || x == W - 1 || y == H - 1) v = 0;
      if (x == 1 || y == 1 || x == W - 2 || y == H - 2) v = 0;
      h[c] = v;
    }
  free(s);
}

static void nshift_of(int W, int nshift[8]) {
  /* fastscape_RB.cpp:137 -- W, NW, N, NE, E, SE, S, SW */
  nshift[0] = -1;     nshift[1] = -W - 1; nshift[2] = -W; nshift[3] = -W + 1;
  nshift[4] = 1;      nshift[5] = W + 1;  nshift[6] = W;  nshift[7] = W - 1;
}

static void dr_of(const fso_params *p, double dr[8]) {
  for (int n = 0; n < 8; n++) dr[n] = (n & 1) ? p->dr_diag : p->dr_orth;
}

/* fastscape_RB.cpp:160-182 (+ ring initialisation :361-362) */
void fso_receivers(const double *h, int W, int H, const fso_params *p,
                   int32_t *rec) {
  int nshift[8];
  double dr[8];
  nshift_of(W, nshift);
  dr_of(p, dr);
  const size_t size = (size_t)W * H;
  for (size_t i = 0; i < size; i++) rec[i] = NO_FLOW;
  for (int y = 2; y < H - 2; y++)
    for (int x = 2; x < W - 2; x++) {
      const size_t c = (size_t)y * W + x;
      double max_slope = 0;
      int max_n = NO_FLOW;
      for (int n = 0; n < 8; n++) {
        const double slope = (h[c] - h[c + nshift[n]]) / dr[n];
        if (slope > max_slope) {
          max_slope = slope;
          max_n = n;
        }
      }
      rec[c] = max_n;
    }
}

/* fastscape_RB.cpp:188-203 */
void fso_donors(const int32_t *rec, int W, int H, int32_t *ndon,
                int32_t *donor) {
  int nshift[8];
  nshift_of(W, nshift);
  const long size = (long)W * H;
  for (long i = 0; i < size; i++) ndon[i] = 0;
  for (long c = 0; c < size; c++) {
    if (rec[c] == NO_FLOW) continue;
    const long n = c + nshift[rec[c]];
    donor[8 * n + ndon[n]] = (int32_t)c;
    ndon[n]++;
  }
}

/* fastscape_RB.cpp:213-254 */
int fso_order(const int32_t *rec, const int32_t *ndon, const int32_t *donor,
              int W, int H, int32_t *stack, int32_t *levels) {
  const long size = (long)W * H;
  long nstack = 0;
  int nlevel = 0;
  levels[nlevel++] = 0;
  for (long c = 0; c < size; c++)
    if (rec[c] == NO_FLOW) stack[nstack++] = (int32_t)c;
  levels[nlevel++] = (int32_t)nstack;
  long level_bottom = -1, level_top = 0;
  while (level_bottom < level_top) {
    level_bottom = level_top;
    level_top = nstack;
    for (long si = level_bottom; si < level_top; si++) {
      const long c = stack[si];
      for (int k = 0; k < ndon[c]; k++) stack[nstack++] = donor[8 * c + k];
    }
    levels[nlevel++] = (int32_t)nstack;
  }
  nlevel--;
  return nlevel;
}

/* fastscape_BW.cpp:201-221; stack_start as fastscape_BW+P.cpp:223-240 */
int fso_order_bw(const int32_t *rec, const int32_t *ndon, const int32_t *donor,
                 int W, int H, int32_t *stack, int32_t *stack_start) {
  const long size = (long)W * H;
  /* explicit DFS stack of (cell, next donor slot) instead of recursion */
  int32_t *node = (int32_t *)malloc(size * sizeof(int32_t));
  int8_t *next = (int8_t *)malloc(size);
  long nstack = 0;
  int nroots = 0;
  for (long c = 0; c < size; c++) {
    if (rec[c] != NO_FLOW) continue;
    if (stack_start) stack_start[nroots] = (int32_t)nstack;
    nroots++;
    stack[nstack++] = (int32_t)c;
    long depth = 0;
    node[0] = (int32_t)c;
    next[0] = 0;
    depth = 1;
    while (depth > 0) {
      const long u = node[depth - 1];
      if (next[depth - 1] < ndon[u]) {
        const int32_t v = donor[8 * u + next[depth - 1]];
        next[depth - 1]++;
        stack[nstack++] = v;
        node[depth] = v;
        next[depth] = 0;
        depth++;
      } else {
        depth--;
      }
    }
  }
  if (stack_start) stack_start[nroots] = (int32_t)nstack;
  free(node);
  free(next);
  return nroots;
}

/* fastscape_RB.cpp:262-279 */
void fso_flowacc(const int32_t *rec, const int32_t *stack, int W, int H,
                 const fso_params *p, double *accum) {
  int nshift[8];
  nshift_of(W, nshift);
  const long size = (long)W * H;
  for (long i = 0; i < size; i++) accum[i] = p->cell_area;
  for (long s = size - 1; s >= 0; s--) {
    const long c = stack[s];
    if (rec[c] != NO_FLOW) {
      const long n = c + nshift[rec[c]];
      accum[n] += accum[c];
    }
  }
}

/* fastscape_RB.cpp:285-296 */
void fso_uplift(double *h, int W, int H, const fso_params *p) {
  for (int y = 2; y < H - 2; y++)
    for (int x = 2; x < W - 2; x++) {
      const size_t c = (size_t)y * W + x;
      h[c] += p->ueq * p->dt;
    }
}

/* One cell of fastscape_RB.cpp:308-326. */
static inline double erode_cell(const double *h, long c, long n, double length,
                                double A, const fso_params *p) {
  const double fact = p->keq * p->dt * pow(A, p->meq) / pow(length, p->neq);
  const double h0 = h[c];
  const double hn = h[n];
  double hnew = h0;
  double hp = h0;
  double diff = 2 * p->tol;
  while (fabs(diff) > p->tol) {
    hnew -= (hnew - h0 + fact * pow(hnew - hn, p->neq)) /
            (1. + fact * p->neq * pow(hnew - hn, p->neq - 1));
    diff = hnew - hp;
    hp = hnew;
  }
  return hnew;
}

/* fastscape_RB.cpp:306-328 */
void fso_erode(double *h, const int32_t *rec, const int32_t *stack,
               const double *accum, int W, int H, const fso_params *p) {
  int nshift[8];
  double dr[8];
  nshift_of(W, nshift);
  dr_of(p, dr);
  const long size = (long)W * H;
  for (long s = 0; s < size; s++) {
    const long c = stack[s];
    if (rec[c] == NO_FLOW) continue;
    const long n = c + nshift[rec[c]];
    h[c] = erode_cell(h, c, n, dr[rec[c]], accum[c], p);
  }
}

/* fastscape_RB+P.cpp:313-351 */
void fso_erode_levels(double *h, const int32_t *rec, const int32_t *stack,
                      const int32_t *levels, int nlevel, const double *accum,
                      int W, int H, const fso_params *p) {
  int nshift[8];
  double dr[8];
  nshift_of(W, nshift);
  dr_of(p, dr);
  (void)H;
  for (int li = 1; li < nlevel - 1; li++) {
    const int lvlstart = levels[li];
    const int lvlend = levels[li + 1];
    const int lvlsize = lvlend - lvlstart;
#pragma omp parallel for if (lvlsize > 500)
    for (int si = lvlstart; si < lvlend; si++) {
      const long c = stack[si];
      const long n = c + nshift[rec[c]];
      h[c] = erode_cell(h, c, n, dr[rec[c]], accum[c], p);
    }
  }
}

int fso_work_init(fso_work *w, int W, int H) {
  const size_t size = (size_t)W * H;
  memset(w, 0, sizeof(*w));
  w->W = W;
  w->H = H;
  w->rec = (int32_t *)malloc(size * sizeof(int32_t));
  w->ndon = (int32_t *)malloc(size * sizeof(int32_t));
  w->donor = (int32_t *)malloc(8 * size * sizeof(int32_t));
  w->stack = (int32_t *)malloc(size * sizeof(int32_t));
  w->levels = (int32_t *)malloc((size + 2) * sizeof(int32_t));
  w->accum = (double *)malloc(size * sizeof(double));
  if (!w->rec || !w->ndon || !w->donor || !w->stack || !w->levels || !w->accum) {
    fso_work_free(w);
    return -1;
  }
  for (size_t i = 0; i < size; i++) w->rec[i] = NO_FLOW;
  return 0;
}

void fso_work_free(fso_work *w) {
  free(w->rec); free(w->ndon); free(w->donor);
  free(w->stack); free(w->levels); free(w->accum);
  memset(w, 0, sizeof(*w));
}

static double now_s(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

/* fastscape_RB.cpp:366-373 */
void fso_step(fso_work *w, double *h, const fso_params *p, int parallel,
              double *phase_s) {
  double t0 = now_s();
  fso_receivers(h, w->W, w->H, p, w->rec);
  double t1 = now_s();
  fso_donors(w->rec, w->W, w->H, w->ndon, w->donor);
  double t2 = now_s();
  w->nlevel = fso_order(w->rec, w->ndon, w->donor, w->W, w->H, w->stack, w->levels);
  double t3 = now_s();
  fso_flowacc(w->rec, w->stack, w->W, w->H, p, w->accum);
  double t4 = now_s();
  fso_uplift(h, w->W, w->H, p);
  double t5 = now_s();
  if (parallel)
    fso_erode_levels(h, w->rec, w->stack, w->levels, w->nlevel, w->accum, w->W, w->H, p);
  else
    fso_erode(h, w->rec, w->stack, w->accum, w->W, w->H, p);
  double t6 = now_s();
  if (phase_s) {
    phase_s[0] += t1 - t0; phase_s[1] += t2 - t1; phase_s[2] += t3 - t2;
    phase_s[3] += t4 - t3; phase_s[4] += t5 - t4; phase_s[5] += t6 - t5;
  }
}

/* fastscape_RB.cpp:341-398 */
void fso_run(double *h, int W, int H, const fso_params *p, int nstep,
             int parallel) {
  fso_work w;
  if (fso_work_init(&w, W, H) != 0) return;
  for (int step = 0; step <= nstep; step++) fso_step(&w, h, p, parallel, NULL);
  fso_work_free(&w);
}

void fso_level_ids(const int32_t *stack, const int32_t *levels, int nlevel,
                   int W, int H, int32_t *level_id) {
  const long size = (long)W * H;
  for (long i = 0; i < size; i++) level_id[i] = -1;
  for (int li = 0; li < nlevel - 1; li++)
    for (int s = levels[li]; s < levels[li + 1]; s++) level_id[stack[s]] = li;
}

int fso_omp_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
