// ref_harness.cpp -- C API around the reference's own FastScape_RB and
// FastScape_RBP classes, used to PIN the oracle restatement. Test
// infrastructure only: oracle/build.py (--ref) compiles this file together with
// the reference sources read from where they lie (never copied), and writes
// the result only to oracle/_ref/. Nothing in the product path loads it.
//
// oracle/build.py emits one translation unit:
//     <this file's PRELUDE section>
//     namespace fsref_rb  { <fastscape_RB.cpp>   }
//     namespace fsref_rbp { <fastscape_RB+P.cpp> }
//     namespace fsref_bw  { <fastscape_BW.cpp>   }
//     <this file's DRIVER section>
// The standard headers, random.hpp and CumulativeTimer.hpp are included
// first, so the includes inside the reference files are no-ops and the two
// classes land in separate namespaces. `private` is mapped to `public` (after
// the standard headers) so the driver can call the six phase methods and read
// the scratch arrays directly. In the "param" build the eight physical
// constants of fastscape_RB.cpp:58-65 are replaced by reads of fsref_p[] so
// the reference can run the workload's constants; the "pristine" build
// compiles the reference text unchanged.

//@@PRELUDE
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fenv.h>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>
#include "random.hpp"
#include "CumulativeTimer.hpp"

// keq, neq, meq, ueq, dt, dr_orth, dr_diag, tol, cell_area
extern "C" {
double fsref_p[9] = {2e-6, 2, 0.8, 2e-3, 1000., 1,
                     1.414213562373095048801688724209698078569671875376948,
                     1e-3, 40000};
}

#define private public
#define main fsref_unused_cli_main
//@@DRIVER
#undef main
#undef private

namespace {

// Mirrors the allocation at fastscape_RB.cpp:346-362, with the level table
// sized for the worst case (size+2) instead of the perimeter (:358).
template <class M>
void prepare_common(M &m) {
  m.accum.assign(m.size, 0.0);
  m.rec.assign(m.size, -1);
  m.ndon.assign(m.size, 0);
  m.donor.assign(8 * static_cast<size_t>(m.size), 0);
  m.stack.assign(m.size, 0);
  m.levels.assign(m.size + 2, 0);
  m.nlevel = 0;
}

void prepare(fsref_rb::FastScape_RB &m) { prepare_common(m); }

// fastscape_BW.cpp:307-315 (no level table in the Braun-Willett variant).
void prepare(fsref_bw::FastScape_BW &m) {
  m.accum.assign(m.size, 0.0);
  m.rec.assign(m.size, -1);
  m.ndon.assign(m.size, 0);
  m.donor.assign(8 * static_cast<size_t>(m.size), 0);
  m.stack.assign(m.size, 0);
}

// fastscape_RB+P.cpp:368-370 also sets the capacities used by its asserts.
void prepare(fsref_rbp::FastScape_RBP &m) {
  m.stack_width = m.size;
  m.level_width = m.size + 2;
  prepare_common(m);
}

template <class M>
void phase(M &m, int p) {
  switch (p) {
    case 0: m.ComputeReceivers(); break;
    case 1: m.ComputeDonors(); break;
    case 2: m.GenerateOrder(); break;
    case 3: m.ComputeFlowAcc(); break;
    case 4: m.AddUplift(); break;
    case 5: m.Erode(); break;
    default: break;
  }
}

}  // namespace

// Variants 0 (RB) and 1 (RB+P), which have a level table.
#define FSREF_DISPATCH(variant, obj, EXPR)                                   \
  do {                                                                       \
    if ((variant) == 0) {                                                    \
      auto &m = *static_cast<fsref_rb::FastScape_RB *>(obj);                 \
      EXPR;                                                                  \
    } else if ((variant) == 1) {                                             \
      auto &m = *static_cast<fsref_rbp::FastScape_RBP *>(obj);               \
      EXPR;                                                                  \
    }                                                                        \
  } while (0)

// All three variants, 2 being BW (fastscape_BW.cpp, the DFS stack order).
#define FSREF_DISPATCH3(variant, obj, EXPR)                                  \
  do {                                                                       \
    if ((variant) == 2) {                                                    \
      auto &m = *static_cast<fsref_bw::FastScape_BW *>(obj);                 \
      EXPR;                                                                  \
    } else {                                                                 \
      FSREF_DISPATCH(variant, obj, EXPR);                                    \
    }                                                                        \
  } while (0)

extern "C" {

int fsref_is_param_build(void) {
#ifdef FSREF_PARAM_BUILD
  return 1;
#else
  return 0;
#endif
}

void fsref_set_params(const double *p) {
  for (int i = 0; i < 9; i++) fsref_p[i] = p[i];
}

void fsref_seed(unsigned long seed) { seed_rand(seed); }

void *fsref_create(int variant, int W, int H) {
  if (variant == 0) return new fsref_rb::FastScape_RB(W, H);
  if (variant == 2) return new fsref_bw::FastScape_BW(W, H);
  return new fsref_rbp::FastScape_RBP(W, H);
}

void fsref_destroy(int variant, void *obj) {
  if (variant == 0)
    delete static_cast<fsref_rb::FastScape_RB *>(obj);
  else if (variant == 2)
    delete static_cast<fsref_bw::FastScape_BW *>(obj);
  else
    delete static_cast<fsref_rbp::FastScape_RBP *>(obj);
}

void fsref_constants(int variant, void *obj, double *out) {
  FSREF_DISPATCH3(variant, obj, {
    out[0] = m.keq; out[1] = m.neq; out[2] = m.meq; out[3] = m.ueq;
    out[4] = m.dt; out[5] = m.dr[0]; out[6] = m.dr[1]; out[7] = m.tol;
    out[8] = m.cell_area;
  });
}

void fsref_get_h(int variant, void *obj, double *out) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(out, m.h.data(), sizeof(double) * m.size));
}

void fsref_set_h(int variant, void *obj, const double *in) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(m.h.data(), in, sizeof(double) * m.size));
}

void fsref_prepare(int variant, void *obj) {
  FSREF_DISPATCH3(variant, obj, prepare(m));
}

void fsref_phase(int variant, void *obj, int p) {
  FSREF_DISPATCH3(variant, obj, phase(m, p));
}

void fsref_step(int variant, void *obj) {
  FSREF_DISPATCH3(variant, obj, for (int p = 0; p < 6; p++) phase(m, p));
}

int fsref_nlevel(int variant, void *obj) {
  int r = 0;
  FSREF_DISPATCH(variant, obj, r = m.nlevel);
  return r;
}

void fsref_get_rec(int variant, void *obj, int32_t *out) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(out, m.rec.data(), sizeof(int) * m.size));
}
void fsref_get_ndon(int variant, void *obj, int32_t *out) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(out, m.ndon.data(), sizeof(int) * m.size));
}
void fsref_get_donor(int variant, void *obj, int32_t *out) {
  FSREF_DISPATCH3(variant, obj,
                  std::memcpy(out, m.donor.data(), sizeof(int) * 8 * static_cast<size_t>(m.size)));
}
void fsref_get_stack(int variant, void *obj, int32_t *out) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(out, m.stack.data(), sizeof(int) * m.size));
}
void fsref_get_levels(int variant, void *obj, int32_t *out, int n) {
  FSREF_DISPATCH(variant, obj, std::memcpy(out, m.levels.data(), sizeof(int) * n));
}
void fsref_get_accum(int variant, void *obj, double *out) {
  FSREF_DISPATCH3(variant, obj, std::memcpy(out, m.accum.data(), sizeof(double) * m.size));
}

// The reference's PrintDEM (fastscape_RB.cpp:20-40) of the current h.
void fsref_print_dem(int variant, void *obj, const char *path) {
  FSREF_DISPATCH3(variant, obj, fsref_rb::PrintDEM(path, m.h, m.width, m.height));
}

// The reference's own run(): nstep+1 timesteps, prints its `p`/`t` lines.
void fsref_run(int variant, void *obj, int nstep) {
  FSREF_DISPATCH3(variant, obj, m.run(nstep));
  std::cout.flush();
}

}  // extern "C"
