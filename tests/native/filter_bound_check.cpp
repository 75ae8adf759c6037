// Host check of the receiver filter's decisions (k_receivers_filter in
// barnes2019-landscape_gb300/csrc/fs_kernels.cu, restated here operation for
// operation in FP32): on random tiles, every cell the filter settles must get
// the receiver of the reference formula (fastscape_RB.cpp:160-182) evaluated
// in FP64. Both stagings are exercised -- FP32 truncations with the tile's
// bound, and heights of 128 m and more relative to the tile's first cell
// (fs::fixed_in_binade) with a per-cell bound -- on tilted planes with
// bumps and noise from sea level to 1e6 m, relief from 1e-9 to 1e2 m per
// cell, heights rounded to coarse grids (exact ties), copied neighbours
// (equal slopes), base-level rows of zeros beside high ground, negative
// ground, zeros, subnormals and heights beyond the relative range.
// Usage: filter_bound_check <tiles> <seed>; exit 1 on the first wrong
// decision.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "fs_bits.h"

namespace {

constexpr int kTw = 32, kTh = 24;               // interior cells of a tile
constexpr int kSw = kTw + 2, kSh = kTh + 2;     // staged with the halo
constexpr int kRelEmin = 1030, kRelEmax = 1123;  // the kernel's constants
constexpr int kPit = -2;

uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }

// nshift order W, NW, N, NE, E, SE, S, SW as (dx, dy)
const int kDx[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
const int kDy[8] = {0, -1, -1, -1, 0, 1, 1, 1};

int exact_receiver(const double *h, int x, int y, double dr_orth, double dr_diag) {
  const double hc = h[y * kSw + x];
  double max_slope = 0;
  int max_n = -1;
  for (int n = 0; n < 8; n++) {
    const double slope = (hc - h[(y + kDy[n]) * kSw + x + kDx[n]]) / ((n & 1) ? dr_diag : dr_orth);
    if (slope > max_slope) {
      max_slope = slope;
      max_n = n;
    }
  }
  return max_n < 0 ? kPit : max_n;
}

}  // namespace

int main(int argc, char **argv) {
  const long ntiles = argc > 1 ? std::atol(argv[1]) : 20000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const double dr_orth = 100.0, dr_diag = 100.0 * 1.4142135623730951;
  const float g_orth = (float)(1.0 / dr_orth), g_diag = (float)(1.0 / dr_diag);
  const float gmax = g_orth > g_diag ? g_orth : g_diag;
  std::vector<double> h(kSw * kSh);
  std::vector<float> f(kSw * kSh);
  long decided = 0, queued = 0, rel_tiles = 0;
  for (long t = 0; t < ntiles; t++) {
    // ---- a tile of terrain ------------------------------------------------
    const unsigned kind = (unsigned)(g() % 8);
    double base;
    if (kind == 0) base = U(g) * 100.0;                                 // low ground
    else if (kind == 1) base = -std::exp(std::log(128.0) + U(g) * std::log(1e6 / 128.0));
    else if (kind == 2) base = std::ldexp(1.0, 7 + (int)(g() % 14));     // on a binade edge
    else base = std::exp(std::log(128.0) + U(g) * std::log(1e6 / 128.0));
    const double S = std::exp(std::log(1e-9) + U(g) * std::log(1e11));  // relief per cell
    const double ax = (2 * U(g) - 1) * S, ay = (2 * U(g) - 1) * S;
    const double bump = U(g) < 0.5 ? 0.0 : S * 30 * U(g);
    const double noise = U(g) < 0.3 ? 0.0 : S * std::exp(-10 * U(g));
    const double grid = U(g) < 0.2 ? std::ldexp(1.0, -(int)(g() % 30)) : 0.0;
    for (int y = 0; y < kSh; y++)
      for (int x = 0; x < kSw; x++) {
        double v = base + ax * x + ay * y + bump * std::sin(x * 0.37) * std::cos(y * 0.29) +
                   noise * (2 * U(g) - 1);
        if (grid > 0) v = std::round(v / grid) * grid;
        h[y * kSw + x] = v;
      }
    if (U(g) < 0.2) {  // copied neighbours: equal slopes
      for (int k = 0; k < 40; k++) {
        const int x = 1 + (int)(g() % kTw), y = 1 + (int)(g() % kTh);
        const int n = (int)(g() % 8), m = (int)(g() % 8);
        h[(y + kDy[n]) * kSw + x + kDx[n]] = h[(y + kDy[m]) * kSw + x + kDx[m]];
      }
    }
    if (U(g) < 0.5) {  // planted near-ties: two downhill slopes a relative 2^-k apart
      for (int k = 0; k < 60; k++) {
        const int x = 1 + (int)(g() % kTw), y = 1 + (int)(g() % kTh);
        const double hc = h[y * kSw + x];
        const double a = std::exp(std::log(1e-9) + U(g) * std::log(1e9)) * (1 + std::fabs(hc) * 1e-7);
        const int n1 = (int)(g() % 8), n2 = (n1 + 1 + (int)(g() % 7)) % 8;
        const double d1 = (n1 & 1) ? dr_diag : dr_orth, d2 = (n2 & 1) ? dr_diag : dr_orth;
        const double rel = std::ldexp(g() & 1 ? 1.0 : -1.0, -(int)(8 + g() % 45));
        for (int n = 0; n < 8; n++)  // the others uphill
          h[(y + kDy[n]) * kSw + x + kDx[n]] = hc + a * d1 * (1 + U(g));
        h[(y + kDy[n1]) * kSw + x + kDx[n1]] = hc - a * d1;
        h[(y + kDy[n2]) * kSw + x + kDx[n2]] = g() % 4 ? hc - a * d2 * (1 + rel)
                                                        : hc - a * d1 * rel;  // or one near zero
      }
    }
    if (U(g) < 0.1) {  // a base-level row or column of zeros
      if (g() & 1) for (int x = 0; x < kSw; x++) h[(g() & 1 ? 0 : kSh - 1) * kSw + x] = 0.0;
      else for (int y = 0; y < kSh; y++) h[y * kSw + (g() & 1 ? 0 : kSw - 1)] = 0.0;
    }
    if (U(g) < 0.1) {  // special values
      const double sp[] = {0.0, -0.0, 5e-324, 1e-300, -1e-310, 1e35, -1e35, 3e30};
      for (int k = 0; k < 6; k++) h[g() % (kSw * kSh)] = sp[g() % 8];
    }
    // ---- the filter, as the kernel computes it ----------------------------
    float m = 0.f;
    bool bad = false;
    int et = 0;
    for (int i = 0; i < kSw * kSh; i++) {
      const uint64_t b = bits(h[i]);
      f[i] = fs::trunc_bits_to_float(b);
      m = std::fmax(m, std::fabs(f[i]));
      bad |= !(f[i] == f[i]);
      et = std::max(et, (int)(b >> 52) & 0x7FF);
    }
    const bool rel = et >= kRelEmin && et <= kRelEmax;
    float absterm = 0x1p-100f;
    if (rel) {
      ++rel_tiles;
      const long long xr = fs::fixed_in_binade(bits(h[kSw + 1]), et);
      const float unit = fs::float_from_bits((uint32_t)(et - 1084 + 127) << 23);
      absterm = fs::float_from_bits((uint32_t)(et - 1062 + 127) << 23);
      for (int i = 0; i < kSw * kSh; i++)
        f[i] = (float)(fs::fixed_in_binade(bits(h[i]), et) - xr) * unit;
    }
    const float M = m;
    const float cE = 0x1p-19f * gmax;
    for (int y = 1; y <= kTh; y++)
      for (int x = 1; x <= kTw; x++) {
        auto F = [&](int dx, int dy) { return f[(y + dy) * kSw + x + dx]; };
        const float u0 = F(-1, -1), u1 = F(0, -1), u2 = F(1, -1);
        const float m0 = F(-1, 0), m1 = F(0, 0), m2 = F(1, 0);
        const float d0 = F(-1, 1), d1 = F(0, 1), d2 = F(1, 1);
        float E = cE * (M + absterm);
        if (rel) {
          const float cu = std::fmax(std::fabs(u0), std::fmax(std::fabs(u1), std::fabs(u2)));
          const float cm = std::fmax(std::fabs(m0), std::fmax(std::fabs(m1), std::fabs(m2)));
          const float cd = std::fmax(std::fabs(d0), std::fmax(std::fabs(d1), std::fabs(d2)));
          E = cE * (std::fmax(cu, std::fmax(cm, cd)) + absterm);
        }
        const float fc = m1;
        const float lo1 = std::fmin(m0, m2), hi1 = std::fmax(m0, m2);
        const float lo2 = std::fmin(u1, d1), hi2 = std::fmax(u1, d1);
        const float lo3 = std::fmin(u0, u2), hi3 = std::fmax(u0, u2);
        const float lo4 = std::fmin(d2, d0), hi4 = std::fmax(d2, d0);
        const float omin = std::fmin(lo1, lo2), osec = std::fmin(std::fmax(lo1, lo2), std::fmin(hi1, hi2));
        const float dmin = std::fmin(lo3, lo4), dsec = std::fmin(std::fmax(lo3, lo4), std::fmin(hi3, hi4));
        const int oi = lo2 < lo1 ? (d1 < u1 ? 6 : 2) : (m2 < m0 ? 4 : 0);
        const int di = lo4 < lo3 ? (d0 < d2 ? 7 : 5) : (u2 < u0 ? 3 : 1);
        const float bo = (fc - omin) * g_orth, so = (fc - osec) * g_orth;
        const float bd = (fc - dmin) * g_diag, sd = (fc - dsec) * g_diag;
        const float best = std::fmax(bo, bd);
        const float second = std::fmax(std::fmin(bo, bd), std::fmax(so, sd));
        const int bn = bo > bd ? oi : di;
        int code = -1;
        if (!bad) {
          if (best - second > 2.f * E && best > E) code = bn;
          else if (best < -E) code = kPit;
        }
        if (code == -1) {
          ++queued;
          continue;
        }
        ++decided;
        const int want = exact_receiver(h.data(), x, y, dr_orth, dr_diag);
        if (code != want) {
          std::printf("wrong decision: tile %ld cell (%d,%d) got %d want %d (rel %d, et %d)\n", t,
                      x, y, code, want, (int)rel, et);
          return 1;
        }
      }
  }
  std::printf("%ld tiles (%ld relative), %ld cells decided, %ld queued: all decisions exact\n",
              ntiles, rel_tiles, decided, queued);
  return 0;
}
