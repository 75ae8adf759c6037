// fastscape_gb300.hpp -- header-only C++ wrapper over the C ABI that restores
// the reference's object interface:
//
//     FastScape_RBP tm(width, height);   // fastscape_RB+P.cpp:138-154
//     tm.run(nstep);                     // fastscape_RB+P.cpp:363-424
//     std::vector<double>& h = tm.getH(); // fastscape_RB+P.cpp:429-431
//
// getH() returns a reference to a host vector that the wrapper refreshes
// from the device on every call (the reference returns its own storage).
// Errors come back as fs::Error exceptions on this side of the boundary; no
// exception crosses the C ABI.
#ifndef FASTSCAPE_GB300_HPP
#define FASTSCAPE_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "fastscape_gb300.h"

namespace fs {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status) {
  if (status != FS_OK) {
    char buf[512];
    fs_last_error(buf, sizeof(buf));
    throw Error(status, buf);
  }
}

inline fs_params reference_params() {
  fs_params p;
  fs_params_reference(&p);
  return p;
}

inline fs_params workload_params(double dx = 100.0) {
  fs_params p;
  fs_params_workload(&p, dx);
  return p;
}

// One realization on the current CUDA device.
class Model {
 public:
  Model(int width, int height, const fs_params &params = reference_params(),
        int init_mode = FS_INIT_REFERENCE, uint64_t seed = 123)
      : width_(width), height_(height) {
    int st = FS_OK;
    m_ = fs_create(width, height, &params, init_mode, seed, &st);
    if (!m_) check(st == FS_OK ? FS_ERR_CUDA : st);
  }
  Model(const Model &) = delete;
  Model &operator=(const Model &) = delete;
  Model(Model &&o) noexcept : m_(o.m_), width_(o.width_), height_(o.height_), h_(std::move(o.h_)) {
    o.m_ = nullptr;
  }
  ~Model() { fs_destroy(m_); }

  // nstep+1 timesteps, like the reference (fastscape_RB.cpp:366).
  void run(int nstep) { check(fs_run(m_, nstep)); }
  // exactly k timesteps
  void step(int k) { check(fs_step(m_, k)); }

  std::vector<double> &getH() {
    h_.resize(static_cast<size_t>(width_) * height_);
    check(fs_get_elevation(m_, h_.data()));
    return h_;
  }
  void setH(const std::vector<double> &h) {
    if (h.size() != static_cast<size_t>(width_) * height_) check(FS_ERR_ARG);
    check(fs_set_elevation(m_, h.data()));
  }
  std::vector<double> accumulation() const {
    std::vector<double> a(static_cast<size_t>(width_) * height_);
    check(fs_get_accumulation(m_, a.data()));
    return a;
  }
  std::vector<int32_t> receivers() const {
    std::vector<int32_t> r(static_cast<size_t>(width_) * height_);
    check(fs_get_receivers(m_, r.data()));
    return r;
  }
  std::vector<int32_t> levels(int32_t *nlevels = nullptr) const {
    std::vector<int32_t> l(static_cast<size_t>(width_) * height_);
    check(fs_get_levels(m_, l.data(), nlevels));
    return l;
  }
  int width() const { return width_; }
  int height() const { return height_; }
  fs_model *handle() { return m_; }

 private:
  fs_model *m_ = nullptr;
  int width_, height_;
  std::vector<double> h_;
};

}  // namespace fs

// The reference's class names, for code written against fastscape_RB*.cpp.
using FastScape_RBP = fs::Model;
using FastScape_RB = fs::Model;

#endif  // FASTSCAPE_GB300_HPP
