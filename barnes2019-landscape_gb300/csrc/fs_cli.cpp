// fs_cli.cpp -- command-line program with the reference's interface
// (fastscape_RB.cpp:414-449):
//
//     fastscape_gb300 <Dimension> <Steps> <Output Name> <Seed> [--workload]
//
// runs a Dimension x Dimension model for Steps+1 timesteps on the GPU,
// prints the RichDEM-style tagged lines the reference prints (A algorithm,
// C citation, h git hash, m seed, p progress every 20 timesteps, t timings;
// consumed by the reference's tests/d.make_tabular) and writes the final
// elevation as an ArcGIS ASCII grid without the halo ring, formatted like
// the reference's PrintDEM (fastscape_RB.cpp:20-40), so compare.sh-style
// diffs against the reference's output work unchanged. The constants are
// the reference's own (fastscape_RB.cpp:58-65) unless --workload selects the
// 1000^2/10000^2 workload's (n 1, m 0.4, dx 100).
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "fastscape_gb300.hpp"

#ifndef FS_GIT_HASH
#define FS_GIT_HASH "unknown"
#endif

namespace {

// fastscape_RB.cpp:20-40: the ASCII grid without the outer (halo) ring, with
// the reference's header values and the stream's default formatting.
void print_dem(const std::string &filename, const std::vector<double> &h, int width,
               int height) {
  std::ofstream fout(filename.c_str());
  fout << "ncols " << (width - 2) << "\n";
  fout << "nrows " << (height - 2) << "\n";
  fout << "xllcorner 637500.000\n";
  fout << "yllcorner 206000.000\n";
  fout << "cellsize 500.000\n";
  fout << "NODATA_value -9999\n";
  for (int y = 1; y < height - 1; y++) {
    for (int x = 1; x < width - 1; x++) fout << h[static_cast<size_t>(y) * width + x] << " ";
    fout << "\n";
  }
}

}  // namespace

int main(int argc, char **argv) {
  bool workload = false;
  std::vector<std::string> pos;
  for (int i = 1; i < argc; i++) {
    if (std::strcmp(argv[i], "--workload") == 0)
      workload = true;
    else
      pos.push_back(argv[i]);
  }
  if (pos.size() != 4) {
    std::cerr << "Syntax: " << argv[0] << " <Dimension> <Steps> <Output Name> <Seed> [--workload]"
              << std::endl;
    return -1;
  }
  const int width = std::stoi(pos[0]);
  const int height = std::stoi(pos[0]);
  const int nstep = std::stoi(pos[1]);
  const std::string output_name = pos[2];
  const auto rand_seed = std::stoul(pos[3]);

  std::cout << "A FastScape GB300" << std::endl;
  std::cout << "C Richard Barnes TODO" << std::endl;
  std::cout << "h git_hash    = " << FS_GIT_HASH << std::endl;
  std::cout << "m Random seed = " << rand_seed << std::endl;

  const auto t0 = std::chrono::steady_clock::now();
  try {
    const fs_params p = workload ? fs::workload_params() : fs::reference_params();
    fs::Model tm(width, height, p, FS_INIT_REFERENCE, rand_seed);
    fs::check(fs_set_timing(tm.handle(), 1));
    fs::check(fs_synchronize(tm.handle()));
    // Step1 is the set-up before the first timestep: the reference times its
    // allocations and receiver reset inside run() (fastscape_RB.cpp:346-364);
    // here the model allocates its device buffers and draws the field when
    // it is created, so that (host clock) is Step1.
    const auto t_init = std::chrono::steady_clock::now();
    // The reference executes timesteps 0..nstep and prints progress after
    // every timestep that is a multiple of 20 (fastscape_RB.cpp:366-376).
    int done = 0;
    while (done <= nstep) {
      const int next = done == 0 ? 1 : std::min(nstep + 1, (done / 20 + 1) * 20 + 1);
      tm.step(next - done);
      done = next;
      if ((done - 1) % 20 == 0) std::cout << "p Step = " << done - 1 << std::endl;
    }
    double ms[FS_NUM_TIMERS];
    fs::check(fs_get_phase_times(tm.handle(), ms, 0));
    auto us = [](double x) { return static_cast<long long>(x * 1e3); };
    const long long init_us =
        std::chrono::duration_cast<std::chrono::microseconds>(t_init - t0).count();
    // The reference's timer lines, names and widths unchanged
    // (fastscape_RB.cpp:380-387), so its tests/d.make_tabular columns
    // (Step1_Initialize ... Step7_Erosion, Overall) come out the same.
    // Steps 2-5 and 7 are device times (CUDA events, and the GPU clock inside
    // the level walk). The uplift is fused into the kernels that need the
    // uplifted heights -- interior cells inside the erosion, pits inside the
    // accumulation's level-0 pass -- so Step6 reports 0 and its time is
    // counted under Step7 (and, for pits, Step5).
    std::cout << "t Step1: Initialize         = " << std::setw(15) << init_us << " microseconds"
              << std::endl;
    std::cout << "t Step2: DetermineReceivers = " << std::setw(15) << us(ms[0]) << " microseconds"
              << std::endl;
    std::cout << "t Step3: DetermineDonors    = " << std::setw(15) << us(ms[1]) << " microseconds"
              << std::endl;
    std::cout << "t Step4: GenerateOrder      = " << std::setw(15) << us(ms[4]) << " microseconds"
              << std::endl;
    std::cout << "t Step5: FlowAcc            = " << std::setw(15) << us(ms[5]) << " microseconds"
              << std::endl;
    std::cout << "t Step6: Uplift             = " << std::setw(15) << 0 << " microseconds"
              << std::endl;
    std::cout << "t Step7: Erosion            = " << std::setw(15) << us(ms[6]) << " microseconds"
              << std::endl;
    std::cout << "t Overall                   = " << std::setw(15) << init_us + us(ms[3])
              << " microseconds" << std::endl;
    const double cell_steps = static_cast<double>(width) * height * (nstep + 1);
    std::cout << "t cell_steps_per_s          = " << std::setw(15)
              << static_cast<long long>(cell_steps / (ms[3] * 1e-3)) << std::endl;
    const auto t1 = std::chrono::steady_clock::now();
    std::cout << "t Total calculation time    = " << std::setw(15)
              << std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count()
              << " microseconds" << std::endl;
    print_dem(output_name, tm.getH(), width, height);
  } catch (const fs::Error &e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}
