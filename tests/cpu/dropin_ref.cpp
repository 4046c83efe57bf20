// The C++ drop-in (include/gba_solve_ba.hpp) compiled against the
// reference's OWN slamplay::BALProblem (utils/datasets/BALProblem.h and
// .cpp, built from where they lie in the reference tree with the
// declaration shims of oracle/ref_shim): the reference's main()
// (backend/slam_ba_simple_g2o_ceres/test_bundle_adjustment_ceres.cpp:37-56)
// with SolveBA replaced by slamplay_gb300::SolveBA.
// Usage: dropin_ref bal_file [quaternions(0|1)] [raw_out]
// Prints "status <gba_status>" and, on success, the final cost; with
// raw_out it writes the solved parameters as raw doubles.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "datasets/BALProblem.h"
#include "gba_solve_ba.hpp"

int main(int argc, char **argv) {
  if (argc < 2) return 1;
  const bool quat = argc > 2 && std::atoi(argv[2]) != 0;
  slamplay::BALProblem bal_problem(argv[1], quat);
  bal_problem.Normalize();
  bal_problem.Perturb(0.1, 0.5, 0.5);
  slamplay_gb300::SolveBAOptions opts;
  opts.print_report = false;
  gba_summary s{};
  const gba_status st = slamplay_gb300::SolveBA(bal_problem, opts, &s);
  std::printf("status %d block %d\n", (int)st, bal_problem.camera_block_size());
  if (st == GBA_OK) {
    std::printf("final_cost %.17g\n", s.final_cost);
    if (argc > 3) {
      FILE *f = std::fopen(argv[3], "wb");
      if (!f) return 3;
      std::fwrite(bal_problem.parameters(), sizeof(double), (size_t)bal_problem.num_parameters(), f);
      std::fclose(f);
    }
  }
  return 0;
}
