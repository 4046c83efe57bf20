// bundle_adjustment_gb300 — the reference demo's main()
// (backend/slam_ba_simple_g2o_ceres/test_bundle_adjustment_ceres.cpp:37-56)
// with SolveBA running on the GPU through libgba:
//   read BAL -> Normalize -> Perturb(0.1, 0.5, 0.5) -> initial.ply ->
//   SolveBA -> final.ply
// Usage: bundle_adjustment_gb300 bal_data.txt [--mixed] [--g2o] [--raw out.bin]
//   --g2o: the g2o variant's SolveBA (test_bundle_adjustment_g2o.cpp:166-232)
//   --raw: also writes the solved parameters (9 per camera, then 3 per point)
//          as raw doubles, and prints the final cost to 17 digits
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gba_solve_ba.hpp"

int main(int argc, char **argv) {
  if (argc < 2) {
    std::printf("usage: %s bal_data.txt [--mixed] [--g2o]\n", argv[0]);
    return 1;
  }
  try {
    slamplay_gb300::BALProblem bal_problem(argv[1]);
    bal_problem.Normalize();
    bal_problem.Perturb(0.1, 0.5, 0.5);
    bal_problem.WriteToPLYFile("initial.ply");
    bool mixed = false, g2o = false;
    const char *raw = nullptr;
    for (int i = 2; i < argc; ++i) {
      mixed |= std::strcmp(argv[i], "--mixed") == 0;
      g2o |= std::strcmp(argv[i], "--g2o") == 0;
      if (std::strcmp(argv[i], "--raw") == 0 && i + 1 < argc) raw = argv[++i];
    }
    slamplay_gb300::SolveBAOptions opts = g2o ? slamplay_gb300::SolveBAOptions::G2OVariant() : slamplay_gb300::SolveBAOptions();
    if (mixed) opts.options.precision = GBA_PRECISION_MIXED;
    gba_summary summary{};
    const gba_status st = slamplay_gb300::SolveBA(bal_problem, opts, &summary);
    bal_problem.WriteToPLYFile("final.ply");
    if (raw && st == GBA_OK) {
      std::printf("final_cost %.17g\n", summary.final_cost);
      FILE *f = std::fopen(raw, "wb");
      if (!f) return 3;
      const size_t n = (size_t)bal_problem.num_parameters();
      const bool ok = std::fwrite(bal_problem.parameters(), sizeof(double), n, f) == n;
      std::fclose(f);
      if (!ok) return 3;
    }
    return st == GBA_OK ? 0 : 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
}
