// gba_solve_ba.hpp — header-only C++ drop-in for the reference's
//   void SolveBA(BALProblem &bal_problem)
// (backend/slam_ba_simple_g2o_ceres/test_bundle_adjustment_ceres.cpp:58-101).
//
// Works with any type exposing the accessors of slamplay::BALProblem
// (utils/datasets/BALProblem.h:55-98): num_cameras(), num_points(),
// num_observations(), camera_block_size(), camera_index(), point_index(),
// observations(), mutable_cameras().  Cameras in the 9-parameter angle-axis
// layout (camera_block_size() == 9, what the reference's
// AutoDiffCostFunction<SnavelyReprojectionError, 2, 9, 3> assumes) or in
// BALProblem's use_quaternions layout (camera_block_size() == 10,
// BALProblem.cpp:117-138), which the library converts to angle-axis for the
// solve and back (gba_options::camera_layout).
//
// Like the reference: one Snavely residual block per observation with
// HuberLoss(1.0) (:78), Levenberg-Marquardt with the points eliminated
// (:97), parameters updated in place (the reference hands Ceres pointers into
// parameters_, :83-86), a report printed afterwards (:101).  Unlike the
// reference, failures come back as a gba_status.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "gba.h"

namespace slamplay_gb300 {

struct SolveBAOptions {
  gba_options options;
  bool print_report = true;
  SolveBAOptions() {
    gba_options_init(&options);
    options.loss = GBA_LOSS_HUBER;  // test_bundle_adjustment_ceres.cpp:78
    options.loss_scale = 1.0;
  }
  // The g2o variant's SolveBA (test_bundle_adjustment_g2o.cpp:166-232):
  // SO3 left camera update (:84-90), g2o's Levenberg (:174-176), Huber 1.0
  // per edge (:213), 40 iterations (:218), no tolerance tests.
  static SolveBAOptions G2OVariant() {
    SolveBAOptions o;
    o.options.camera_update = GBA_CAMERA_UPDATE_SO3_LEFT;
    o.options.lm_policy = GBA_LM_POLICY_G2O;
    o.options.max_num_iterations = 40;
    o.options.function_tolerance = 0.0;
    o.options.gradient_tolerance = 0.0;
    o.options.parameter_tolerance = 0.0;
    return o;
  }
};

// Solves in place; returns the status (and fills *summary when given).
template <typename BALProblemT>
gba_status SolveBA(BALProblemT &bal_problem, const SolveBAOptions &opts = SolveBAOptions(),
                   gba_summary *summary = nullptr) {
  const int cbs = bal_problem.camera_block_size();
  if (cbs != 9 && cbs != 10) return GBA_ERR_INVALID_ARGUMENT;
  gba_options options = opts.options;
  options.camera_layout = cbs == 10 ? GBA_CAMERA_QUATERNION : GBA_CAMERA_ANGLE_AXIS;
  gba_problem_view v;
  v.num_cameras = bal_problem.num_cameras();
  v.num_points = bal_problem.num_points();
  v.num_observations = bal_problem.num_observations();
  v.camera_index = bal_problem.camera_index();
  v.point_index = bal_problem.point_index();
  v.observations = bal_problem.observations();
  v.parameters = bal_problem.mutable_cameras();  // cameras, then points, contiguous
  gba_handle *h = nullptr;
  gba_status st = gba_create(&options, &h);
  if (st != GBA_OK) {
    std::fprintf(stderr, "gba_create: %s\n", gba_last_error(nullptr));
    return st;
  }
  gba_summary s{};
  // one trace row per trial: up to 10 per iteration under g2o's policy
  const int per = opts.options.lm_policy == GBA_LM_POLICY_G2O ? 10 : 1;
  std::vector<double> cost((size_t)opts.options.max_num_iterations * per + 1);
  s.trace_capacity = (int32_t)cost.size();
  s.trace_cost = cost.data();
  st = gba_solve(h, &v, &s);
  if (st != GBA_OK) {
    std::fprintf(stderr, "gba_solve: %s\n", gba_last_error(h));
  } else if (opts.print_report) {
    std::printf("bal problem have %d cameras and %d points. Forming %d observations.\n", v.num_cameras,
                v.num_points, v.num_observations);
    for (int k = 0; k < s.trace_length; ++k) std::printf("%4d  cost %.6e\n", k, cost[k]);
    std::printf("Initial cost %.6e  Final cost %.6e  Iterations %d (%d successful)  PCG iterations %lld\n"
                "Termination %s  solve %.3f ms  total %.3f ms\n",
                s.initial_cost, s.final_cost, s.num_iterations, s.num_successful_steps,
                (long long)s.num_linear_solver_iterations,
                s.termination_type == GBA_TERMINATION_CONVERGENCE      ? "CONVERGENCE"
                : s.termination_type == GBA_TERMINATION_NO_CONVERGENCE ? "NO_CONVERGENCE"
                                                                       : "FAILURE",
                s.solve_time_s * 1e3, s.total_time_s * 1e3);
  }
  if (summary) *summary = s;
  gba_destroy(h);
  return st;
}

// Minimal owner of a BAL problem with the reference's accessors, backed by
// libgba's BAL reader / writer (utils/datasets/BALProblem.cpp:78-336).
class BALProblem {
 public:
  explicit BALProblem(const std::string &filename) {
    int32_t nc, np, no;
    if (gba_bal_read_header(filename.c_str(), &nc, &np, &no) != GBA_OK)
      throw std::runtime_error("unable to open file " + filename);
    nc_ = nc, np_ = np, no_ = no;
    cam_.resize(no), pt_.resize(no), obs_.resize(2 * (size_t)no), par_.resize(9 * (size_t)nc + 3 * (size_t)np);
    gba_problem_view v = view();
    if (gba_bal_read(filename.c_str(), &v) != GBA_OK) throw std::runtime_error("invalid BAL file " + filename);
  }
  int camera_block_size() const { return 9; }
  int point_block_size() const { return 3; }
  int num_cameras() const { return nc_; }
  int num_points() const { return np_; }
  int num_observations() const { return no_; }
  int num_parameters() const { return (int)par_.size(); }
  const int *camera_index() const { return cam_.data(); }
  const int *point_index() const { return pt_.data(); }
  const double *observations() const { return obs_.data(); }
  const double *parameters() const { return par_.data(); }
  double *mutable_cameras() { return par_.data(); }
  double *mutable_points() { return par_.data() + 9 * (size_t)nc_; }
  void Normalize() {
    gba_problem_view v = view();
    gba_bal_normalize(&v);
  }
  void Perturb(double rotation_sigma, double translation_sigma, double point_sigma) {
    gba_problem_view v = view();
    gba_bal_perturb(&v, rotation_sigma, translation_sigma, point_sigma, 0);
  }
  void WriteToFile(const std::string &filename) const {
    gba_problem_view v = view();
    gba_bal_write(filename.c_str(), &v);
  }
  void WriteToPLYFile(const std::string &filename) const {
    gba_problem_view v = view();
    gba_bal_write_ply(filename.c_str(), &v);
  }

 private:
  gba_problem_view view() const {
    gba_problem_view v;
    v.num_cameras = nc_;
    v.num_points = np_;
    v.num_observations = no_;
    v.camera_index = cam_.data();
    v.point_index = pt_.data();
    v.observations = obs_.data();
    v.parameters = const_cast<double *>(par_.data());
    return v;
  }
  int nc_ = 0, np_ = 0, no_ = 0;
  std::vector<int32_t> cam_, pt_;
  std::vector<double> obs_, par_;
};

}  // namespace slamplay_gb300
