/*
 * oracle.h — CPU oracle for the bundle-adjustment hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU solver in slamplay_gb300/ is compared
 * against this oracle; nothing in the product links it.
 *
 * What it restates (file:line in luigifreda/slamplay):
 *   - residual model: utils/camera/SnavelyReprojectionError.h:42-53, :61-87
 *   - Rodrigues rotation with the theta^2 <= DBL_EPSILON first-order branch:
 *     utils/geometry/rotation.h:133-199 (dot/cross :57-67)
 *   - exact Jacobian as ceres::AutoDiffCostFunction<...,2,9,3>
 *     (SnavelyReprojectionError.h:89-92): forward-mode dual numbers over the
 *     12 parameters, evaluated through the same formula and branch
 *   - problem build and solve: backend/slam_ba_simple_g2o_ceres/
 *     test_bundle_adjustment_ceres.cpp:70-100 (one block per observation,
 *     optional HuberLoss(1.0) at :78, SPARSE_SCHUR at :97)
 *   - the solver is Ceres Solver 2.2.0 (cloned by build_thirdparty.sh:190-197,
 *     not present in the reference tree): trust-region Levenberg-Marquardt
 *     with Jacobi scaling, Ceres' radius schedule, its function / gradient /
 *     parameter tolerance tests, the robust-loss corrector, and an exact
 *     Schur-complement solve (points eliminated, dense Cholesky of the
 *     reduced camera system).  These follow Ceres' published documentation
 *     and algorithm description; the Ceres source is not available here.
 *
 * Parity status: the residual, Jacobian, rotation and BAL I/O restatements
 * are pinned against the reference's own sources compiled by
 * oracle/build_ref.sh (oracle/_ref).  The LM / Schur solver level is
 * "parity unpinned": Ceres itself cannot be built here.
 */
#ifndef GBA_ORACLE_H_
#define GBA_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem {
  int nc, np, no;
  const int *camera_index;
  const int *point_index;
  const double *observations;
  double *parameters; /* 9*nc + 3*np, in/out */
} orc_problem;

enum { ORC_LOSS_TRIVIAL = 0, ORC_LOSS_HUBER = 1, ORC_LOSS_CAUCHY = 2 };
enum { ORC_SOLVER_DENSE_SCHUR = 0, ORC_SOLVER_PCG_SCHUR = 1 };
enum { ORC_PCG_RESIDUAL = 0, ORC_PCG_QUADRATIC_MODEL = 1 };
/* camera update: Ceres' additive angle-axis, or g2o's R <- exp(dw) R */
enum { ORC_UPDATE_ADDITIVE = 0, ORC_UPDATE_SO3_LEFT = 1 };
/* The local-BA window's camera model (full_slam/include/myslam/g2o_types.h
 * EdgeProjection, full_slam/src/backend.cpp:67-199): a stereo rig of two
 * pinhole cameras sharing K, each with its extrinsic E_k (body -> camera);
 * camera blocks hold a keyframe pose T_cw as angle-axis (3), translation (3)
 * and three unused slots; obs_camera[i] says which rig camera saw
 * observation i (0 left, 1 right). */
typedef struct orc_rig {
  double fx, fy, cx, cy;
  double ext[2][6]; /* angle-axis (3), translation (3) of E_0, E_1 */
  const unsigned char *obs_camera;
} orc_rig;

/* LM damping policy: Ceres' LevenbergMarquardtStrategy, or g2o's
 * OptimizationAlgorithmLevenberg (g2o tag 20230223_git) */
enum { ORC_LM_CERES = 0, ORC_LM_G2O = 1 };

typedef struct orc_options {
  int max_num_iterations;
  double function_tolerance, gradient_tolerance, parameter_tolerance;
  double initial_trust_region_radius, max_trust_region_radius, min_trust_region_radius;
  double min_relative_decrease, min_lm_diagonal, max_lm_diagonal;
  int max_num_consecutive_invalid_steps;
  int jacobi_scaling;
  int loss;
  double loss_scale;
  int linear_solver;
  int pcg_criterion;
  int max_linear_solver_iterations, min_linear_solver_iterations;
  double pcg_tolerance, eta;
  int num_threads; /* 0 = OpenMP default */
  int verbose;
  int camera_update; /* ORC_UPDATE_* */
  int lm_policy;     /* ORC_LM_* */
  const orc_rig *rig; /* NULL: BAL cameras (Snavely model); else the rig model */
} orc_options;

typedef struct orc_summary {
  double initial_cost, final_cost;
  int num_iterations, num_successful_steps, num_unsuccessful_steps, num_invalid_steps;
  long long num_linear_solver_iterations;
  int termination_type;   /* 0 convergence, 1 no convergence, 2 failure */
  int termination_reason; /* same codes as gba_termination_reason */
  double final_trust_region_radius, gradient_max_norm;
  int trace_capacity, trace_length;
  double *trace_cost, *trace_radius;
  int *trace_linear_iterations, *trace_successful;
} orc_summary;

void orc_options_init(orc_options *o);

/* Rodrigues rotation in double, same branch as rotation.h:133-199. */
void orc_angle_axis_rotate_point(const double aa[3], const double pt[3], double out[3]);

/* Residual and 2x12 Jacobian of one observation (row-major: row u then v;
 * columns 0..8 camera, 9..11 point), no loss.  Returns 0 when non-finite. */
int orc_residual_jacobian(const double cam[9], const double pt[3], const double uv[2],
                          double r[2], double J[24]);

/* w' = log(exp(dw) exp(w)) in angle-axis form (the g2o camera update). */
void orc_compose_left(const double dw[3], const double w[3], double out[3]);

/* Rig model: residual (measurement - pixel) and the reference's Jacobian of
 * one observation seen by rig camera `cam`; J as orc_residual_jacobian
 * (camera slots: rotation 0-2, translation 3-5, 6-8 zero). */
int orc_rig_residual_jacobian(const double pose[9], const double pt[3], const double uv[2], const orc_rig *rig,
                              int cam, double r[2], double J[24]);
/* T <- exp(xi) T on SE3 (VertexPose::oplusImpl, g2o_types.h:55-60):
 * xi = (rotation dw, translation du); pose = angle-axis (3), translation (3). */
void orc_se3_compose_left(const double dw[3], const double du[3], const double pose[6], double out[6]);
/* backend.cpp:156-187: chi2 threshold doubled (at most max_doublings times)
 * until more than half the observations are inliers; outlier[i] = chi2[i] >
 * final threshold.  Returns the final threshold. */
double orc_window_outliers(const double *chi2, int no, double threshold, int max_doublings, unsigned char *outlier,
                           int *num_inliers, int *num_outliers);

/* Residuals (2*no) and Jacobians (24*no) of every observation in input order
 * (either may be NULL) and the cost 0.5*sum rho(|r|^2).  Returns 0 on a
 * non-finite evaluation. */
int orc_evaluate_ex(const orc_problem *p, int loss, double loss_scale, int camera_update, double *residuals,
                    double *jacobians, double *cost);
int orc_evaluate_rig(const orc_problem *p, const orc_rig *rig, int loss, double loss_scale, double *residuals,
                     double *jacobians, double *cost);
int orc_evaluate(const orc_problem *p, int loss, double loss_scale, double *residuals,
                 double *jacobians, double *cost);

/* One LM linear solve at p->parameters (the iteration-0 Jacobi scaling of
 * that point, radius `radius`): writes delta (parameter units) and the model
 * cost change.  Returns 0 if the linear solve failed. */
int orc_compute_step(const orc_problem *p, const orc_options *o, double radius, double *delta,
                     double *model_cost_change, int *linear_iterations);

/* Full solve; p->parameters updated in place.  Returns 0 on success. */
int orc_solve(const orc_problem *p, const orc_options *o, orc_summary *s);

/* The benchmark configurations' seeded synthetic problems (synth.c): sizes,
 * then the arrays (caller-allocated; parameters = the perturbed initial
 * guess).  config 0-4, `index` selects a window (3) or a request (4).
 * Return 0 on an unknown configuration, a size mismatch or no memory. */
int orc_synth_size(int config, int index, uint64_t seed, int *nc, int *np, int *no);
int orc_synth_generate(int config, int index, uint64_t seed, int nc, int np, int no, int *camera_index,
                       int *point_index, double *observations, double *parameters);

#ifdef __cplusplus
}
#endif
#endif
