/*
 * gba.h — C ABI of the GB300-native bundle-adjustment solver (libgba.so).
 *
 * Drop-in replacement for the Ceres solve in slamplay's
 * backend/slam_ba_simple_g2o_ceres/test_bundle_adjustment_ceres.cpp:58-101
 * (`void SolveBA(BALProblem&)`).  The problem keeps the BALProblem layout of
 * utils/datasets/BALProblem.h:31-119:
 *   parameters  = double[9*nc + 3*np], cameras first (BALProblem.h:80,82);
 *                 camera = [angle-axis(3), translation(3), f, k1, k2]
 *                 (utils/camera/SnavelyReprojectionError.h:55-59), point = xyz;
 *   camera_index, point_index = int32[no] (BALProblem.h:67-69);
 *   observations = double[2*no], interleaved u,v (BALProblem.h:71).
 * One residual block per observation, r = predict(camera, point) - (u, v)
 * (SnavelyReprojectionError.h:42-53), optional Huber loss
 * (test_bundle_adjustment_ceres.cpp:78), additive update of all 9 camera
 * parameters (no manifold, test_bundle_adjustment_ceres.cpp:86).
 *
 * Memory: every pointer in this header is caller-owned HOST memory.  The
 * library copies in, solves on one GPU, and copies `parameters` back in place.
 * Threading: a gba_handle owns one CUDA stream and is used from one host
 * thread at a time.  Every entry point returns a gba_status; the message of
 * the last failure is available from gba_last_error().
 */
#ifndef GBA_H_
#define GBA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBA_ABI_VERSION 1

/* ------------------------------------------------------------------------ */
/* Status codes.  The reference has none: BALProblem prints parse errors and  */
/* carries on (utils/datasets/BALProblem.cpp:60-64, :81-84); Ceres reports    */
/* failures only through Solver::Summary::termination_type.                  */
/* ------------------------------------------------------------------------ */
typedef enum gba_status {
  GBA_OK = 0,
  GBA_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, index out of range */
  GBA_ERR_OUT_OF_MEMORY = 2,    /* device or host allocation failed / footprint too large */
  GBA_ERR_NON_FINITE = 3,       /* NaN/Inf in observations or parameters */
  GBA_ERR_CUDA = 4,             /* CUDA runtime error (message in gba_last_error) */
  GBA_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up */
  GBA_ERR_IO = 6,               /* file could not be opened / parsed */
  GBA_ERR_NO_DEVICE = 7,        /* no CUDA device or the kernels' image cannot load */
  GBA_ERR_QUEUE_FULL = 8,       /* serving: admission refused, queue at capacity */
  GBA_ERR_NOT_FOUND = 9,        /* serving: unknown ticket */
  GBA_ERR_INTERNAL = 10
} gba_status;

/* Ceres::TerminationType equivalents (Solver::Summary::termination_type). */
typedef enum gba_termination {
  GBA_TERMINATION_CONVERGENCE = 0,
  GBA_TERMINATION_NO_CONVERGENCE = 1, /* max_num_iterations reached */
  GBA_TERMINATION_FAILURE = 2         /* evaluation failed / too many invalid steps */
} gba_termination;

/* Which test ended the minimiser (Ceres' Summary::message, as a code). */
typedef enum gba_termination_reason {
  GBA_REASON_NONE = 0,
  GBA_REASON_MAX_ITERATIONS = 1,
  GBA_REASON_FUNCTION_TOLERANCE = 2,
  GBA_REASON_GRADIENT_TOLERANCE = 3,
  GBA_REASON_PARAMETER_TOLERANCE = 4,
  GBA_REASON_MIN_TRUST_REGION_RADIUS = 5,
  GBA_REASON_INVALID_STEPS = 6,
  GBA_REASON_EVALUATION_FAILED = 7,
  GBA_REASON_LM_TRIALS = 8 /* GBA_LM_POLICY_G2O: the damping trials of one
                              iteration ran out, or a trial left the cost
                              exactly unchanged                              */
} gba_termination_reason;

typedef enum gba_loss {
  GBA_LOSS_TRIVIAL = 0, /* rho(s) = s                       (no LossFunction)     */
  GBA_LOSS_HUBER = 1,   /* ceres::HuberLoss(a), test_bundle_adjustment_ceres.cpp:78 */
  GBA_LOSS_CAUCHY = 2   /* ceres::CauchyLoss(a), backend/ceres/test_ceres_bundle_adjuster_simple.cpp:192-193 */
} gba_loss;

typedef enum gba_precision {
  GBA_PRECISION_FP64 = 0,  /* plain: every kernel in FP64 */
  GBA_PRECISION_MIXED = 1  /* FP32 Jacobians / Schur products / PCG mat-vecs with
                              compensated sums; FP64 cost, step ratio, dots, norms
                              and the 3x3 / 9x9 block inverses */
} gba_precision;

typedef enum gba_pcg_criterion {
  GBA_PCG_RESIDUAL = 0,        /* stop when |r_k| <= pcg_tolerance * |r_0|          */
  GBA_PCG_QUADRATIC_MODEL = 1  /* Ceres ITERATIVE_SCHUR's eta (Nash-Sofer) test    */
} gba_pcg_criterion;

/* How the PCG applies the reduced camera matrix S = B + D^2 - W C^-1 W^T
 * (Ceres' Solver::Options::use_explicit_schur_complement). */
typedef enum gba_schur {
  GBA_SCHUR_AUTO = 0,     /* explicit when the co-visible observation pairs are
                             at most 16 per observation, else implicit          */
  GBA_SCHUR_IMPLICIT = 1, /* every PCG iteration applies J: no S is formed      */
  GBA_SCHUR_EXPLICIT = 2  /* the camera-camera blocks of S are formed once per LM
                             iteration; each PCG iteration multiplies by them    */
} gba_schur;

/* How an accepted step updates a camera's rotation (the first three camera
 * parameters, angle-axis w).  ADDITIVE is the Ceres reference's
 * (test_bundle_adjustment_ceres.cpp: parameters plus step); SO3_LEFT is the
 * g2o variant's VertexPoseAndIntrinsics::oplusImpl
 * (test_bundle_adjustment_g2o.cpp:84-90): R <- exp(dw) R, the Jacobian's
 * rotation columns taken with respect to dw.  Translation, focal length and
 * distortion are additive in both. */
typedef enum gba_camera_update {
  GBA_CAMERA_UPDATE_ADDITIVE = 0,
  GBA_CAMERA_UPDATE_SO3_LEFT = 1
} gba_camera_update;

/* Camera parameter layout of gba_problem_view::parameters (gba_solve,
 * gba_batch_solve): BALProblem's 9 angle-axis parameters per camera, or its
 * use_quaternions layout of 10 (unit quaternion, translation, f, k1, k2;
 * utils/datasets/BALProblem.cpp:117-138, camera_block_size() == 10 at
 * BALProblem.h:55).  Quaternion cameras are converted to angle-axis for the
 * solve and back afterwards, with the reference's own conversions
 * (utils/geometry/rotation.h:72-131), as BALProblem does on load and write. */
typedef enum gba_camera_layout {
  GBA_CAMERA_ANGLE_AXIS = 0,
  GBA_CAMERA_QUATERNION = 1
} gba_camera_layout;

/* Levenberg-Marquardt damping policy.  CERES: LevenbergMarquardtStrategy
 * (trust-region radius, D^2 = clamp(diag J^T J) / radius, Jacobi scaling,
 * Ceres' termination tests).  G2O: the g2o variant's
 * OptimizationAlgorithmLevenberg (test_bundle_adjustment_g2o.cpp:174-176, g2o
 * tag 20230223_git): lambda I damping of the unscaled normal equations
 * (jacobi_scaling ignored), lambda_0 = 1e-5 max diag(J^T J), gain
 * (chi2 - chi2') / (dx.(lambda dx + b) + 1e-3), accept when it is > 0,
 * lambda *= max(1/3, min(2/3, 1 - (2 rho - 1)^3)) then, else lambda *= nu,
 * nu *= 2; up to 10 trials per iteration; max_num_iterations counts
 * iterations (accepted steps), num_iterations in the summary counts trials;
 * the tolerances and the radius bounds are not used.  final_trust_region_radius
 * reports 1 / lambda. */
typedef enum gba_lm_policy {
  GBA_LM_POLICY_CERES = 0,
  GBA_LM_POLICY_G2O = 1
} gba_lm_policy;

/* ------------------------------------------------------------------------ */
/* Options.  Defaults (gba_options_init) are Ceres 2.2's Solver::Options     */
/* defaults for the fields the reference leaves unset                        */
/* (test_bundle_adjustment_ceres.cpp:96-98), plus the GPU-side knobs.         */
/* ------------------------------------------------------------------------ */
typedef struct gba_options {
  uint32_t abi_version;               /* = GBA_ABI_VERSION                          */
  int32_t max_num_iterations;         /* 50                                          */
  double function_tolerance;          /* 1e-6                                        */
  double gradient_tolerance;          /* 1e-10                                       */
  double parameter_tolerance;         /* 1e-8                                        */
  double initial_trust_region_radius; /* 1e4                                         */
  double max_trust_region_radius;     /* 1e16                                        */
  double min_trust_region_radius;     /* 1e-32                                       */
  double min_relative_decrease;       /* 1e-3                                        */
  double min_lm_diagonal;             /* 1e-6                                        */
  double max_lm_diagonal;             /* 1e32                                        */
  int32_t max_num_consecutive_invalid_steps; /* 5                                    */
  int32_t jacobi_scaling;             /* 1                                           */
  int32_t loss;                       /* gba_loss, GBA_LOSS_TRIVIAL                  */
  double loss_scale;                  /* a of Huber/Cauchy, 1.0                      */
  int32_t precision;                  /* gba_precision, GBA_PRECISION_FP64           */
  int32_t pcg_criterion;              /* gba_pcg_criterion, GBA_PCG_RESIDUAL         */
  int32_t max_linear_solver_iterations; /* PCG cap, 500                              */
  int32_t min_linear_solver_iterations; /* 0                                         */
  double pcg_tolerance;               /* relative residual for GBA_PCG_RESIDUAL, 1e-10 */
  double eta;                         /* forcing term for GBA_PCG_QUADRATIC_MODEL, 0.1 */
  int32_t minimizer_progress_to_stdout; /* 0                                         */
  int32_t device;                     /* CUDA device ordinal, 0                      */
  void *stream;                       /* cudaStream_t to run on; NULL = own stream   */
  int32_t chunk_observations;         /* point-segment tile (obs per CTA), 0 = auto  */
  int32_t reorder_points;             /* 1 = group points by first camera (locality) */
  int32_t use_graphs;                 /* 1 = run the LM loop as one CUDA graph       */
  int32_t pcg_unroll;                 /* PCG iterations per graph body, 0 = auto (2) */
  int32_t autotune;                   /* 1 = run gba_autotune on the first solve of a
                                         new problem-size bucket                     */
  int32_t schur;                      /* gba_schur, GBA_SCHUR_AUTO                   */
  int32_t persistent_pcg;             /* 1 = with the explicit Schur complement, run
                                         the whole PCG of an LM iteration in one
                                         launch where the form allows: the mixed
                                         precision as a thread-block cluster per
                                         problem, the FP64 form of a single problem
                                         over the whole GPU (grid-wide barriers; it
                                         expects the GPU to itself: beside other
                                         kernels it runs on the SMs it finds free,
                                         correct but slower; the server's slots
                                         keep the two-kernel FP64 PCG);
                                         0 = one launch pair per PCG iteration      */
  int32_t camera_update;              /* gba_camera_update, GBA_CAMERA_UPDATE_ADDITIVE */
  int32_t lm_policy;                  /* gba_lm_policy, GBA_LM_POLICY_CERES          */
  int32_t camera_layout;              /* gba_camera_layout, GBA_CAMERA_ANGLE_AXIS    */
  int32_t server_slots;               /* serving: cohorts solved concurrently (engine
                                         slots, one stream each), 1..16, 0 = 8     */
} gba_options;

/* Per-solve report, the subset of ceres::Solver::Summary the reference
 * prints with FullReport() (test_bundle_adjustment_ceres.cpp:101). */
typedef struct gba_summary {
  double initial_cost;            /* 0.5 * sum rho(|r|^2) at the start            */
  double final_cost;              /* cost at the returned parameters              */
  int32_t num_iterations;         /* LM iterations after iteration 0              */
  int32_t num_successful_steps;
  int32_t num_unsuccessful_steps;
  int32_t num_invalid_steps;
  int64_t num_linear_solver_iterations; /* PCG iterations, summed                 */
  int32_t termination_type;       /* gba_termination                              */
  int32_t termination_reason;     /* gba_termination_reason                       */
  double final_trust_region_radius;
  double gradient_max_norm;       /* at the returned parameters                   */
  double setup_time_s;            /* host prep + H2D + device setup               */
  double solve_time_s;            /* device LM loop (CUDA events); for a served
                                     request, as total_time_s                    */
  double total_time_s;            /* wall time of the call; for a served request,
                                     from admission to delivery                  */
  /* Optional per-iteration trace, caller-allocated; may be NULL.  Entry k is
   * iteration k (0 = initial point): cost, trust radius, PCG iterations and
   * step_is_successful, as in Ceres' IterationSummary. */
  int32_t trace_capacity;
  int32_t trace_length;
  double *trace_cost;
  double *trace_radius;
  int32_t *trace_linear_iterations;
  int32_t *trace_successful;
} gba_summary;

/* A problem in the BALProblem layout (see header comment). */
typedef struct gba_problem_view {
  int32_t num_cameras;
  int32_t num_points;
  int32_t num_observations;
  const int32_t *camera_index;  /* [num_observations]                 */
  const int32_t *point_index;   /* [num_observations]                 */
  const double *observations;   /* [2 * num_observations] u,v         */
  double *parameters;           /* [9*num_cameras + 3*num_points] in/out */
} gba_problem_view;

typedef struct gba_handle gba_handle;

/* ---- lifecycle --------------------------------------------------------- */
/* Fills `o` with the defaults listed in gba_options. */
void gba_options_init(gba_options *o);
/* Creates a solver bound to o->device.  Fails with GBA_ERR_NO_DEVICE when no
 * GPU is present or the sm_103a kernels cannot load. */
gba_status gba_create(const gba_options *o, gba_handle **out);
void gba_destroy(gba_handle *h);
/* Message of the last failure on `h` (or of the last failed gba_create when
 * h == NULL).  Valid until the next call on the same handle. */
const char *gba_last_error(const gba_handle *h);
/* Version string "gba <abi> sm_103a". */
const char *gba_version(void);

/* ---- solving ----------------------------------------------------------- */
/* Replaces ceres::Solve(options, &problem, &summary) as called at
 * test_bundle_adjustment_ceres.cpp:100 for the problem built at :70-87.
 * p->parameters is updated in place with the best accepted iterate. */
gba_status gba_solve(gba_handle *h, const gba_problem_view *p, gba_summary *s);

/* Solves `n` independent problems together: one work list over all
 * (problem, point-segment) tiles, one LM iteration per graph launch, each
 * problem with its own trust region and termination.  summaries[i] may be
 * NULL-filled (pass summaries == NULL to skip reports). */
gba_status gba_batch_solve(gba_handle *h, const gba_problem_view *problems, int32_t n,
                           gba_summary *summaries);

/* ---- local bundle adjustment (full_slam's backend) --------------------- */
/* The problem Backend::Optimize (full_slam/src/backend.cpp:67-199) hands to
 * g2o: the active keyframes' poses, the active landmarks and one edge per
 * feature, seen by the left or right camera of a stereo rig (EdgeProjection,
 * full_slam/include/myslam/g2o_types.h:127-175):
 *   pos_cam = E_k (T X),  pixel = K pos_cam / z,  error = measurement - pixel,
 * with the reference's analytic Jacobian (the pose columns of a rotation
 * about the rig camera's origin) and the left SE3 update T <- exp(xi) T
 * (VertexPose::oplusImpl, g2o_types.h:55-60).  Poses and extrinsics are
 * angle-axis (3) then translation (3); a pose maps world to body
 * (Frame::Pose(), T_cw), an extrinsic body to camera (Camera::pose()).  The
 * solve uses the handle's options (full_slam: gba_local_ba_options_init);
 * its tolerances, loss, LM policy and precision apply as in gba_solve, and
 * camera_update does not (the pose moves on SE3).  After the solve, the
 * outlier test of backend.cpp:156-187 runs on chi2 = |error|^2 at the
 * returned estimate: the threshold starts at chi2_threshold and doubles, at
 * most max_threshold_doublings times, until more than half the edges are
 * inliers. */
typedef struct gba_rig {
  double fx, fy, cx, cy;   /* K shared by both cameras (backend.cpp:99)     */
  double extrinsic[2][6];  /* E_0 (left), E_1 (right): angle-axis, translation */
} gba_rig;

typedef struct gba_window_view {
  int32_t num_keyframes;
  int32_t num_landmarks;
  int32_t num_observations;
  const int32_t *keyframe_index;  /* [num_observations]                       */
  const int32_t *landmark_index;  /* [num_observations]                       */
  const uint8_t *rig_camera;      /* [num_observations] 0 left image, 1 right  */
  const double *observations;     /* [2 * num_observations] pixel u, v        */
  double *poses;                  /* [6 * num_keyframes] in/out               */
  double *landmarks;              /* [3 * num_landmarks] in/out               */
  gba_rig rig;
  double chi2_threshold;          /* 5.991 (backend.cpp:104)                  */
  int32_t max_threshold_doublings;/* 5 (backend.cpp:161)                      */
  uint8_t *outlier;               /* [num_observations] out: 1 = outlier; may be NULL */
} gba_window_view;

typedef struct gba_window_result {
  int32_t num_inliers, num_outliers;  /* of the threshold loop's last pass   */
  double chi2_threshold;              /* the final threshold                 */
} gba_window_result;

/* Options of full_slam's local BA: g2o's Levenberg, 10 iterations
 * (backend.cpp:152), Huber with delta 5.991 (backend.cpp:137-139), no
 * tolerance tests. */
void gba_local_ba_options_init(gba_options *o);
/* Window defaults: chi2_threshold 5.991, max_threshold_doublings 5. */
void gba_window_view_init(gba_window_view *w);
/* Solves `n` windows as one batch (each with its own LM state); results may
 * be NULL, summaries may be NULL. */
gba_status gba_local_ba(gba_handle *h, gba_window_view *windows, int32_t n, gba_summary *summaries,
                        gba_window_result *results);

/* ---- serving (continuous batching) ------------------------------------- */
/* Starts the serving loop on the handle: problems submitted with gba_submit
 * are admitted while their estimated device footprint fits in
 * `device_budget_bytes` (0 = 90% of free memory) and at most `max_live`
 * solves are on the device at once; live solves advance one LM iteration
 * per step, finished ones free their slot immediately. */
gba_status gba_server_start(gba_handle *h, size_t device_budget_bytes, int32_t max_live,
                            int32_t max_queue);
/* Queues a solve.  The view's arrays must stay valid until gba_poll reports
 * it done; parameters are written back in place then. */
gba_status gba_submit(gba_handle *h, const gba_problem_view *p, uint64_t *ticket);
/* done = 1 when the ticket's solve finished (summary filled, ticket freed). */
gba_status gba_poll(gba_handle *h, uint64_t ticket, gba_summary *s, int32_t *done);
/* Blocks until every submitted problem is done, then stops the loop. */
gba_status gba_server_stop(gba_handle *h);

typedef struct gba_server_stats {
  int64_t submitted, admitted, completed, rejected;
  int32_t live, queued, peak_live;
  int64_t steps;                 /* batched LM iterations run */
  size_t device_bytes_in_use, device_bytes_peak;
  int64_t reforms;               /* cohorts re-formed at an LM-iteration boundary
                                    (finished members out, queued requests in) */
  double host_prep_s;            /* host time laying out and uploading cohorts, on
                                    worker threads beside the serving loop      */
} gba_server_stats;
gba_status gba_server_get_stats(gba_handle *h, gba_server_stats *st);

/* Estimated device footprint of one problem in bytes (the admission rule). */
size_t gba_estimate_footprint(int32_t num_cameras, int32_t num_points, int32_t num_observations,
                              int32_t precision);

/* ---- kernel-level entry points (parity tests, profiling) --------------- */
/* Evaluates residuals and Jacobians on the GPU at p->parameters, in the
 * original observation order: residuals[2*i+k] and jacobians[24*i + 12*k + j]
 * (row k = u,v; columns 0..8 camera, 9..11 point), as
 * ceres::AutoDiffCostFunction<SnavelyReprojectionError,2,9,3>
 * (utils/camera/SnavelyReprojectionError.h:89-92) would produce before the
 * loss.  cost = 0.5 * sum rho(|r_i|^2) with the handle's loss.  Either
 * output pointer may be NULL. */
gba_status gba_evaluate(gba_handle *h, const gba_problem_view *p, double *residuals,
                        double *jacobians, double *cost);

/* One LM linear solve at p->parameters with trust radius `radius` and the
 * Jacobi scaling of that point: writes the parameter update delta
 * (9*nc+3*np, in parameter units) that Ceres' LevenbergMarquardtStrategy +
 * Schur solver would produce, and the model cost change.  pcg_iterations may
 * be NULL. */
gba_status gba_compute_step(gba_handle *h, const gba_problem_view *p, double radius,
                            double *delta, double *model_cost_change, int32_t *pcg_iterations);

/* Re-runs the problem (or batch) last solved on this handle `repeats` times
 * from its uploaded initial point, entirely on the device: no host prep and
 * no transfers, results stay in device memory.  Asynchronous on the handle's
 * stream (gba_options.stream when given).  For benchmarks with inputs
 * resident in HBM; no counterpart in the reference. */
gba_status gba_solve_resident(gba_handle *h, int32_t repeats);
/* Waits for all work queued on the handle's stream. */
gba_status gba_synchronize(gba_handle *h);

/* ---- autotuner ------------------------------------------------------------
 * Times short trial solves of the given problem(s) on a scratch engine and
 * sets the fastest choices on the handle (later solves use them), one knob
 * after another:
 *  1. launch shapes (3 LM iterations, tolerances off, PCG capped at 20
 *     iterations): the point-segment tile, i.e. the observations (and so
 *     the warps, 32 observations a warp) that one CTA of the point kernels
 *     takes (256, 192, 128), x PCG iterations per graph body (1, 2, 4; one
 *     value when the PCG runs as one launch);
 *  2. with the cluster PCG (mixed form, explicit Schur complement): the
 *     cameras of a problem that one CTA of its cluster takes (16, 32, 64);
 *     with the grid PCG (FP64 form, one problem): its CTAs (every SM, 3/4,
 *     1/2, 1/4 of them; the result does not depend on the count);
 *  3. only when the handle's options.autotune is 2: the PCG iteration cap
 *     (5 LM iterations at the handle's PCG tolerance): the configured cap
 *     and its halvings down to 10; a smaller cap is taken only when its
 *     trial ends within 1e-6 relative of the configured cap's cost, and
 *     then the fastest such one.
 * Steps 1-2 change which thread adds which partial sum, never what is
 * solved; step 3 changes how far each linear solve goes.  The problems are
 * not modified.  Results are cached per size bucket (number of problems,
 * log2 of observations and cameras, precision) for the process.  No
 * counterpart in the reference (Ceres has no launch shapes to tune). */
#define GBA_TUNE_MAX_TRIALS 32
typedef struct gba_tune_result {
  int32_t chunk_observations; /* chosen tile size                           */
  int32_t pcg_unroll;         /* chosen PCG iterations per graph body       */
  int32_t num_trials;         /* 0 when the answer came from the cache      */
  int32_t from_cache;
  double best_ms;             /* device time of the chosen launch-shape trial */
  int32_t pcg_cameras_per_cta; /* chosen cameras per CTA of the cluster PCG
                                  (0: not a cluster PCG, defaults kept)     */
  int32_t pcg_cap;            /* chosen PCG iteration cap (0: not tuned)    */
  int32_t pcg_grid_ctas;      /* chosen CTAs of the grid PCG (0: not a grid
                                 PCG, every SM kept)                        */
  int32_t reserved_;
  double trial_ms[GBA_TUNE_MAX_TRIALS];
  int32_t trial_step[GBA_TUNE_MAX_TRIALS];   /* 1, 2 or 3 (the knob above) */
  int32_t trial_chunk[GBA_TUNE_MAX_TRIALS];
  int32_t trial_unroll[GBA_TUNE_MAX_TRIALS];
  int32_t trial_cameras_per_cta[GBA_TUNE_MAX_TRIALS];
  int32_t trial_cap[GBA_TUNE_MAX_TRIALS];
  int32_t trial_grid_ctas[GBA_TUNE_MAX_TRIALS];
  double trial_final_cost[GBA_TUNE_MAX_TRIALS];
} gba_tune_result;
gba_status gba_autotune(gba_handle *h, const gba_problem_view *problems, int32_t num_problems,
                        gba_tune_result *result);

/* ---- allocation-free evaluation ----------------------------------------- */
/* A problem whose arrays are already in DEVICE memory (BALProblem layout,
 * cameras and points in separate arrays). */
typedef struct gba_device_problem {
  int32_t num_cameras;
  int32_t num_points;
  int32_t num_observations;
  const int32_t *camera_index;  /* device, [num_observations]     */
  const int32_t *point_index;   /* device, [num_observations]     */
  const double *observations;   /* device, [2 * num_observations] */
  const double *cameras;        /* device, [9 * num_cameras]      */
  const double *points;         /* device, [3 * num_points]       */
} gba_device_problem;

/* Residuals (device, 2 per observation, may be NULL) and cost (device, one
 * double) of a device-resident problem, computed without allocating any
 * memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc — real-time tracking threads that must not take
 * cudaMalloc's implicit device synchronisation and unbounded latency, hosts
 * that own every device byte through their own pool.  Scratch lives in a
 * fixed file-scope device array (~6.3 MB, held by every GPU that loads the
 * library until exit); at most 16384 cameras and 16777216 observations per
 * call, larger problems are rejected with GBA_ERR_INVALID_ARGUMENT.  The
 * first call on a device sets up the array's address for that device (make
 * it before any stream capture).  Calls share the array: calls that overlap
 * on the GPU race.  The array's address is looked up once per device and
 * kept for the life of the process: do not call this after a
 * cudaDeviceReset of that device.  Asynchronous on `stream` (a
 * cudaStream_t, NULL = the default stream); errors via gba_last_error(NULL). */
gba_status gba_evaluate_noalloc(const gba_device_problem *p, int32_t loss, double loss_scale,
                                double *residuals, double *cost, void *stream);

/* Per-kernel device times of the last gba_solve / gba_batch_solve when
 * profiling is on: kernel names, launches and total milliseconds. */
gba_status gba_set_profiling(gba_handle *h, int32_t on);
int32_t gba_profile_count(const gba_handle *h);
gba_status gba_profile_entry(const gba_handle *h, int32_t i, const char **name,
                             int64_t *launches, double *total_ms, double *bytes);

/* ---- BALProblem I/O and preparation (host only, no GPU needed) --------- */
/* Header of a BAL text file (BALProblem.cpp:87-89). */
gba_status gba_bal_read_header(const char *path, int32_t *nc, int32_t *np, int32_t *no);
/* Reads the body into caller-allocated arrays sized from the header
 * (BALProblem.cpp:78-114). */
gba_status gba_bal_read(const char *path, const gba_problem_view *out);
/* Writes a BAL text file as BALProblem::WriteToFile (BALProblem.cpp:141-183). */
gba_status gba_bal_write(const char *path, const gba_problem_view *p);
/* Writes camera centres + points as BALProblem::WriteToPLYFile (BALProblem.cpp:185-228). */
gba_status gba_bal_write_ply(const char *path, const gba_problem_view *p);
/* BALProblem::Normalize (BALProblem.cpp:263-303). */
gba_status gba_bal_normalize(const gba_problem_view *p);
/* BALProblem::Perturb (BALProblem.cpp:305-336).  seed == 0 draws from the C
 * library's rand() exactly as the reference does; otherwise a private
 * generator seeded with `seed` is used. */
gba_status gba_bal_perturb(const gba_problem_view *p, double rotation_sigma,
                           double translation_sigma, double point_sigma, uint64_t seed);
/* Angle-axis <-> quaternion (utils/geometry/rotation.h:73-131), for the
 * BALProblem use_quaternions layout (BALProblem.cpp:117-138). */
void gba_angle_axis_to_quaternion(const double *angle_axis, double *quaternion);
void gba_quaternion_to_angle_axis(const double *quaternion, double *angle_axis);
/* Rodrigues rotation R(w)*pt with the reference's small-angle branch
 * (utils/geometry/rotation.h:133-199). */
void gba_angle_axis_rotate_point(const double *angle_axis, const double *pt, double *result);

/* ---- synthetic problems (seeded; host only) ---------------------------- */
/* Problem families of the benchmark configurations:
 *   GBA_SYNTH_RING     16-camera ring, uniform points, uniform 4..10 views;
 *   GBA_SYNTH_WALK     random-walk trajectory, box of points, geometric views;
 *   GBA_SYNTH_LOOPS    several random-walk loops with coincident starts, Zipf views;
 *   GBA_SYNTH_WINDOW   short random-walk segment (local-BA window), uniform views. */
typedef enum gba_synth_layout {
  GBA_SYNTH_RING = 0,
  GBA_SYNTH_WALK = 1,
  GBA_SYNTH_LOOPS = 2,
  GBA_SYNTH_WINDOW = 3
} gba_synth_layout;

typedef struct gba_synth_spec {
  int32_t layout;           /* gba_synth_layout                         */
  int32_t num_cameras;
  int32_t num_points;
  int32_t min_views, max_views;
  int32_t view_distribution; /* 0 uniform, 1 geometric tail, 2 Zipf     */
  double view_param;         /* p of the geometric tail / s of Zipf     */
  double focal;              /* 500                                     */
  double k1_range, k2_range; /* 0.05, 0.005                             */
  double pixel_noise;        /* 0.5 px                                  */
  double rotation_noise;     /* 0.01 rad                                */
  double translation_noise;  /* 0.1                                     */
  double point_noise;        /* 0.1                                     */
  double focal_noise;        /* 0.01 (relative)                         */
  uint64_t seed;
} gba_synth_spec;

/* Fills `spec` for benchmark configuration 0, 1 or 2 (single problems) or,
 * for config 3, problem `index` of the 1,024-window batch, and for config 4
 * request `index` of the serving stream. */
gba_status gba_synth_preset(int32_t config, int32_t index, uint64_t seed, gba_synth_spec *spec);
/* Sizes of the problem `spec` generates. */
gba_status gba_synth_size(const gba_synth_spec *spec, int32_t *nc, int32_t *np, int32_t *no);
/* Generates it into caller-allocated arrays: observations are projections of
 * the true scene plus pixel noise; parameters hold the perturbed initial
 * guess; `truth` (may be NULL) receives the true parameters. */
gba_status gba_synth_generate(const gba_synth_spec *spec, const gba_problem_view *out,
                              double *truth);

#ifdef __cplusplus
}
#endif

#endif /* GBA_H_ */
