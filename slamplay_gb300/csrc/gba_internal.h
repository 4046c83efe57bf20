// gba_internal.h — definitions shared by the host library and the CUDA
// kernels of libgba (not part of the public ABI).
#pragma once

#include <cstddef>
#include <cstdint>

#include <vector_types.h>

#include "gba.h"

namespace gba {

// Point-segment tile: one CTA of the chunk kernels processes one chunk, one
// thread per observation.  A chunk is a run of consecutive points (in the
// internal point order) whose observations fit in kChunkCap.
constexpr int kChunkCap = 256;
constexpr int kCamPieceObs = 256;  // observations of one piece of a camera's list (FP64 K1c)

// Per-chunk metadata (all indices global over the batch).
struct ChunkInfo {
  int32_t obs_begin;
  int32_t obs_count;
  int32_t pt_begin;
  int32_t pt_count;
  int32_t seg_begin;  // first camera segment of this chunk
  int32_t seg_count;  // number of distinct cameras observed in this chunk
  int32_t problem;
  int32_t pad;
};

// Per-problem ranges inside the batch arrays.
struct ProblemInfo {
  int32_t cam_begin, cam_count;
  int32_t pt_begin, pt_count;
  int32_t obs_begin, obs_count;
  int32_t chunk_begin, chunk_count;
  int32_t seg_begin, seg_count;
  int32_t cam_block_begin, cam_block_count;  // camera-kernel CTAs of this problem
};

// Solver options as the kernels need them (copied from gba_options).
struct DeviceOptions {
  double function_tolerance, gradient_tolerance, parameter_tolerance;
  double initial_radius, max_radius, min_radius, min_relative_decrease;
  double min_diagonal, max_diagonal;
  double loss_scale;
  double pcg_tolerance, eta;
  int32_t max_iterations, max_invalid_steps, jacobi_scaling, loss;
  int32_t pcg_criterion, max_pcg_iterations, min_pcg_iterations, mixed;
  int32_t so3_left;  // camera rotation update R <- exp(dw) R (else additive)
  int32_t g2o;       // g2o's Levenberg policy (else Ceres' trust region)
  int32_t max_bodies;  // LM bodies (trials) a solve may run
  int32_t pinhole;     // local-BA windows: the stereo-rig pinhole model, SE3 poses
  int32_t bodies_cap;  // > 0: the LM loop of one launch stops after this many counted bodies
  int32_t grid_wait_test;  // failure test of the grid PCG (environment GBA_TEST_GRID_WAIT=1 at
                           // handle creation): every barrier waits for one CTA more than
                           // registered, so its bounded wait runs out (GBA_ERR_TIMEOUT)
                       // (the problems stay active; a later launch continues them)
};

// Per problem of a local-BA batch: fx, fy, cx, cy, then R (9, row-major) and
// t (3) of the rig's two extrinsics.
constexpr int kRig = 28;

// g2o's OptimizationAlgorithmLevenberg constants: lambda_0 = tau max diag(H),
// at most this many damping trials per iteration.
constexpr double kG2oTau = 1e-5;
constexpr int kG2oMaxTrials = 10;

// LM / trust-region state of one problem, resident on the device.
// Follows Ceres' TrustRegionMinimizer + LevenbergMarquardtStrategy.
struct LMState {
  double radius;
  double decrease_factor;
  double x_cost;           // cost at the current point
  double x_norm;           // |x| over parameter blocks that appear in a residual
  double gradient_max_norm;
  double candidate_cost;
  double model_cost_change;
  double step_norm;
  double minimum_cost;
  double relative_decrease;
  double initial_cost;
  // PCG scalars
  double rz, pq, alpha, beta, r0_norm, rr, q0;
  int32_t iteration;       // LM iteration index (0 = initial point)
  int32_t active;          // 1 while the problem is still iterating
  int32_t need_jacobian;   // 1 after an accepted step
  int32_t parity;          // which parameter buffer holds the current point
  int32_t termination_type, termination_reason;
  int32_t successful_steps, unsuccessful_steps, invalid_steps, invalid_run;
  int32_t pcg_active, pcg_iterations, linear_ok, last_linear_ok;
  int32_t trials, outer;  // g2o policy: trials of this iteration, iterations done
  int32_t resumed;        // 1 from a resumed upload until its first evaluation
  int32_t pad_;
  int64_t total_pcg_iterations;
};

// Everything a kernel may touch, as raw device pointers.  Built by the host
// (solver.cpp) and passed by value to every launch.
struct DeviceBatch {
  int32_t num_problems, nc, np, no, nchunks, nseg;
  int32_t cam_blocks;        // camera blocks of the PCG camera kernel (kPcgBlockCams cameras each)
  const ProblemInfo *prob;
  const ChunkInfo *chunk;
  // observations, internal (point-major) order
  const int32_t *obs_cam;    // global camera
  const int32_t *obs_pt;     // global internal point
  const double2 *obs_uv;
  const uint8_t *obs_rig;    // local-BA windows: rig camera of each observation
  const double *prob_rig;    // local-BA windows: kRig per problem
  double *obs_chi2;          // local-BA windows: |error|^2 at the returned estimate
  const uint16_t *obs_seg;   // local camera-segment index inside its chunk
  const uint16_t *obs_slot;  // position in the chunk's camera-sorted order
  const int32_t *pt_obs_begin;  // np + 1
  const int32_t *pt_problem;
  const int32_t *cam_problem;
  const uint8_t *pt_used, *cam_used;
  const uint16_t *seg_pos;   // start (sorted position) of each segment in its chunk
  const int32_t *seg_cam;
  const int32_t *cam_seg_begin;  // nc + 1: each camera's run of partials (camera-major)
  const int32_t *seg_slot;       // camera-major position of each segment's partial
  const int32_t *cam_obs_begin, *cam_obs_list;
  // the FP64 camera kernel's pieces: camera c's observation list in pieces
  // of kCamPieceObs, pieces [cam_piece_begin[c], cam_piece_begin[c + 1]);
  // per piece its 54 sums, per camera the count of its pieces done
  const int32_t *cam_piece_begin;
  int32_t npieces;
  double *piece_part;
  uint32_t *cam_counter;
  // parameters: the uploaded initial point, and two working buffers of
  // which LMState::parity picks the current one
  const double *cam_init;    // nc * 9
  const double *pt_init;     // np * 4 (xyz + pad)
  double *cam_param[2];      // nc * 9
  double *pt_param[2];       // np * 4
  double *cam_table;         // nc * kCamTable: R, dR/dw, t, f, k1, k2 of one buffer
  float *cam_tablef;         // nc * kCamTable: FP32 copy for the mixed-form Jacobian
  float2 *cam_tabledf;       // nc * kCamTable: double-float copy (mixed form: the gradient's Jacobian)
  // Jacobian (scaled, loss-corrected), SoA by column pair; element type by mode
  void *jac;                 // 13 * no of double2 (FP64) or float2 (mixed)
  // per point
  double *pt_C;              // 6 sym (J_p^T J_p)
  double *pt_g;              // 3
  double *pt_scale;          // 3
  float *pt_scalef;          // 3, FP32 copy
  float2 *pt_scaledf;        // 3, double-float copy
  double *pt_t;              // 3: Cinv g_p
  void *pt_Cinv;             // 6 sym, double (FP64) or float (mixed)
  double *pt_Cinv64;         // 6 sym, double (both modes, for the back-substitution)
  // per camera
  double *cam_B;             // 45 sym packed (J_c^T J_c)
  double *cam_g;             // 9
  double *cam_scale;         // 9
  float *cam_scalef;         // 9, FP32 copy
  float2 *cam_scaledf;       // 9, double-float copy
  double *cam_Minv;          // 81 block-Jacobi inverse of S_ii
  float *cam_Minvf;          // 81, FP32 copy (mixed form)
  float *cam_Bf;             // 45, FP32 copy of cam_B (mixed form)
  double *cam_D2;            // 9: squared LM diagonal of the camera parameters
  // PCG vectors, 9 * nc each: x, r, z (= M r), p (direction), v (rhs); FP32
  // copies of z and p (the mixed form's mat-vec forms its direction from them)
  double *pcg_x, *pcg_r, *pcg_z, *pcg_p, *pcg_v;
  float *pcg_zf, *pcg_pf;
  double *cam_colnorm;       // 9 * nc: column norms of the first evaluation
  double *pt_colnorm;        // 3 * np
  void *seg_partial;         // 9 * nseg, double (FP64) or float (mixed)
  void *schur_partial;       // 54 * nseg: per segment 45 packed Schur-block and 9 rhs partials
  double *seg_grad;          // 9 * nseg: per segment FP64 J_c^T r (mixed form: the camera gradient)
  // per chunk / per camera / per camera-block scalars (deterministic partials)
  double *chunk_scal;        // kChunkScal per chunk
  double *cam_scal;          // kCamScal per camera
  const int4 *camblk;        // camera blocks: (problem, first camera, count, 0)
  LMState *lm;
  DeviceOptions opt;
  // cross-CTA completion counters (last-block reductions)
  uint32_t *prob_counter;    // 4 per problem
  uint32_t *global_counter;  // 8
  int32_t *status;           // [0] error word, [1] any LM active, [2] any PCG active
  // per-iteration trace, [num_problems][trace_cap]
  int32_t trace_cap;
  double *trace_cost, *trace_radius;
  int32_t *trace_pcg, *trace_succ;
  // graph conditional handles (0 when the host drives the loops)
  unsigned long long lm_cond, pcg_cond;
  int32_t use_cond;
  // PCG reductions: per chunk its share of p.q, then per group of kRedGroup
  // chunks ([nchunks + first chunk of the group]); per camera block its
  // r.z, r.r, x.(v + r)
  double *chunk_red;         // 2 * nchunks (mixed form: double-float pairs, hi then lo)
  uint32_t *chunk_counter;   // nchunks (one per group, at its first chunk)
  double *blk_red;           // 3 * cam_blocks
  // explicit Schur complement (explicit_schur != 0): the off-diagonal
  // camera-camera blocks by row camera, each block's transpose, the blocks
  // on and above the diagonal with their observation pairs, per observation
  // F = J_c^T J_p L (L L^T = C^-1 of its point), the blocks' values (9x9
  // row-major, working precision), the diagonal blocks, S p of the current
  // direction, and per camera its share of p.q
  int32_t explicit_schur;
  int32_t nblk, nup;
  long long npairs;
  int32_t sblk_max;          // the most blocks of a row of S (the diagonal one included)
  const int32_t *sblk_row;   // nc + 1
  const int32_t *sblk_col;   // nblk
  const int32_t *sblk_tr;    // nblk
  const int32_t *sblk_up;    // nup: block index
  const int32_t *sblk_pair;  // nup + 1
  const int2 *spair;         // npairs: (row camera's, column camera's observation), F positions
  const int32_t *obs_fpos;   // no: each observation's F row (camera-major order)
  void *obs_F;               // kObsF * no (9x3 row-major + pad), camera-major
  void *sblk_val;            // 81 * nblk
  void *cam_Sii;             // 81 * nc
  double *pcg_q;             // 9 * nc
  double *spmv_red;          // nc
  // the grid PCG (FP64, one problem): the second direction buffer (the
  // directions alternate between pcg_p and pcg_p2 by iteration parity) and
  // its control words (kGrid* slots), zeroed by K3b before each launch
  double *pcg_p2;            // 9 * nc
  // a resumed batch (a problem continued in a new batch at an LM-iteration
  // boundary): per problem a flag and the LM state to continue from, per
  // camera / point the Jacobi scales of its first evaluation (internal
  // order); all null when no problem of the batch is resumed
  const int32_t *prob_resume;
  const LMState *lm_resume;
  const double *cam_scale_in, *pt_scale_in;
  double *pq_row;            // 9 * nc: each row's p_i q_i, [row of the camera][camera of the problem]
  uint32_t *grid_ctl;        // 8
};

constexpr int kCamTable = 44;    // R(9) dR(27) t(3) f k1 k2 + pad
// chunk_scal slots
constexpr int kChunkScal = 6;
constexpr int kCS_COST = 0, kCS_GMAX = 1, kCS_XN2 = 2, kCS_MODEL = 3, kCS_STEP2 = 4, kCS_BAD = 5;
// cam_scal slots
constexpr int kCamScal = 6;
constexpr int kCC_GMAX = 0, kCC_XN2 = 1, kCC_STEP2 = 2, kCC_RZ = 3, kCC_RR = 4, kCC_YG = 5;
// PCG iterations per body of the graph's PCG loop
constexpr int kPcgUnroll = 2;
// cameras per block of the camera-side PCG kernel
constexpr int kPcgBlockCams = 8;
// p.q of the PCG: problems of up to kRedDirect chunks have their chunk
// values summed by the camera kernel directly, larger ones in groups of
// kRedGroup chunks first
constexpr int kRedDirect = 2048;
constexpr int kRedGroup = 64;
// explicit Schur complement: chosen automatically up to this many ordered
// observation pairs per observation, and supported up to kExplicitPairsMax
constexpr long long kExplicitPairsPerObs = 16;
constexpr long long kExplicitPairsMax = 1LL << 28;
constexpr int kObsF = 28;  // reals per observation of obs_F (27 + pad: 16-byte rows)
// prob_counter slots (4 per problem) and global_counter slots
constexpr int kPC_SCHUR = 0, kPC_REDUCE = 1, kPC_UPDATE = 2;
constexpr int kGC_SCHUR = 0, kGC_UPDATE = 1, kGC_POST = 2, kGC_LMBODIES = 3;
// status words: [0] error, [1] any LM active, [2] any PCG active, [3] PCG-active problem count
// grid PCG: threads per CTA (16 warps: four per SM sub-partition, so up to
// 128 registers a thread) and the control words: registration (64-bit:
// count, and the closed bit), the published participant count + 1, the
// barrier counter, the abort word
constexpr int kPcgGridThreads = 512;
// chunk sums (32 cameras each) of the explicit FP64 form's p.q in the camera
// kernel: problems of up to 32 * kPcgChunkSums cameras
constexpr int kPcgChunkSums = 1024;
constexpr int kGridReg = 0, kGridCount = 2, kGridBar = 3, kGridAbort = 4;

// A problem without observations has no parameter blocks in the
// reference's problem (each observation adds its camera and point through
// AddResidualBlock, test_bundle_adjustment_ceres.cpp:70-87), and Ceres'
// Solver::Solve returns before the minimizer for such a problem: CONVERGENCE
// ("Function tolerance reached.  No non-constant parameter blocks found."),
// cost 0, no iterations.  The library does the same without touching the
// device; the parameters are left as they are.  The caller's trace buffers
// are kept (no entries).
inline void empty_problem_summary(gba_summary *s, double radius) {
  if (!s) return;
  s->initial_cost = 0.0;
  s->final_cost = 0.0;
  s->num_iterations = 0;
  s->num_successful_steps = 0;
  s->num_unsuccessful_steps = 0;
  s->num_invalid_steps = 0;
  s->num_linear_solver_iterations = 0;
  s->termination_type = GBA_TERMINATION_CONVERGENCE;
  s->termination_reason = GBA_REASON_FUNCTION_TOLERANCE;
  s->final_trust_region_radius = radius;
  s->gradient_max_norm = 0.0;
  s->setup_time_s = 0.0;
  s->solve_time_s = 0.0;
  s->total_time_s = 0.0;
  s->trace_length = 0;
}

}  // namespace gba
