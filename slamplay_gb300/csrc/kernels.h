// kernels.h — host-side launchers of the libgba kernels (one per kernel
// family; the precision mode picks the template instance).
#pragma once

#include <cuda_runtime.h>

#include "gba_internal.h"

namespace gba {

// LM state initialisation (per problem).
void launch_init_state(const DeviceBatch &b, cudaStream_t s);
// K0: camera tables (R, dR/dw, t, f, k1, k2) of the current parameters.
void launch_camera_table(const DeviceBatch &b, cudaStream_t s);
// K1 + K1c: residuals, scaled & corrected Jacobian, point blocks (chunk
// kernel) and camera blocks (camera kernel).  norms = first pass of the
// solve: unscaled column norms only.
void launch_eval_jacobian(const DeviceBatch &b, bool mixed, bool norms, cudaStream_t s);
// Jacobi scaling from the column norms of the first pass.
void launch_scale_init(const DeviceBatch &b, cudaStream_t s);
// K7: per-problem cost / gradient / |x| after a Jacobian evaluation, the
// trust-region termination tests, and the LM loop condition.
void launch_post_eval(const DeviceBatch &b, cudaStream_t s);
// K3a: damped point blocks, their FP64 inverses, Cinv g_p.
void launch_point_prepare(const DeviceBatch &b, bool mixed, cudaStream_t s);
// K3b: camera-diagonal Schur blocks, reduced rhs, block-Jacobi inverse, PCG init.
void launch_camera_schur(const DeviceBatch &b, bool mixed, cudaStream_t s);
// K3c: the off-diagonal camera-camera blocks of the explicit Schur complement.
void launch_schur_form(const DeviceBatch &b, bool mixed, cudaStream_t s);
// K4a': q = S p_k with the explicit complement (launch_schur_matvec calls it
// when the batch forms S).
cudaError_t launch_schur_spmv(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl);
// K4 cluster form: the whole PCG of every problem in one launch, one thread
// block cluster of plan.cs CTAs per problem (mixed form, explicit Schur
// complement, problems of at most kClMaxCams cameras).
constexpr int kClThreads = 512;
constexpr int kClMaxCS = 16;
constexpr int kClMaxOwn = 64;    // cameras per CTA
constexpr int kClMaxCams = 1024; // cameras per problem
struct ClusterPlan {
  int cs = 0, n_max = 0, own_max = 0;
  int threads = 0;
  int cache_blocks = 0;  // > 0: each CTA keeps its rows of S (this many 9x9 blocks at most) in shared memory
  size_t smem = 0;
};
// Chooses the cluster size, the block size and whether the rows of S stay
// in shared memory, from the batch's problems (camera ranges) and the
// explicit complement's row structure (sblk_row, nc + 1); false when the
// form does not apply or cannot be launched.
// cams_per_cta: the cameras of a problem one CTA of its cluster takes (the
// cluster size follows); 0 = 16 for a single problem, 64 for a batch.
bool pcg_cluster_plan(const ProblemInfo *prob, int num_problems, const int32_t *sblk_row, int cams_per_cta,
                      ClusterPlan *plan);
cudaError_t launch_pcg_cluster(const DeviceBatch &b, const ClusterPlan &plan, cudaStream_t s);
// K4 grid form: the whole PCG of one problem in one launch, one CTA per SM
// with grid-wide barriers (FP64 form, explicit Schur complement).
struct GridPlan {
  int grid = 0;        // CTAs launched (the ones that register share the work)
  int cap_blocks = 0;  // blocks of S a CTA's shared-memory layout holds
  int cache_s = 0;     // 1: the blocks' values too (else only the staged direction)
  int cap_pairs = 0;   // (row, block) pairs of one pass of the product
  size_t smem = 0;
};
// Sizes the launch from the problem's explicit-complement rows (sblk_row,
// nc + 1); false when the form does not apply (a batch, the mixed form,
// the implicit complement), when the CTAs' blocks of S would not stay in
// shared memory, or when its kernel cannot be resident.  ctas: the
// CTAs of the launch (one per SM at most; 0 = every SM).
bool pcg_grid_plan(int num_problems, bool mixed, bool explicit_schur, int nc, const int32_t *sblk_row, int ctas,
                   GridPlan *plan);
cudaError_t launch_pcg_grid(const DeviceBatch &b, const GridPlan &plan, cudaStream_t s);
// K4a-b: one PCG iteration (implicit Schur mat-vec, camera-side update).
void launch_pcg_iteration(const DeviceBatch &b, bool mixed, cudaStream_t s);
cudaError_t launch_schur_matvec(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl);
// K4b alone (one CTA per block of kPcgBlockCams cameras).
cudaError_t launch_pcg_camera(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl);
void launch_prof_delay(cudaStream_t s);
void point_schur_init();
// Raises a kernel's dynamic shared memory limit on the current device to at
// least `bytes`, never lowering it: the limit is process-wide, and several
// engines (the serving slots) plan and capture launches of the same kernel
// with different sizes at different times.
cudaError_t raise_smem_limit(const void *func, size_t bytes);
// Kernel attributes of the PCG kernels (once per device).
void pcg_init();
// K5: point back-substitution, model cost change, candidate points.
void launch_back_substitute(const DeviceBatch &b, bool mixed, cudaStream_t s);
// K5b + K2: candidate cameras (+ their tables) and the candidate cost.
void launch_candidate_cost(const DeviceBatch &b, cudaStream_t s);
// K6: accept / reject, trust-region radius update, termination tests.
void launch_decide(const DeviceBatch &b, cudaStream_t s);
// Copies the uploaded initial parameters into both working buffers.
void launch_sync_param_buffers(const DeviceBatch &b, cudaStream_t s);
// Gathers each problem's current parameters (the buffer its parity selects)
// into out_cam (9 per camera) / out_pt (4 per point).
void launch_gather_results(const DeviceBatch &b, double *out_cam, double *out_pt, cudaStream_t s);
// Local-BA windows: camera tables at the gathered estimate, then each
// observation's chi2 = |error|^2 (B.obs_chi2).
void launch_window_chi2(const DeviceBatch &b, const double *out_cam, const double *out_pt, cudaStream_t s);

}  // namespace gba
