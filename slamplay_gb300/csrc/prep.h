// prep.h — host-side preparation of a batch of BAL problems into the
// device layout (observation orderings, point-segment chunks, camera
// segments).  Pure host code, testable without a GPU.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "gba_internal.h"

namespace gba {

struct PrepOptions {
  int chunk_cap = kChunkCap;  // observations per chunk (CTA)
  bool reorder_points = true; // group points by their first camera
  int schur = GBA_SCHUR_AUTO; // gba_schur: whether the batch forms S explicitly
};

struct HostBatch {
  int P = 0, nc = 0, np = 0, no = 0, nchunks = 0, nseg = 0, cam_blocks = 0;
  std::vector<ProblemInfo> prob;
  std::vector<ChunkInfo> chunk;
  std::vector<int32_t> obs_cam, obs_pt;
  std::vector<double> obs_uv;  // 2 per observation
  std::vector<uint16_t> obs_seg, obs_slot;
  std::vector<int32_t> pt_obs_begin, pt_problem, cam_problem;
  std::vector<uint8_t> pt_used, cam_used;
  std::vector<uint16_t> seg_pos;
  std::vector<int32_t> seg_cam;
  std::vector<int32_t> cam_seg_begin, seg_slot, cam_obs_begin, cam_obs_list;
  std::vector<int32_t> cam_piece_begin;  // nc + 1: pieces of kCamPieceObs of each camera's list
  std::vector<int4> camblk;
  // explicit Schur complement (explicit_schur): the off-diagonal camera-camera
  // blocks of S by row camera (CSR over the batch's cameras; a block with
  // the row's own camera holds the cross terms of a camera that observes a
  // point more than once) and each block's transpose; the blocks on and
  // above the diagonal (sblk_up) with their observation pairs (row camera's,
  // column camera's) of the points both see, in point order
  bool explicit_schur = false;
  long long nblk = 0, nup = 0, npairs = 0;
  std::vector<int32_t> sblk_row, sblk_col, sblk_tr, sblk_up, sblk_pair;
  std::vector<int32_t> spair;     // 2 per pair: camera-major positions (obs_fpos)
  std::vector<int32_t> obs_fpos;  // observation -> its position in cam_obs_list
  // output mapping
  std::vector<int32_t> obs_orig;  // internal observation -> index in its problem's input
  std::vector<int32_t> pt_orig;   // internal point -> point index in its problem's input
  // initial parameters in the internal layout
  std::vector<double> cam_param;  // 9 per camera
  std::vector<double> pt_param;   // 4 per point
  // local-BA windows (empty otherwise): the rig camera of each internal
  // observation, and per problem fx, fy, cx, cy, then (R, t) of E_0 and E_1
  std::vector<uint8_t> obs_rig;
  std::vector<double> prob_rig;   // kRig per problem
  // resumed problems (set_resume; empty when none): per problem a flag and
  // the LM state to continue from, the Jacobi scales in the internal layout
  std::vector<int32_t> resume;
  std::vector<LMState> resume_lm;
  std::vector<double> resume_cam_scale;  // 9 per camera
  std::vector<double> resume_pt_scale;   // 3 per point
  // Starts a new batch: counts, offsets and appended arrays emptied; the
  // arrays prepare_batch overwrites entirely keep their size and storage (a
  // handle re-preparing problems of similar size neither touches fresh
  // pages nor re-zeroes them).
  void reset();
};

// The host thread pool of the prep (and of other host-side data-parallel
// copies): fn(task) for task in [0, ntasks), on the pool's threads and the
// caller's; fn must write disjoint outputs per task.  Runs on the calling
// thread alone when the pool is busy.
int host_threads();
void host_parallel(int ntasks, const std::function<void(int)> &fn);

// Validates and lays out `n` problems.  Returns GBA_OK or an error with a
// message in *err.
gba_status prepare_batch(const gba_problem_view *views, int n, const PrepOptions &opt, HostBatch *out,
                         std::string *err);

// Checks one problem view (sizes, pointers, indices, finiteness).
gba_status validate_problem(const gba_problem_view *v, std::string *err);

// The state of a problem at an LM-iteration boundary, enough to continue its
// solve in another batch with the same bits: the LM state and the Jacobi
// scales of its first evaluation (user order: 9 per camera, 3 per point);
// its current parameters are the problem view's.
struct ProblemState {
  LMState lm;
  std::vector<double> cam_scale, pt_scale;
};
// Marks problem p of a prepared batch as resumed from `st`.
void set_resume(HostBatch &hb, int p, const ProblemState &st);
// Maps the internal-layout scales of problem p to user order.
void gather_scales(const HostBatch &hb, int p, const double *cam_scale, const double *pt_scale, ProblemState *st);

// Writes the internal-layout parameters of problem p back to the caller's array.
void scatter_parameters(const HostBatch &hb, int p, const double *cam_param, const double *pt_param,
                        double *out);

}  // namespace gba
