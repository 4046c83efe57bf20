// engine.h — one GPU solver instance (behind a gba_handle).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include <string>
#include <vector>

#include "gba_internal.h"
#include "kernels.h"
#include "prep.h"

namespace gba {

struct ProfileEntry {
  std::string name;
  long long launches = 0;
  double total_ms = 0.0;
  double bytes = 0.0;  // algorithmic bytes moved, summed over launches
};

class Engine {
 public:
  explicit Engine(const gba_options &o);
  ~Engine();
  gba_status init(std::string *err);

  gba_status solve(const gba_problem_view *v, int n, gba_summary *s, std::string *err);
  gba_status evaluate(const gba_problem_view *v, double *residuals, double *jacobians, double *cost,
                      std::string *err);
  gba_status compute_step(const gba_problem_view *v, double radius, double *delta, double *model,
                          int *pcg_iterations, std::string *err);
  // Local-BA windows (the rig camera model) solved as one batch, then each
  // window's outlier test.
  gba_status solve_windows(gba_window_view *w, int n, gba_summary *s, gba_window_result *res, std::string *err);

  void set_profiling(bool on) { profiling_ = on; }
  const std::vector<ProfileEntry> &profile() const { return profile_; }
  const gba_options &options() const { return o_; }
  // Launch shapes chosen by the autotuner (takes effect on the next upload).
  // The autotuner's choices: tile size, PCG iterations per graph body, the
  // cameras per CTA of the cluster PCG (0 = default), when > 0 the PCG
  // iteration cap, and the CTAs of the grid PCG (0 = every SM).
  void set_tuning(int chunk_observations, int pcg_unroll, int cluster_cams = 0, int pcg_cap = 0, int grid_ctas = 0);
  bool cluster_pcg() const { return cl_plan_.cs > 0; }
  int grid_pcg_ctas() const { return gr_plan_.grid; }
  bool one_launch_pcg() const { return cl_plan_.cs > 0 || gr_plan_.grid > 0; }
  double last_solve_ms() const { return last_solve_ms_; }
  PrepOptions prep_options() const;
  cudaStream_t stream() const { return stream_; }
  size_t device_bytes() const { return d_cap_; }

  // Prepared-batch level entry points (used by the serving loop).
  gba_status upload(const HostBatch &hb, std::string *err);
  gba_status run_solve(std::string *err);
  // Segment runs (the serving loop): at most `lm_bodies` LM iterations a
  // launch (0 = to the end); run_segment(false) starts the uploaded batch
  // (setup, then the loop), run_segment(true) continues it from the device
  // state.  fetch_states() queues the copy of the problems' LM states to the
  // host staging area, states() reads them once the stream has passed it.
  void set_segment(int lm_bodies) { segment_bodies_ = std::max(0, lm_bodies); }
  gba_status run_segment(bool cont, std::string *err);
  // Builds the continue graph of the uploaded batch ahead of its use (the
  // capture does not wait for the stream).
  gba_status prepare_continue(std::string *err);
  gba_status fetch_states(std::string *err);
  const LMState *states(const HostBatch &hb);
  // The batch's device-side error word as fetched (GBA_OK when clear).
  gba_status device_status(std::string *err);
  // Once the stream has passed a segment: the parameters of problems
  // `probs` into their views (their current point; for a finished problem
  // its result) and, if s, their summaries from the fetched LM states.  The
  // batch stays on the device.
  gba_status deliver(const HostBatch &hb, const std::vector<int> &probs, const gba_problem_view *v, gba_summary *s,
                     std::string *err);
  // Each problem's state for a resumed upload: the fetched LM state and the
  // Jacobi scales in user order.
  gba_status download_states(const HostBatch &hb, std::vector<ProblemState> *out, std::string *err);
  // Re-runs the last uploaded batch from its initial point (device only,
  // asynchronous on the handle's stream).
  gba_status rerun(std::string *err);
  gba_status download(const HostBatch &hb, const gba_problem_view *v, gba_summary *s, std::string *err);

 private:
  gba_status ensure_capacity(size_t dev_bytes, size_t host_bytes, std::string *err);
  size_t layout(const HostBatch &hb, char *dbase, DeviceBatch *db, size_t *upload_bytes,
                size_t *download_off, size_t *download_bytes);
  gba_status build_graph(std::string *err, bool cont = false);
  void summarize(const DeviceBatch &hdb, int p, double solve_s, gba_summary *out);
  void end_captures();
  void enqueue_gather(cudaStream_t s);
  void destroy_graph();
  gba_status run_host_driven(std::string *err);
  gba_status check(cudaError_t e, const char *what, std::string *err);
  void enqueue_setup(cudaStream_t s);
  void zero_counters(cudaStream_t s);
  void enqueue_lm_head(cudaStream_t s);
  void enqueue_lm_tail(cudaStream_t s);
  // profiling helpers (host-driven mode)
  void prof_begin(cudaStream_t s);
  void prof_end(cudaStream_t s, int entry, double bytes);

  gba_options o_;
  bool mixed_ = false;
  bool profiling_ = false;
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  cudaStream_t cap_[2] = {nullptr, nullptr};
  char *d_arena_ = nullptr;
  size_t d_cap_ = 0;
  char *h_stage_ = nullptr;
  size_t h_cap_ = 0;
  DeviceBatch db_{};
  size_t upload_bytes_ = 0, download_off_ = 0, download_bytes_ = 0;
  // graph cache: valid while the arena and the batch shape are unchanged
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  std::vector<long long> graph_key_;
  // the continue graph (no setup) of segment runs, and the segment length
  cudaGraph_t graph_c_ = nullptr;
  cudaGraphExec_t exec_c_ = nullptr;
  std::vector<long long> graph_c_key_;
  int segment_bodies_ = 0;
  int cluster_cams_ = 0;  // cameras per CTA of the cluster PCG (0 = default)
  int grid_ctas_ = 0;     // CTAs of the grid PCG (0 = every SM)
  bool grid_wait_test_ = false;  // the grid PCG's wait-runs-out test (DeviceOptions::grid_wait_test)
  int graph_segment_ = -1, graph_c_segment_ = -1;
  std::vector<long long> cur_key_;
  // events
  cudaEvent_t ev_start_ = nullptr, ev_stop_ = nullptr;
  cudaEvent_t pev_[2] = {nullptr, nullptr};
  std::vector<ProfileEntry> profile_;
  double last_setup_ms_ = 0.0, last_solve_ms_ = 0.0;
  int trace_cap_ = 0;
  // LM bodies (trials) one solve may run: max_num_iterations, times g2o's
  // trials per iteration under that policy
  int max_lm_bodies() const {
    const long long k = (long long)o_.max_num_iterations * (o_.lm_policy == GBA_LM_POLICY_G2O ? kG2oMaxTrials : 1);
    return (int)std::min<long long>(k, 1 << 28);
  }
  int sm_count_ = 0;
  bool pdl_ = true;        // programmatic dependent launches inside the PCG body
  ClusterPlan cl_plan_;    // cs > 0: the PCG runs as one cluster launch per LM iteration
  GridPlan gr_plan_;       // grid > 0: the PCG runs as one grid-wide launch per LM iteration
  HostBatch hb_;           // the last solve's prepared batch (storage reused)
  gba_status enqueue_pcg_one_launch(cudaStream_t s, std::string *err);
};

}  // namespace gba
