// server.h — continuous-batching request loop over several engine slots.
#pragma once

#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace gba {

class Server {
 public:
  explicit Server(const gba_options &o) : o_(o) {}
  ~Server() { stop(); }

  // Estimated device bytes of one problem (admission rule).
  // Upper bound of one problem's device bytes; explicit_bound adds what the
  // explicit Schur complement may take when the options allow it.
  static size_t estimate_footprint(int nc, int np, int no, bool mixed, bool explicit_bound);

  gba_status start(size_t budget, int max_live, int max_queue, std::string *err);
  gba_status submit(const gba_problem_view *p, uint64_t *ticket, std::string *err);
  gba_status poll(uint64_t ticket, gba_summary *s, int32_t *done, std::string *err);
  gba_status drain_and_stop(std::string *err);
  void stop();
  bool running() const { return running_; }
  void stats(gba_server_stats *st);

 private:
  struct Request {
    uint64_t ticket;
    gba_problem_view view;
    size_t footprint;
    gba_summary summary;
    gba_status status = GBA_OK;
    std::string error;
    bool done = false;
  };
  // A slot is idle, preparing (a worker thread lays out, uploads and starts
  // its cohort while the loop serves the other slots) or running (its
  // segment's completion event pending).
  enum class SlotState { kIdle, kPreparing, kRunning };
  struct Slot {
    std::unique_ptr<Engine> engine;
    std::vector<std::shared_ptr<Request>> reqs;
    std::vector<gba_problem_view> views;
    std::vector<double> t_start;  // per member: when it was admitted
    std::vector<char> delivered;  // per member: finished, result delivered
    std::vector<ProblemState> resume;  // the continuing members' states, for the worker
    HostBatch hb;
    cudaEvent_t done_ev = nullptr;
    size_t bytes = 0;
    SlotState state = SlotState::kIdle;
    std::thread worker;
    std::atomic<int> prep_done{0};
    gba_status prep_status = GBA_OK;
    std::string prep_error;
  };
  void loop();
  // The queued requests (in order) that fit the live cap, the device budget
  // and `max_obs` observations (the first one always, if it fits the
  // budget): take_queued removes and admits them (their bytes in *bytes),
  // peek_queued counts them and their observations.
  std::vector<std::shared_ptr<Request>> take_queued(long long max_obs, size_t *bytes);
  int peek_queued(long long max_obs, long long *obs);
  // Starts a cohort on a worker thread: `keep` members continue from
  // `states` (their views hold their current parameters), `fresh` ones
  // start.
  void launch_cohort(Slot &s, std::vector<std::shared_ptr<Request>> &&keep, std::vector<double> &&keep_t,
                     std::vector<ProblemState> &&states, std::vector<std::shared_ptr<Request>> &&fresh);
  void prepare_and_start(Slot &s);
  // At a segment boundary: continue, re-form (finished members out, queued
  // requests in) or retire the whole cohort.
  void boundary(Slot &s);
  void finish(Slot &s, const std::vector<int> &members, const std::vector<gba_summary> &sums);
  void fail_cohort(Slot &s, gba_status st, const std::string &err);
  template <typename F>
  void guarded(Slot &s, F &&f);

  gba_options o_;
  std::thread thread_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::condition_variable done_cv_;
  std::deque<std::shared_ptr<Request>> queue_;
  std::map<uint64_t, std::shared_ptr<Request>> tickets_;
  std::vector<std::unique_ptr<Slot>> slots_;
  uint64_t next_ticket_ = 1;
  size_t budget_ = 0;
  int max_live_ = 0, max_queue_ = 0;
  bool running_ = false, stopping_ = false;
  std::string init_error_;
  gba_status init_status_ = GBA_OK;
  bool init_done_ = false;
  gba_server_stats st_{};
};

}  // namespace gba
