// server.cpp — continuous batching at LM-iteration granularity.  Requests
// arrive at any time.  A cohort (the problems of one engine slot, laid out
// as one batch of at most kCohortObs observations) runs one LM iteration
// per launch on the slot's own stream, the cohorts of the slots overlapping
// on the device.  Free slots take queued requests as new cohorts.  At each
// iteration boundary the loop reads the members' LM states: members that
// finished get their results at once (their parameters and summaries are
// copied out while the batch stays on the device).  When queued requests
// are waiting, no slot is free and the change is worth a re-layout (the
// finished members and the joining requests are at least 1/kReformDiv of
// the cohort), the cohort is re-formed: finished members leave, queued
// requests join, and the members still running continue in the new batch
// from their exact state (LM state, Jacobi scales, current point), so a
// request joins a running batch at an LM-iteration boundary and every
// result keeps the bits of the problem solved alone.  Otherwise the cohort
// continues on the device (a graph without the setup).
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <stdexcept>

namespace gba {

namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
constexpr int kDefaultSlots = 8;
constexpr int kSegmentBodies = 1;            // LM iterations a cohort runs between boundaries
constexpr long long kCohortObs = 1LL << 21;  // observations a cohort takes in (one request more if alone)
constexpr int kReformDiv = 4;                // re-form when leavers + joiners >= 1/kReformDiv of the cohort
}  // namespace

size_t Server::estimate_footprint(int nc, int np, int no, bool mixed, bool explicit_bound) {
  const double per_obs = 32.0 + 4.0 + 13.0 * (mixed ? 8.0 : 16.0) + 84.0;  // indices, J, segment share
  const double per_pt = 16.0 + 64.0 + 8.0 * 24.0 + (mixed ? 24.0 : 48.0);
  const double per_cam = 8.0 * (18.0 + 44.0 + 45.0 + 9.0 + 9.0 + 81.0 + 9.0 + 54.0 + 9.0 + 6.0) + 64.0;
  double bytes = per_obs * no + per_pt * np + per_cam * nc;
  if (explicit_bound) {
    // the explicit Schur complement as GBA_SCHUR_AUTO may choose it: at most
    // kExplicitPairsPerObs observation pairs per observation, and at most
    // that many (and nc^2) camera-camera blocks of 81 values
    const double rs = mixed ? 4.0 : 8.0;
    const double pairs = (double)kExplicitPairsPerObs * no;
    const double blocks = std::min(pairs, (double)nc * (double)nc);
    bytes += pairs * 8.0 + blocks * (81.0 * rs + 8.0) + (double)nc * (81.0 * rs + 80.0);
  }
  return (size_t)(bytes * 1.15) + (1u << 20);
}

gba_status Server::start(size_t budget, int max_live, int max_queue, std::string *err) {
  if (running_) {
    *err = "server already running";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  max_live_ = max_live > 0 ? max_live : 1 << 30;
  max_queue_ = max_queue > 0 ? max_queue : 1 << 30;
  budget_ = budget;
  st_ = gba_server_stats{};
  stopping_ = false;
  init_done_ = false;
  thread_ = std::thread([this] { loop(); });
  std::unique_lock<std::mutex> lk(mu_);
  done_cv_.wait(lk, [this] { return init_done_; });
  if (init_status_ != GBA_OK) {
    lk.unlock();
    thread_.join();
    *err = init_error_;
    return init_status_;
  }
  running_ = true;
  return GBA_OK;
}

gba_status Server::submit(const gba_problem_view *p, uint64_t *ticket, std::string *err) {
  const gba_status vs = validate_problem(p, err);
  if (vs != GBA_OK) return vs;
  const bool mixed = o_.precision == GBA_PRECISION_MIXED;
  const size_t fp = estimate_footprint(p->num_cameras, p->num_points, p->num_observations, mixed,
                                      o_.schur != GBA_SCHUR_IMPLICIT);
  std::lock_guard<std::mutex> lk(mu_);
  if (!running_ || stopping_) {
    *err = "server not running";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  const bool empty = p->num_observations == 0;  // nothing to solve: done at once, as gba_solve
  if (!empty && fp > budget_) {
    ++st_.rejected;
    *err = "problem footprint exceeds the device budget";
    return GBA_ERR_OUT_OF_MEMORY;
  }
  if (!empty && (int)queue_.size() >= max_queue_) {
    ++st_.rejected;
    *err = "request queue full";
    return GBA_ERR_QUEUE_FULL;
  }
  auto r = std::make_shared<Request>();
  r->ticket = next_ticket_++;
  r->view = *p;
  r->footprint = fp;
  std::memset(&r->summary, 0, sizeof r->summary);
  tickets_[r->ticket] = r;
  ++st_.submitted;
  *ticket = r->ticket;
  if (empty) {
    empty_problem_summary(&r->summary, o_.initial_trust_region_radius);
    r->done = true;
    ++st_.completed;
    done_cv_.notify_all();
    return GBA_OK;
  }
  queue_.push_back(r);
  st_.queued = (int32_t)queue_.size();
  cv_.notify_all();
  return GBA_OK;
}

gba_status Server::poll(uint64_t ticket, gba_summary *s, int32_t *done, std::string *err) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = tickets_.find(ticket);
  if (it == tickets_.end()) {
    *err = "unknown ticket";
    return GBA_ERR_NOT_FOUND;
  }
  Request &r = *it->second;
  *done = r.done ? 1 : 0;
  if (!r.done) return GBA_OK;
  if (s) {
    // keep the caller's trace buffers; copy scalars
    const int cap = s->trace_capacity;
    double *tc = s->trace_cost, *tr = s->trace_radius;
    int32_t *tl = s->trace_linear_iterations, *ts = s->trace_successful;
    *s = r.summary;
    s->trace_capacity = cap;
    s->trace_cost = tc, s->trace_radius = tr, s->trace_linear_iterations = tl, s->trace_successful = ts;
    s->trace_length = 0;
  }
  const gba_status st = r.status;
  if (st != GBA_OK) *err = r.error;
  tickets_.erase(it);
  return st;
}

void Server::stats(gba_server_stats *out) {
  std::lock_guard<std::mutex> lk(mu_);
  *out = st_;
}

auto Server::take_queued(long long max_obs, size_t *bytes) -> std::vector<std::shared_ptr<Request>> {
  std::vector<std::shared_ptr<Request>> take;
  *bytes = 0;
  long long obs = 0;
  std::lock_guard<std::mutex> lk(mu_);
  while (!queue_.empty()) {
    const auto &r = queue_.front();
    if (st_.live + (int)take.size() >= max_live_) break;
    if (st_.device_bytes_in_use + *bytes + r->footprint > budget_) break;
    if (!take.empty() && obs + r->view.num_observations > max_obs) break;
    *bytes += r->footprint;
    obs += r->view.num_observations;
    take.push_back(r);
    queue_.pop_front();
  }
  if (!take.empty()) {
    st_.live += (int32_t)take.size();
    st_.peak_live = std::max(st_.peak_live, st_.live);
    st_.admitted += (int64_t)take.size();
    st_.device_bytes_in_use += *bytes;
    st_.device_bytes_peak = std::max(st_.device_bytes_peak, st_.device_bytes_in_use);
    st_.queued = (int32_t)queue_.size();
  }
  return take;
}

int Server::peek_queued(long long max_obs, long long *obs) {
  std::lock_guard<std::mutex> lk(mu_);
  int n = 0;
  size_t bytes = 0;
  *obs = 0;
  for (const auto &r : queue_) {
    if (st_.live + n >= max_live_) break;
    if (st_.device_bytes_in_use + bytes + r->footprint > budget_) break;
    if (*obs + r->view.num_observations > max_obs) break;
    bytes += r->footprint;
    *obs += r->view.num_observations;
    ++n;
  }
  return n;
}

void Server::launch_cohort(Slot &s, std::vector<std::shared_ptr<Request>> &&keep, std::vector<double> &&keep_t,
                           std::vector<ProblemState> &&states, std::vector<std::shared_ptr<Request>> &&fresh) {
  const double t = now_s();
  s.reqs = std::move(keep);
  s.t_start = std::move(keep_t);
  s.resume = std::move(states);
  for (auto &r : fresh) {
    s.reqs.push_back(r);
    s.t_start.push_back(t);
  }
  s.delivered.assign(s.reqs.size(), 0);
  s.views.clear();
  for (auto &r : s.reqs) s.views.push_back(r->view);
  s.prep_done.store(0, std::memory_order_relaxed);
  s.worker = std::thread([this, &s] { prepare_and_start(s); });  // may throw: the slot is not marked yet
  s.state = SlotState::kPreparing;
}

// On the slot's worker thread: the loop does not touch the slot until
// prep_done is set.
void Server::prepare_and_start(Slot &s) {
  std::string err;
  const double t0 = now_s();
  double t1 = t0;
  gba_status st = GBA_OK;
  try {
    const PrepOptions po = s.engine->prep_options();
    st = prepare_batch(s.views.data(), (int)s.views.size(), po, &s.hb, &err);
    if (st == GBA_OK)
      for (size_t i = 0; i < s.resume.size(); ++i) set_resume(s.hb, (int)i, s.resume[i]);
    s.resume.clear();
    if (st == GBA_OK) st = s.engine->upload(s.hb, &err);
  } catch (const std::bad_alloc &) {
    st = GBA_ERR_OUT_OF_MEMORY;
    err = "host memory exhausted while laying out a cohort";
  } catch (const std::exception &e) {
    st = GBA_ERR_INTERNAL;
    err = std::string("laying out a cohort: ") + e.what();
  }
  t1 = now_s();
  if (st == GBA_OK) st = s.engine->run_segment(false, &err);
  if (st == GBA_OK) st = s.engine->fetch_states(&err);
  if (st == GBA_OK && cudaEventRecord(s.done_ev, s.engine->stream()) != cudaSuccess) {
    st = GBA_ERR_CUDA;
    err = "event record";
  }
  // the graph of the next segments, built while the first one runs (a
  // failure here is not the cohort's: the first continue builds it again)
  if (st == GBA_OK) {
    std::string ignored;
    s.engine->prepare_continue(&ignored);
  }
  s.prep_status = st;
  s.prep_error = err;
  {
    std::lock_guard<std::mutex> lk(mu_);
    st_.host_prep_s += t1 - t0;
    if (st == GBA_OK) ++st_.steps;
    s.prep_done.store(1, std::memory_order_release);
  }
  cv_.notify_all();
}

// Every member not yet delivered fails with `st`; the slot is emptied.
void Server::fail_cohort(Slot &s, gba_status st, const std::string &err) {
  std::lock_guard<std::mutex> lk(mu_);
  for (size_t i = 0; i < s.reqs.size(); ++i) {
    if (i < s.delivered.size() && s.delivered[i]) continue;
    Request &r = *s.reqs[i];
    r.status = st;
    r.error = err;
    r.done = true;
    ++st_.completed;
    --st_.live;
  }
  st_.device_bytes_in_use -= s.bytes;
  s.reqs.clear();
  s.views.clear();
  s.t_start.clear();
  s.delivered.clear();
  s.state = SlotState::kIdle;
  s.bytes = 0;
  done_cv_.notify_all();
}

void Server::finish(Slot &s, const std::vector<int> &members, const std::vector<gba_summary> &sums) {
  const double t = now_s();
  std::lock_guard<std::mutex> lk(mu_);
  for (int i : members) {
    Request &r = *s.reqs[i];
    r.summary = sums[i];
    r.summary.total_time_s = t - s.t_start[i];
    r.summary.solve_time_s = r.summary.total_time_s;
    r.status = GBA_OK;
    r.done = true;
    s.delivered[i] = 1;
    ++st_.completed;
    --st_.live;
    st_.device_bytes_in_use -= r.footprint;
    s.bytes -= r.footprint;
  }
  done_cv_.notify_all();
}

void Server::boundary(Slot &s) {
  std::string err;
  gba_status st = s.engine->device_status(&err);
  if (st != GBA_OK) {
    fail_cohort(s, st, err);
    return;
  }
  const LMState *lm = s.engine->states(s.hb);
  const int n = (int)s.reqs.size();
  std::vector<int> newly, live_m;
  long long live_obs = 0, gone_obs = 0;
  for (int i = 0; i < n; ++i) {
    const long long o = s.reqs[i]->view.num_observations;
    if (lm[i].active) {
      live_m.push_back(i);
      live_obs += o;
    } else {
      if (!s.delivered[i]) newly.push_back(i);
      gone_obs += o;
    }
  }
  // results of the members that finished in this segment
  if (!newly.empty()) {
    std::vector<gba_summary> sums(n);
    for (auto &x : sums) std::memset(&x, 0, sizeof x);
    if ((st = s.engine->deliver(s.hb, newly, s.views.data(), sums.data(), &err)) != GBA_OK) {
      fail_cohort(s, st, err);
      return;
    }
    finish(s, newly, sums);
  }
  if (live_m.empty()) {
    // every member done: the slot is free
    s.reqs.clear();
    s.views.clear();
    s.t_start.clear();
    s.delivered.clear();
    s.state = SlotState::kIdle;
    s.bytes = 0;
    return;
  }
  long long join_obs = 0;
  const int joiners = peek_queued(kCohortObs - live_obs, &join_obs);
  if (joiners > 0 && (gone_obs + join_obs) * kReformDiv >= live_obs + gone_obs) {
    // re-form: the running members' current point into their views, their
    // states carried over; the finished ones leave, queued requests join
    std::vector<ProblemState> states;
    if ((st = s.engine->deliver(s.hb, live_m, s.views.data(), nullptr, &err)) != GBA_OK ||
        (st = s.engine->download_states(s.hb, &states, &err)) != GBA_OK) {
      fail_cohort(s, st, err);
      return;
    }
    std::vector<std::shared_ptr<Request>> keep;
    std::vector<double> keep_t;
    std::vector<ProblemState> keep_states;
    for (int i : live_m) {
      keep.push_back(s.reqs[i]);
      keep_t.push_back(s.t_start[i]);
      keep_states.push_back(std::move(states[i]));
    }
    size_t bytes = 0;
    std::vector<std::shared_ptr<Request>> fresh = take_queued(kCohortObs - live_obs, &bytes);
    s.bytes += bytes;
    {
      std::lock_guard<std::mutex> lk(mu_);
      ++st_.reforms;
    }
    launch_cohort(s, std::move(keep), std::move(keep_t), std::move(keep_states), std::move(fresh));
    return;
  }
  // nothing joins: the next LM iteration on the device
  st = s.engine->run_segment(true, &err);
  if (st == GBA_OK) st = s.engine->fetch_states(&err);
  if (st == GBA_OK && cudaEventRecord(s.done_ev, s.engine->stream()) != cudaSuccess) {
    st = GBA_ERR_CUDA;
    err = "event record";
  }
  if (st != GBA_OK) {
    fail_cohort(s, st, err);
    return;
  }
  std::lock_guard<std::mutex> lk(mu_);
  ++st_.steps;
}

// Runs a step of the loop for slot s; a host exception (memory, thread
// creation) fails the slot's requests instead of ending the process.  The
// steps start a worker only as their last action, so no worker is running
// when one throws.
template <typename F>
void Server::guarded(Slot &s, F &&f) {
  try {
    f();
  } catch (const std::bad_alloc &) {
    if (s.state != SlotState::kPreparing) fail_cohort(s, GBA_ERR_OUT_OF_MEMORY, "host memory exhausted");
  } catch (const std::exception &e) {
    if (s.state != SlotState::kPreparing) fail_cohort(s, GBA_ERR_INTERNAL, e.what());
  }
}

void Server::loop() {
  // engines are created on this thread, bound to the configured device
  {
    std::lock_guard<std::mutex> lk(mu_);
    const int n = o_.server_slots > 0 ? o_.server_slots : kDefaultSlots;
    for (int i = 0; i < n; ++i) {
      slots_.emplace_back(new Slot);
      Slot &s = *slots_.back();
      gba_options so = o_;
      so.stream = nullptr;
      so.use_graphs = 1;
      // the FP64 grid PCG spreads one problem over every SM; cohorts of
      // other slots run beside it, and a grid launch that finds the SMs
      // taken proceeds with the CTAs that start (correct, but slow), so the
      // slots keep the two-kernel FP64 PCG (the mixed form's clusters hold
      // 16 SMs each and share the GPU)
      if (so.precision == GBA_PRECISION_FP64) so.persistent_pcg = 0;
      s.engine.reset(new Engine(so));
      std::string err;
      const gba_status st = s.engine->init(&err);
      if (st != GBA_OK) {
        init_status_ = st;
        init_error_ = err;
        break;
      }
      s.engine->set_segment(kSegmentBodies);
      cudaEventCreateWithFlags(&s.done_ev, cudaEventDisableTiming);
    }
    if (init_status_ == GBA_OK && budget_ == 0) {
      size_t fr = 0, tot = 0;
      cudaMemGetInfo(&fr, &tot);
      budget_ = (size_t)(0.9 * (double)fr);
    }
    init_done_ = true;
    done_cv_.notify_all();
    if (init_status_ != GBA_OK) {
      for (auto &s : slots_)
        if (s->done_ev) cudaEventDestroy(s->done_ev);
      slots_.clear();
      return;
    }
  }
  for (;;) {
    bool did = false;
    // cohorts whose worker finished laying out and starting them
    for (auto &sp : slots_) {
      Slot &s = *sp;
      if (s.state != SlotState::kPreparing || !s.prep_done.load(std::memory_order_acquire)) continue;
      s.worker.join();
      if (s.prep_status != GBA_OK)
        fail_cohort(s, s.prep_status, s.prep_error);
      else
        s.state = SlotState::kRunning;
      did = true;
    }
    // free slots take queued requests as new cohorts
    for (auto &sp : slots_) {
      Slot &s = *sp;
      if (s.state != SlotState::kIdle) continue;
      size_t bytes = 0;
      std::vector<std::shared_ptr<Request>> take = take_queued(kCohortObs, &bytes);
      if (take.empty()) break;
      s.bytes = bytes;
      guarded(s, [&] { launch_cohort(s, {}, {}, {}, std::move(take)); });
      did = true;
    }
    // cohorts at an LM-iteration boundary: results out, continue or re-form
    for (auto &sp : slots_) {
      Slot &s = *sp;
      if (s.state == SlotState::kRunning && cudaEventQuery(s.done_ev) == cudaSuccess) {
        guarded(s, [&] { boundary(s); });
        did = true;
      }
    }
    std::unique_lock<std::mutex> lk(mu_);
    bool any_busy = false;
    for (auto &s : slots_) any_busy |= s->state != SlotState::kIdle;
    if (stopping_ && queue_.empty() && !any_busy) break;
    if (!did) {
      if (any_busy)
        cv_.wait_for(lk, std::chrono::microseconds(20));
      else
        cv_.wait_for(lk, std::chrono::milliseconds(5), [this] { return !queue_.empty() || stopping_; });
    }
  }
  for (auto &s : slots_) {
    if (s->done_ev) cudaEventDestroy(s->done_ev);
    s->engine.reset();
  }
  slots_.clear();
}

gba_status Server::drain_and_stop(std::string *err) {
  (void)err;
  stop();
  return GBA_OK;
}

void Server::stop() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (!running_ && !thread_.joinable()) return;
    stopping_ = true;
    cv_.notify_all();
  }
  if (thread_.joinable()) thread_.join();
  running_ = false;
}

}  // namespace gba
