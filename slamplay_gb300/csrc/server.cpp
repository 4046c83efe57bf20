// server.cpp — continuous batching: requests arrive at any time; the loop
// admits queued requests into a free engine slot as long as their estimated
// device footprint fits the remaining budget and the live-problem cap, lays
// them out as one batch (problems batched per LM iteration inside one CUDA
// graph), and launches it on the slot's own stream while other slots are
// still running, so cohorts overlap on the device.  A finished cohort is
// retired (results written back, memory budget returned) as soon as its
// completion event fires.  Each problem's arithmetic depends only on the
// problem, never on its cohort, so a result is the same alone and in the mix.
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace gba {

namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
constexpr int kSlots = 4;
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
  if (fp > budget_) {
    ++st_.rejected;
    *err = "problem footprint exceeds the device budget";
    return GBA_ERR_OUT_OF_MEMORY;
  }
  if ((int)queue_.size() >= max_queue_) {
    ++st_.rejected;
    *err = "request queue full";
    return GBA_ERR_QUEUE_FULL;
  }
  auto r = std::make_shared<Request>();
  r->ticket = next_ticket_++;
  r->view = *p;
  r->footprint = fp;
  std::memset(&r->summary, 0, sizeof r->summary);
  queue_.push_back(r);
  tickets_[r->ticket] = r;
  ++st_.submitted;
  st_.queued = (int32_t)queue_.size();
  *ticket = r->ticket;
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

bool Server::launch_cohort(Slot &s, std::vector<std::shared_ptr<Request>> &&reqs) {
  s.reqs = std::move(reqs);
  s.views.clear();
  for (auto &r : s.reqs) s.views.push_back(r->view);
  std::string err;
  const PrepOptions po = s.engine->prep_options();
  gba_status st = prepare_batch(s.views.data(), (int)s.views.size(), po, &s.hb, &err);
  if (st == GBA_OK) st = s.engine->upload(s.hb, &err);
  if (st == GBA_OK) st = s.engine->run_solve(&err);
  if (st == GBA_OK && cudaEventRecord(s.done_ev, s.engine->stream()) != cudaSuccess) {
    st = GBA_ERR_CUDA;
    err = "event record";
  }
  if (st != GBA_OK) {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto &r : s.reqs) {
      r->status = st;
      r->error = err;
      r->done = true;
      ++st_.completed;
    }
    s.reqs.clear();
    done_cv_.notify_all();
    return false;
  }
  s.busy = true;
  s.t_start = now_s();
  return true;
}

void Server::retire(Slot &s) {
  std::string err;
  std::vector<gba_summary> sums(s.reqs.size());
  for (auto &x : sums) std::memset(&x, 0, sizeof x);
  const gba_status st = s.engine->download(s.hb, s.views.data(), sums.data(), &err);
  const double t = now_s();
  std::lock_guard<std::mutex> lk(mu_);
  for (size_t i = 0; i < s.reqs.size(); ++i) {
    Request &r = *s.reqs[i];
    r.summary = sums[i];
    r.summary.total_time_s = t - s.t_start;
    r.status = st;
    r.error = err;
    r.done = true;
    ++st_.completed;
  }
  st_.live -= (int32_t)s.reqs.size();
  st_.device_bytes_in_use -= s.bytes;
  s.reqs.clear();
  s.busy = false;
  s.bytes = 0;
  done_cv_.notify_all();
}

void Server::loop() {
  // engines are created on this thread, bound to the configured device
  {
    std::lock_guard<std::mutex> lk(mu_);
    slots_.resize(kSlots);
    for (Slot &s : slots_) {
      gba_options so = o_;
      so.stream = nullptr;
      so.use_graphs = 1;
      s.engine.reset(new Engine(so));
      std::string err;
      const gba_status st = s.engine->init(&err);
      if (st != GBA_OK) {
        init_status_ = st;
        init_error_ = err;
        break;
      }
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
      for (Slot &s : slots_)
        if (s.done_ev) cudaEventDestroy(s.done_ev);
      slots_.clear();
      return;
    }
  }
  for (;;) {
    bool did = false;
    // retire finished cohorts
    for (Slot &s : slots_)
      if (s.busy && cudaEventQuery(s.done_ev) == cudaSuccess) {
        retire(s);
        did = true;
      }
    // admit queued requests into free slots
    for (Slot &s : slots_) {
      if (s.busy) continue;
      std::vector<std::shared_ptr<Request>> take;
      size_t bytes = 0;
      {
        std::lock_guard<std::mutex> lk(mu_);
        while (!queue_.empty()) {
          const auto &r = queue_.front();
          if (st_.live + (int)take.size() >= max_live_) break;
          if (st_.device_bytes_in_use + bytes + r->footprint > budget_) break;
          bytes += r->footprint;
          take.push_back(r);
          queue_.pop_front();
        }
        if (take.empty()) break;
        st_.live += (int32_t)take.size();
        st_.peak_live = std::max(st_.peak_live, st_.live);
        st_.admitted += (int64_t)take.size();
        st_.device_bytes_in_use += bytes;
        st_.device_bytes_peak = std::max(st_.device_bytes_peak, st_.device_bytes_in_use);
        st_.queued = (int32_t)queue_.size();
        ++st_.steps;
      }
      s.bytes = bytes;
      const int32_t count = (int32_t)take.size();
      if (!launch_cohort(s, std::move(take))) {
        std::lock_guard<std::mutex> lk(mu_);
        st_.live -= count;
        st_.device_bytes_in_use -= bytes;
        s.bytes = 0;
      }
      did = true;
    }
    std::unique_lock<std::mutex> lk(mu_);
    bool any_busy = false;
    for (Slot &s : slots_) any_busy |= s.busy;
    if (stopping_ && queue_.empty() && !any_busy) break;
    if (!did) {
      if (any_busy)
        cv_.wait_for(lk, std::chrono::microseconds(50));
      else
        cv_.wait_for(lk, std::chrono::milliseconds(5), [this] { return !queue_.empty() || stopping_; });
    }
  }
  for (Slot &s : slots_) {
    if (s.done_ev) cudaEventDestroy(s.done_ev);
    s.engine.reset();
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
