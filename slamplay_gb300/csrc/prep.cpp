// prep.cpp — host-side layout of a batch of BAL problems.
//
// Input: the BALProblem arrays of each problem (utils/datasets/BALProblem.h:
// 109-118), in any observation order.  Output: observations sorted by
// (internal point, camera, input index) — point-major as BAL files usually
// are (data/bal/ladybug49.txt) — with every point's observations contiguous;
// chunks of whole points; per chunk the camera-sorted order of its
// observations and its camera segments; per camera its segments and its
// observations.  All orderings are deterministic functions of the input.
// The data-parallel loops run on a pool of host threads; no result depends
// on how their work is split.
#include "prep.h"

#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>

namespace gba {

static std::string fmt(const char *f, long long a, long long b = 0, long long c = 0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, f, a, b, c);
  return buf;
}

// ---------------------------------------------------------------------------
// Host thread pool for the data-parallel loops: hardware threads (at most
// 32, or GBA_HOST_THREADS) made on first use and kept (starting threads costs far more than a
// loop's wake-up), the calling thread working too; tasks are taken from a
// shared counter, and no result depends on which thread runs a task.  A loop
// that finds the pool busy (another handle preparing at the same time), runs
// inside a task, or runs in a forked child works on the calling thread alone.
// The pool is never destroyed: a forked child (which has none of the
// parent's threads) and the parent at exit end without joining or locking
// anything.  An exception from a task ends the loop's other tasks early and
// is rethrown by run() once every worker has left the loop.
namespace {
thread_local bool tl_in_task = false;  // this thread is running a pool task

class Pool {
 public:
  static Pool &get() {
    static Pool *p = new Pool;  // never destroyed
    return *p;
  }
  int threads() const { return (int)workers_.size() + 1; }
  void run(int ntasks, const std::function<void(int)> &fn) {
    if (ntasks <= 0) return;
    std::unique_lock<std::mutex> busy(run_mu_, std::defer_lock);
    if (ntasks == 1 || workers_.empty() || tl_in_task || getpid() != pid_ || !busy.try_lock()) {
      for (int t = 0; t < ntasks; ++t) fn(t);
      return;
    }
    {
      std::lock_guard<std::mutex> g(mu_);
      fn_ = &fn;
      ntasks_ = ntasks;
      next_.store(0, std::memory_order_relaxed);
      done_ = 0;
      error_ = nullptr;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::exception_ptr err;
    {
      std::unique_lock<std::mutex> g(mu_);
      done_cv_.wait(g, [&] { return done_ == (int)workers_.size(); });
      fn_ = nullptr;
      err = error_;
      error_ = nullptr;
    }
    if (err) std::rethrow_exception(err);
  }

 private:
  Pool() : pid_(getpid()) {
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    // GBA_HOST_THREADS caps the host threads (1: every loop on the caller's)
    if (const char *env = std::getenv("GBA_HOST_THREADS")) {
      const long v = std::strtol(env, nullptr, 10);
      if (v >= 1) hw = std::min<unsigned>(hw, (unsigned)v);
    }
    const int n = (int)std::min(hw, 32u) - 1;
    try {
      for (int i = 0; i < n; ++i) workers_.emplace_back([this] { loop(); });
    } catch (...) {
      // fewer threads than asked: the loop counts only those that started
    }
  }
  // the tasks of the current loop, until none is left; a task's exception
  // is kept (the first one) and the remaining tasks are skipped
  void work() {
    struct InTask {
      InTask() { tl_in_task = true; }
      ~InTask() { tl_in_task = false; }
    } in_task;
    for (;;) {
      const int t = next_.fetch_add(1, std::memory_order_relaxed);
      if (t >= ntasks_) break;
      try {
        (*fn_)(t);
      } catch (...) {
        std::lock_guard<std::mutex> g(mu_);
        if (!error_) error_ = std::current_exception();
        next_.store(ntasks_, std::memory_order_relaxed);
      }
    }
  }
  void loop() {
    long long seen = 0;
    std::unique_lock<std::mutex> g(mu_);
    for (;;) {
      cv_.wait(g, [&] { return gen_ != seen; });
      seen = gen_;
      g.unlock();
      work();
      g.lock();
      if (++done_ == (int)workers_.size()) done_cv_.notify_one();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)> *fn_ = nullptr;
  int ntasks_ = 0;
  std::atomic<int> next_{0};
  int done_ = 0;
  long long gen_ = 0;
  std::exception_ptr error_;
  const pid_t pid_;
};
}  // namespace

int host_threads() { return Pool::get().threads(); }

void host_parallel(int ntasks, const std::function<void(int)> &fn) { Pool::get().run(ntasks, fn); }

// Runs fn(begin, end) over [0, n) in contiguous runs (one run when n is
// small); fn must write disjoint outputs per index.
static void parallel_runs(long long n, long long min_per_run, const std::function<void(long long, long long)> &fn) {
  const long long runs =
      std::min<long long>(4LL * host_threads(), std::max<long long>(1, n / std::max(1LL, min_per_run)));
  if (runs <= 1) {
    fn(0, n);
    return;
  }
  host_parallel((int)runs, [&](int r) { fn(n * r / runs, n * (r + 1) / runs); });
}

static inline void atomic_min_i64(std::atomic<long long> &a, long long v) {
  long long cur = a.load(std::memory_order_relaxed);
  while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
  }
}

// Loops with fewer elements than this run on the calling thread.
constexpr long long kParMin = 32768;

gba_status validate_problem(const gba_problem_view *v, std::string *err) {
  if (!v) {
    *err = "null problem view";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  if (v->num_cameras < 0 || v->num_points < 0 || v->num_observations < 0) {
    *err = "negative problem size";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  if (v->num_observations > 0 &&
      (!v->camera_index || !v->point_index || !v->observations))
    return *err = "null observation array", GBA_ERR_INVALID_ARGUMENT;
  if ((v->num_cameras > 0 || v->num_points > 0) && !v->parameters)
    return *err = "null parameter array", GBA_ERR_INVALID_ARGUMENT;
  const int nc = v->num_cameras, np = v->num_points;
  // the first bad observation and the first bad parameter (runs in
  // parallel; the reported one is the lowest index, as a sequential scan)
  auto bad_obs = [&](long long i) {
    const int c = v->camera_index[i], p = v->point_index[i];
    return c < 0 || c >= nc || p < 0 || p >= np || !std::isfinite(v->observations[2 * i]) ||
           !std::isfinite(v->observations[2 * i + 1]);
  };
  const long long no = v->num_observations, npar = 9LL * nc + 3LL * np;
  std::atomic<long long> first_obs{no}, first_par{npar};
  parallel_runs(no, kParMin, [&](long long b, long long e) {
    for (long long i = b; i < e && i < first_obs.load(std::memory_order_relaxed); ++i)
      if (bad_obs(i)) {
        atomic_min_i64(first_obs, i);
        return;
      }
  });
  parallel_runs(npar, 4 * kParMin, [&](long long b, long long e) {
    for (long long k = b; k < e && k < first_par.load(std::memory_order_relaxed); ++k)
      if (!std::isfinite(v->parameters[k])) {
        atomic_min_i64(first_par, k);
        return;
      }
  });
  if (first_obs.load() < no) {
    const long long i = first_obs.load();
    const int c = v->camera_index[i], p = v->point_index[i];
    if (c < 0 || c >= nc) {
      *err = fmt("observation %lld: camera index %lld out of range [0, %lld)", i, c, nc);
      return GBA_ERR_INVALID_ARGUMENT;
    }
    if (p < 0 || p >= np) {
      *err = fmt("observation %lld: point index %lld out of range [0, %lld)", i, p, np);
      return GBA_ERR_INVALID_ARGUMENT;
    }
    *err = fmt("observation %lld is not finite", i);
    return GBA_ERR_NON_FINITE;
  }
  if (first_par.load() < npar) {
    *err = fmt("parameter %lld is not finite", first_par.load());
    return GBA_ERR_NON_FINITE;
  }
  return GBA_OK;
}

// Per-thread scratch tables indexed by camera, stamped so that they need no
// clearing between uses: a slot is valid when its stamp is the caller's.
namespace {
std::atomic<long long> g_stamp_base{0};
struct CamScratch {
  std::vector<long long> mark;
  std::vector<int32_t> a, b, c;
};
CamScratch &cam_scratch(int n) {
  static thread_local CamScratch s;
  if ((int)s.mark.size() < n) {
    s.mark.resize(n, -1);
    s.a.resize(n);
    s.b.resize(n);
    s.c.resize(n);
  }
  return s;
}
// A fresh range of 2^32 stamps.
long long new_stamps() { return g_stamp_base.fetch_add(1, std::memory_order_relaxed) << 32; }
}  // namespace

// The explicit Schur complement's structure, row camera by row camera: the
// row's co-visible cameras (sorted; the row's own camera when it observes a
// point more than once), the transpose of every block, and for the blocks
// on and above the diagonal (column camera >= row camera: the formation
// kernel forms those and writes each transpose) the ordered observation
// pairs (a of the row camera, b of the column camera, a != b, same point;
// stored as the two observations' camera-major positions) in point order,
// so the formation sums have a fixed order.  A camera's observations
// (cam_obs_list) are in point order, so walking them and each point's
// observations lists every block's pairs in that order.  O(pairs) with a
// per-row lookup table; the rows are independent, so the pool's threads
// take runs of rows (the result does not depend on the split).
static void build_schur_structure(HostBatch *hbp) {
  HostBatch &hb = *hbp;
  const int nc = hb.nc;
  // F rows are stored camera-major (a camera's observations together, in
  // point order): the pairs of a block read two cameras' runs of rows
  hb.obs_fpos.resize(hb.no);
  parallel_runs(hb.no, kParMin, [&](long long b, long long e) {
    for (long long i = b; i < e; ++i) hb.obs_fpos[hb.cam_obs_list[i]] = (int32_t)i;
  });
  std::vector<std::vector<int32_t>> rows(nc), cnts(nc);  // per row: columns; pair counts of its upper blocks
  std::vector<int32_t> first_up(nc, 0);                  // per row: index of its first column >= the row
  // runs of rows of about equal observation counts
  std::vector<int> rb(1, 0);
  {
    const long long target = std::max<long long>(4096, (long long)hb.no / (8LL * host_threads()) + 1);
    for (int c = 0; c < nc;) {
      long long acc = 0;
      int c1 = c;
      do {
        acc += hb.cam_obs_begin[c1 + 1] - hb.cam_obs_begin[c1];
        ++c1;
      } while (c1 < nc && acc < target);
      rb.push_back(c1);
      c = c1;
    }
  }
  const int nruns = (int)rb.size() - 1;
  // 1. per row: sorted co-visible cameras, pair counts of the upper blocks
  const long long stamp = new_stamps();
  host_parallel(nruns, [&](int r) {
    CamScratch &s = cam_scratch(nc);
    int32_t *pairs_of = s.a.data();  // per column camera: the row's pair count
    for (int c = rb[r]; c < rb[r + 1]; ++c) {
      const long long mk = stamp | c;
      const int a0 = hb.cam_obs_begin[c], a1 = hb.cam_obs_begin[c + 1];
      std::vector<int32_t> &row = rows[c];
      for (int ia = a0; ia < a1; ++ia) {
        const int a = hb.cam_obs_list[ia], j = hb.obs_pt[a];
        for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b) {
          const int k = hb.obs_cam[b];
          if (b == a) continue;
          if (s.mark[k] != mk) s.mark[k] = mk, row.push_back(k), pairs_of[k] = 0;
          ++pairs_of[k];
        }
      }
      std::sort(row.begin(), row.end());
      const int nb = (int)row.size();
      const int u0 = (int)(std::lower_bound(row.begin(), row.end(), c) - row.begin());
      first_up[c] = u0;
      std::vector<int32_t> &cnt = cnts[c];
      cnt.resize(nb - u0);
      for (int u = u0; u < nb; ++u) cnt[u - u0] = pairs_of[row[u]];
    }
  });
  // 2. prefix sums: the CSR, the upper blocks, their pair ranges
  hb.sblk_row.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) hb.sblk_row[c + 1] = hb.sblk_row[c] + (int32_t)rows[c].size();
  hb.nblk = hb.sblk_row[nc];
  hb.sblk_col.resize(hb.nblk);
  std::vector<long long> up_begin(nc + 1, 0);  // per row: its first upper block (index into sblk_up)
  for (int c = 0; c < nc; ++c) up_begin[c + 1] = up_begin[c] + (long long)cnts[c].size();
  hb.nup = up_begin[nc];
  hb.sblk_up.resize(hb.nup);
  hb.sblk_pair.resize(hb.nup + 1);
  hb.sblk_pair[0] = 0;
  for (int c = 0; c < nc; ++c) {
    std::copy(rows[c].begin(), rows[c].end(), hb.sblk_col.begin() + hb.sblk_row[c]);
    for (size_t u = 0; u < cnts[c].size(); ++u) {
      const long long k = up_begin[c] + (long long)u;
      hb.sblk_up[k] = hb.sblk_row[c] + first_up[c] + (int32_t)u;
      hb.sblk_pair[k + 1] = hb.sblk_pair[k] + cnts[c][u];
    }
  }
  hb.npairs = hb.sblk_pair[hb.nup];
  hb.spair.resize(2 * (size_t)hb.npairs);
  // 3. the pairs, in point order per block
  host_parallel(nruns, [&](int r) {
    CamScratch &s = cam_scratch(nc);
    std::vector<int32_t> &pos = s.a;
    std::vector<int32_t> next;
    for (int c = rb[r]; c < rb[r + 1]; ++c) {
      const std::vector<int32_t> &row = rows[c];
      const int u0 = first_up[c], nu = (int)row.size() - u0;
      next.resize(nu);
      for (int u = 0; u < nu; ++u) {
        pos[row[u0 + u]] = u;
        next[u] = hb.sblk_pair[up_begin[c] + u];
      }
      for (int ia = hb.cam_obs_begin[c]; ia < hb.cam_obs_begin[c + 1]; ++ia) {
        const int a = hb.cam_obs_list[ia], j = hb.obs_pt[a];
        for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b)
          if (b != a && hb.obs_cam[b] >= c) {
            const size_t k = (size_t)next[pos[hb.obs_cam[b]]]++;
            hb.spair[2 * k] = hb.obs_fpos[a];
            hb.spair[2 * k + 1] = hb.obs_fpos[b];
          }
      }
    }
  });
  // 4. the transpose of block (c, k) is block (k, c), in row k
  hb.sblk_tr.resize(hb.nblk);
  host_parallel(nruns, [&](int r) {
    for (int c = rb[r]; c < rb[r + 1]; ++c)
      for (int e = hb.sblk_row[c]; e < hb.sblk_row[c + 1]; ++e) {
        const int k = hb.sblk_col[e];
        const auto b0 = hb.sblk_col.begin() + hb.sblk_row[k], b1 = hb.sblk_col.begin() + hb.sblk_row[k + 1];
        hb.sblk_tr[e] = (int32_t)(std::lower_bound(b0, b1, c) - hb.sblk_col.begin());
      }
  });
}

// Counts, offsets and appended arrays start empty; the arrays prepare_batch
// overwrites entirely keep their size, so a batch of the same size is laid
// out without re-zeroing them.
void HostBatch::reset() {
  P = nc = np = no = nchunks = nseg = cam_blocks = 0;
  explicit_schur = false;
  nblk = nup = npairs = 0;
  for (auto *v : {&pt_obs_begin, &seg_cam, &cam_seg_begin, &cam_obs_begin, &cam_piece_begin, &sblk_row, &sblk_up,
                  &sblk_pair})
    v->clear();
  seg_pos.clear();
  cam_used.clear();
  obs_rig.clear();
  prob_rig.clear();
  resume.clear();
  resume_lm.clear();
  resume_cam_scale.clear();
  resume_pt_scale.clear();
  prob.clear();
  chunk.clear();
  camblk.clear();
}

gba_status prepare_batch(const gba_problem_view *views, int n, const PrepOptions &opt, HostBatch *out,
                         std::string *err) {
  HostBatch &hb = *out;
  hb.reset();
  if (n <= 0 || !views) {
    *err = "empty batch";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  const int cap = opt.chunk_cap;
  long long tc = 0, tp = 0, to = 0;
  for (int p = 0; p < n; ++p) {
    const gba_status st = validate_problem(&views[p], err);
    if (st != GBA_OK) {
      if (n > 1) *err = fmt("problem %lld: ", p) + *err;
      return st;
    }
    tc += views[p].num_cameras;
    tp += views[p].num_points;
    to += views[p].num_observations;
  }
  if (tc > (1LL << 30) || tp > (1LL << 30) || to > (1LL << 30)) {
    *err = "batch too large for 32-bit indices";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  hb.P = n;
  hb.nc = (int)tc;
  hb.np = (int)tp;
  hb.no = (int)to;
  hb.prob.resize(n);
  hb.obs_cam.resize(to);
  hb.obs_pt.resize(to);
  hb.obs_uv.resize(2 * to);
  hb.obs_seg.resize(to);
  hb.obs_slot.resize(to);
  hb.obs_orig.resize(to);
  hb.pt_obs_begin.assign(tp + 1, 0);
  hb.pt_problem.resize(tp);
  hb.cam_problem.resize(tc);
  hb.pt_used.resize(tp);
  hb.cam_used.assign(tc, 0);
  hb.pt_orig.resize(tp);
  hb.cam_param.resize(9 * tc);
  hb.pt_param.resize(4 * tp);
  hb.cam_obs_begin.assign(tc + 1, 0);
  hb.cam_obs_list.resize(to);

  int cam0 = 0, pt0 = 0, obs0 = 0;
  std::vector<int32_t> deg, key, order, inv, fill, part_deg, part_key;
  std::vector<uint8_t> part_used;
  for (int p = 0; p < n; ++p) {
    const gba_problem_view &v = views[p];
    const int nc = v.num_cameras, np = v.num_points, no = v.num_observations;
    ProblemInfo &pi = hb.prob[p];
    pi.cam_begin = cam0;
    pi.cam_count = nc;
    pi.pt_begin = pt0;
    pi.pt_count = np;
    pi.obs_begin = obs0;
    pi.obs_count = no;
    pi.chunk_begin = (int)hb.chunk.size();
    // degrees, first camera of each point.  A large problem takes runs of
    // its observations on host threads, each counting into its own
    // per-point arrays (merged over the runs); the same runs then place
    // their observations in the points' ranges after the earlier runs', so
    // each point keeps its input order as in one sequential pass.
    const long long runs =
        std::min<long long>({(long long)host_threads(), (long long)no / 16384, (1LL << 22) / std::max(1, np)});
    auto run_begin = [&](long long r) { return (int)((long long)no * r / runs); };
    deg.assign(np, 0);
    key.assign(np, nc);
    if (runs > 1) {
      part_deg.assign((size_t)runs * np, 0);
      part_key.assign((size_t)runs * np, nc);
      part_used.assign((size_t)runs * nc, 0);
      host_parallel((int)runs, [&](int r) {
        int32_t *d = part_deg.data() + (size_t)r * np, *k = part_key.data() + (size_t)r * np;
        uint8_t *u = part_used.data() + (size_t)r * nc;
        for (int i = run_begin(r); i < run_begin(r + 1); ++i) {
          const int c = v.camera_index[i], j = v.point_index[i];
          ++d[j];
          if (c < k[j]) k[j] = c;
          u[c] = 1;
        }
      });
      parallel_runs(np, 8192, [&](long long j0, long long j1) {
        for (long long j = j0; j < j1; ++j) {
          int32_t dj = 0, kj = nc;
          for (long long r = 0; r < runs; ++r) {
            dj += part_deg[(size_t)r * np + j];
            kj = std::min(kj, part_key[(size_t)r * np + j]);
          }
          deg[j] = dj;
          key[j] = kj;
        }
      });
      for (int c = 0; c < nc; ++c)
        for (long long r = 0; r < runs; ++r) hb.cam_used[cam0 + c] |= part_used[(size_t)r * nc + c];
    } else {
      for (int i = 0; i < no; ++i) {
        const int c = v.camera_index[i], j = v.point_index[i];
        ++deg[j];
        if (c < key[j]) key[j] = c;
        hb.cam_used[cam0 + c] = 1;
      }
    }
    // internal point order: by first camera (locality of the camera
    // segments in the chunk kernels), stable in the input index
    order.resize(np);
    if (opt.reorder_points) {
      fill.assign(nc + 2, 0);
      for (int j = 0; j < np; ++j) ++fill[key[j] + 1];
      for (int c = 0; c <= nc; ++c) fill[c + 1] += fill[c];
      for (int j = 0; j < np; ++j) order[fill[key[j]]++] = j;
    } else {
      for (int j = 0; j < np; ++j) order[j] = j;
    }
    inv.resize(np);
    // CSR by internal point, observations stable in input index
    parallel_runs(np, 8192, [&](long long j0, long long j1) {
      for (int ji = (int)j0; ji < (int)j1; ++ji) {
        const int j = order[ji];
        inv[j] = ji;
        hb.pt_orig[pt0 + ji] = j;
        hb.pt_problem[pt0 + ji] = p;
        hb.pt_used[pt0 + ji] = deg[j] > 0;
        hb.pt_obs_begin[pt0 + ji + 1] = deg[j];
        double *x = hb.pt_param.data() + 4 * (size_t)(pt0 + ji);
        for (int q = 0; q < 3; ++q) x[q] = v.parameters[9 * (size_t)nc + 3 * (size_t)j + q];
        x[3] = 0.0;
      }
    });
    hb.pt_obs_begin[pt0] = obs0;
    for (int ji = 0; ji < np; ++ji) hb.pt_obs_begin[pt0 + ji + 1] += hb.pt_obs_begin[pt0 + ji];
    if (runs > 1) {
      // per (run, point): where the run's observations of the point start
      parallel_runs(np, 8192, [&](long long j0, long long j1) {
        for (long long j = j0; j < j1; ++j) {
          int32_t base = hb.pt_obs_begin[pt0 + inv[j]];
          for (long long r = 0; r < runs; ++r) {
            const int32_t d = part_deg[(size_t)r * np + j];
            part_deg[(size_t)r * np + j] = base;
            base += d;
          }
        }
      });
      host_parallel((int)runs, [&](int r) {
        int32_t *at = part_deg.data() + (size_t)r * np;
        for (int i = run_begin(r); i < run_begin(r + 1); ++i) hb.obs_orig[at[v.point_index[i]]++] = i;
      });
    } else {
      fill.assign(hb.pt_obs_begin.begin() + pt0, hb.pt_obs_begin.begin() + pt0 + np + 1);
      for (int i = 0; i < no; ++i) hb.obs_orig[fill[inv[v.point_index[i]]]++] = i;
    }
    // within a point: by camera, then input index (insertion sort, stable);
    // points and observations are independent (host threads)
    parallel_runs(np, 20000, [&](long long j0, long long j1) {
      for (int ji = (int)j0; ji < (int)j1; ++ji) {
        const int b = hb.pt_obs_begin[pt0 + ji], e = hb.pt_obs_begin[pt0 + ji + 1];
        for (int k = b + 1; k < e; ++k) {
          const int x = hb.obs_orig[k];
          const int cx = v.camera_index[x];
          int m = k - 1;
          while (m >= b && v.camera_index[hb.obs_orig[m]] > cx) {
            hb.obs_orig[m + 1] = hb.obs_orig[m];
            --m;
          }
          hb.obs_orig[m + 1] = x;
        }
      }
    });
    parallel_runs(no, 50000, [&](long long k0, long long k1) {
      for (int k = obs0 + (int)k0; k < obs0 + (int)k1; ++k) {
        const int i = hb.obs_orig[k];
        hb.obs_cam[k] = cam0 + v.camera_index[i];
        hb.obs_pt[k] = pt0 + inv[v.point_index[i]];
        hb.obs_uv[2 * (size_t)k] = v.observations[2 * (size_t)i];
        hb.obs_uv[2 * (size_t)k + 1] = v.observations[2 * (size_t)i + 1];
      }
    });
    for (int c = 0; c < nc; ++c) hb.cam_problem[cam0 + c] = p;
    if (nc > 0) std::memcpy(hb.cam_param.data() + 9 * (size_t)cam0, v.parameters, sizeof(double) * 9 * (size_t)nc);
    // chunks of whole points (their camera orders below, for the whole batch)
    int ji = 0;
    while (ji < np) {
      ChunkInfo ci;
      std::memset(&ci, 0, sizeof ci);
      ci.problem = p;
      ci.pt_begin = pt0 + ji;
      ci.obs_begin = hb.pt_obs_begin[pt0 + ji];
      int nobs = 0, npts = 0;
      while (ji < np && npts < cap) {
        const int d = hb.pt_obs_begin[pt0 + ji + 1] - hb.pt_obs_begin[pt0 + ji];
        if (d > cap) {
          *err = fmt("point %lld is observed %lld times; at most %lld observations per point are supported",
                     order[ji], d, cap);
          return GBA_ERR_INVALID_ARGUMENT;
        }
        if (nobs + d > cap) break;
        nobs += d;
        ++npts;
        ++ji;
      }
      ci.obs_count = nobs;
      ci.pt_count = npts;
      hb.chunk.push_back(ci);
    }
    pi.chunk_count = (int)hb.chunk.size() - pi.chunk_begin;
    // camera blocks of the PCG kernels
    pi.cam_block_begin = (int)hb.camblk.size();
    for (int c = 0; c < nc; c += kPcgBlockCams) {
      int4 b;
      b.x = p;
      b.y = cam0 + c;
      b.z = std::min(kPcgBlockCams, nc - c);
      b.w = 0;
      hb.camblk.push_back(b);
    }
    pi.cam_block_count = (int)hb.camblk.size() - pi.cam_block_begin;
    cam0 += nc;
    pt0 += np;
    obs0 += no;
  }
  hb.nchunks = (int)hb.chunk.size();
  hb.cam_blocks = (int)hb.camblk.size();
  // per chunk, the camera-sorted order of its observations, stable: the
  // chunk's distinct cameras (a stamped table), sorted, then each
  // observation's position from its camera's running count.  Two passes
  // over runs of chunks: the segment counts, then (at their offsets) the
  // segments and the orders.
  const int nch = hb.nchunks;
  const long long chunk_runs = std::max<long long>(1, std::min<long long>(4LL * host_threads(), (long long)to / 16384));
  std::vector<int32_t> seg_off(nch + 1, 0);
  {
    const long long st = new_stamps();
    host_parallel((int)chunk_runs, [&](int r) {
      CamScratch &s = cam_scratch((int)tc);
      for (int ch = (int)((long long)nch * r / chunk_runs); ch < (int)((long long)nch * (r + 1) / chunk_runs); ++ch) {
        const ChunkInfo &ci = hb.chunk[ch];
        const long long mk = st | ch;
        int segs = 0;
        for (int k = 0; k < ci.obs_count; ++k) {
          const int cam = hb.obs_cam[ci.obs_begin + k];
          if (s.mark[cam] != mk) s.mark[cam] = mk, ++segs;
        }
        seg_off[ch + 1] = segs;
      }
    });
  }
  for (int ch = 0; ch < nch; ++ch) seg_off[ch + 1] += seg_off[ch];
  hb.nseg = seg_off[nch];
  hb.seg_pos.resize(hb.nseg);
  hb.seg_cam.resize(hb.nseg);
  {
    const long long st = new_stamps();
    host_parallel((int)chunk_runs, [&](int r) {
      CamScratch &s = cam_scratch((int)tc);
      std::vector<int32_t> distinct;
      int32_t *count = s.a.data(), *start = s.b.data(), *segi = s.c.data();
      for (int ch = (int)((long long)nch * r / chunk_runs); ch < (int)((long long)nch * (r + 1) / chunk_runs); ++ch) {
        ChunkInfo &ci = hb.chunk[ch];
        const long long mk = st | ch;
        distinct.clear();
        for (int k = 0; k < ci.obs_count; ++k) {
          const int cam = hb.obs_cam[ci.obs_begin + k];
          if (s.mark[cam] != mk) s.mark[cam] = mk, count[cam] = 0, distinct.push_back(cam);
          ++count[cam];
        }
        std::sort(distinct.begin(), distinct.end());
        ci.seg_begin = seg_off[ch];
        ci.seg_count = (int)distinct.size();
        for (int sg = 0, pos = 0; sg < ci.seg_count; ++sg) {
          const int cam = distinct[sg];
          hb.seg_pos[ci.seg_begin + sg] = (uint16_t)pos;
          hb.seg_cam[ci.seg_begin + sg] = cam;
          start[cam] = pos;
          segi[cam] = sg;
          pos += count[cam];
        }
        for (int k = 0; k < ci.obs_count; ++k) {
          const int cam = hb.obs_cam[ci.obs_begin + k];
          hb.obs_slot[ci.obs_begin + k] = (uint16_t)start[cam]++;
          hb.obs_seg[ci.obs_begin + k] = (uint16_t)segi[cam];
        }
      }
    });
  }
  for (int p = 0; p < n; ++p) {
    ProblemInfo &pi = hb.prob[p];
    pi.seg_begin = seg_off[pi.chunk_begin];
    pi.seg_count = seg_off[pi.chunk_begin + pi.chunk_count] - pi.seg_begin;
  }
  // per camera: its segments (chunk order) and its observations (internal order)
  hb.cam_seg_begin.assign(hb.nc + 1, 0);
  for (int s = 0; s < hb.nseg; ++s) ++hb.cam_seg_begin[hb.seg_cam[s] + 1];
  for (int c = 0; c < hb.nc; ++c) hb.cam_seg_begin[c + 1] += hb.cam_seg_begin[c];
  // each segment's partial goes to its camera-major position, so a camera's
  // partials are contiguous for the camera reduce
  hb.seg_slot.resize(hb.nseg);
  fill.assign(hb.cam_seg_begin.begin(), hb.cam_seg_begin.end());
  for (int s = 0; s < hb.nseg; ++s) hb.seg_slot[s] = fill[hb.seg_cam[s]]++;
  // explicit Schur complement: chosen by the option, AUTO when a point's
  // ordered observation pairs (sum over points of m (m - 1)) are at most
  // kExplicitPairsPerObs per observation (forming S then costs less than the
  // implicit mat-vec saves over a PCG solve)
  {
    std::atomic<long long> pairs{0};
    parallel_runs(hb.np, kParMin, [&](long long j0, long long j1) {
      long long s = 0;
      for (long long j = j0; j < j1; ++j) {
        const long long m = hb.pt_obs_begin[j + 1] - hb.pt_obs_begin[j];
        s += m * (m - 1);
      }
      pairs.fetch_add(s, std::memory_order_relaxed);
    });
    hb.explicit_schur = opt.schur == GBA_SCHUR_EXPLICIT ||
                        (opt.schur == GBA_SCHUR_AUTO && pairs.load() <= kExplicitPairsPerObs * (long long)hb.no);
    if (hb.explicit_schur && pairs.load() > kExplicitPairsMax) {
      *err = fmt("the explicit Schur complement needs %lld observation pairs; at most %lld are supported",
                 pairs.load(), (long long)kExplicitPairsMax);
      return GBA_ERR_INVALID_ARGUMENT;
    }
    // the FP64 explicit form sums a problem's cameras' p.q in chunks of 32
    // held in shared memory: at most 32 kPcgChunkSums cameras a problem
    int most_cams = 0;
    for (const ProblemInfo &pi : hb.prob) most_cams = std::max(most_cams, (int)pi.cam_count);
    if (most_cams > 32 * kPcgChunkSums) {
      if (opt.schur == GBA_SCHUR_EXPLICIT) {
        *err = fmt("the explicit Schur complement supports problems of at most %d cameras", 32 * kPcgChunkSums);
        return GBA_ERR_INVALID_ARGUMENT;
      }
      hb.explicit_schur = false;
    }
  }
  // each camera's observations in internal order: a stable counting sort by
  // camera over runs of observations (per-run counts, then offsets)
  {
    const long long runs = std::min<long long>(std::max<long long>(1, to / kParMin), 2LL * host_threads());
    if (runs <= 1 || runs * tc > (1LL << 24)) {
      for (int k = 0; k < hb.no; ++k) ++hb.cam_obs_begin[hb.obs_cam[k] + 1];
      for (int c = 0; c < hb.nc; ++c) hb.cam_obs_begin[c + 1] += hb.cam_obs_begin[c];
      fill.assign(hb.cam_obs_begin.begin(), hb.cam_obs_begin.end());
      for (int k = 0; k < hb.no; ++k) hb.cam_obs_list[fill[hb.obs_cam[k]]++] = k;
    } else {
      std::vector<int32_t> cnt((size_t)runs * tc, 0);
      host_parallel((int)runs, [&](int r) {
        int32_t *c = cnt.data() + (size_t)r * tc;
        for (long long k = to * r / runs; k < to * (r + 1) / runs; ++k) ++c[hb.obs_cam[k]];
      });
      long long acc = 0;
      for (long long c = 0; c < tc; ++c) {
        hb.cam_obs_begin[c] = (int32_t)acc;
        for (long long r = 0; r < runs; ++r) {
          const int32_t x = cnt[(size_t)r * tc + c];
          cnt[(size_t)r * tc + c] = (int32_t)acc;
          acc += x;
        }
      }
      hb.cam_obs_begin[tc] = (int32_t)acc;
      host_parallel((int)runs, [&](int r) {
        int32_t *c = cnt.data() + (size_t)r * tc;
        for (long long k = to * r / runs; k < to * (r + 1) / runs; ++k) hb.cam_obs_list[c[hb.obs_cam[k]]++] = (int32_t)k;
      });
    }
  }
  hb.cam_piece_begin.assign((size_t)tc + 1, 0);
  for (long long c = 0; c < tc; ++c) {
    const int n = hb.cam_obs_begin[c + 1] - hb.cam_obs_begin[c];
    hb.cam_piece_begin[c + 1] = hb.cam_piece_begin[c] + std::max(1, (n + kCamPieceObs - 1) / kCamPieceObs);
  }
  if (hb.explicit_schur) build_schur_structure(&hb);
  return GBA_OK;
}

void set_resume(HostBatch &hb, int p, const ProblemState &st) {
  if (hb.resume.empty()) {
    hb.resume.assign((size_t)hb.P, 0);
    hb.resume_lm.assign((size_t)hb.P, LMState{});
    hb.resume_cam_scale.assign(9 * (size_t)hb.nc, 1.0);
    hb.resume_pt_scale.assign(3 * (size_t)hb.np, 1.0);
  }
  const ProblemInfo &pi = hb.prob[p];
  hb.resume[p] = 1;
  hb.resume_lm[p] = st.lm;
  std::copy(st.cam_scale.begin(), st.cam_scale.begin() + 9 * (size_t)pi.cam_count,
            hb.resume_cam_scale.begin() + 9 * (size_t)pi.cam_begin);
  for (int ji = 0; ji < pi.pt_count; ++ji) {
    const int j = hb.pt_orig[pi.pt_begin + ji];
    for (int q = 0; q < 3; ++q) hb.resume_pt_scale[3 * (size_t)(pi.pt_begin + ji) + q] = st.pt_scale[3 * (size_t)j + q];
  }
}

void gather_scales(const HostBatch &hb, int p, const double *cam_scale, const double *pt_scale, ProblemState *st) {
  const ProblemInfo &pi = hb.prob[p];
  st->cam_scale.assign(cam_scale + 9 * (size_t)pi.cam_begin, cam_scale + 9 * (size_t)(pi.cam_begin + pi.cam_count));
  st->pt_scale.assign(3 * (size_t)pi.pt_count, 1.0);
  for (int ji = 0; ji < pi.pt_count; ++ji) {
    const int j = hb.pt_orig[pi.pt_begin + ji];
    for (int q = 0; q < 3; ++q) st->pt_scale[3 * (size_t)j + q] = pt_scale[3 * (size_t)(pi.pt_begin + ji) + q];
  }
}

void scatter_parameters(const HostBatch &hb, int p, const double *cam_param, const double *pt_param,
                        double *out) {
  const ProblemInfo &pi = hb.prob[p];
  std::memcpy(out, cam_param + 9 * (size_t)pi.cam_begin, sizeof(double) * 9 * (size_t)pi.cam_count);
  double *pts = out + 9 * (size_t)pi.cam_count;
  parallel_runs(pi.pt_count, kParMin, [&](long long j0, long long j1) {
    for (long long ji = j0; ji < j1; ++ji) {
      const int j = hb.pt_orig[pi.pt_begin + ji];
      for (int q = 0; q < 3; ++q) pts[3 * (size_t)j + q] = pt_param[4 * (size_t)(pi.pt_begin + ji) + q];
    }
  });
}

}  // namespace gba
