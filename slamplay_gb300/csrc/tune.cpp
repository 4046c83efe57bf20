// tune.cpp — the autotuner behind gba_autotune: short timed trial solves of
// the caller's problem(s) over a grid of launch shapes on a scratch engine.
// The shapes change which thread adds which partial sum, never what is
// computed, so every choice solves the same problem; only the speed differs.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.h"
#include "gba.h"

namespace gba {

namespace {

struct TuneKey {
  int n, log_obs, log_cams, precision;
  bool operator<(const TuneKey &o) const {
    return std::tie(n, log_obs, log_cams, precision) < std::tie(o.n, o.log_obs, o.log_cams, o.precision);
  }
};

std::mutex g_tune_mu;
std::map<TuneKey, gba_tune_result> g_tune_cache;

int ilog2(long long v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    ++r;
  }
  return r;
}

TuneKey key_of(const gba_problem_view *v, int n, int precision) {
  long long obs = 0, cams = 0;
  for (int i = 0; i < n; ++i) {
    obs += v[i].num_observations;
    cams += v[i].num_cameras;
  }
  return TuneKey{n, ilog2(obs), ilog2(cams), precision};
}

}  // namespace

gba_status autotune(Engine &target, const gba_problem_view *problems, int n, gba_tune_result *out,
                    std::string *err) {
  std::memset(out, 0, sizeof *out);
  const gba_options base = target.options();
  const TuneKey key = key_of(problems, n, base.precision);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *out = it->second;
      out->num_trials = 0;
      out->from_cache = 1;
      target.set_tuning(out->chunk_observations, out->pcg_unroll);
      return GBA_OK;
    }
  }
  // the trial solves write into private copies of the parameter arrays
  std::vector<std::vector<double>> params(n);
  std::vector<gba_problem_view> views(problems, problems + n);
  for (int i = 0; i < n; ++i) {
    const size_t np = 9 * (size_t)views[i].num_cameras + 3 * (size_t)views[i].num_points;
    params[i].assign(views[i].parameters, views[i].parameters + np);
    views[i].parameters = params[i].data();
  }
  gba_options o = base;
  o.max_num_iterations = 3;
  o.function_tolerance = 0.0;
  o.gradient_tolerance = 0.0;
  o.parameter_tolerance = 0.0;
  o.max_linear_solver_iterations = std::min(20, std::max(1, (int)base.max_linear_solver_iterations));
  o.minimizer_progress_to_stdout = 0;
  o.use_graphs = 1;
  o.autotune = 0;
  o.stream = nullptr;
  Engine eng(o);
  gba_status st = eng.init(err);
  if (st != GBA_OK) return st;
  const int chunks[] = {256, 192, 128};
  const int unrolls[] = {1, 2, 4};
  std::vector<gba_summary> sums(n);
  double best = 1e300;
  int t = 0;
  for (int c : chunks)
    for (int u : unrolls) {
      eng.set_tuning(c, u);
      double ms = 1e300;
      for (int rep = 0; rep < 2; ++rep) {  // the first run also builds the graph
        for (int i = 0; i < n; ++i)
          std::memcpy(params[i].data(), problems[i].parameters, params[i].size() * sizeof(double));
        std::memset(sums.data(), 0, sizeof(gba_summary) * sums.size());
        st = eng.solve(views.data(), n, sums.data(), err);
        if (st != GBA_OK) return st;
        ms = eng.last_solve_ms();
      }
      if (t < GBA_TUNE_MAX_TRIALS) {
        out->trial_ms[t] = ms;
        out->trial_chunk[t] = c;
        out->trial_unroll[t] = u;
      }
      ++t;
      if (ms < best) {
        best = ms;
        out->chunk_observations = c;
        out->pcg_unroll = u;
        out->best_ms = ms;
      }
    }
  out->num_trials = t;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = *out;
  }
  target.set_tuning(out->chunk_observations, out->pcg_unroll);
  return GBA_OK;
}

bool tune_cached(const gba_problem_view *problems, int n, int precision) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune_cache.count(key_of(problems, n, precision)) != 0;
}

}  // namespace gba
