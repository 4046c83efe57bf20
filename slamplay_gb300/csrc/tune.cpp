// tune.cpp — the autotuner behind gba_autotune: short timed trial solves of
// the caller's problem(s) on scratch engines, one knob after another: the
// launch shapes (point-segment tile x PCG iterations per graph body), the
// cameras per CTA of the cluster PCG, and (opted into) the PCG iteration
// cap.  The launch shapes change which thread adds which partial sum, never
// what is computed; a smaller PCG cap is kept only when its trial ends
// within 1e-6 relative of the configured cap's cost.
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
  int cap;  // the configured PCG cap when the cap is tuned, else 0
  bool operator<(const TuneKey &o) const {
    return std::tie(n, log_obs, log_cams, precision, cap) < std::tie(o.n, o.log_obs, o.log_cams, o.precision, o.cap);
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

TuneKey key_of(const gba_problem_view *v, int n, int precision, int cap) {
  long long obs = 0, cams = 0;
  for (int i = 0; i < n; ++i) {
    obs += v[i].num_observations;
    cams += v[i].num_cameras;
  }
  return TuneKey{n, ilog2(obs), ilog2(cams), precision, cap};
}

constexpr double kCapCostTol = 1e-6;  // a smaller PCG cap must end within this of the configured one

}  // namespace

gba_status autotune(Engine &target, const gba_problem_view *problems, int n, gba_tune_result *out,
                    std::string *err) {
  std::memset(out, 0, sizeof *out);
  const gba_options base = target.options();
  const bool tune_cap = base.autotune >= 2;
  const TuneKey key = key_of(problems, n, base.precision, tune_cap ? base.max_linear_solver_iterations : 0);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *out = it->second;
      out->num_trials = 0;
      out->from_cache = 1;
      target.set_tuning(out->chunk_observations, out->pcg_unroll, out->pcg_cameras_per_cta, out->pcg_cap,
                        out->pcg_grid_ctas);
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
  std::vector<gba_summary> sums(n);
  int t = 0;
  // one trial: the solve twice (the first run also builds the graph), the
  // second one's device time; the summed final cost
  auto trial = [&](Engine &eng, int step, int chunk, int unroll, int cams, int cap, int ctas, double *ms,
                   double *cost) -> gba_status {
    eng.set_tuning(chunk, unroll, cams, cap, ctas);
    for (int rep = 0; rep < 2; ++rep) {
      for (int i = 0; i < n; ++i)
        std::memcpy(params[i].data(), problems[i].parameters, params[i].size() * sizeof(double));
      std::memset(sums.data(), 0, sizeof(gba_summary) * sums.size());
      const gba_status st = eng.solve(views.data(), n, sums.data(), err);
      if (st != GBA_OK) return st;
      *ms = eng.last_solve_ms();
    }
    *cost = 0.0;
    for (const gba_summary &x : sums) *cost += x.final_cost;
    if (t < GBA_TUNE_MAX_TRIALS) {
      out->trial_ms[t] = *ms;
      out->trial_step[t] = step;
      out->trial_chunk[t] = chunk;
      out->trial_unroll[t] = unroll;
      out->trial_cameras_per_cta[t] = cams;
      out->trial_cap[t] = cap;
      out->trial_grid_ctas[t] = ctas;
      out->trial_final_cost[t] = *cost;
    }
    ++t;
    return GBA_OK;
  };
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
  gba_status st;
  {
    Engine eng(o);
    if ((st = eng.init(err)) != GBA_OK) return st;
    // 1. tile size x PCG iterations per graph body (one value when the PCG
    //    is one launch per LM iteration: the unroll has no effect there)
    const int chunks[] = {256, 192, 128};
    std::vector<int> unrolls = {1, 2, 4};
    double best = 1e300, ms = 0.0, cost = 0.0;
    for (int c : chunks)
      for (size_t k = 0; k < unrolls.size(); ++k) {
        const int u = unrolls[k];
        if ((st = trial(eng, 1, c, u, 0, 0, 0, &ms, &cost)) != GBA_OK) return st;
        if (eng.one_launch_pcg()) unrolls.assign(1, u);
        if (ms < best) {
          best = ms;
          out->chunk_observations = c;
          out->pcg_unroll = u;
          out->best_ms = ms;
        }
      }
    // 2. cameras per CTA of the cluster PCG, or the CTAs of the grid PCG
    //    (the defaults are step 1's best trial)
    if (eng.cluster_pcg()) {
      double best2 = best;
      for (int cams : {16, 32, 64}) {
        if ((st = trial(eng, 2, out->chunk_observations, out->pcg_unroll, cams, 0, 0, &ms, &cost)) != GBA_OK)
          return st;
        if (ms < best2) {
          best2 = ms;
          out->pcg_cameras_per_cta = cams;
        }
      }
    } else if (eng.grid_pcg_ctas() > 0) {
      const int full = eng.grid_pcg_ctas();
      double best2 = best;
      for (int ctas : {3 * full / 4, full / 2, full / 4}) {
        if (ctas < 1) continue;
        if ((st = trial(eng, 2, out->chunk_observations, out->pcg_unroll, 0, 0, ctas, &ms, &cost)) != GBA_OK)
          return st;
        if (ms < best2) {
          best2 = ms;
          out->pcg_grid_ctas = ctas;
        }
      }
    }
  }
  // 3. the PCG iteration cap, at the handle's PCG tolerance
  if (tune_cap) {
    gba_options oc = o;
    oc.max_num_iterations = 5;
    oc.max_linear_solver_iterations = base.max_linear_solver_iterations;
    Engine eng(oc);
    if ((st = eng.init(err)) != GBA_OK) return st;
    const int cap0 = std::max(1, (int)base.max_linear_solver_iterations);
    double ms0 = 0.0, cost0 = 0.0;
    if ((st = trial(eng, 3, out->chunk_observations, out->pcg_unroll, out->pcg_cameras_per_cta, cap0,
                    out->pcg_grid_ctas, &ms0, &cost0)) != GBA_OK)
      return st;
    out->pcg_cap = cap0;
    double best3 = ms0;
    for (int cap = cap0 / 2; cap >= 10; cap /= 2) {
      double ms = 0.0, cost = 0.0;
      if ((st = trial(eng, 3, out->chunk_observations, out->pcg_unroll, out->pcg_cameras_per_cta, cap,
                      out->pcg_grid_ctas, &ms, &cost)) != GBA_OK)
        return st;
      if (!(cost <= cost0 * (1.0 + kCapCostTol))) break;  // smaller caps go further off
      if (ms < best3) {
        best3 = ms;
        out->pcg_cap = cap;
      }
    }
  }
  out->num_trials = t;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = *out;
  }
  target.set_tuning(out->chunk_observations, out->pcg_unroll, out->pcg_cameras_per_cta, out->pcg_cap,
                    out->pcg_grid_ctas);
  return GBA_OK;
}

}  // namespace gba
