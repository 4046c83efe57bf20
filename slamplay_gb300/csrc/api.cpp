// api.cpp — the extern "C" surface of libgba (declared in include/gba.h).
#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "engine.h"
#include "gba.h"
#include "server.h"

struct gba_handle {
  std::unique_ptr<gba::Engine> engine;
  std::unique_ptr<gba::Server> server;
  std::string last_error;
};

namespace {
thread_local std::string g_create_error;

gba_status fail(gba_handle *h, gba_status st, const std::string &msg) {
  if (h) h->last_error = msg;
  return st;
}
}  // namespace

const char *gba_io_last_error(void);

namespace gba {
// The calling thread's handle-less error message (gba_last_error(NULL)).
std::string &thread_error_message() { return g_create_error; }
gba_status autotune(Engine &target, const gba_problem_view *problems, int n, gba_tune_result *out, std::string *err);
}  // namespace gba

namespace {
// gba_options.autotune: tune on the first solve of a new size bucket.
gba_status maybe_autotune(gba_handle *h, const gba_problem_view *p, int n, std::string *err) {
  const gba_options &o = h->engine->options();
  if (!o.autotune) return GBA_OK;
  gba_tune_result r;
  return gba::autotune(*h->engine, p, n, &r, err);
}
}  // namespace

extern "C" {

void gba_options_init(gba_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->abi_version = GBA_ABI_VERSION;
  o->max_num_iterations = 50;
  o->function_tolerance = 1e-6;
  o->gradient_tolerance = 1e-10;
  o->parameter_tolerance = 1e-8;
  o->initial_trust_region_radius = 1e4;
  o->max_trust_region_radius = 1e16;
  o->min_trust_region_radius = 1e-32;
  o->min_relative_decrease = 1e-3;
  o->min_lm_diagonal = 1e-6;
  o->max_lm_diagonal = 1e32;
  o->max_num_consecutive_invalid_steps = 5;
  o->jacobi_scaling = 1;
  o->loss = GBA_LOSS_TRIVIAL;
  o->loss_scale = 1.0;
  o->precision = GBA_PRECISION_FP64;
  o->pcg_criterion = GBA_PCG_RESIDUAL;
  o->max_linear_solver_iterations = 500;
  o->min_linear_solver_iterations = 0;
  o->pcg_tolerance = 1e-10;
  o->eta = 0.1;
  o->minimizer_progress_to_stdout = 0;
  o->device = 0;
  o->stream = nullptr;
  o->chunk_observations = 0;
  o->reorder_points = 1;
  o->use_graphs = 1;
  o->pcg_unroll = 0;
  o->autotune = 0;
  o->schur = GBA_SCHUR_AUTO;
  o->persistent_pcg = 1;
  o->camera_update = GBA_CAMERA_UPDATE_ADDITIVE;
  o->lm_policy = GBA_LM_POLICY_CERES;
}

void gba_local_ba_options_init(gba_options *o) {
  gba_options_init(o);
  o->lm_policy = GBA_LM_POLICY_G2O;  // OptimizationAlgorithmLevenberg, backend.cpp:71-74
  o->max_num_iterations = 10;        // optimizer.optimize(10), backend.cpp:152
  o->loss = GBA_LOSS_HUBER;          // RobustKernelHuber, delta 5.991, backend.cpp:137-139
  o->loss_scale = 5.991;
  o->function_tolerance = 0.0;
  o->gradient_tolerance = 0.0;
  o->parameter_tolerance = 0.0;
}

void gba_window_view_init(gba_window_view *w) {
  std::memset(w, 0, sizeof *w);
  w->chi2_threshold = 5.991;
  w->max_threshold_doublings = 5;
}

const char *gba_version(void) { return "gba 1 sm_103a"; }

gba_status gba_create(const gba_options *o, gba_handle **out) {
  if (!out) return GBA_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gba_options opt;
  if (o) {
    opt = *o;
    if (opt.abi_version != GBA_ABI_VERSION) {
      g_create_error = "gba_options.abi_version mismatch (call gba_options_init)";
      return GBA_ERR_INVALID_ARGUMENT;
    }
  } else {
    gba_options_init(&opt);
  }
  if (opt.max_num_iterations < 0 || opt.max_linear_solver_iterations < 0 || opt.loss < 0 || opt.loss > 2 ||
      opt.precision < 0 || opt.precision > 1 || opt.schur < 0 || opt.schur > 2 ||
      opt.camera_update < 0 || opt.camera_update > 1 || opt.lm_policy < 0 || opt.lm_policy > 1 ||
      opt.camera_layout < 0 || opt.camera_layout > 1 || opt.server_slots < 0 || opt.server_slots > 16 ||
      !(opt.initial_trust_region_radius > 0) ||
      !(opt.loss_scale > 0) || opt.max_num_consecutive_invalid_steps < 1) {
    g_create_error = "invalid solver options";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  gba_handle *h = new (std::nothrow) gba_handle();
  if (!h) return GBA_ERR_OUT_OF_MEMORY;
  h->engine.reset(new gba::Engine(opt));
  std::string err;
  const gba_status st = h->engine->init(&err);
  if (st != GBA_OK) {
    g_create_error = err;
    delete h;
    return st;
  }
  *out = h;
  return GBA_OK;
}

void gba_destroy(gba_handle *h) {
  if (!h) return;
  if (h->server) h->server->stop();
  delete h;
}

const char *gba_last_error(const gba_handle *h) {
  if (!h) return g_create_error.c_str();
  return h->last_error.c_str();
}

// Solves n problems; with the quaternion camera layout the cameras are
// converted to angle-axis copies first and the results converted back into
// the callers' arrays (BALProblem.cpp:117-138 loads and writes the same way).
static gba_status solve_nonempty(gba_handle *h, const gba_problem_view *problems, int32_t n, gba_summary *summaries,
                                 std::string *err) {
  if (h->engine->options().camera_layout != GBA_CAMERA_QUATERNION) {
    gba_status st = maybe_autotune(h, problems, n, err);
    if (st == GBA_OK) st = h->engine->solve(problems, n, summaries, err);
    return st;
  }
  std::vector<gba_problem_view> views(problems, problems + n);
  std::vector<std::vector<double>> aa((size_t)n);
  for (int32_t p = 0; p < n; ++p) {
    const gba_problem_view &v = problems[p];
    if (v.num_cameras < 0 || v.num_points < 0 || ((v.num_cameras > 0 || v.num_points > 0) && !v.parameters)) {
      *err = "invalid problem view";
      return GBA_ERR_INVALID_ARGUMENT;
    }
    const size_t nc = (size_t)v.num_cameras, np = (size_t)v.num_points;
    aa[p].resize(9 * nc + 3 * np);
    for (size_t c = 0; c < nc; ++c) {
      const double *q = v.parameters + 10 * c;
      gba_quaternion_to_angle_axis(q, &aa[p][9 * c]);
      std::copy(q + 4, q + 10, &aa[p][9 * c + 3]);
    }
    std::copy(v.parameters + 10 * nc, v.parameters + 10 * nc + 3 * np, aa[p].begin() + 9 * nc);
    views[p].parameters = aa[p].data();
  }
  gba_status st = maybe_autotune(h, views.data(), n, err);
  if (st == GBA_OK) st = h->engine->solve(views.data(), n, summaries, err);
  if (st != GBA_OK) return st;
  for (int32_t p = 0; p < n; ++p) {
    const gba_problem_view &v = problems[p];
    const size_t nc = (size_t)v.num_cameras, np = (size_t)v.num_points;
    for (size_t c = 0; c < nc; ++c) {
      double *q = v.parameters + 10 * c;
      gba_angle_axis_to_quaternion(&aa[p][9 * c], q);
      std::copy(&aa[p][9 * c + 3], &aa[p][9 * c + 9], q + 4);
    }
    std::copy(aa[p].begin() + 9 * nc, aa[p].begin() + 9 * nc + 3 * np, v.parameters + 10 * nc);
  }
  return GBA_OK;
}

// Problems without observations are answered on the host
// (empty_problem_summary); the others are solved together, in their order.
static gba_status solve_views(gba_handle *h, const gba_problem_view *problems, int32_t n, gba_summary *summaries,
                              std::string *err) {
  std::vector<int32_t> live;
  live.reserve((size_t)n);
  for (int32_t p = 0; p < n; ++p) {
    const gba_problem_view &v = problems[p];
    if (v.num_observations != 0) {
      live.push_back(p);
      continue;
    }
    const gba_status vs = gba::validate_problem(&v, err);
    if (vs != GBA_OK) return vs;
  }
  if ((int32_t)live.size() == n) return solve_nonempty(h, problems, n, summaries, err);
  if (!live.empty()) {
    std::vector<gba_problem_view> lv;
    std::vector<gba_summary> ls;
    for (int32_t p : live) {
      lv.push_back(problems[p]);
      if (summaries) ls.push_back(summaries[p]);
    }
    const gba_status st = solve_nonempty(h, lv.data(), (int32_t)lv.size(), summaries ? ls.data() : nullptr, err);
    if (st != GBA_OK) return st;
    if (summaries)
      for (size_t j = 0; j < live.size(); ++j) summaries[live[j]] = ls[j];
  }
  if (summaries) {
    const double radius = h->engine->options().initial_trust_region_radius;
    for (int32_t p = 0, j = 0; p < n; ++p) {
      if (j < (int32_t)live.size() && live[j] == p) {
        ++j;
        continue;
      }
      gba::empty_problem_summary(&summaries[p], radius);
    }
  }
  return GBA_OK;
}

gba_status gba_solve(gba_handle *h, const gba_problem_view *p, gba_summary *s) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (!p) return fail(h, GBA_ERR_INVALID_ARGUMENT, "null problem");
  if (h->server && h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "handle is serving");
  std::string err;
  const gba_status st = solve_views(h, p, 1, s, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_batch_solve(gba_handle *h, const gba_problem_view *problems, int32_t n, gba_summary *summaries) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (!problems || n <= 0) return fail(h, GBA_ERR_INVALID_ARGUMENT, "empty batch");
  if (h->server && h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "handle is serving");
  std::string err;
  const gba_status st = solve_views(h, problems, n, summaries, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_local_ba(gba_handle *h, gba_window_view *windows, int32_t n, gba_summary *summaries,
                        gba_window_result *results) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (h->engine->options().camera_layout == GBA_CAMERA_QUATERNION)
    return fail(h, GBA_ERR_INVALID_ARGUMENT, "the quaternion camera layout is taken by gba_solve and gba_batch_solve only");
  if (!windows || n <= 0) return fail(h, GBA_ERR_INVALID_ARGUMENT, "empty batch");
  if (h->server && h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "handle is serving");
  std::string err;
  const gba_status st = h->engine->solve_windows(windows, n, summaries, results, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_autotune(gba_handle *h, const gba_problem_view *problems, int32_t n, gba_tune_result *result) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (!problems || n <= 0 || !result) return fail(h, GBA_ERR_INVALID_ARGUMENT, "empty batch or null result");
  if (h->server && h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "handle is serving");
  for (int i = 0; i < n; ++i) {
    std::string verr;
    const gba_status vs = gba::validate_problem(&problems[i], &verr);
    if (vs != GBA_OK) return fail(h, vs, verr);
  }
  std::string err;
  const gba_status st = gba::autotune(*h->engine, problems, n, result, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_evaluate(gba_handle *h, const gba_problem_view *p, double *residuals, double *jacobians,
                        double *cost) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (h->engine->options().camera_layout == GBA_CAMERA_QUATERNION)
    return fail(h, GBA_ERR_INVALID_ARGUMENT, "the quaternion camera layout is taken by gba_solve and gba_batch_solve only");
  if (!p) return fail(h, GBA_ERR_INVALID_ARGUMENT, "null problem");
  std::string err;
  const gba_status st = h->engine->evaluate(p, residuals, jacobians, cost, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_compute_step(gba_handle *h, const gba_problem_view *p, double radius, double *delta,
                            double *model_cost_change, int32_t *pcg_iterations) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (h->engine->options().camera_layout == GBA_CAMERA_QUATERNION)
    return fail(h, GBA_ERR_INVALID_ARGUMENT, "the quaternion camera layout is taken by gba_solve and gba_batch_solve only");
  if (!p || !delta || !(radius > 0)) return fail(h, GBA_ERR_INVALID_ARGUMENT, "invalid step arguments");
  std::string err;
  int it = 0;
  const gba_status st = h->engine->compute_step(p, radius, delta, model_cost_change, &it, &err);
  if (pcg_iterations) *pcg_iterations = it;
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_solve_resident(gba_handle *h, int32_t repeats) {
  if (!h || repeats < 0) return GBA_ERR_INVALID_ARGUMENT;
  std::string err;
  for (int32_t r = 0; r < repeats; ++r) {
    const gba_status st = h->engine->rerun(&err);
    if (st != GBA_OK) return fail(h, st, err);
  }
  return GBA_OK;
}

gba_status gba_synchronize(gba_handle *h) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  const cudaError_t e = cudaStreamSynchronize(h->engine->stream());
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(h, GBA_ERR_CUDA, cudaGetErrorString(e));
  }
  return GBA_OK;
}

gba_status gba_set_profiling(gba_handle *h, int32_t on) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  h->engine->set_profiling(on != 0);
  return GBA_OK;
}

int32_t gba_profile_count(const gba_handle *h) { return h ? (int32_t)h->engine->profile().size() : 0; }

gba_status gba_profile_entry(const gba_handle *h, int32_t i, const char **name, int64_t *launches,
                             double *total_ms, double *bytes) {
  if (!h || i < 0 || i >= (int32_t)h->engine->profile().size()) return GBA_ERR_INVALID_ARGUMENT;
  const gba::ProfileEntry &e = h->engine->profile()[i];
  if (name) *name = e.name.c_str();
  if (launches) *launches = e.launches;
  if (total_ms) *total_ms = e.total_ms;
  if (bytes) *bytes = e.bytes;
  return GBA_OK;
}

size_t gba_estimate_footprint(int32_t nc, int32_t np, int32_t no, int32_t precision) {
  return gba::Server::estimate_footprint(nc, np, no, precision == GBA_PRECISION_MIXED, true);
}

gba_status gba_server_start(gba_handle *h, size_t budget, int32_t max_live, int32_t max_queue) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (h->server && h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "server already running");
  h->server.reset(new gba::Server(h->engine->options()));
  std::string err;
  const gba_status st = h->server->start(budget, max_live, max_queue, &err);
  if (st != GBA_OK) {
    h->server.reset();
    return fail(h, st, err);
  }
  return GBA_OK;
}

gba_status gba_submit(gba_handle *h, const gba_problem_view *p, uint64_t *ticket) {
  if (!h || !ticket) return GBA_ERR_INVALID_ARGUMENT;
  if (h->engine->options().camera_layout == GBA_CAMERA_QUATERNION)
    return fail(h, GBA_ERR_INVALID_ARGUMENT, "the quaternion camera layout is taken by gba_solve and gba_batch_solve only");
  if (!h->server || !h->server->running()) return fail(h, GBA_ERR_INVALID_ARGUMENT, "server not started");
  std::string err;
  const gba_status st = h->server->submit(p, ticket, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_poll(gba_handle *h, uint64_t ticket, gba_summary *s, int32_t *done) {
  if (!h || !done) return GBA_ERR_INVALID_ARGUMENT;
  if (!h->server) return fail(h, GBA_ERR_INVALID_ARGUMENT, "server not started");
  std::string err;
  const gba_status st = h->server->poll(ticket, s, done, &err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_server_stop(gba_handle *h) {
  if (!h) return GBA_ERR_INVALID_ARGUMENT;
  if (!h->server) return GBA_OK;
  std::string err;
  const gba_status st = h->server->drain_and_stop(&err);
  if (st != GBA_OK) return fail(h, st, err);
  return GBA_OK;
}

gba_status gba_server_get_stats(gba_handle *h, gba_server_stats *st) {
  if (!h || !st) return GBA_ERR_INVALID_ARGUMENT;
  std::memset(st, 0, sizeof *st);
  if (h->server) h->server->stats(st);
  return GBA_OK;
}

}  // extern "C"
