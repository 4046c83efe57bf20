"""GPU bundle-adjustment solver: the Python side of include/gba.h.

``solve_ba(bal_problem)`` is the drop-in for the reference's
``void SolveBA(BALProblem&)`` (backend/slam_ba_simple_g2o_ceres/
test_bundle_adjustment_ceres.cpp:58-101): one Snavely residual block per
observation with HuberLoss(1.0), Levenberg-Marquardt with the points
eliminated, parameters updated in place, and a report of the fields
Ceres' ``Summary::FullReport()`` prints.
"""
from __future__ import annotations

import dataclasses
from typing import Sequence

import numpy as np

from . import _native as N
from .bal_problem import BALProblem


@dataclasses.dataclass
class SolveSummary:
    initial_cost: float
    final_cost: float
    num_iterations: int
    num_successful_steps: int
    num_unsuccessful_steps: int
    num_invalid_steps: int
    num_linear_solver_iterations: int
    termination_type: str
    termination_reason: str
    final_trust_region_radius: float
    gradient_max_norm: float
    setup_time_s: float
    solve_time_s: float
    total_time_s: float
    trace_cost: np.ndarray
    trace_radius: np.ndarray
    trace_linear_iterations: np.ndarray
    trace_successful: np.ndarray

    def FullReport(self) -> str:
        return (
            "GB300 bundle adjustment report\n"
            f"  Initial cost          {self.initial_cost:.6e}\n"
            f"  Final cost            {self.final_cost:.6e}\n"
            f"  Change                {self.initial_cost - self.final_cost:.6e}\n"
            f"  Minimizer iterations  {self.num_iterations}\n"
            f"  Successful steps      {self.num_successful_steps}\n"
            f"  Unsuccessful steps    {self.num_unsuccessful_steps}\n"
            f"  Linear solver iters   {self.num_linear_solver_iterations}\n"
            f"  Solve time (s)        {self.solve_time_s:.6f}\n"
            f"  Total time (s)        {self.total_time_s:.6f}\n"
            f"  Termination           {self.termination_type} ({self.termination_reason})\n")


class _Trace:
    def __init__(self, cap: int):
        self.cost = np.zeros(cap)
        self.radius = np.zeros(cap)
        self.lin = np.zeros(cap, np.int32)
        self.succ = np.zeros(cap, np.int32)

    def attach(self, s: N.Summary) -> None:
        s.trace_capacity = len(self.cost)
        s.trace_cost = N.f64p(self.cost)
        s.trace_radius = N.f64p(self.radius)
        s.trace_linear_iterations = N.i32p(self.lin)
        s.trace_successful = N.i32p(self.succ)


def _summary(s: N.Summary, tr: _Trace | None) -> SolveSummary:
    n = s.trace_length if tr is not None else 0
    return SolveSummary(
        initial_cost=s.initial_cost, final_cost=s.final_cost, num_iterations=s.num_iterations,
        num_successful_steps=s.num_successful_steps, num_unsuccessful_steps=s.num_unsuccessful_steps,
        num_invalid_steps=s.num_invalid_steps, num_linear_solver_iterations=s.num_linear_solver_iterations,
        termination_type=N.TERMINATION.get(s.termination_type, str(s.termination_type)),
        termination_reason=N.REASON.get(s.termination_reason, str(s.termination_reason)),
        final_trust_region_radius=s.final_trust_region_radius, gradient_max_norm=s.gradient_max_norm,
        setup_time_s=s.setup_time_s, solve_time_s=s.solve_time_s, total_time_s=s.total_time_s,
        trace_cost=tr.cost[:n].copy() if tr else np.zeros(0),
        trace_radius=tr.radius[:n].copy() if tr else np.zeros(0),
        trace_linear_iterations=tr.lin[:n].copy() if tr else np.zeros(0, np.int32),
        trace_successful=tr.succ[:n].copy() if tr else np.zeros(0, np.int32))


def make_options(**kw) -> N.Options:
    """gba_options with Ceres' defaults, overridden by keyword (loss,
    precision, pcg_criterion, schur, camera_update, lm_policy and
    camera_layout accept names: loss='huber', precision='mixed',
    schur='explicit', camera_update='so3_left', lm_policy='g2o',
    camera_layout='quaternion')."""
    o = N.Options()
    N.lib().gba_options_init(N.C.byref(o))
    for k, v in kw.items():
        if k == "loss" and isinstance(v, str):
            v = N.LOSS[v]
        elif k == "precision" and isinstance(v, str):
            v = N.PRECISION[v]
        elif k == "pcg_criterion" and isinstance(v, str):
            v = N.PCG_CRITERION[v]
        elif k == "schur" and isinstance(v, str):
            v = N.SCHUR[v]
        elif k == "camera_update" and isinstance(v, str):
            v = N.CAMERA_UPDATE[v]
        elif k == "lm_policy" and isinstance(v, str):
            v = N.LM_POLICY[v]
        elif k == "camera_layout" and isinstance(v, str):
            v = N.CAMERA_LAYOUT[v]
        elif k == "stream" and v is not None and not isinstance(v, int):
            v = int(v)
        if not hasattr(o, k):
            raise TypeError(f"unknown solver option {k!r}")
        setattr(o, k, v)
    return o


class Solver:
    """One GPU solver handle (gba_handle): a CUDA stream, a device workspace
    reused across solves and the cached LM graph."""

    def __init__(self, **options):
        self.options = make_options(**options)
        h = N.C.c_void_p()
        N.check(N.lib().gba_create(N.C.byref(self.options), N.C.byref(h)), None, "gba_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().gba_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _cap(self) -> int:
        # one trace row per LM trial: g2o's policy runs up to 10 per iteration
        per = 10 if self.options.lm_policy == N.LM_POLICY["g2o"] else 1
        return max(1, self.options.max_num_iterations * per + 1)

    def _view(self, problem: BALProblem) -> N.ProblemView:
        quat = self.options.camera_layout == N.CAMERA_LAYOUT["quaternion"]
        if problem.use_quaternions != quat:
            raise ValueError("the problem's camera layout (use_quaternions=%s) differs from the solver's "
                             "camera_layout option" % problem.use_quaternions)
        return problem.view(allow_quaternions=quat)

    def solve(self, problem: BALProblem) -> SolveSummary:
        """ceres::Solve replacement; problem.parameters() updated in place.
        A use_quaternions problem needs camera_layout='quaternion'."""
        v = self._view(problem)
        s = N.Summary()
        tr = _Trace(self._cap())
        tr.attach(s)
        N.check(N.lib().gba_solve(self._h, N.C.byref(v), N.C.byref(s)), self._h, "gba_solve")
        return _summary(s, tr)

    def batch_solve(self, problems: Sequence[BALProblem]) -> list[SolveSummary]:
        n = len(problems)
        views = (N.ProblemView * n)(*[self._view(p) for p in problems])
        sums = (N.Summary * n)()
        trs = [_Trace(self._cap()) for _ in range(n)]
        for s, t in zip(sums, trs):
            t.attach(s)
        N.check(N.lib().gba_batch_solve(self._h, views, n, sums), self._h, "gba_batch_solve")
        return [_summary(s, t) for s, t in zip(sums, trs)]

    def local_ba(self, windows, chi2_threshold: float = 5.991, max_threshold_doublings: int = 5):
        """Solves local-BA windows (slamplay_gb300.window.LocalBAWindow; one
        or a list, solved as one batch) in place and runs full_slam's outlier
        test on each (full_slam/src/backend.cpp:67-199).  Returns, per window,
        (summary, {"num_inliers", "num_outliers", "chi2_threshold",
        "outlier": uint8 per observation})."""
        single = not isinstance(windows, (list, tuple))
        ws = [windows] if single else list(windows)
        n = len(ws)
        views = (N.WindowView * n)()
        flags = []
        for v, w in zip(views, ws):
            N.lib().gba_window_view_init(N.C.byref(v))
            v.num_keyframes, v.num_landmarks, v.num_observations = w.num_keyframes, w.num_landmarks, w.num_observations
            v.keyframe_index, v.landmark_index = N.i32p(w.keyframe_index), N.i32p(w.landmark_index)
            v.rig_camera = w.rig_camera.ctypes.data_as(N.C.POINTER(N.C.c_uint8))
            v.observations, v.poses, v.landmarks = N.f64p(w.observations), N.f64p(w.poses), N.f64p(w.landmarks)
            v.rig.fx, v.rig.fy, v.rig.cx, v.rig.cy = w.fx, w.fy, w.cx, w.cy
            for k in range(2):
                for q in range(6):
                    v.rig.extrinsic[k][q] = float(w.extrinsics[k, q])
            v.chi2_threshold, v.max_threshold_doublings = chi2_threshold, max_threshold_doublings
            f = np.zeros(w.num_observations, np.uint8)
            flags.append(f)
            v.outlier = f.ctypes.data_as(N.C.POINTER(N.C.c_uint8))
        sums = (N.Summary * n)()
        trs = [_Trace(self._cap()) for _ in range(n)]
        for s, t in zip(sums, trs):
            t.attach(s)
        res = (N.WindowResult * n)()
        N.check(N.lib().gba_local_ba(self._h, views, n, sums, res), self._h, "gba_local_ba")
        out = [(_summary(s, t), {"num_inliers": r.num_inliers, "num_outliers": r.num_outliers,
                                 "chi2_threshold": r.chi2_threshold, "outlier": f})
               for s, t, r, f in zip(sums, trs, res, flags)]
        return out[0] if single else out

    def autotune(self, problems: BALProblem | Sequence[BALProblem]) -> dict:
        """Picks the fastest launch shapes (tile size, PCG iterations per
        graph body, cameras per CTA of the cluster PCG) and, with
        autotune=2, the PCG iteration cap for these problems by timed trial
        solves; later solves on this handle use them.  The problems are not
        modified."""
        if isinstance(problems, BALProblem):
            problems = [problems]
        views = (N.ProblemView * len(problems))(*[p.view() for p in problems])
        r = N.TuneResult()
        N.check(N.lib().gba_autotune(self._h, views, len(problems), N.C.byref(r)), self._h, "gba_autotune")
        n = min(r.num_trials, N.TUNE_MAX_TRIALS)
        return {"chunk_observations": r.chunk_observations, "pcg_unroll": r.pcg_unroll, "best_ms": r.best_ms,
                "pcg_cameras_per_cta": r.pcg_cameras_per_cta, "pcg_cap": r.pcg_cap, "pcg_grid_ctas": r.pcg_grid_ctas,
                "from_cache": bool(r.from_cache),
                "trials": [{"step": r.trial_step[i], "chunk_observations": r.trial_chunk[i],
                            "pcg_unroll": r.trial_unroll[i], "pcg_cameras_per_cta": r.trial_cameras_per_cta[i],
                            "pcg_cap": r.trial_cap[i], "pcg_grid_ctas": r.trial_grid_ctas[i], "ms": r.trial_ms[i],
                            "final_cost": r.trial_final_cost[i]}
                           for i in range(n)]}

    def evaluate(self, problem: BALProblem):
        """(residuals [no,2], jacobians [no,2,12], cost) evaluated on the GPU."""
        no = problem.num_observations()
        r = np.zeros(2 * no)
        J = np.zeros(24 * no)
        c = N.C.c_double()
        N.check(N.lib().gba_evaluate(self._h, N.C.byref(problem.view()), N.f64p(r), N.f64p(J), N.C.byref(c)),
                self._h, "gba_evaluate")
        return r.reshape(no, 2), J.reshape(no, 2, 12), c.value

    def compute_step(self, problem: BALProblem, radius: float):
        """One LM linear solve: (delta, model_cost_change, pcg_iterations)."""
        d = np.zeros(problem.num_parameters())
        m = N.C.c_double()
        it = N.C.c_int32()
        N.check(N.lib().gba_compute_step(self._h, N.C.byref(problem.view()), float(radius), N.f64p(d),
                                         N.C.byref(m), N.C.byref(it)), self._h, "gba_compute_step")
        return d, m.value, it.value

    def solve_resident(self, repeats: int = 1) -> None:
        """Re-run the last solved problem from its initial point on the device
        (asynchronous; no host transfers)."""
        N.check(N.lib().gba_solve_resident(self._h, int(repeats)), self._h, "gba_solve_resident")

    def synchronize(self) -> None:
        N.check(N.lib().gba_synchronize(self._h), self._h, "gba_synchronize")

    # ---- profiling ---------------------------------------------------------
    def set_profiling(self, on: bool) -> None:
        N.check(N.lib().gba_set_profiling(self._h, 1 if on else 0), self._h)

    def profile(self) -> list[dict]:
        L = N.lib()
        out = []
        for i in range(L.gba_profile_count(self._h)):
            name = N.C.c_char_p()
            n = N.C.c_int64()
            ms = N.C.c_double()
            b = N.C.c_double()
            N.check(L.gba_profile_entry(self._h, i, N.C.byref(name), N.C.byref(n), N.C.byref(ms), N.C.byref(b)))
            out.append({"name": name.value.decode(), "launches": n.value, "total_ms": ms.value, "bytes": b.value})
        return out

    # ---- serving -------------------------------------------------------------
    def start_server(self, device_budget_bytes: int = 0, max_live: int = 0, max_queue: int = 0) -> None:
        N.check(N.lib().gba_server_start(self._h, device_budget_bytes, max_live, max_queue), self._h,
                "gba_server_start")
        self._pending: dict[int, BALProblem] = {}

    def submit(self, problem: BALProblem) -> int:
        t = N.C.c_uint64()
        N.check(N.lib().gba_submit(self._h, N.C.byref(problem.view()), N.C.byref(t)), self._h, "gba_submit")
        self._pending[t.value] = problem  # keep arrays alive until done
        return t.value

    def poll(self, ticket: int):
        s = N.Summary()
        done = N.C.c_int32()
        N.check(N.lib().gba_poll(self._h, ticket, N.C.byref(s), N.C.byref(done)), self._h, "gba_poll")
        if not done.value:
            return None
        self._pending.pop(ticket, None)
        return _summary(s, None)

    def stop_server(self) -> None:
        N.check(N.lib().gba_server_stop(self._h), self._h, "gba_server_stop")

    def server_stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.lib().gba_server_get_stats(self._h, N.C.byref(st)), self._h)
        return {k: getattr(st, k) for k, _ in N.ServerStats._fields_}


# The g2o variant's SolveBA (test_bundle_adjustment_g2o.cpp:166-232): SO3 left
# camera update (:84-90), g2o's Levenberg (:174-176), Huber 1.0 per edge
# (:213), 40 iterations (:218), no tolerance tests.
G2O_VARIANT = dict(camera_update="so3_left", lm_policy="g2o", loss="huber", loss_scale=1.0, max_num_iterations=40,
                   function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)


# full_slam's local BA (Backend::Optimize, full_slam/src/backend.cpp:67-199):
# g2o's Levenberg, 10 iterations, Huber with delta 5.991, no tolerance tests
# (the same set gba_local_ba_options_init fills in).
LOCAL_BA = dict(lm_policy="g2o", max_num_iterations=10, loss="huber", loss_scale=5.991, function_tolerance=0.0,
                gradient_tolerance=0.0, parameter_tolerance=0.0)


def solve_ba(bal_problem: BALProblem, **options) -> SolveSummary:
    """Drop-in for SolveBA(BALProblem&) (test_bundle_adjustment_ceres.cpp:58-101):
    HuberLoss(1.0) per observation unless `loss` is given; other options are
    Ceres' defaults unless overridden."""
    options.setdefault("loss", "huber")
    options.setdefault("loss_scale", 1.0)
    with Solver(**options) as s:
        return s.solve(bal_problem)


def estimate_footprint(num_cameras: int, num_points: int, num_observations: int, precision: str = "fp64") -> int:
    return int(N.lib().gba_estimate_footprint(num_cameras, num_points, num_observations, N.PRECISION[precision]))
