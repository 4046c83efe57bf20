"""Regenerates tests/golden/small_problem.npz: a small seeded synthetic BAL
problem (product generator) and the CPU oracle's solve of it (exact Schur,
dense Cholesky, 15 LM iterations, trivial and Huber loss).  The GPU tests
compare against these stored oracle results, so they do not depend on the
generator staying unchanged.

And tests/golden/variants.npz: the same problem solved with the g2o
variant's options (SO3 left camera update, g2o's Levenberg, Huber 1.0), and
a small local-BA window (its arrays, the oracle's solve with full_slam's
options, each edge's chi2 and the outlier flags).

Usage: python tests/golden/make_golden.py [--variants-only]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from slamplay_gb300 import BALProblem  # noqa: E402

OPTS = dict(max_num_iterations=15, function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
            linear_solver="dense_schur")


def variants():
    from slamplay_gb300 import G2O_VARIANT, LOCAL_BA, LocalBAWindow
    b = BALProblem.synthetic(0, seed=123, num_cameras=10, num_points=250)
    out = {}
    g2o = dict(G2O_VARIANT, max_num_iterations=15)
    r = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", **g2o)
    out["g2o_trace_cost"] = r["trace_cost"]
    out["g2o_trace_radius"] = r["trace_radius"]
    out["g2o_final_parameters"] = r["parameters"]
    w = LocalBAWindow.synthetic(seed=77, num_keyframes=5, num_landmarks=120)
    for k in ("keyframe_index", "landmark_index", "rig_camera", "observations", "poses", "landmarks", "extrinsics"):
        out["window_" + k] = getattr(w, k)
    out["window_K"] = np.array([w.fx, w.fy, w.cx, w.cy])
    rig = O.rig_from_window(w)
    r = O.solve(O.window_problem(w), rig=rig, linear_solver="dense_schur", **LOCAL_BA)
    out["window_trace_cost"] = r["trace_cost"]
    out["window_final_parameters"] = r["parameters"]
    p = O.window_problem(w)
    p.params[:] = r["parameters"]
    res, _, _, ok = O.evaluate_rig(p, rig)
    assert ok
    chi2 = np.sum(res * res, axis=1)
    flags, ni, no_, th = O.window_outliers(chi2)
    out["window_chi2"] = chi2
    out["window_outlier"] = flags
    out["window_threshold"] = np.array([th])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "variants.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    from slamplay_gb300 import build
    build.build()
    if "--variants-only" in sys.argv:
        variants()
        return
    variants()
    b = BALProblem.synthetic(0, seed=123, num_cameras=10, num_points=250)
    out = {"num_cameras": b.num_cameras(), "num_points": b.num_points(), "camera_index": b.camera_index(),
           "point_index": b.point_index(), "observations": b.observations(), "parameters": b.parameters()}
    for loss in ("trivial", "huber"):
        r = O.solve(O.Problem.from_bal(b), loss=loss, **OPTS)
        out[f"{loss}_trace_cost"] = r["trace_cost"]
        out[f"{loss}_final_cost"] = r["final_cost"]
        out[f"{loss}_final_parameters"] = r["parameters"]
        out[f"{loss}_initial_cost"] = r["initial_cost"]
    step, mcc, _, ok = O.compute_step(O.Problem.from_bal(b), 1e4, linear_solver="dense_schur")
    assert ok
    out["step_radius_1e4"] = step
    out["step_model_cost_change"] = mcc
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_problem.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
