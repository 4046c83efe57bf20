"""Regenerates tests/golden/small_problem.npz: a small seeded synthetic BAL
problem (product generator) and the CPU oracle's solve of it (exact Schur,
dense Cholesky, 15 LM iterations, trivial and Huber loss).  The GPU tests
compare against these stored oracle results, so they do not depend on the
generator staying unchanged.

Usage: python tests/golden/make_golden.py
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


def main():
    from slamplay_gb300 import build
    build.build()
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
