"""The g2o variant of the solve (test_bundle_adjustment_g2o.cpp) on the GPU
vs the CPU oracle, through the C ABI: its camera update (:84-90, R <- exp(dw)
R, the rest additive; camera_update=so3_left) and its Levenberg policy
(:174-176, g2o's OptimizationAlgorithmLevenberg; lm_policy=g2o), with the
Huber kernel of :213 and the 40 iterations of :218.

Tolerances: FP64 Jacobian entries <= 1e-10 (1 + |row|_max); FP64 final cost
relative difference <= 1e-9; mixed final cost <= 1e-6 from the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem, Solver

pytestmark = pytest.mark.gpu

FIXED = dict(function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)
LEFT = dict(camera_update="so3_left")


def test_evaluate_so3_left_matches_oracle():
    b = BALProblem.synthetic(0, seed=11)
    with Solver(**LEFT) as s:
        r, J, cost = s.evaluate(b)
    ro, Jo, co, ok = O.evaluate(O.Problem.from_bal(b), camera_update="so3_left")
    assert ok
    scale = 1.0 + np.abs(Jo).max(axis=2, keepdims=True)
    assert np.all(np.abs(r - ro) <= 1e-10 * (1.0 + np.abs(ro)))
    assert np.all(np.abs(J - Jo) <= 1e-10 * scale), np.abs(J - Jo).max()
    assert abs(cost - co) <= 1e-12 * co


def test_solve_so3_left_fp64_matches_oracle():
    b = BALProblem.synthetic(0, seed=11)
    opts = dict(max_num_iterations=20, **FIXED, **LEFT)
    g = b.copy()
    with Solver(pcg_tolerance=1e-12, max_linear_solver_iterations=1000, **opts) as s:
        sg = s.solve(g)
    so = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", **opts)
    sa = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=20, **FIXED)
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-9, (sg.final_cost, so["final_cost"], rel)
    n = min(len(sg.trace_cost), len(so["trace_cost"]), 4)
    np.testing.assert_allclose(sg.trace_cost[:n], so["trace_cost"][:n], rtol=1e-9)
    # the update is a different path from the additive one
    assert not np.allclose(so["trace_cost"][1:n], sa["trace_cost"][1:n], rtol=1e-9)
    cams = g.parameters()[: 9 * b.num_cameras()].reshape(-1, 9)
    assert np.all(np.linalg.norm(cams[:, :3], axis=1) <= np.pi + 1e-12)


@pytest.mark.parametrize("schur", ["explicit", "implicit"])
def test_solve_so3_left_mixed_within_1e6_of_fp64_oracle(schur):
    b = BALProblem.synthetic(0, seed=11)
    opts = dict(max_num_iterations=20, **FIXED, **LEFT)
    g = b.copy()
    with Solver(precision="mixed", schur=schur, pcg_tolerance=1e-6, max_linear_solver_iterations=200, **opts) as s:
        sg = s.solve(g)
    so = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", **opts)
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-6, rel


def test_batch_so3_left_equals_alone_bitwise():
    probs = [BALProblem.synthetic(3, index=i, seed=2) for i in range(3)]
    with Solver(max_num_iterations=6, precision="mixed", **FIXED, **LEFT) as s:
        alone = []
        for p in probs:
            q = p.copy()
            sm = s.solve(q)
            alone.append((q.parameters().copy(), sm.final_cost))
        qs = [p.copy() for p in probs]
        sums = s.batch_solve(qs)
    for (pa, ca), q, sm in zip(alone, qs, sums):
        assert np.array_equal(pa, q.parameters())
        assert ca == sm.final_cost


G2O = dict(camera_update="so3_left", lm_policy="g2o", loss="huber", **FIXED)


def test_solve_g2o_policy_fp64_matches_oracle():
    b = BALProblem.synthetic(0, seed=11)
    g = b.copy()
    with Solver(pcg_tolerance=1e-12, max_linear_solver_iterations=1000, max_num_iterations=12, **G2O) as s:
        sg = s.solve(g)
    so = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=12, **G2O)
    assert sg.trace_radius[0] == pytest.approx(so["trace_radius"][0], rel=1e-12)  # 1 / lambda_0
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-9, (sg.final_cost, so["final_cost"], rel)
    n = min(len(sg.trace_cost), len(so["trace_cost"]), 6)
    np.testing.assert_allclose(sg.trace_cost[:n], so["trace_cost"][:n], rtol=1e-9)
    np.testing.assert_array_equal(sg.trace_successful[:n], so["trace_successful"][:n])
    assert sg.num_successful_steps == so["num_successful_steps"]


def test_g2o_policy_counts_iterations_not_trials():
    b = BALProblem.synthetic(0, seed=11)
    with Solver(pcg_tolerance=1e-12, max_linear_solver_iterations=1000, max_num_iterations=4, **G2O) as s:
        sg = s.solve(b.copy())
    assert sg.num_successful_steps == 4
    assert sg.termination_reason == "max_iterations"
    assert sg.num_iterations == len(sg.trace_cost) - 1 >= 4


@pytest.mark.parametrize("schur", ["explicit", "implicit"])
def test_solve_g2o_variant_mixed_within_1e6_of_fp64_oracle(schur):
    b = BALProblem.synthetic(0, seed=11)
    with Solver(precision="mixed", schur=schur, pcg_tolerance=1e-6, max_linear_solver_iterations=200,
                max_num_iterations=40, **G2O) as s:
        sg = s.solve(b.copy())
    so = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=40, **G2O)
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-6, rel


def test_batch_g2o_variant_equals_alone_bitwise():
    probs = [BALProblem.synthetic(3, index=i, seed=4) for i in range(3)]
    with Solver(max_num_iterations=6, precision="mixed", **G2O) as s:
        alone = []
        for p in probs:
            q = p.copy()
            sm = s.solve(q)
            alone.append((q.parameters().copy(), sm.final_cost, sm.num_iterations))
        qs = [p.copy() for p in probs]
        sums = s.batch_solve(qs)
    for (pa, ca, ia), q, sm in zip(alone, qs, sums):
        assert np.array_equal(pa, q.parameters())
        assert ca == sm.final_cost and ia == sm.num_iterations
