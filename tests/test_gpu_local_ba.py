"""Local-BA windows (full_slam's Backend::Optimize, full_slam/src/backend.cpp:67-199)
on the GPU vs the CPU oracle, through the C ABI (gba_local_ba).

Tolerances: FP64 final cost relative difference <= 1e-9 and cost trace
rtol 1e-9; mixed final cost <= 1e-6 from the FP64 oracle; outlier flags
equal except where the oracle's chi2 lies within 1e-6 (relative) of the
final threshold.
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import LOCAL_BA, BALProblem, LocalBAWindow, Solver

pytestmark = pytest.mark.gpu

EXACT = dict(pcg_tolerance=1e-12, max_linear_solver_iterations=1000)


def _oracle(w, **opts):
    rig = O.rig_from_window(w)
    s = O.solve(O.window_problem(w), rig=rig, linear_solver="dense_schur", **opts)
    p = O.window_problem(w)
    p.params[:] = s["parameters"]
    r, _, _, ok = O.evaluate_rig(p, rig)
    assert ok
    chi2 = np.sum(r * r, axis=1)
    flags, ni, no_, th = O.window_outliers(chi2)
    return s, chi2, flags, ni, no_, th


def _check_flags(res, chi2, flags, th):
    near = np.abs(chi2 - th) <= 1e-6 * th
    assert res["chi2_threshold"] == pytest.approx(th, rel=1e-12)
    assert np.all((res["outlier"] == flags) | near)


def test_local_ba_fp64_matches_oracle():
    w = LocalBAWindow.synthetic(seed=7)
    g = w.copy()
    with Solver(**LOCAL_BA, **EXACT) as s:
        sg, res = s.local_ba(g)
    so, chi2, flags, ni, no_, th = _oracle(w, **LOCAL_BA)
    assert sg.initial_cost == pytest.approx(so["initial_cost"], rel=1e-12)
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-9, (sg.final_cost, so["final_cost"], rel)
    n = min(len(sg.trace_cost), len(so["trace_cost"]), 6)
    np.testing.assert_allclose(sg.trace_cost[:n], so["trace_cost"][:n], rtol=1e-9)
    assert sg.num_successful_steps == so["num_successful_steps"]
    _check_flags(res, chi2, flags, th)
    assert abs(res["num_outliers"] - no_) <= int(np.sum(np.abs(chi2 - th) <= 1e-6 * th))
    # the outliers planted by the generator (5 %, 20-60 px) are among the flagged
    assert res["num_outliers"] >= 0.05 * w.num_observations - 1
    # poses and landmarks were written back
    assert not np.array_equal(g.poses, w.poses) and not np.array_equal(g.landmarks, w.landmarks)


def test_local_ba_ceres_policy_matches_oracle():
    w = LocalBAWindow.synthetic(seed=8, num_landmarks=400)
    opts = dict(LOCAL_BA, lm_policy="ceres")
    with Solver(**opts, **EXACT) as s:
        sg, res = s.local_ba(w.copy())
    so, chi2, flags, ni, no_, th = _oracle(w, **opts)
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-9, rel
    _check_flags(res, chi2, flags, th)


@pytest.mark.parametrize("schur", ["explicit", "implicit"])
def test_local_ba_mixed_within_1e6_of_fp64_oracle(schur):
    w = LocalBAWindow.synthetic(seed=9)
    with Solver(**LOCAL_BA, precision="mixed", schur=schur, pcg_tolerance=1e-6,
                max_linear_solver_iterations=200) as s:
        sg, res = s.local_ba(w.copy())
    so = _oracle(w, **LOCAL_BA)[0]
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-6, rel


def test_local_ba_batch_equals_alone_bitwise():
    ws = [LocalBAWindow.synthetic(seed=20 + i, num_keyframes=5 + i, num_landmarks=300 + 50 * i) for i in range(4)]
    with Solver(**LOCAL_BA) as s:
        alone = []
        for w in ws:
            g = w.copy()
            sm, res = s.local_ba(g)
            alone.append((g.poses.copy(), g.landmarks.copy(), sm.final_cost, res["outlier"].copy()))
        gs = [w.copy() for w in ws]
        out = s.local_ba(gs)
    for (pa, la, ca, fa), g, (sm, res) in zip(alone, gs, out):
        assert np.array_equal(pa, g.poses) and np.array_equal(la, g.landmarks)
        assert ca == sm.final_cost and np.array_equal(fa, res["outlier"])


def test_bal_solve_after_windows_on_the_same_handle():
    b = BALProblem.synthetic(0, seed=11)
    with Solver(max_num_iterations=5) as fresh:
        q = b.copy()
        ref = fresh.solve(q)
    with Solver(max_num_iterations=5) as s:
        s.local_ba(LocalBAWindow.synthetic(seed=3, num_landmarks=200))
        q2 = b.copy()
        got = s.solve(q2)
    assert got.final_cost == ref.final_cost and np.array_equal(q.parameters(), q2.parameters())
