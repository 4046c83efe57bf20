"""GPU kernels and solver vs the CPU oracle, through the C ABI (libgba.so).

Tolerances (stated per test):
  FP64 residual / Jacobian: |gpu - oracle| <= 1e-10 (1 + |row|_max) per entry
  FP64 final cost: relative difference <= 1e-9 (the FP64 parity bar)
  mixed final cost: relative difference <= 1e-6 from the FP64 oracle
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem, GBAError, Solver

pytestmark = pytest.mark.gpu

# Iteration-count runs: tolerances off so both sides run the stated number
# of LM iterations (benchmark configurations "run N LM iterations").
FIXED = dict(function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)


def small_problem(config=0, **over):
    return BALProblem.synthetic(config, seed=11, **over)


def branch_problem():
    """Cameras whose angle-axis norm sits on both sides of the reference's
    theta^2 <= DBL_EPSILON branch (rotation.h:136), plus exactly zero."""
    b = BALProblem.synthetic(0, seed=5, num_cameras=8, num_points=300)
    cams = b.mutable_cameras().reshape(-1, 9)
    rng = np.random.default_rng(3)
    for i, th in enumerate([0.0, 1e-9, 1.0e-8, 1.45e-8, 1.5e-8, 1e-7, 1e-4, 2.0]):
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        cams[i, :3] = axis * th
    return b


@pytest.mark.parametrize("make", [small_problem, branch_problem])
def test_evaluate_fp64_matches_oracle(make):
    b = make()
    with Solver() as s:
        r, J, cost = s.evaluate(b)
    ro, Jo, co, ok = O.evaluate(O.Problem.from_bal(b))
    assert ok
    scale = 1.0 + np.abs(Jo).max(axis=2, keepdims=True)
    assert np.all(np.abs(r - ro) <= 1e-10 * (1.0 + np.abs(ro))), np.abs(r - ro).max()
    assert np.all(np.abs(J - Jo) <= 1e-10 * scale), np.abs(J - Jo).max()
    assert abs(cost - co) <= 1e-12 * co


def test_evaluate_mixed_matches_oracle():
    b = small_problem()
    with Solver(precision="mixed") as s:
        r, J, cost = s.evaluate(b)
    ro, Jo, co, _ = O.evaluate(O.Problem.from_bal(b))
    scale = 1.0 + np.abs(Jo).max(axis=2, keepdims=True)
    # residual stored in FP32 after an FP64 evaluation; J computed in FP32
    assert np.all(np.abs(r - ro) <= 1e-6 * (1.0 + np.abs(ro)))
    assert np.all(np.abs(J - Jo) <= 2e-5 * scale), np.abs(J - Jo).max()
    assert abs(cost - co) <= 1e-12 * co  # cost is FP64 in both modes


@pytest.mark.parametrize("loss", ["trivial", "huber", "cauchy"])
def test_compute_step_matches_oracle(loss):
    b = small_problem()
    radius = 1e4
    with Solver(loss=loss, pcg_tolerance=1e-12, max_linear_solver_iterations=1000) as s:
        d, m, it = s.compute_step(b, radius)
    p = O.Problem.from_bal(b)
    do, mo, _, ok = O.compute_step(p, radius, loss=loss, linear_solver="pcg_schur", pcg_tolerance=1e-12,
                                   max_linear_solver_iterations=1000)
    assert ok and it > 0
    rel = np.linalg.norm(d - do) / np.linalg.norm(do)
    assert rel < 1e-8, rel
    assert abs(m - mo) <= 1e-9 * abs(mo)
    # and against the exact (dense Cholesky) Schur solve
    dd, md, _, ok = O.compute_step(O.Problem.from_bal(b), radius, loss=loss, linear_solver="dense_schur")
    assert ok
    assert np.linalg.norm(d - dd) / np.linalg.norm(dd) < 1e-6


def _solve_pair(b, gpu_opts, orc_opts):
    g = b.copy()
    with Solver(**gpu_opts) as s:
        sg = s.solve(g)
    po = O.Problem.from_bal(b)
    so = O.solve(po, **orc_opts)
    return g, sg, so


@pytest.mark.parametrize("loss", ["trivial", "huber", "cauchy"])
def test_solve_fp64_matches_oracle(loss):
    b = small_problem()
    opts = dict(max_num_iterations=20, loss=loss, **FIXED)
    g, sg, so = _solve_pair(b, dict(opts, pcg_tolerance=1e-12, max_linear_solver_iterations=1000),
                            dict(opts, linear_solver="dense_schur"))
    assert abs(sg.initial_cost - so["initial_cost"]) <= 1e-12 * so["initial_cost"]
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-9, (sg.final_cost, so["final_cost"], rel)
    # the two cost histories agree until the cost stops changing
    n = min(len(sg.trace_cost), len(so["trace_cost"]), 4)
    np.testing.assert_allclose(sg.trace_cost[:n], so["trace_cost"][:n], rtol=1e-9)
    dp = g.parameters() - so["parameters"]
    print("camera RMS diff", np.sqrt(np.mean(dp[: 9 * b.num_cameras()] ** 2)),
          "point RMS diff", np.sqrt(np.mean(dp[9 * b.num_cameras():] ** 2)))


def test_solve_default_tolerances_same_termination():
    b = small_problem()
    g, sg, so = _solve_pair(b, dict(pcg_tolerance=1e-12, max_linear_solver_iterations=1000),
                            dict(linear_solver="dense_schur"))
    assert sg.num_iterations == so["num_iterations"]
    assert sg.termination_type == "CONVERGENCE" and so["termination_type"] == 0
    assert abs(sg.final_cost - so["final_cost"]) <= 1e-9 * so["final_cost"]


def test_solve_mixed_within_1e6_of_fp64_oracle():
    b = small_problem()
    opts = dict(max_num_iterations=20, **FIXED)
    g, sg, so = _solve_pair(b, dict(opts, precision="mixed", pcg_tolerance=1e-6, max_linear_solver_iterations=200),
                            dict(opts, linear_solver="dense_schur"))
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= 1e-6, rel


def test_solve_is_deterministic_and_graph_equals_host_loop():
    b = small_problem(num_points=800)
    outs = []
    for use_graphs in (1, 1, 0):
        g = b.copy()
        with Solver(max_num_iterations=10, use_graphs=use_graphs, **FIXED) as s:
            sm = s.solve(g)
        outs.append((g.parameters().copy(), sm.final_cost, sm.num_linear_solver_iterations))
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0])
        assert o[1] == outs[0][1] and o[2] == outs[0][2]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_alone_bitwise(precision):
    # a problem's arithmetic depends only on itself: the same bits alone and
    # in a batch (the mixed form's batch and single-problem mat-vec kernels
    # differ in how they load, not in what they compute)
    probs = [BALProblem.synthetic(3, index=i, seed=2) for i in range(4)]
    alone = []
    with Solver(max_num_iterations=8, precision=precision, schur="implicit", **FIXED) as s:
        for p in probs:
            q = p.copy()
            sm = s.solve(q)
            alone.append((q.parameters().copy(), sm.final_cost))
        qs = [p.copy() for p in probs]
        sums = s.batch_solve(qs)
    for (pa, ca), q, sm in zip(alone, qs, sums):
        assert np.array_equal(pa, q.parameters())
        assert ca == sm.final_cost


def test_unobserved_blocks_unchanged():
    b = small_problem(num_points=400)
    # add one camera and one point that no observation uses
    nc, np_ = b.num_cameras(), b.num_points()
    params = np.concatenate([b.cameras(), [0.1, 0.2, 0.3, 1, 2, -10, 500, 0, 0], b.points(), [7.0, 8.0, 9.0]])
    e = BALProblem.from_arrays(nc + 1, np_ + 1, b.camera_index(), b.point_index(), b.observations(), params)
    before = e.parameters().copy()
    with Solver(max_num_iterations=5) as s:
        s.solve(e)
    np.testing.assert_array_equal(e.parameters()[9 * nc: 9 * nc + 9], before[9 * nc: 9 * nc + 9])
    np.testing.assert_array_equal(e.parameters()[-3:], before[-3:])


def test_invalid_inputs_raise():
    b = small_problem(num_points=100)
    with Solver() as s:
        bad = b.copy()
        bad.camera_index()[3] = b.num_cameras()
        with pytest.raises(GBAError) as ei:
            s.solve(bad)
        assert ei.value.status == 1
        bad = b.copy()
        bad.observations()[5] = np.nan
        with pytest.raises(GBAError) as ei:
            s.solve(bad)
        assert ei.value.status == 3
        # a point observed more than 256 times does not fit a chunk
        k = 300
        ci = np.concatenate([b.camera_index(), np.arange(k, dtype=np.int32) % b.num_cameras()])
        pi = np.concatenate([b.point_index(), np.zeros(k, np.int32)])
        uv = np.concatenate([b.observations(), np.tile(b.observations()[:2], k)])
        big = BALProblem.from_arrays(b.num_cameras(), b.num_points(), ci, pi, uv, b.parameters().copy())
        with pytest.raises(GBAError) as ei:
            s.solve(big)
        assert ei.value.status == 1 and "observed" in str(ei.value)
        # the handle stays usable after an error
        ok = b.copy()
        sm = s.solve(ok)
        assert sm.final_cost < sm.initial_cost


def test_problem_without_observations():
    """A problem without observations has no parameter blocks in the
    reference's problem, and Ceres returns at once for it (CONVERGENCE, cost
    0, no iterations): so do gba_solve, gba_batch_solve (the other problems
    of the batch get the bits they get alone) and the server (the ticket is
    done at once).  The parameters are left as they are."""
    b = small_problem(num_points=300)
    none = np.zeros(0, np.int32)
    e = BALProblem.from_arrays(b.num_cameras(), b.num_points(), none, none, np.zeros(0), b.parameters().copy())
    z = BALProblem.from_arrays(0, 0, none, none, np.zeros(0), np.zeros(0))
    before = e.parameters().copy()
    with Solver(max_num_iterations=5) as s:
        sm = s.solve(e)
        alone = b.copy()
        sa = s.solve(alone)
        mix = [e.copy(), b.copy(), z.copy()]
        sums = s.batch_solve(mix)
    assert sm.termination_type == "CONVERGENCE" and sm.num_iterations == 0
    assert sm.initial_cost == 0.0 and sm.final_cost == 0.0
    np.testing.assert_array_equal(e.parameters(), before)
    assert np.array_equal(mix[1].parameters(), alone.parameters()) and sums[1].final_cost == sa.final_cost
    assert sums[0].num_iterations == 0 and sums[2].num_iterations == 0 and sums[2].final_cost == 0.0
    np.testing.assert_array_equal(mix[0].parameters(), before)
    with Solver(max_num_iterations=5) as s:
        s.start_server()
        t = s.submit(e.copy())
        r = s.poll(t)
        s.stop_server()
    assert r is not None and r.num_iterations == 0 and r.termination_type == "CONVERGENCE"


@pytest.mark.parametrize("crit", ["residual", "quadratic_model"])
def test_many_camera_problem_matches_oracle_pcg(crit):
    """700 cameras: 88 blocks of the camera-side PCG kernel, whose last block
    decides for the problem.  FP64 against the oracle's PCG Schur solver with
    the same criterion; relative cost difference <= 1e-9 with the residual
    criterion at 1e-12, <= 1e-8 with the quadratic-model criterion at eta
    1e-6 (a rounding-level change of where the model test stops may move one
    PCG iteration)."""
    b = BALProblem.synthetic(0, seed=21, num_cameras=700, num_points=6000)
    opts = dict(max_num_iterations=6, pcg_criterion=crit, schur="implicit", **FIXED)
    tol = dict(pcg_tolerance=1e-12, max_linear_solver_iterations=1000) if crit == "residual" else dict(eta=1e-6)
    g, sg, so = _solve_pair(b, dict(opts, **tol), dict(opts, linear_solver="pcg_schur", **tol))
    rel = abs(sg.final_cost - so["final_cost"]) / so["final_cost"]
    assert rel <= (1e-9 if crit == "residual" else 1e-8), (sg.final_cost, so["final_cost"], rel)
    # graph-driven and host-driven loops agree bitwise on this shape too
    h = b.copy()
    with Solver(use_graphs=0, **opts, **tol) as s:
        sh = s.solve(h)
    assert np.array_equal(h.parameters(), g.parameters())
    assert sh.num_linear_solver_iterations == sg.num_linear_solver_iterations


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_problem_reduction_path(precision):
    """More than 2,048 chunks: the mat-vec first sums its p.q values in groups
    of 64 chunks (the group's last CTA) and the camera kernel reads the group
    sums.  The same problem in chunks of at most 32 observations (~4,000
    chunks: the group path) and of 256 (~550 chunks: the direct path) is the
    same solve up to the order of the sums: final costs within 1e-9 (FP64)
    or 1e-6 (mixed) of each other, and of the FP64 oracle."""
    b = BALProblem.synthetic(0, seed=5, num_points=20000)
    opts = dict(max_num_iterations=6, pcg_tolerance=1e-10, max_linear_solver_iterations=300,
                precision=precision, schur="implicit", **FIXED)
    with Solver(chunk_observations=32, **opts) as s:
        grouped = s.solve(b.copy())
    with Solver(**opts) as s:
        direct = s.solve(b.copy())
    so = O.solve(O.Problem.from_bal(b), max_num_iterations=6, linear_solver="dense_schur", **FIXED)
    tol = 1e-9 if precision == "fp64" else 1e-6
    assert abs(grouped.final_cost - direct.final_cost) <= tol * direct.final_cost
    assert abs(grouped.final_cost - so["final_cost"]) <= tol * so["final_cost"], (grouped.final_cost, so["final_cost"])


@pytest.mark.parametrize("loss", ["trivial", "huber"])
def test_golden_fixture_fp64(loss):
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "small_problem.npz"))
    b = BALProblem.from_arrays(int(g["num_cameras"]), int(g["num_points"]), g["camera_index"], g["point_index"],
                               g["observations"], g["parameters"])
    with Solver(max_num_iterations=15, loss=loss, pcg_tolerance=1e-12, max_linear_solver_iterations=1000,
                **FIXED) as s:
        sm = s.solve(b)
    assert abs(sm.initial_cost - g[f"{loss}_initial_cost"]) <= 1e-12 * g[f"{loss}_initial_cost"]
    assert abs(sm.final_cost - g[f"{loss}_final_cost"]) <= 1e-9 * g[f"{loss}_final_cost"]
    np.testing.assert_allclose(sm.trace_cost[:4], g[f"{loss}_trace_cost"][:4], rtol=1e-9)
    if loss == "trivial":
        with Solver(pcg_tolerance=1e-12, max_linear_solver_iterations=1000) as s:
            d, m, _ = s.compute_step(BALProblem.from_arrays(int(g["num_cameras"]), int(g["num_points"]),
                                                            g["camera_index"], g["point_index"], g["observations"],
                                                            g["parameters"]), 1e4)
        ref = g["step_radius_1e4"]
        assert np.linalg.norm(d - ref) <= 1e-6 * np.linalg.norm(ref)


def test_autotune_picks_a_shape_and_keeps_the_solution():
    """The tuner's launch shapes change which thread adds which partial,
    never what is solved: FP64 final cost within 1e-9 relative of the
    untuned solve; the problem is not modified by tuning; the second call
    for the same size bucket comes from the cache."""
    b = small_problem(num_points=1200)
    before = b.parameters().copy()
    opts = dict(max_num_iterations=10, pcg_tolerance=1e-12, max_linear_solver_iterations=500, **FIXED)
    with Solver(**opts) as s:
        ref = s.solve(b.copy())
    with Solver(**opts) as s:
        r = s.autotune(b)
        assert np.array_equal(b.parameters(), before)
        assert r["chunk_observations"] in (128, 192, 256) and r["pcg_unroll"] in (1, 2, 4)
        shapes = [t for t in r["trials"] if t["step"] == 1]
        assert len(shapes) in (3, 9) and min(t["ms"] for t in shapes) == r["best_ms"]
        assert r["pcg_cap"] == 0  # the cap is tuned only with autotune=2
        tuned = s.solve(b.copy())
        assert s.autotune(b)["from_cache"]
    assert abs(tuned.final_cost - ref.final_cost) <= 1e-9 * ref.final_cost


def test_autotune_cluster_split_and_pcg_cap():
    """A mixed batch on the cluster PCG: the tuner also picks the cameras
    per CTA (16, 32, 64, or 0 = the default split) and, with autotune=2, the
    PCG cap: a smaller cap only when its 5-iteration trial ends within 1e-6
    relative of the configured cap's, and then the fastest such one.  The
    tuned solve ends within 1e-6 relative of the untuned one (10 LM
    iterations; a smaller cap changes each linear solve's length)."""
    probs = [BALProblem.synthetic(0, seed=20 + i, num_points=600) for i in range(8)]
    opts = dict(precision="mixed", max_num_iterations=10, pcg_tolerance=1e-6, max_linear_solver_iterations=80,
                persistent_pcg=1, **FIXED)
    with Solver(**opts) as s:
        ref = s.batch_solve([p.copy() for p in probs])
    with Solver(autotune=2, **opts) as s:
        r = s.autotune(probs)
        steps = {t["step"] for t in r["trials"]}
        assert steps >= {1, 3}
        if 2 in steps:
            assert r["pcg_cameras_per_cta"] in (0, 16, 32, 64)
        caps = [t for t in r["trials"] if t["step"] == 3]
        assert caps[0]["pcg_cap"] == 80 and r["pcg_cap"] in [t["pcg_cap"] for t in caps]
        chosen = next(t for t in caps if t["pcg_cap"] == r["pcg_cap"])
        assert chosen["final_cost"] <= caps[0]["final_cost"] * (1 + 1e-6)
        tuned = s.batch_solve([p.copy() for p in probs])
    print("tune:", {k: r[k] for k in ("chunk_observations", "pcg_unroll", "pcg_cameras_per_cta", "pcg_cap")},
          [(t["step"], t["pcg_cap"], round(t["ms"], 3)) for t in r["trials"]])
    for a, b in zip(tuned, ref):
        assert abs(a.final_cost - b.final_cost) <= 1e-6 * b.final_cost
