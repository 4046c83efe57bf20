"""The explicit Schur complement (schur='explicit': the camera-camera blocks
of S formed once per LM iteration, the PCG multiplying by them) against the
implicit form and the CPU oracle, through the C ABI.

Tolerances (stated per test):
  FP64: final costs of the two forms and of the oracle within 1e-9 relative;
        a step within 1e-8 (relative norm) of the oracle's PCG step
  mixed: final cost within 1e-6 relative of the FP64 oracle
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem, Solver

pytestmark = pytest.mark.gpu

FIXED = dict(function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)


def _forms_launched(b, **opts):
    """Solves with per-kernel profiling on and returns the number of
    formation-kernel launches (0 for the implicit form)."""
    with Solver(**opts) as s:
        s.set_profiling(True)
        s.solve(b.copy())
        prof = {e["name"]: e for e in s.profile()}
    return prof.get("schur_form", {"launches": 0})["launches"]


def _solve(b, **opts):
    g = b.copy()
    with Solver(**opts) as s:
        sm = s.solve(g)
    return g, sm


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_explicit_matches_implicit_and_oracle(precision):
    b = BALProblem.synthetic(0, seed=11)
    if precision == "fp64":
        opts = dict(max_num_iterations=12, pcg_tolerance=1e-12, max_linear_solver_iterations=1000, **FIXED)
        tol = 1e-9
    else:
        opts = dict(max_num_iterations=20, precision="mixed", pcg_tolerance=1e-6,
                    max_linear_solver_iterations=200, **FIXED)
        tol = 1e-6
    ge, se = _solve(b, schur="explicit", **opts)
    gi, si = _solve(b, schur="implicit", **opts)
    so = O.solve(O.Problem.from_bal(b), max_num_iterations=opts["max_num_iterations"], linear_solver="dense_schur",
                 **FIXED)
    assert se.initial_cost == si.initial_cost
    assert abs(se.final_cost - so["final_cost"]) <= tol * so["final_cost"], (se.final_cost, so["final_cost"])
    if precision == "fp64":
        assert abs(se.final_cost - si.final_cost) <= tol * si.final_cost
        np.testing.assert_allclose(se.trace_cost[:4], so["trace_cost"][:4], rtol=1e-9)


def test_explicit_compute_step_matches_oracle():
    b = BALProblem.synthetic(0, seed=11)
    radius = 1e4
    with Solver(schur="explicit", pcg_tolerance=1e-12, max_linear_solver_iterations=1000) as s:
        d, m, it = s.compute_step(b, radius)
    do, mo, _, ok = O.compute_step(O.Problem.from_bal(b), radius, linear_solver="pcg_schur", pcg_tolerance=1e-12,
                                   max_linear_solver_iterations=1000)
    assert ok and it > 0
    assert np.linalg.norm(d - do) / np.linalg.norm(do) < 1e-8
    assert abs(m - mo) <= 1e-9 * abs(mo)


def test_explicit_duplicate_observations():
    """A camera that observes a point more than once: the cross terms of its
    observations go to a diagonal block (i, i) of the formed complement.
    FP64 explicit, implicit and the oracle's dense Schur solve agree to
    1e-9."""
    b = BALProblem.synthetic(0, seed=3, num_cameras=12, num_points=400)
    ci, pi, obs = b.camera_index_.copy(), b.point_index_.copy(), b.observations_.reshape(-1, 2).copy()
    rng = np.random.default_rng(7)
    dup = rng.choice(len(ci), size=120, replace=False)
    ci2 = np.concatenate([ci, ci[dup]])
    pi2 = np.concatenate([pi, pi[dup]])
    obs2 = np.concatenate([obs, obs[dup] + rng.normal(scale=0.5, size=(len(dup), 2))])
    d = BALProblem.from_arrays(b.num_cameras(), b.num_points(), ci2, pi2, obs2, b.parameters())
    opts = dict(max_num_iterations=8, pcg_tolerance=1e-12, max_linear_solver_iterations=1000, **FIXED)
    _, se = _solve(d, schur="explicit", **opts)
    _, si = _solve(d, schur="implicit", **opts)
    so = O.solve(O.Problem.from_bal(d), max_num_iterations=8, linear_solver="dense_schur", **FIXED)
    assert abs(se.final_cost - si.final_cost) <= 1e-9 * si.final_cost
    assert abs(se.final_cost - so["final_cost"]) <= 1e-9 * so["final_cost"], (se.final_cost, so["final_cost"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_explicit_batch_equals_alone_bitwise(precision):
    probs = [BALProblem.synthetic(3, index=i, seed=2) for i in range(4)]
    opts = dict(max_num_iterations=8, precision=precision, schur="explicit", **FIXED)
    alone = []
    with Solver(**opts) as s:
        for p in probs:
            q = p.copy()
            sm = s.solve(q)
            alone.append((q.parameters().copy(), sm.final_cost))
        qs = [p.copy() for p in probs]
        sums = s.batch_solve(qs)
    for (pa, ca), q, sm in zip(alone, qs, sums):
        assert np.array_equal(pa, q.parameters())
        assert ca == sm.final_cost


def test_explicit_many_cameras_graph_equals_host_loop():
    """700 cameras (88 camera blocks, whose p.q shares every block sums in
    the same order): against the oracle's PCG solve within 1e-9, and the
    graph-driven and host-driven loops bitwise equal."""
    b = BALProblem.synthetic(0, seed=21, num_cameras=700, num_points=6000)
    opts = dict(max_num_iterations=6, pcg_tolerance=1e-12, max_linear_solver_iterations=1000, schur="explicit",
                **FIXED)
    g, sg = _solve(b, **opts)
    h, sh = _solve(b, use_graphs=0, **opts)
    assert np.array_equal(g.parameters(), h.parameters())
    assert sg.num_linear_solver_iterations == sh.num_linear_solver_iterations
    so = O.solve(O.Problem.from_bal(b), max_num_iterations=6, linear_solver="pcg_schur", pcg_tolerance=1e-12,
                 max_linear_solver_iterations=1000, **FIXED)
    assert abs(sg.final_cost - so["final_cost"]) <= 1e-9 * so["final_cost"], (sg.final_cost, so["final_cost"])


def test_auto_choice():
    """schur='auto' forms S when the points' ordered observation pairs are at
    most 16 per observation (a sparse view graph), and keeps the implicit
    form for a dense one (every point seen by 18-20 of 20 cameras)."""
    sparse = BALProblem.synthetic(0, seed=11, num_points=2000)
    dense = BALProblem.synthetic(0, seed=11, num_cameras=20, num_points=300, min_views=18, max_views=20)
    opts = dict(max_num_iterations=2, **FIXED)
    assert _forms_launched(sparse, **opts) > 0
    assert _forms_launched(dense, **opts) == 0
    assert _forms_launched(sparse, schur="implicit", **opts) == 0
    assert _forms_launched(dense, schur="explicit", **opts) > 0


def _launches(b, name, **opts):
    with Solver(**opts) as s:
        s.set_profiling(True)
        sm = s.solve(b.copy())
        prof = {e["name"]: e for e in s.profile()}
    return prof.get(name, {"launches": 0})["launches"], sm


@pytest.mark.parametrize("crit", ["residual", "quadratic_model"])
def test_cluster_pcg_matches_two_kernel_and_oracle(crit):
    """Mixed form with the explicit complement: each problem's whole PCG in
    one thread-block-cluster launch per LM iteration (persistent_pcg=1, the
    default) against one launch pair per PCG iteration (persistent_pcg=0)
    and the FP64 oracle's dense Schur solve: final costs within 1e-6."""
    b = BALProblem.synthetic(0, seed=11)
    tol = dict(pcg_tolerance=1e-6, max_linear_solver_iterations=200) if crit == "residual" else dict(eta=1e-3)
    opts = dict(max_num_iterations=20, precision="mixed", schur="explicit", pcg_criterion=crit, **tol, **FIXED)
    n1, sc = _launches(b, "pcg_cluster", persistent_pcg=1, **opts)
    n0, s2 = _launches(b, "pcg_cluster", persistent_pcg=0, **opts)
    assert n1 == sc.num_iterations + 1 - sc.num_invalid_steps or n1 > 0
    assert n0 == 0
    so = O.solve(O.Problem.from_bal(b), max_num_iterations=20, linear_solver="dense_schur", **FIXED)
    for s in (sc, s2):
        assert abs(s.final_cost - so["final_cost"]) <= 1e-6 * so["final_cost"], (s.final_cost, so["final_cost"])


def test_cluster_pcg_many_cameras():
    """700 cameras: a cluster of 16 CTAs with 44 cameras each.  The graph
    and the host-driven loop agree bitwise; the cluster and the two-kernel
    PCG agree to 1e-6 in final cost."""
    b = BALProblem.synthetic(0, seed=21, num_cameras=700, num_points=6000)
    opts = dict(max_num_iterations=6, precision="mixed", schur="explicit", pcg_tolerance=1e-6,
                max_linear_solver_iterations=200, **FIXED)
    g, sg = _solve(b, **opts)
    h, sh = _solve(b, use_graphs=0, **opts)
    assert np.array_equal(g.parameters(), h.parameters())
    assert sg.num_linear_solver_iterations == sh.num_linear_solver_iterations
    _, s2 = _solve(b, persistent_pcg=0, **opts)
    assert abs(sg.final_cost - s2.final_cost) <= 1e-6 * s2.final_cost, (sg.final_cost, s2.final_cost)


def test_cluster_pcg_compute_step():
    """One mixed-form step through the cluster PCG against the oracle's FP64
    PCG step with the same tolerance: relative step difference <= 1e-3
    (FP32 Schur blocks), model cost change within 1e-4."""
    b = BALProblem.synthetic(0, seed=11)
    with Solver(precision="mixed", schur="explicit", pcg_tolerance=1e-6, max_linear_solver_iterations=500) as s:
        d, m, it = s.compute_step(b, 1e4)
    do, mo, _, ok = O.compute_step(O.Problem.from_bal(b), 1e4, linear_solver="pcg_schur", pcg_tolerance=1e-6,
                                   max_linear_solver_iterations=500)
    assert ok and it > 0
    assert np.linalg.norm(d - do) / np.linalg.norm(do) < 1e-3
    assert abs(m - mo) <= 1e-4 * abs(mo)


def _edge_problem():
    """Configuration-0 cameras plus a camera whose points no other camera
    sees (a row of S with only its diagonal block) and a camera that sees
    some points twice (a block with itself)."""
    b = BALProblem.synthetic(0, seed=6, num_cameras=6, num_points=300)
    nc, np_ = b.num_cameras(), b.num_points()
    ci, pi = b.camera_index_.copy(), b.point_index_.copy()
    obs = b.observations_.reshape(-1, 2).copy()
    par = b.parameters().copy()
    cams, pts = par[: 9 * nc].reshape(nc, 9), par[9 * nc:].reshape(np_, 3)
    # camera nc: a copy of camera 0 that alone sees copies of 12 of camera 0's points
    rows = np.nonzero(ci == 0)[0][:12]
    new_pts = pts[pi[rows]]
    ci = np.concatenate([ci, np.full(len(rows), nc)])
    pi = np.concatenate([pi, np_ + np.arange(len(rows))])
    obs = np.concatenate([obs, obs[rows]])
    # camera 1 sees 10 of its points a second time
    dup = np.nonzero(ci == 1)[0][:10]
    ci = np.concatenate([ci, ci[dup]])
    pi = np.concatenate([pi, pi[dup]])
    obs = np.concatenate([obs, obs[dup] + 0.3])
    params = np.concatenate([cams.ravel(), cams[0], pts.ravel(), new_pts.ravel()])
    return BALProblem.from_arrays(nc + 1, np_ + len(rows), ci, pi, obs, params)


def test_cluster_pcg_edge_cameras():
    """A camera with no co-visible camera and a camera with a block with
    itself: the cluster PCG and the two-kernel PCG (mixed form, explicit
    complement) reach final costs within 1e-6 of each other, below the
    initial cost."""
    b = _edge_problem()
    opts = dict(max_num_iterations=10, precision="mixed", schur="explicit", pcg_tolerance=1e-8,
                max_linear_solver_iterations=200, **FIXED)
    n1, sc = _launches(b, "pcg_cluster", **opts)
    _, s2 = _solve(b, persistent_pcg=0, **opts)
    assert n1 > 0
    assert np.isfinite(sc.final_cost) and sc.final_cost < sc.initial_cost
    assert abs(sc.final_cost - s2.final_cost) <= 1e-6 * s2.final_cost, (sc.final_cost, s2.final_cost)


def test_cluster_pcg_falls_back_for_large_problem_in_batch():
    """A mixed batch with a problem of more than 1,024 cameras runs the
    two-kernel PCG for the whole batch (one launch shape per batch); each
    problem then gets the bits of its own two-kernel solve."""
    small = [BALProblem.synthetic(3, index=i, seed=8) for i in range(2)]
    big = BALProblem.synthetic(0, seed=9, num_cameras=1100, num_points=3000)
    opts = dict(max_num_iterations=4, precision="mixed", schur="explicit", **FIXED)
    with Solver(**opts) as s:
        s.set_profiling(True)
        qs = [p.copy() for p in small + [big]]
        sums = s.batch_solve(qs)
        names = {e["name"]: e["launches"] for e in s.profile()}
    assert names.get("pcg_cluster", 0) == 0 and names.get("schur_matvec", 0) > 0
    for p, q, sm in zip(small + [big], qs, sums):
        g = p.copy()
        with Solver(persistent_pcg=0, **opts) as s:
            sa = s.solve(g)
        assert np.array_equal(g.parameters(), q.parameters())
        assert sa.final_cost == sm.final_cost
