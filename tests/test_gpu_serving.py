"""Serving (continuous batching) through the C ABI: requests submitted
together are admitted into several engine slots and solved in overlapping
cohorts; each result must equal the same request solved alone.  Requests
arriving while cohorts run join them at LM-iteration boundaries: the
members still running continue in the re-formed batch from their carried
state (LM state, Jacobi scales, current point), and their results must
still equal the request solved alone.

Tolerance: exact (bitwise) parameters and final cost -- every reduction of a
problem has a fixed order that depends only on that problem."""
import time

import numpy as np
import pytest

from slamplay_gb300 import BALProblem, Solver

pytestmark = pytest.mark.gpu

OPTS = dict(precision="mixed", max_num_iterations=15, function_tolerance=1e-6, pcg_tolerance=1e-6,
            max_linear_solver_iterations=100)


def _requests(n=10):
    return [BALProblem.synthetic(4, index=i, seed=3, num_points=1500) for i in range(n)]


def test_served_results_equal_alone():
    reqs = _requests()
    alone = []
    with Solver(**OPTS) as s:
        for r in reqs:
            g = r.copy()
            sm = s.solve(g)
            alone.append((g.parameters().copy(), sm.final_cost, sm.num_iterations))
    served = [r.copy() for r in reqs]
    results = {}
    with Solver(**OPTS) as s:
        s.start_server()
        tickets = [s.submit(p) for p in served]
        deadline = time.time() + 120
        while len(results) < len(tickets) and time.time() < deadline:
            for t in tickets:
                if t not in results:
                    r = s.poll(t)
                    if r is not None:
                        results[t] = r
            time.sleep(0.001)
        stats = s.server_stats()
        s.stop_server()
    assert len(results) == len(tickets)
    assert stats["peak_live"] > 1  # requests were on the device together
    assert stats["host_prep_s"] > 0.0  # cohorts laid out on the slots' worker threads
    for i, t in enumerate(tickets):
        assert np.array_equal(served[i].parameters(), alone[i][0]), i
        assert results[t].final_cost == alone[i][1]
        assert results[t].num_iterations == alone[i][2]


G2O = dict(camera_update="so3_left", lm_policy="g2o", loss="huber", loss_scale=1.0, function_tolerance=0.0,
           gradient_tolerance=0.0, parameter_tolerance=0.0)


def _serve(opts, reqs, first, max_live):
    """Submits `first` requests, waits for three batched LM iterations, then
    submits the rest; returns the results by request and the server stats.
    One engine slot: every request that arrives while the cohort runs joins
    it at an LM-iteration boundary."""
    served = [r.copy() for r in reqs]
    results = {}
    with Solver(server_slots=1, **opts) as s:
        s.start_server(max_live=max_live)
        tickets = [s.submit(p) for p in served[:first]]
        deadline = time.time() + 60
        while s.server_stats()["steps"] < 3 and time.time() < deadline:
            time.sleep(0.0005)
        tickets += [s.submit(p) for p in served[first:]]
        deadline = time.time() + 120
        while len(results) < len(tickets) and time.time() < deadline:
            for t in tickets:
                if t not in results:
                    r = s.poll(t)
                    if r is not None:
                        results[t] = r
            time.sleep(0.0005)
        stats = s.server_stats()
        s.stop_server()
    assert len(results) == len(tickets)
    return served, [results[t] for t in tickets], stats


@pytest.mark.parametrize("form", ["mixed", "fp64", "fp64_g2o"])
def test_requests_join_running_cohorts_bitwise(form):
    # 40 iterations at most: the requests stop at different iterations
    # (relative decrease below 1e-6), so cohorts re-form with members running
    opts = dict(OPTS, precision=form.split("_")[0], max_num_iterations=40)
    if form.endswith("g2o"):  # a fixed count of iterations, a varying count of LM trials
        opts.update(G2O, max_num_iterations=12)
    reqs = [BALProblem.synthetic(4, index=i, seed=5, num_points=1200) for i in range(12)]
    alone = []
    with Solver(**opts) as s:
        for r in reqs:
            g = r.copy()
            sm = s.solve(g)
            alone.append((g.parameters().copy(), sm))
    served, res, stats = _serve(opts, reqs, first=3, max_live=8)
    print(form, {k: stats[k] for k in ("steps", "reforms", "peak_live", "completed")},
          [a[1].num_iterations for a in alone])
    assert stats["reforms"] > 0  # members continued in re-formed batches
    assert stats["peak_live"] > 1
    for i in range(len(reqs)):
        assert np.array_equal(served[i].parameters(), alone[i][0]), i
        assert res[i].final_cost == alone[i][1].final_cost, i
        assert res[i].initial_cost == alone[i][1].initial_cost, i
        assert res[i].num_iterations == alone[i][1].num_iterations, i
        assert res[i].num_successful_steps == alone[i][1].num_successful_steps, i
        assert res[i].termination_type == alone[i][1].termination_type, i
        assert res[i].num_linear_solver_iterations == alone[i][1].num_linear_solver_iterations, i


def test_server_rejects_oversize_and_survives():
    with Solver(**OPTS) as s:
        s.start_server(device_budget_bytes=1 << 20)  # 1 MiB: no real problem fits
        from slamplay_gb300 import GBAError

        with pytest.raises(GBAError):
            s.submit(_requests(1)[0])
        # a request without observations needs no device memory: done at once
        b = _requests(1)[0]
        none = np.zeros(0, np.int32)
        e = BALProblem.from_arrays(b.num_cameras(), b.num_points(), none, none, np.zeros(0), b.parameters().copy())
        r = s.poll(s.submit(e))
        st = s.server_stats()
        s.stop_server()
    assert st["rejected"] == 1
    assert r is not None and r.num_iterations == 0 and r.final_cost == 0.0
