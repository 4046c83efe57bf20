"""Serving (continuous batching) through the C ABI: requests submitted
together are admitted into several engine slots and solved in overlapping
cohorts; each result must equal the same request solved alone.

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
    for i, t in enumerate(tickets):
        assert np.array_equal(served[i].parameters(), alone[i][0]), i
        assert results[t].final_cost == alone[i][1]
        assert results[t].num_iterations == alone[i][2]


def test_server_rejects_oversize_and_survives():
    with Solver(**OPTS) as s:
        s.start_server(device_budget_bytes=1 << 20)  # 1 MiB: no real problem fits
        from slamplay_gb300 import GBAError

        with pytest.raises(GBAError):
            s.submit(_requests(1)[0])
        st = s.server_stats()
        s.stop_server()
    assert st["rejected"] == 1
