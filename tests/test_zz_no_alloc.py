"""gba_evaluate_noalloc: the allocation-free evaluation entry point.

It serves callers that cannot call cudaMalloc (real-time tracking threads
that must not take its implicit synchronisation, hosts that own every
device byte through their own pool): they hand in device inputs and outputs and the library
uses only a fixed file-scope device array as scratch.  This test (collected
last on purpose) allocates the caller's device buffers with torch, calls the
entry point through the C ABI twice in a row on two different problems, and
checks each result against the existing gba_evaluate entry point with the
FP64 evaluation tolerances used elsewhere:
  residuals: |a - b| <= 1e-10 (1 + |b|),  cost: relative difference <= 1e-12.
"""
import ctypes

import numpy as np
import pytest

from slamplay_gb300 import BALProblem, Solver
from slamplay_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _device_problem(torch, b):
    cams = torch.tensor(b.cameras().reshape(-1), dtype=torch.float64, device="cuda")
    pts = torch.tensor(b.points().reshape(-1), dtype=torch.float64, device="cuda")
    obs = torch.tensor(b.observations(), dtype=torch.float64, device="cuda")
    ci = torch.tensor(b.camera_index(), dtype=torch.int32, device="cuda")
    pi = torch.tensor(b.point_index(), dtype=torch.int32, device="cuda")
    dp = N.DeviceProblem(b.num_cameras(), b.num_points(), b.num_observations(), ci.data_ptr(), pi.data_ptr(),
                         obs.data_ptr(), cams.data_ptr(), pts.data_ptr())
    return dp, (cams, pts, obs, ci, pi)


def _noalloc(torch, b, loss=0, scale=1.0):
    dp, keep = _device_problem(torch, b)
    res = torch.full((2 * b.num_observations(),), float("nan"), dtype=torch.float64, device="cuda")
    cost = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    st = N.lib().gba_evaluate_noalloc(ctypes.byref(dp), loss, scale, ctypes.c_void_p(res.data_ptr()),
                                      ctypes.c_void_p(cost.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    N.check(st, None, "gba_evaluate_noalloc")
    torch.cuda.synchronize()
    return res.cpu().numpy().reshape(-1, 2), float(cost.cpu().item())


def test_noalloc_matches_evaluate_on_two_calls():
    torch = pytest.importorskip("torch")
    problems = [BALProblem.synthetic(0, seed=31, num_points=1500), BALProblem.synthetic(3, index=2, seed=32)]
    for b in problems:  # two calls in a row; the second problem is smaller, so stale scratch would show
        with Solver() as s:
            r_ref, _, c_ref = s.evaluate(b)
        r, c = _noalloc(torch, b)
        assert np.all(np.abs(r - r_ref) <= 1e-10 * (1.0 + np.abs(r_ref))), np.abs(r - r_ref).max()
        assert abs(c - c_ref) <= 1e-12 * c_ref, (c, c_ref)


def test_noalloc_rejects_sizes_beyond_the_limit():
    dp = N.DeviceProblem(16385, 1, 1, None, None, None, None, None)
    cost = ctypes.c_double()
    st = N.lib().gba_evaluate_noalloc(ctypes.byref(dp), 0, 1.0, None, ctypes.c_void_p(ctypes.addressof(cost)), None)
    assert st == 1  # GBA_ERR_INVALID_ARGUMENT, before any GPU work
    assert b"16384" in N.lib().gba_last_error(None)
