"""The C++ drop-in on the GPU: the demo app bundle_adjustment_gb300 (the
reference's main() of backend/slam_ba_simple_g2o_ceres with SolveBA from
include/gba_solve_ba.hpp) run as its own process on ladybug49 written as a
BAL file, against the same path through the Python / ctypes binding
(parse, Normalize, Perturb from the C library's rand() in its initial
state, HuberLoss(1.0), Ceres' defaults): the solved parameters and final
cost bit for bit.  And BALProblem's use_quaternions camera layout through
the C ABI (gba_options::camera_layout): the same bits as solving the
angle-axis conversion and converting back.

Tolerance: exact (bitwise) in both tests."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from slamplay_gb300 import BALProblem, Solver, solve_ba
from slamplay_gb300 import _native as N
from slamplay_gb300 import build as B
from test_ladybug_prepare import load_fixture, raw_problem

pytestmark = pytest.mark.gpu


def test_demo_app_equals_ctypes_bitwise(tmp_path):
    app = os.path.join(os.path.dirname(B.build()), "bundle_adjustment_gb300")
    assert os.path.exists(app)
    bal = str(tmp_path / "ladybug49.txt")
    raw_problem(load_fixture()).WriteToFile(bal)
    out = str(tmp_path / "final.bin")
    r = subprocess.run([app, bal, "--raw", out], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    app_cost = float(re.search(r"final_cost (\S+)", r.stdout).group(1))
    app_params = np.fromfile(out, dtype=np.float64)
    b = BALProblem(bal)  # the reader the app uses
    b.Normalize()
    ctypes.CDLL(None).srand(ctypes.c_uint(1))  # the app's process never seeds rand()
    b.Perturb(0.1, 0.5, 0.5, seed=0)
    s = solve_ba(b)
    assert app_params.size == b.num_parameters()
    assert np.array_equal(app_params, b.parameters())
    assert app_cost == s.final_cost


def _to_quaternion_params(aa_params, nc):
    out = np.zeros(10 * nc + aa_params.size - 9 * nc)
    L = N.lib()
    for i in range(nc):
        q = np.zeros(4)
        L.gba_angle_axis_to_quaternion(N.f64p(np.ascontiguousarray(aa_params[9 * i: 9 * i + 3])), N.f64p(q))
        out[10 * i: 10 * i + 4] = q
        out[10 * i + 4: 10 * i + 10] = aa_params[9 * i + 3: 9 * i + 9]
    out[10 * nc:] = aa_params[9 * nc:]
    return out


def test_quaternion_layout_equals_angle_axis_solve():
    b = BALProblem.synthetic(0, seed=4, num_points=800)
    nc = b.num_cameras()
    q = b.copy()
    q.parameters_ = _to_quaternion_params(b.parameters(), nc)
    q.use_quaternions = True
    assert q.camera_block_size() == 10
    opts = dict(max_num_iterations=8, loss="huber")
    # what the library does: quaternions -> angle-axis, solve, -> quaternions
    a = b.copy()
    a.parameters_ = q.to_angle_axis_parameters()
    with Solver(**opts) as s:
        sa = s.solve(a)
    with Solver(camera_layout="quaternion", **opts) as s:
        sq = s.solve(q)
        with pytest.raises(Exception):
            s.evaluate(q)  # only gba_solve / gba_batch_solve take the quaternion layout
    assert sq.final_cost == sa.final_cost
    assert np.array_equal(q.parameters(), _to_quaternion_params(a.parameters(), nc))
    with Solver(**opts) as s, pytest.raises(ValueError):
        s.solve(q)  # a quaternion problem on an angle-axis solver
