"""The reference's own input path on its shipped BAL file (ladybug49:
parse, Normalize(), Perturb(0.1, 0.5, 0.5) from the C library's rand() in
its initial state; test_bundle_adjustment_ceres.cpp:48-50) reproduced by
this library's host code, bit for bit, against the fixture that the
reference's own BALProblem.cpp produced (tests/golden/make_ladybug.py).
Needs no GPU and no reference tree."""
import ctypes
import os

import numpy as np

from slamplay_gb300 import BALProblem

HERE = os.path.dirname(os.path.abspath(__file__))


def load_fixture():
    return np.load(os.path.join(HERE, "golden", "ladybug49_prepared.npz"))


def raw_problem(g):
    return BALProblem.from_arrays(int(g["num_cameras"]), int(g["num_points"]), g["camera_index"], g["point_index"],
                                  g["observations"], g["parameters_raw"])


def test_ladybug_normalize_perturb_equal_reference_bitwise():
    g = load_fixture()
    b = raw_problem(g)
    assert (b.num_cameras(), b.num_points(), b.num_observations()) == (49, 7776, 31843)
    b.Normalize()
    ctypes.CDLL(None).srand(ctypes.c_uint(1))  # the reference's main() never seeds rand()
    b.Perturb(0.1, 0.5, 0.5, seed=0)
    assert np.array_equal(b.parameters(), g["parameters_prepared"])
