"""Pins the oracle restatement and the product's BALProblem host code to the
reference's OWN sources (utils/camera/SnavelyReprojectionError.h,
utils/geometry/rotation.h, utils/datasets/BALProblem.cpp), compiled by
oracle/build_ref.sh into oracle/_ref with declaration shims for Ceres/Eigen.
Skipped where the reference tree is not available."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem
from slamplay_gb300 import _native as N

REF_ROOT = O.reference_root()
LADYBUG = os.path.join(REF_ROOT, "data", "bal", "ladybug49.txt") if REF_ROOT else ""

ref = O.reference_lib() if REF_ROOT else None
pytestmark = pytest.mark.skipif(ref is None, reason="reference tree / oracle/_ref unavailable")


def random_cameras(n, seed):
    rng = np.random.default_rng(seed)
    scales = [2.0, 1.0, 1e-4, 1e-7, 1.48e-8, 1.5e-8, 1e-9, 0.0]
    out = []
    for i in range(n):
        cam = np.zeros(9)
        cam[:3] = rng.normal(size=3) * scales[i % len(scales)]
        cam[3:6] = rng.normal(size=3)
        cam[5] -= 10.0
        cam[6] = 500.0 * (1 + 0.01 * rng.normal())
        cam[7] = rng.uniform(-0.05, 0.05)
        cam[8] = rng.uniform(-0.005, 0.005)
        out.append(cam)
    return out


def test_oracle_residual_and_jacobian_equal_reference_bitwise():
    rng = np.random.default_rng(1)
    for cam in random_cameras(4000, 2):
        pt = rng.uniform(-2, 2, 3)
        uv = rng.normal(size=2) * 100
        r1, J1, r2, J2 = np.zeros(2), np.zeros(24), np.zeros(2), np.zeros(24)
        O.oracle().orc_residual_jacobian(O.f64(cam), O.f64(pt), O.f64(uv), O.f64(r1), O.f64(J1))
        ref.ref_residual_jacobian(O.f64(cam), O.f64(pt), O.f64(uv), O.f64(r2), O.f64(J2))
        assert np.array_equal(r1, r2) and np.array_equal(J1, J2)
        r3 = np.zeros(2)
        ref.ref_residual(O.f64(cam), O.f64(pt), O.f64(uv), O.f64(r3))
        assert np.array_equal(r3, r2)


def test_rotation_and_quaternions_equal_reference():
    L = N.lib()
    rng = np.random.default_rng(4)
    for cam in random_cameras(2000, 5):
        aa = np.ascontiguousarray(cam[:3])
        pt = rng.normal(size=3)
        a, b, c = np.zeros(3), np.zeros(3), np.zeros(3)
        L.gba_angle_axis_rotate_point(N.f64p(aa), N.f64p(pt), N.f64p(a))
        ref.ref_rotate(O.f64(aa), O.f64(pt), O.f64(b))
        O.oracle().orc_angle_axis_rotate_point(O.f64(aa), O.f64(pt), O.f64(c))
        assert np.array_equal(a, b) and np.array_equal(c, b)
        q1, q2 = np.zeros(4), np.zeros(4)
        L.gba_angle_axis_to_quaternion(N.f64p(aa), N.f64p(q1))
        ref.ref_aa_to_quat(O.f64(aa), O.f64(q2))
        assert np.array_equal(q1, q2)
        a1, a2 = np.zeros(3), np.zeros(3)
        L.gba_quaternion_to_angle_axis(N.f64p(q1), N.f64p(a1))
        ref.ref_quat_to_aa(O.f64(q2), O.f64(a2))
        assert np.array_equal(a1, a2)


def load_ref(path, use_quaternions=0):
    nc, np_, no, npar = (ctypes.c_int() for _ in range(4))
    ref.ref_bal_load(path.encode(), use_quaternions, ctypes.byref(nc), ctypes.byref(np_), ctypes.byref(no),
                     ctypes.byref(npar), None, None, None, None)
    ci = np.zeros(no.value, np.int32)
    pi = np.zeros(no.value, np.int32)
    ob = np.zeros(2 * no.value)
    pa = np.zeros(npar.value)
    ref.ref_bal_load(path.encode(), use_quaternions, ctypes.byref(nc), ctypes.byref(np_), ctypes.byref(no),
                     ctypes.byref(npar), O.i32(ci), O.i32(pi), O.f64(ob), O.f64(pa))
    return nc.value, np_.value, ci, pi, ob, pa


@pytest.fixture(scope="module")
def bal_file(tmp_path_factory):
    if os.path.exists(LADYBUG):
        return LADYBUG
    b = BALProblem.synthetic(0, seed=8, num_points=300)
    f = str(tmp_path_factory.mktemp("bal") / "synthetic.txt")
    b.WriteToFile(f)
    return f


@pytest.mark.parametrize("use_q", [0, 1])
def test_bal_read_equals_reference(bal_file, use_q):
    nc, np_, ci, pi, ob, pa = load_ref(bal_file, use_q)
    b = BALProblem(bal_file, use_quaternions=bool(use_q))
    assert (b.num_cameras(), b.num_points()) == (nc, np_)
    assert np.array_equal(b.camera_index(), ci) and np.array_equal(b.point_index(), pi)
    assert np.array_equal(b.observations(), ob)
    assert np.array_equal(b.parameters(), pa)


def test_bal_write_equals_reference_after_header(bal_file, tmp_path):
    mine, theirs = str(tmp_path / "mine.txt"), str(tmp_path / "ref.txt")
    BALProblem(bal_file).WriteToFile(mine)
    ref.ref_bal_write(bal_file.encode(), theirs.encode())
    a = open(mine).read().splitlines()
    b = open(theirs).read().splitlines()
    # the reference header repeats the camera count (BALProblem.cpp:149)
    nc, np_, no = a[0].split()
    assert b[0].split() == [nc, nc, np_, no]
    assert a[1:] == b[1:]


def test_ply_equals_reference(bal_file, tmp_path):
    mine, theirs = str(tmp_path / "mine.ply"), str(tmp_path / "ref.ply")
    BALProblem(bal_file).WriteToPLYFile(mine)
    ref.ref_bal_write_ply(bal_file.encode(), theirs.encode())
    assert open(mine).read() == open(theirs).read()


def test_normalize_and_perturb_equal_reference(bal_file):
    libc = ctypes.CDLL(None)
    for normalize, perturb, seed in [(1, 0, 1), (0, 1, 1), (1, 1, 7)]:
        expect = np.zeros(BALProblem(bal_file).num_parameters())
        ref.ref_bal_prepare(bal_file.encode(), normalize, perturb, seed, 0.1, 0.5, 0.5, O.f64(expect))
        b = BALProblem(bal_file)
        if normalize:
            b.Normalize()
        if perturb:
            libc.srand(ctypes.c_uint(seed))
            b.Perturb(0.1, 0.5, 0.5, seed=0)  # the C library's rand(), as the reference
        assert np.array_equal(b.parameters(), expect)
