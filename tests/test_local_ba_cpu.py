"""The local-BA window model on the CPU: the oracle's rig camera (EdgeProjection,
full_slam/include/myslam/g2o_types.h:127-175), the SE3 left update (VertexPose,
:48-66) and the outlier-threshold loop (full_slam/src/backend.cpp:156-187),
checked against independent restatements (numpy, scipy's matrix exponential,
central differences)."""
import os

import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300.window import LocalBAWindow

FIXED = dict(function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)


def _hat(v):
    return np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])


def _R(w):
    out = np.zeros((3, 3))
    for j in range(3):
        e = np.zeros(3)
        e[j] = 1.0
        c = np.zeros(3)
        O.oracle().orc_angle_axis_rotate_point(O.f64(np.ascontiguousarray(w, dtype=np.float64)), O.f64(e), O.f64(c))
        out[:, j] = c
    return out


@pytest.mark.parametrize("scale", [1.0, 1e-3, 1e-6, 0.0])
def test_se3_compose_left_is_the_matrix_exponential(scale):
    expm = pytest.importorskip("scipy.linalg").expm
    rng = np.random.default_rng(int(scale * 1e6) + 1)
    for _ in range(50):
        pose = np.concatenate([rng.normal(size=3), rng.normal(size=3)])
        dw, du = rng.normal(size=3) * scale, rng.normal(size=3)
        out = O.se3_compose_left(dw, du, pose)
        X = np.zeros((4, 4))
        X[:3, :3], X[:3, 3] = _hat(dw), du
        T = np.eye(4)
        T[:3, :3], T[:3, 3] = _R(pose[:3]), pose[3:]
        T2 = expm(X) @ T
        np.testing.assert_allclose(_R(out[:3]), T2[:3, :3], atol=1e-13)
        np.testing.assert_allclose(out[3:], T2[:3, 3], atol=1e-13)


def _obs(w, i):
    pose = np.zeros(9)
    pose[:6] = w.poses.reshape(-1, 6)[w.keyframe_index[i]]
    X = w.landmarks.reshape(-1, 3)[w.landmark_index[i]].copy()
    return pose, X, w.observations[2 * i: 2 * i + 2].copy(), int(w.rig_camera[i])


def _rj(rig, pose, X, uv, cam):
    r, J = np.zeros(2), np.zeros(24)
    O.oracle().orc_rig_residual_jacobian(O.f64(pose), O.f64(X), O.f64(uv), rig, cam, O.f64(r), O.f64(J))
    return r, J.reshape(2, 12)


def test_rig_residual_matches_the_window_projection():
    w = LocalBAWindow.synthetic(seed=3, num_landmarks=200)
    rig = O.rig_from_window(w)
    r, _, cost, ok = O.evaluate_rig(O.window_problem(w), rig)
    uv, depth = w.project()
    assert ok and np.all(depth > 0)
    np.testing.assert_allclose(r, w.observations.reshape(-1, 2) - uv, rtol=1e-12, atol=1e-9)
    assert cost == pytest.approx(0.5 * np.sum(r ** 2), rel=1e-12)


def test_rig_jacobian_is_the_reference_formula():
    """Left camera (identity extrinsic): the pose and point columns are the
    derivatives of the SE3 left update (central differences).  Right camera:
    the point columns are exact; the pose columns are EdgeProjection's
    formula evaluated at the rig camera's point (a rotation taken about the
    rig camera's origin), which differs from the derivative of the update by
    the baseline coupling, as in the reference."""
    w = LocalBAWindow.synthetic(seed=4, num_landmarks=300)
    rig = O.rig_from_window(w)
    h = 1e-6
    seen = {0: 0, 1: 0}
    for i in range(0, w.num_observations, 23):
        pose, X, uv, cam = _obs(w, i)
        seen[cam] += 1
        r, J = _rj(rig, pose, X, uv, cam)
        fdp = np.zeros((2, 3))
        for c in range(3):
            Xp, Xm = X.copy(), X.copy()
            Xp[c] += h
            Xm[c] -= h
            fdp[:, c] = (_rj(rig, pose, Xp, uv, cam)[0] - _rj(rig, pose, Xm, uv, cam)[0]) / (2 * h)
        np.testing.assert_allclose(J[:, 9:], fdp, rtol=1e-5, atol=1e-6 * np.abs(fdp).max())
        np.testing.assert_array_equal(J[:, 6:9], 0.0)
        # the reference's pose columns, restated from its formula
        R = _R(pose[:3])
        Re, te = _R(w.extrinsics[cam, :3]), w.extrinsics[cam, 3:]
        Xc, Yc, Zc = Re @ (R @ X + pose[3:6]) + te
        fx, fy = w.fx, w.fy
        zi = 1.0 / (Zc + 1e-18)
        ref = np.array([[-fx * zi, 0, fx * Xc * zi * zi, fx * Xc * Yc * zi * zi, -fx - fx * Xc * Xc * zi * zi, fx * Yc * zi],
                        [0, -fy * zi, fy * Yc * zi * zi, fy + fy * Yc * Yc * zi * zi, -fy * Xc * Yc * zi * zi, -fy * Xc * zi]])
        np.testing.assert_allclose(J[:, 0:3], ref[:, 3:6], rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(J[:, 3:6], ref[:, 0:3], rtol=1e-12, atol=1e-9)
        if cam == 0:
            fd = np.zeros((2, 6))
            for c in range(6):
                xi = np.zeros(6)
                xi[c] = h
                pp, pm = np.zeros(9), np.zeros(9)
                pp[:6] = O.se3_compose_left(xi[:3], xi[3:], pose[:6])
                pm[:6] = O.se3_compose_left(-xi[:3], -xi[3:], pose[:6])
                fd[:, c] = (_rj(rig, pp, X, uv, cam)[0] - _rj(rig, pm, X, uv, cam)[0]) / (2 * h)
            np.testing.assert_allclose(J[:, :6], fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())
    assert seen[0] > 0 and seen[1] > 0


def test_window_outlier_threshold_loop():
    chi2 = np.array([1.0, 2.0, 7.0, 3.0, 9.0, 0.5, 20.0, 1.0, 2.0, 4.0])
    fl, ni, no_, th = O.window_outliers(chi2)
    assert th == 5.991 and (ni, no_) == (7, 3)
    np.testing.assert_array_equal(fl, chi2 > 5.991)
    # more than half above: doubled until the inliers are the majority
    chi2 = np.array([7.0, 8.0, 9.0, 13.0, 30.0, 1.0])
    fl, ni, no_, th = O.window_outliers(chi2)
    assert th == pytest.approx(5.991 * 2) and (ni, no_) == (4, 2)
    np.testing.assert_array_equal(fl, chi2 > th)
    # never: five doublings, the counts of the last pass (at 16 x)
    chi2 = np.full(4, 1e6)
    fl, ni, no_, th = O.window_outliers(chi2)
    assert th == pytest.approx(5.991 * 32) and (ni, no_) == (0, 4) and fl.all()


@pytest.mark.parametrize("policy", ["g2o", "ceres"])
def test_oracle_window_without_noise_converges(policy):
    w, truth = LocalBAWindow.synthetic(seed=5, num_landmarks=300, pixel_noise=0.0, outlier_fraction=0.0,
                                       return_truth=True)
    s = O.solve(O.window_problem(w), rig=O.rig_from_window(w), linear_solver="dense_schur", max_num_iterations=30,
                lm_policy=policy, loss="huber", loss_scale=5.991, **FIXED)
    assert s["initial_cost"] > 1e3 and s["final_cost"] < 1e-12 * s["initial_cost"]


def test_oracle_window_flags_the_planted_outliers():
    w = LocalBAWindow.synthetic(seed=6, num_landmarks=400, outlier_fraction=0.05)
    s = O.solve(O.window_problem(w), rig=O.rig_from_window(w), linear_solver="dense_schur", max_num_iterations=10,
                lm_policy="g2o", loss="huber", loss_scale=5.991, **FIXED)
    p = O.window_problem(w)
    p.params[:] = s["parameters"]
    r, _, _, ok = O.evaluate_rig(p, O.rig_from_window(w))
    fl, ni, no_, th = O.window_outliers(np.sum(r * r, axis=1))
    assert ok and th == 5.991 and ni + no_ == w.num_observations
    # the 20-60 px outliers are all flagged; the rest is chi2 with 2 dof
    # of unit pixel noise (about 5 % above 5.991)
    assert 0.05 <= no_ / w.num_observations <= 0.13


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture_window(g):
    K = g["window_K"]
    return LocalBAWindow(g["window_keyframe_index"], g["window_landmark_index"], g["window_rig_camera"],
                         g["window_observations"], g["window_poses"], g["window_landmarks"], K[0], K[1], K[2],
                         K[3], g["window_extrinsics"])


def test_oracle_reproduces_the_variant_fixtures():
    """The oracle's g2o-variant solve and local-BA solve against the stored
    ones (tests/golden/make_golden.py): a change to either restatement shows
    here first."""
    from slamplay_gb300 import G2O_VARIANT, LOCAL_BA
    g = np.load(os.path.join(GOLDEN, "variants.npz"))
    gs = np.load(os.path.join(GOLDEN, "small_problem.npz"))
    p = O.Problem(int(gs["num_cameras"]), int(gs["num_points"]), gs["camera_index"], gs["point_index"],
                  gs["observations"], gs["parameters"])
    r = O.solve(p, linear_solver="dense_schur", **dict(G2O_VARIANT, max_num_iterations=15))
    np.testing.assert_allclose(r["trace_cost"], g["g2o_trace_cost"], rtol=1e-12)
    np.testing.assert_allclose(r["trace_radius"], g["g2o_trace_radius"], rtol=1e-12)
    np.testing.assert_allclose(r["parameters"], g["g2o_final_parameters"], rtol=1e-9, atol=1e-9)
    w = _fixture_window(g)
    rig = O.rig_from_window(w)
    r = O.solve(O.window_problem(w), rig=rig, linear_solver="dense_schur", **LOCAL_BA)
    np.testing.assert_allclose(r["trace_cost"], g["window_trace_cost"], rtol=1e-12)
    np.testing.assert_allclose(r["parameters"], g["window_final_parameters"], rtol=1e-9, atol=1e-9)
    q = O.window_problem(w)
    q.params[:] = r["parameters"]
    res, _, _, ok = O.evaluate_rig(q, rig)
    chi2 = np.sum(res * res, axis=1)
    np.testing.assert_allclose(chi2, g["window_chi2"], rtol=1e-9, atol=1e-12)
    flags, _, _, th = O.window_outliers(chi2)
    assert th == g["window_threshold"][0] and np.array_equal(flags, g["window_outlier"])


def test_se3_left_update_inverse_and_identity():
    rng = np.random.default_rng(11)
    for _ in range(100):
        pose = np.concatenate([rng.normal(size=3) * 0.7, rng.normal(size=3) * 3])
        dw, du = rng.normal(size=3) * rng.choice([1.0, 1e-3, 1e-7]), rng.normal(size=3)
        # the identity: translation exact, rotation through the quaternion round trip
        same = O.se3_compose_left(np.zeros(3), np.zeros(3), pose)
        np.testing.assert_array_equal(same[3:], pose[3:])
        np.testing.assert_allclose(same[:3], pose[:3], rtol=1e-14, atol=1e-15)
        # exp(-xi) exp(xi) T = T
        back = O.se3_compose_left(-dw, -du, O.se3_compose_left(dw, du, pose))
        np.testing.assert_allclose(_R(back[:3]), _R(pose[:3]), atol=1e-12)
        np.testing.assert_allclose(back[3:], pose[3:], atol=1e-11)


def test_synthetic_window_is_deterministic_and_in_spec():
    a, ta = LocalBAWindow.synthetic(seed=12, return_truth=True)
    b = LocalBAWindow.synthetic(seed=12)
    for k in ("keyframe_index", "landmark_index", "rig_camera", "observations", "poses", "landmarks"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    assert a.num_keyframes == 7 and set(np.unique(a.rig_camera)) <= {0, 1}
    assert np.all(np.bincount(a.landmark_index, minlength=a.num_landmarks) >= 2)
    # the truth projects every edge in front of its camera and inside the image
    uv, depth = ta.project()
    ideal = uv.copy()
    assert np.all(depth > 1.0) and np.all((ideal[:, 0] > 0) & (ideal[:, 0] < 1241) & (ideal[:, 1] > 0) & (ideal[:, 1] < 376))
    # the first keyframe is not perturbed (the others are)
    np.testing.assert_array_equal(a.poses[:6], ta.poses[:6])
    assert not np.array_equal(a.poses[6:], ta.poses[6:])


def test_window_rejects_inconsistent_arrays():
    w = LocalBAWindow.synthetic(seed=1, num_landmarks=60)
    args = [w.keyframe_index, w.landmark_index, w.rig_camera, w.observations, w.poses, w.landmarks,
            w.fx, w.fy, w.cx, w.cy, w.extrinsics]
    LocalBAWindow(*args)  # consistent
    for v in (2, 256, 257, -1):  # integers that a byte cast would wrap into 0 or 1 are rejected too
        bad = list(args)
        bad[2] = np.full(w.rig_camera.shape, v, dtype=np.int64)
        with pytest.raises(ValueError):
            LocalBAWindow(*bad)
    bad = list(args)
    bad[0] = w.keyframe_index.copy()
    bad[0][0] = w.num_keyframes
    with pytest.raises(ValueError):
        LocalBAWindow(*bad)
    bad = list(args)
    bad[3] = w.observations[:-2]
    with pytest.raises(ValueError):
        LocalBAWindow(*bad)
