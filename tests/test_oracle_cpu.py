"""The CPU oracle on its own: golden fixture, known answers, and independent
cross-checks (finite differences, scipy least_squares)."""
import os

import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "small_problem.npz")
FIXED = dict(function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0)


def golden_problem():
    g = np.load(GOLDEN)
    return g, O.Problem(int(g["num_cameras"]), int(g["num_points"]), g["camera_index"], g["point_index"],
                        g["observations"], g["parameters"])


@pytest.mark.parametrize("loss", ["trivial", "huber"])
def test_oracle_reproduces_golden_fixture(loss):
    g, p = golden_problem()
    r = O.solve(p, loss=loss, max_num_iterations=15, linear_solver="dense_schur", **FIXED)
    np.testing.assert_allclose(r["trace_cost"], g[f"{loss}_trace_cost"], rtol=1e-12)
    np.testing.assert_allclose(r["parameters"], g[f"{loss}_final_parameters"], rtol=1e-9, atol=1e-9)


def test_jacobian_matches_central_differences():
    b = BALProblem.synthetic(0, seed=2, num_points=30)
    cams = b.cameras().reshape(-1, 9)
    pts = b.points().reshape(-1, 3)
    for i in range(0, b.num_observations(), 17):
        cam = cams[b.camera_index()[i]].copy()
        pt = pts[b.point_index()[i]].copy()
        uv = b.observations()[2 * i: 2 * i + 2].copy()
        r0, J = np.zeros(2), np.zeros(24)
        O.oracle().orc_residual_jacobian(O.f64(cam), O.f64(pt), O.f64(uv), O.f64(r0), O.f64(J))
        J = J.reshape(2, 12)
        x = np.concatenate([cam, pt])
        for k in range(12):
            h = 1e-6 * max(1.0, abs(x[k]))
            rr = []
            for s in (+1, -1):
                y = x.copy()
                y[k] += s * h
                r = np.zeros(2)
                O.oracle().orc_residual_jacobian(O.f64(np.ascontiguousarray(y[:9])), O.f64(np.ascontiguousarray(y[9:])),
                                                 O.f64(uv), O.f64(r), O.f64(np.zeros(24)))
                rr.append(r)
            fd = (rr[0] - rr[1]) / (2 * h)
            assert np.allclose(J[:, k], fd, rtol=1e-5, atol=1e-5 * (1 + np.abs(J).max())), (k, J[:, k], fd)


def test_zero_noise_problem_converges_to_zero_cost():
    b, truth = BALProblem.synthetic(0, seed=5, num_points=400, pixel_noise=0.0, return_truth=True)
    r = O.solve(O.Problem.from_bal(b), max_num_iterations=30, linear_solver="dense_schur")
    assert r["initial_cost"] > 1e3
    assert r["final_cost"] < 1e-12 * r["initial_cost"]


@pytest.mark.parametrize("loss", ["trivial", "cauchy"])
def test_dense_and_pcg_schur_agree(loss):
    b = BALProblem.synthetic(0, seed=6, num_points=500)
    a = O.solve(O.Problem.from_bal(b), max_num_iterations=10, linear_solver="dense_schur", loss=loss, **FIXED)
    c = O.solve(O.Problem.from_bal(b), max_num_iterations=10, linear_solver="pcg_schur", pcg_tolerance=1e-13,
                max_linear_solver_iterations=2000, loss=loss, **FIXED)
    assert a["final_cost"] < 0.1 * a["initial_cost"]
    assert abs(a["final_cost"] - c["final_cost"]) <= 1e-10 * a["final_cost"]


def test_cauchy_cost_formula_and_corrector():
    """CauchyLoss(a) (backend/ceres/test_ceres_bundle_adjuster_simple.cpp:193):
    rho(s) = a^2 log(1 + s / a^2) of each observation's squared residual
    norm.  The evaluation returns the raw residuals and Jacobians (the
    solver applies the corrector; the GPU parity tests solve with it)."""
    b = BALProblem.synthetic(0, seed=7, num_points=100)
    p = O.Problem.from_bal(b)
    r, J, c_triv, _ = O.evaluate(p, "trivial")
    for a in (1.0, 2.5):
        rc, Jc, c_cau, ok = O.evaluate(p, "cauchy", a)
        assert ok
        s = (r ** 2).sum(axis=1)
        b2 = a * a
        assert abs(c_cau - 0.5 * (b2 * np.log1p(s / b2)).sum()) <= 1e-9 * c_cau
        np.testing.assert_array_equal(rc, r)
        np.testing.assert_array_equal(Jc, J)
        assert c_cau < c_triv


def test_huber_cost_formula():
    b = BALProblem.synthetic(0, seed=7, num_points=100)
    p = O.Problem.from_bal(b)
    r, _, c_triv, _ = O.evaluate(p, "trivial")
    _, _, c_hub, _ = O.evaluate(p, "huber", 1.0)
    s = (r ** 2).sum(axis=1)
    rho = np.where(s > 1.0, 2.0 * np.sqrt(s) - 1.0, s)
    assert abs(c_triv - 0.5 * s.sum()) <= 1e-9 * c_triv
    assert abs(c_hub - 0.5 * rho.sum()) <= 1e-9 * c_hub


def test_final_cost_matches_scipy_least_squares():
    scipy_opt = pytest.importorskip("scipy.optimize")
    b = BALProblem.synthetic(0, seed=21, num_cameras=6, num_points=60)
    p = O.Problem.from_bal(b)
    x0 = b.parameters().copy()
    nc = b.num_cameras()
    ci, pi = b.camera_index(), b.point_index()

    def fun(x):
        q = O.Problem(nc, b.num_points(), ci, pi, b.observations(), x)
        r, _, _, _ = O.evaluate(q)
        return r.reshape(-1)

    def jac(x):
        q = O.Problem(nc, b.num_points(), ci, pi, b.observations(), x)
        _, J, _, _ = O.evaluate(q)
        full = np.zeros((2 * len(ci), x.size))
        for i in range(len(ci)):
            full[2 * i: 2 * i + 2, 9 * ci[i]: 9 * ci[i] + 9] = J[i, :, :9]
            full[2 * i: 2 * i + 2, 9 * nc + 3 * pi[i]: 9 * nc + 3 * pi[i] + 3] = J[i, :, 9:]
        return full

    ls = scipy_opt.least_squares(fun, x0, jac=jac, method="trf", x_scale="jac", xtol=1e-15, ftol=1e-15,
                                 gtol=1e-15, max_nfev=400)
    r = O.solve(p, max_num_iterations=100, linear_solver="dense_schur", function_tolerance=1e-15,
                parameter_tolerance=1e-15, gradient_tolerance=1e-15)
    assert abs(r["final_cost"] - ls.cost) <= 1e-6 * ls.cost, (r["final_cost"], ls.cost)


def _rotate(w, x):
    out = np.zeros(3)
    O.oracle().orc_angle_axis_rotate_point(O.f64(np.ascontiguousarray(w, dtype=np.float64)),
                                           O.f64(np.ascontiguousarray(x, dtype=np.float64)), O.f64(out))
    return out


def _rotation_matrix(w):
    return np.stack([_rotate(w, e) for e in np.eye(3)], axis=1)


@pytest.mark.parametrize("scale", [2.0, 0.3, 1e-5, 0.0])
def test_compose_left_is_rotation_product(scale):
    """The g2o camera update R <- exp(dw) R (test_bundle_adjustment_g2o.cpp:84-90) in angle-axis form."""
    rng = np.random.default_rng(int(scale * 1e6) + 3)
    for _ in range(200):
        w = rng.normal(size=3) * scale
        dw = rng.normal(size=3) * rng.choice([1.0, 1e-3, 1e-9])
        out = O.compose_left(dw, w)
        assert np.linalg.norm(out) <= np.pi + 1e-12
        np.testing.assert_allclose(_rotation_matrix(out), _rotation_matrix(dw) @ _rotation_matrix(w), atol=1e-13)
    np.testing.assert_array_equal(O.compose_left(np.zeros(3), np.zeros(3)), np.zeros(3))


def test_so3_left_jacobian_matches_central_differences():
    b = BALProblem.synthetic(0, seed=2, num_points=30)
    p = O.Problem.from_bal(b)
    r0, Ja, _, ok = O.evaluate(p)
    r1, Jl, _, ok1 = O.evaluate(p, camera_update="so3_left")
    assert ok and ok1
    np.testing.assert_array_equal(r0, r1)
    np.testing.assert_array_equal(Ja[:, :, 3:], Jl[:, :, 3:])
    cams = b.cameras().reshape(-1, 9)
    pts = b.points().reshape(-1, 3)
    for i in range(0, b.num_observations(), 13):
        cam = cams[b.camera_index()[i]]
        pt = np.ascontiguousarray(pts[b.point_index()[i]])
        uv = np.ascontiguousarray(b.observations()[2 * i: 2 * i + 2])
        h = 1e-6
        for k in range(3):
            rr = []
            for s in (+1, -1):
                c = cam.copy()
                c[:3] = O.compose_left(s * h * np.eye(3)[k], cam[:3])
                r = np.zeros(2)
                O.oracle().orc_residual_jacobian(O.f64(c), O.f64(pt), O.f64(uv), O.f64(r), O.f64(np.zeros(24)))
                rr.append(r)
            fd = (rr[0] - rr[1]) / (2 * h)
            assert np.allclose(Jl[i, :, k], fd, rtol=1e-5, atol=1e-5 * (1 + np.abs(Jl[i]).max())), (k, Jl[i, :, k], fd)


def test_so3_left_update_reaches_the_additive_minimum():
    b, truth = BALProblem.synthetic(0, seed=5, num_points=400, pixel_noise=0.0, return_truth=True)
    r = O.solve(O.Problem.from_bal(b), max_num_iterations=30, linear_solver="dense_schur", camera_update="so3_left")
    assert r["initial_cost"] > 1e3 and r["final_cost"] < 1e-12 * r["initial_cost"]
    b = BALProblem.synthetic(0, seed=6, num_points=500)
    a = O.solve(O.Problem.from_bal(b), max_num_iterations=40, linear_solver="dense_schur")
    c = O.solve(O.Problem.from_bal(b), max_num_iterations=40, linear_solver="dense_schur", camera_update="so3_left")
    assert a["final_cost"] < a["initial_cost"] and abs(a["final_cost"] - c["final_cost"]) <= 1e-6 * a["final_cost"]
    assert not np.array_equal(a["trace_cost"][1:3], c["trace_cost"][1:3])


def _dense_jacobian(b, camera_update="additive"):
    p = O.Problem.from_bal(b)
    r, J, cost, ok = O.evaluate(p, camera_update=camera_update)
    assert ok
    nc, no = b.num_cameras(), b.num_observations()
    n = 9 * nc + 3 * b.num_points()
    Jd = np.zeros((2 * no, n))
    rows = np.arange(no)
    for k in range(9):
        Jd[2 * rows, 9 * b.camera_index() + k] = J[:, 0, k]
        Jd[2 * rows + 1, 9 * b.camera_index() + k] = J[:, 1, k]
    for k in range(3):
        Jd[2 * rows, 9 * nc + 3 * b.point_index() + k] = J[:, 0, 9 + k]
        Jd[2 * rows + 1, 9 * nc + 3 * b.point_index() + k] = J[:, 1, 9 + k]
    return r.reshape(-1), Jd, cost


@pytest.mark.parametrize("camera_update", ["additive", "so3_left"])
def test_g2o_policy_first_step_is_the_damped_gauss_newton_step(camera_update):
    """g2o's Levenberg step: (J^T J + lambda_0 I) dx = -J^T r with
    lambda_0 = 1e-5 max diag(J^T J), unscaled, solved densely here."""
    b = BALProblem.synthetic(0, seed=3, num_points=60)
    r, Jd, cost0 = _dense_jacobian(b, camera_update)
    H = Jd.T @ Jd
    lam = 1e-5 * np.max(np.diag(H))
    dx = np.linalg.solve(H + lam * np.eye(H.shape[0]), -Jd.T @ r)
    x1 = b.parameters().copy()
    nc = b.num_cameras()
    x1 += dx
    if camera_update == "so3_left":
        for c in range(nc):
            x1[9 * c: 9 * c + 3] = O.compose_left(dx[9 * c: 9 * c + 3], b.parameters()[9 * c: 9 * c + 3])
    q = O.Problem(nc, b.num_points(), b.camera_index(), b.point_index(), b.observations(), x1)
    _, _, cost1, _ = O.evaluate(q)
    s = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=1, lm_policy="g2o",
                camera_update=camera_update, **FIXED)
    assert s["trace_radius"][0] == pytest.approx(1.0 / lam, rel=1e-12)
    assert s["trace_cost"][1] == pytest.approx(cost1, rel=1e-9)
    assert s["num_successful_steps"] == 1 and s["termination_reason"] == 1


def test_g2o_policy_damping_updates_and_limits():
    b = BALProblem.synthetic(0, seed=6, num_points=500)
    s = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=40, lm_policy="g2o",
                loss="huber", **FIXED)
    ok = s["trace_successful"]
    rad = s["trace_radius"]
    assert s["final_cost"] < s["initial_cost"]
    for k in range(1, len(rad)):
        f = rad[k] / rad[k - 1]
        if ok[k]:
            assert 1.5 * (1 - 1e-15) <= f <= 3.0 * (1 + 1e-15), (k, f)  # lambda *= [1/3, 2/3]
        else:
            assert f <= 0.5 * (1 + 1e-15), (k, f)  # lambda *= nu >= 2
    # accepted steps never raise the cost
    c = s["trace_cost"]
    acc = [c[0]] + [c[k] for k in range(1, len(c)) if ok[k]]
    assert all(acc[i + 1] < acc[i] for i in range(len(acc) - 1))
    # max_num_iterations bounds outer iterations (accepted steps), not trials
    t = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=4, lm_policy="g2o",
                loss="huber", **FIXED)
    assert t["num_successful_steps"] == 4 and t["termination_reason"] == 1
    # same minimum as the Ceres policy
    a = O.solve(O.Problem.from_bal(b), linear_solver="dense_schur", max_num_iterations=60, loss="huber", **FIXED)
    assert abs(a["final_cost"] - s["final_cost"]) <= 1e-9 * a["final_cost"]
