"""CPU-only checks of libgba: it loads, exports every symbol include/gba.h
declares, host-side helpers work, and GPU entry points fail cleanly without
a GPU.  No compute kernel is called here."""
import ctypes
import os
import re

import numpy as np
import pytest

from slamplay_gb300 import G2O_VARIANT, LOCAL_BA, BALProblem, GBAError, Solver, estimate_footprint, make_options
from slamplay_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(gba_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol():
    lib = ctypes.CDLL(N.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_option_defaults_are_ceres_defaults():
    o = make_options()
    assert o.abi_version == N.GBA_ABI_VERSION
    assert o.max_num_iterations == 50
    assert o.function_tolerance == 1e-6 and o.gradient_tolerance == 1e-10 and o.parameter_tolerance == 1e-8
    assert o.initial_trust_region_radius == 1e4 and o.max_trust_region_radius == 1e16
    assert o.min_relative_decrease == 1e-3 and o.min_lm_diagonal == 1e-6 and o.max_lm_diagonal == 1e32
    assert o.jacobi_scaling == 1 and o.max_num_consecutive_invalid_steps == 5
    assert o.loss == 0 and o.precision == 0
    assert o.camera_update == 0 and make_options(camera_update="so3_left").camera_update == 1
    assert o.lm_policy == 0 and make_options(lm_policy="g2o").lm_policy == 1
    g = make_options(**G2O_VARIANT)
    assert (g.camera_update, g.lm_policy, g.loss, g.max_num_iterations) == (1, 1, 1, 40)
    with pytest.raises(TypeError):
        make_options(no_such_option=1)


def test_local_ba_defaults():
    o = N.Options()
    N.lib().gba_local_ba_options_init(N.C.byref(o))
    ref = make_options(**LOCAL_BA)
    for k in ("lm_policy", "max_num_iterations", "loss", "loss_scale", "function_tolerance", "gradient_tolerance",
              "parameter_tolerance"):
        assert getattr(o, k) == getattr(ref, k), k
    assert (o.lm_policy, o.max_num_iterations, o.loss, o.loss_scale) == (1, 10, 1, 5.991)
    v = N.WindowView()
    N.lib().gba_window_view_init(N.C.byref(v))
    assert v.chi2_threshold == 5.991 and v.max_threshold_doublings == 5 and v.num_observations == 0


def _gpu_present():
    try:
        Solver().close()
        return True
    except GBAError:
        return False


def test_create_without_gpu_fails_cleanly():
    if _gpu_present():
        pytest.skip("a GPU is present")
    with pytest.raises(GBAError) as ei:
        Solver()
    assert ei.value.status == 7  # GBA_ERR_NO_DEVICE
    assert "device" in ei.value.message


def test_bad_options_rejected_before_device():
    with pytest.raises(GBAError) as ei:
        Solver(loss=7)
    assert ei.value.status == 1
    with pytest.raises(GBAError) as ei:
        Solver(camera_update=2)
    assert ei.value.status == 1
    with pytest.raises(GBAError) as ei:
        Solver(lm_policy=-1)
    assert ei.value.status == 1


@pytest.mark.parametrize("config,index", [(0, 0), (3, 0), (3, 5), (4, 2)])
def test_synthetic_is_deterministic_and_in_spec(config, index):
    a = BALProblem.synthetic(config, index=index, seed=9)
    b = BALProblem.synthetic(config, index=index, seed=9)
    assert np.array_equal(a.parameters(), b.parameters())
    assert np.array_equal(a.observations(), b.observations())
    assert np.array_equal(a.camera_index(), b.camera_index())
    c = BALProblem.synthetic(config, index=index, seed=10)
    assert not np.array_equal(a.observations(), c.observations()) or a.num_observations() != c.num_observations()
    deg = np.bincount(a.point_index(), minlength=a.num_points())
    if config == 0:
        assert a.num_cameras() == 16 and a.num_points() == 2000
        assert deg.min() >= 4 and deg.max() <= 10
        assert 12000 <= a.num_observations() <= 16000
    if config == 3:
        assert 5 <= a.num_cameras() <= 40 and 200 <= a.num_points() <= 5000
        assert deg.max() <= 8
    if config == 4:
        assert 10 <= a.num_cameras() <= 400 and 1000 <= a.num_points() <= 150000
    # every observation pair is unique (a camera sees a point once)
    key = a.point_index().astype(np.int64) * a.num_cameras() + a.camera_index()
    assert len(np.unique(key)) == a.num_observations()


def test_synthetic_truth_has_noise_level_cost():
    b, truth = BALProblem.synthetic(0, seed=3, return_truth=True)
    from oracle import oracle_py as O
    p = O.Problem(b.num_cameras(), b.num_points(), b.camera_index(), b.point_index(), b.observations(), truth)
    _, _, cost, ok = O.evaluate(p)
    # N(0, 0.5 px) per coordinate: E[cost] = 0.5 * 2 * no * 0.25
    assert ok and abs(cost / (0.25 * b.num_observations()) - 1.0) < 0.1


def test_bal_write_read_roundtrip(tmp_path):
    b = BALProblem.synthetic(0, seed=4, num_points=200)
    f = str(tmp_path / "p.txt")
    b.WriteToFile(f)
    r = BALProblem(f)
    assert (r.num_cameras(), r.num_points(), r.num_observations()) == (b.num_cameras(), b.num_points(),
                                                                         b.num_observations())
    assert np.array_equal(r.camera_index(), b.camera_index())
    assert np.array_equal(r.point_index(), b.point_index())
    np.testing.assert_allclose(r.observations(), b.observations(), rtol=1e-5)  # "%g" as the reference
    np.testing.assert_allclose(r.parameters(), b.parameters(), rtol=1e-15, atol=1e-300)  # "%.16g"


def test_bal_read_errors(tmp_path):
    with pytest.raises(GBAError) as ei:
        BALProblem(str(tmp_path / "missing.txt"))
    assert ei.value.status == 6
    f = tmp_path / "bad.txt"
    f.write_text("2 3 4\n0 0 1.0\n")
    with pytest.raises(GBAError):
        BALProblem(str(f))


def test_quaternion_layout_roundtrip(tmp_path):
    b = BALProblem.synthetic(0, seed=4, num_points=50)
    f = str(tmp_path / "p.txt")
    b.WriteToFile(f)
    q = BALProblem(f, use_quaternions=True)
    assert q.camera_block_size() == 10 and q.num_parameters() == 10 * q.num_cameras() + 3 * q.num_points()
    np.testing.assert_allclose(q.to_angle_axis_parameters(), BALProblem(f).parameters(), rtol=1e-12, atol=1e-14)
    with pytest.raises(ValueError):
        q.view()


def test_footprint_estimate_monotone():
    a = estimate_footprint(250, 60000, 300000, "fp64")
    b = estimate_footprint(250, 60000, 300000, "mixed")
    c = estimate_footprint(1800, 1000000, 5000000, "mixed")
    assert b < a < c
    assert 50e6 < a < 400e6


def test_c_abi_header_is_plain_c():
    """include/gba.h is the C ABI: it compiles as C99 with every warning on,
    and a C caller can fill the window view and the options."""
    import shutil
    import subprocess
    import tempfile
    if shutil.which("gcc") is None:
        pytest.skip("gcc missing")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = ("#include \"gba.h\"\n"
           "int main(void) {\n"
           "  gba_options o; gba_window_view w; gba_window_result r;\n"
           "  gba_local_ba_options_init(&o); gba_window_view_init(&w);\n"
           "  o.camera_update = GBA_CAMERA_UPDATE_SO3_LEFT; o.lm_policy = GBA_LM_POLICY_G2O;\n"
           "  w.rig.extrinsic[1][3] = -0.5; r.num_inliers = 0;\n"
           "  return (int)(w.max_threshold_doublings + r.num_inliers - 5);\n"
           "}\n")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        with open(c, "w") as f:
            f.write(src)
        r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                            "-I", os.path.join(root, "include"), c], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
