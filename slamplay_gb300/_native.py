"""ctypes declarations of include/gba.h and the loader of libgba.so.

The library is built in-tree (slamplay_gb300/_build/libgba.so).  There is no
fallback: if it is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgba.so")

GBA_ABI_VERSION = 1

STATUS = {
    0: "GBA_OK", 1: "GBA_ERR_INVALID_ARGUMENT", 2: "GBA_ERR_OUT_OF_MEMORY",
    3: "GBA_ERR_NON_FINITE", 4: "GBA_ERR_CUDA", 5: "GBA_ERR_TIMEOUT", 6: "GBA_ERR_IO",
    7: "GBA_ERR_NO_DEVICE", 8: "GBA_ERR_QUEUE_FULL", 9: "GBA_ERR_NOT_FOUND", 10: "GBA_ERR_INTERNAL",
}
TERMINATION = {0: "CONVERGENCE", 1: "NO_CONVERGENCE", 2: "FAILURE"}
REASON = {0: "none", 1: "max_iterations", 2: "function_tolerance", 3: "gradient_tolerance",
          4: "parameter_tolerance", 5: "min_trust_region_radius", 6: "invalid_steps",
          7: "evaluation_failed", 8: "lm_trials"}
LOSS = {"trivial": 0, "huber": 1, "cauchy": 2}
PRECISION = {"fp64": 0, "mixed": 1}
PCG_CRITERION = {"residual": 0, "quadratic_model": 1}
SCHUR = {"auto": 0, "implicit": 1, "explicit": 2}
CAMERA_UPDATE = {"additive": 0, "so3_left": 1}
LM_POLICY = {"ceres": 0, "g2o": 1}
CAMERA_LAYOUT = {"angle_axis": 0, "quaternion": 1}

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class Options(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32), ("max_num_iterations", C.c_int32),
        ("function_tolerance", C.c_double), ("gradient_tolerance", C.c_double),
        ("parameter_tolerance", C.c_double), ("initial_trust_region_radius", C.c_double),
        ("max_trust_region_radius", C.c_double), ("min_trust_region_radius", C.c_double),
        ("min_relative_decrease", C.c_double), ("min_lm_diagonal", C.c_double),
        ("max_lm_diagonal", C.c_double), ("max_num_consecutive_invalid_steps", C.c_int32),
        ("jacobi_scaling", C.c_int32), ("loss", C.c_int32), ("loss_scale", C.c_double),
        ("precision", C.c_int32), ("pcg_criterion", C.c_int32),
        ("max_linear_solver_iterations", C.c_int32), ("min_linear_solver_iterations", C.c_int32),
        ("pcg_tolerance", C.c_double), ("eta", C.c_double),
        ("minimizer_progress_to_stdout", C.c_int32), ("device", C.c_int32), ("stream", C.c_void_p),
        ("chunk_observations", C.c_int32), ("reorder_points", C.c_int32), ("use_graphs", C.c_int32),
        ("pcg_unroll", C.c_int32), ("autotune", C.c_int32), ("schur", C.c_int32), ("persistent_pcg", C.c_int32),
        ("camera_update", C.c_int32), ("lm_policy", C.c_int32), ("camera_layout", C.c_int32), ("server_slots", C.c_int32),
    ]


class Summary(C.Structure):
    _fields_ = [
        ("initial_cost", C.c_double), ("final_cost", C.c_double),
        ("num_iterations", C.c_int32), ("num_successful_steps", C.c_int32),
        ("num_unsuccessful_steps", C.c_int32), ("num_invalid_steps", C.c_int32),
        ("num_linear_solver_iterations", C.c_int64), ("termination_type", C.c_int32),
        ("termination_reason", C.c_int32), ("final_trust_region_radius", C.c_double),
        ("gradient_max_norm", C.c_double), ("setup_time_s", C.c_double),
        ("solve_time_s", C.c_double), ("total_time_s", C.c_double),
        ("trace_capacity", C.c_int32), ("trace_length", C.c_int32),
        ("trace_cost", _f64p), ("trace_radius", _f64p),
        ("trace_linear_iterations", _i32p), ("trace_successful", _i32p),
    ]


class ProblemView(C.Structure):
    _fields_ = [
        ("num_cameras", C.c_int32), ("num_points", C.c_int32), ("num_observations", C.c_int32),
        ("camera_index", _i32p), ("point_index", _i32p), ("observations", _f64p),
        ("parameters", _f64p),
    ]


class Rig(C.Structure):
    _fields_ = [("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
                ("extrinsic", (C.c_double * 6) * 2)]


class WindowView(C.Structure):
    _fields_ = [
        ("num_keyframes", C.c_int32), ("num_landmarks", C.c_int32), ("num_observations", C.c_int32),
        ("keyframe_index", _i32p), ("landmark_index", _i32p), ("rig_camera", C.POINTER(C.c_uint8)),
        ("observations", _f64p), ("poses", _f64p), ("landmarks", _f64p), ("rig", Rig),
        ("chi2_threshold", C.c_double), ("max_threshold_doublings", C.c_int32),
        ("outlier", C.POINTER(C.c_uint8)),
    ]


class WindowResult(C.Structure):
    _fields_ = [("num_inliers", C.c_int32), ("num_outliers", C.c_int32), ("chi2_threshold", C.c_double)]


class SynthSpec(C.Structure):
    _fields_ = [
        ("layout", C.c_int32), ("num_cameras", C.c_int32), ("num_points", C.c_int32),
        ("min_views", C.c_int32), ("max_views", C.c_int32), ("view_distribution", C.c_int32),
        ("view_param", C.c_double), ("focal", C.c_double), ("k1_range", C.c_double),
        ("k2_range", C.c_double), ("pixel_noise", C.c_double), ("rotation_noise", C.c_double),
        ("translation_noise", C.c_double), ("point_noise", C.c_double),
        ("focal_noise", C.c_double), ("seed", C.c_uint64),
    ]


class DeviceProblem(C.Structure):
    """gba_device_problem: device pointers (as integers) of a resident problem."""
    _fields_ = [
        ("num_cameras", C.c_int32), ("num_points", C.c_int32), ("num_observations", C.c_int32),
        ("camera_index", C.c_void_p), ("point_index", C.c_void_p), ("observations", C.c_void_p),
        ("cameras", C.c_void_p), ("points", C.c_void_p),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
        ("rejected", C.c_int64), ("live", C.c_int32), ("queued", C.c_int32),
        ("peak_live", C.c_int32), ("steps", C.c_int64), ("device_bytes_in_use", C.c_size_t),
        ("device_bytes_peak", C.c_size_t), ("reforms", C.c_int64), ("host_prep_s", C.c_double),
    ]


TUNE_MAX_TRIALS = 32


class TuneResult(C.Structure):
    _fields_ = [
        ("chunk_observations", C.c_int32), ("pcg_unroll", C.c_int32), ("num_trials", C.c_int32),
        ("from_cache", C.c_int32), ("best_ms", C.c_double), ("pcg_cameras_per_cta", C.c_int32),
        ("pcg_cap", C.c_int32), ("pcg_grid_ctas", C.c_int32), ("reserved_", C.c_int32),
        ("trial_ms", C.c_double * TUNE_MAX_TRIALS),
        ("trial_step", C.c_int32 * TUNE_MAX_TRIALS), ("trial_chunk", C.c_int32 * TUNE_MAX_TRIALS),
        ("trial_unroll", C.c_int32 * TUNE_MAX_TRIALS), ("trial_cameras_per_cta", C.c_int32 * TUNE_MAX_TRIALS),
        ("trial_cap", C.c_int32 * TUNE_MAX_TRIALS), ("trial_grid_ctas", C.c_int32 * TUNE_MAX_TRIALS),
        ("trial_final_cost", C.c_double * TUNE_MAX_TRIALS),
    ]


class GBAError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "gba_autotune": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), C.c_int32, C.POINTER(TuneResult)]),
    "gba_options_init": (None, [C.POINTER(Options)]),
    "gba_create": (C.c_int, [C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "gba_destroy": (None, [C.c_void_p]),
    "gba_last_error": (C.c_char_p, [C.c_void_p]),
    "gba_version": (C.c_char_p, []),
    "gba_solve": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), C.POINTER(Summary)]),
    "gba_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), C.c_int32, C.POINTER(Summary)]),
    "gba_local_ba_options_init": (None, [C.POINTER(Options)]),
    "gba_window_view_init": (None, [C.POINTER(WindowView)]),
    "gba_local_ba": (C.c_int, [C.c_void_p, C.POINTER(WindowView), C.c_int32, C.POINTER(Summary),
                               C.POINTER(WindowResult)]),
    "gba_server_start": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int32, C.c_int32]),
    "gba_submit": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), C.POINTER(C.c_uint64)]),
    "gba_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Summary), C.POINTER(C.c_int32)]),
    "gba_server_stop": (C.c_int, [C.c_void_p]),
    "gba_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "gba_estimate_footprint": (C.c_size_t, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "gba_evaluate": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), _f64p, _f64p, _f64p]),
    "gba_compute_step": (C.c_int, [C.c_void_p, C.POINTER(ProblemView), C.c_double, _f64p, _f64p, _i32p]),
    "gba_solve_resident": (C.c_int, [C.c_void_p, C.c_int32]),
    "gba_synchronize": (C.c_int, [C.c_void_p]),
    "gba_evaluate_noalloc": (C.c_int, [C.POINTER(DeviceProblem), C.c_int32, C.c_double, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "gba_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "gba_profile_count": (C.c_int32, [C.c_void_p]),
    "gba_profile_entry": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_int64),
                                    _f64p, _f64p]),
    "gba_bal_read_header": (C.c_int, [C.c_char_p, _i32p, _i32p, _i32p]),
    "gba_bal_read": (C.c_int, [C.c_char_p, C.POINTER(ProblemView)]),
    "gba_bal_write": (C.c_int, [C.c_char_p, C.POINTER(ProblemView)]),
    "gba_bal_write_ply": (C.c_int, [C.c_char_p, C.POINTER(ProblemView)]),
    "gba_bal_normalize": (C.c_int, [C.POINTER(ProblemView)]),
    "gba_bal_perturb": (C.c_int, [C.POINTER(ProblemView), C.c_double, C.c_double, C.c_double, C.c_uint64]),
    "gba_angle_axis_to_quaternion": (None, [_f64p, _f64p]),
    "gba_quaternion_to_angle_axis": (None, [_f64p, _f64p]),
    "gba_angle_axis_rotate_point": (None, [_f64p, _f64p, _f64p]),
    "gba_synth_preset": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, C.POINTER(SynthSpec)]),
    "gba_synth_size": (C.c_int, [C.POINTER(SynthSpec), _i32p, _i32p, _i32p]),
    "gba_synth_generate": (C.c_int, [C.POINTER(SynthSpec), C.POINTER(ProblemView), _f64p]),
}


def lib():
    """The loaded libgba.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"libgba.so not built at {LIB_PATH}; run slamplay_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, handle=None, what: str = "") -> None:
    if status != 0:
        msg = lib().gba_last_error(handle)
        msg = msg.decode() if msg else ""
        raise GBAError(status, (what + ": " if what else "") + msg)


def f64p(a):
    return a.ctypes.data_as(_f64p) if a is not None else None


def i32p(a):
    return a.ctypes.data_as(_i32p) if a is not None else None
