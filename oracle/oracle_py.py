"""ctypes binding of the CPU oracle (oracle.c) and of the reference-built
checker (oracle/_ref).  TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
product package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libslamplay_ref.so")

_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int)


class OrcProblem(C.Structure):
    _fields_ = [("nc", C.c_int), ("np", C.c_int), ("no", C.c_int), ("camera_index", _i32p),
                ("point_index", _i32p), ("observations", _f64p), ("parameters", _f64p)]


class OrcRig(C.Structure):
    _fields_ = [("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
                ("ext", (C.c_double * 6) * 2), ("obs_camera", C.POINTER(C.c_ubyte))]


class OrcOptions(C.Structure):
    _fields_ = [
        ("max_num_iterations", C.c_int), ("function_tolerance", C.c_double),
        ("gradient_tolerance", C.c_double), ("parameter_tolerance", C.c_double),
        ("initial_trust_region_radius", C.c_double), ("max_trust_region_radius", C.c_double),
        ("min_trust_region_radius", C.c_double), ("min_relative_decrease", C.c_double),
        ("min_lm_diagonal", C.c_double), ("max_lm_diagonal", C.c_double),
        ("max_num_consecutive_invalid_steps", C.c_int), ("jacobi_scaling", C.c_int),
        ("loss", C.c_int), ("loss_scale", C.c_double), ("linear_solver", C.c_int),
        ("pcg_criterion", C.c_int), ("max_linear_solver_iterations", C.c_int),
        ("min_linear_solver_iterations", C.c_int), ("pcg_tolerance", C.c_double), ("eta", C.c_double),
        ("num_threads", C.c_int), ("verbose", C.c_int), ("camera_update", C.c_int),
        ("lm_policy", C.c_int), ("rig", C.POINTER(OrcRig)),
    ]


class OrcSummary(C.Structure):
    _fields_ = [
        ("initial_cost", C.c_double), ("final_cost", C.c_double), ("num_iterations", C.c_int),
        ("num_successful_steps", C.c_int), ("num_unsuccessful_steps", C.c_int),
        ("num_invalid_steps", C.c_int), ("num_linear_solver_iterations", C.c_longlong),
        ("termination_type", C.c_int), ("termination_reason", C.c_int),
        ("final_trust_region_radius", C.c_double), ("gradient_max_norm", C.c_double),
        ("trace_capacity", C.c_int), ("trace_length", C.c_int), ("trace_cost", _f64p),
        ("trace_radius", _f64p), ("trace_linear_iterations", _i32p), ("trace_successful", _i32p),
    ]


LOSS = {"trivial": 0, "huber": 1, "cauchy": 2}
SOLVER = {"dense_schur": 0, "pcg_schur": 1}
CAMERA_UPDATE = {"additive": 0, "so3_left": 1}
LM_POLICY = {"ceres": 0, "g2o": 1}
G2O_MAX_TRIALS = 10

_orc = None
_ref = None


def _stale(lib: str, sources: list[str]) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in sources if os.path.exists(os.path.join(HERE, f)))


def ensure_built(reference: bool = False) -> None:
    """Builds the oracle (and with `reference` the reference-built checker)
    when missing or older than its sources."""
    if _stale(ORACLE_LIB, ["oracle.c", "synth.c", "oracle.h"]) or (reference and not os.path.exists(REF_LIB)):
        import subprocess
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "all" if reference else "oracle"], check=True)


def reference_root():
    """The reference tree's path where this machine has it (the environment
    variable REF_ROOT, else build_ref.sh's default), or None."""
    import subprocess
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "root"], stdout=subprocess.PIPE, text=True)
    p = r.stdout.strip()
    return p if p and os.path.isdir(p) else None


def oracle():
    global _orc
    if _orc is None:
        ensure_built()
        L = C.CDLL(ORACLE_LIB)
        L.orc_options_init.argtypes = [C.POINTER(OrcOptions)]
        L.orc_residual_jacobian.argtypes = [_f64p, _f64p, _f64p, _f64p, _f64p]
        L.orc_residual_jacobian.restype = C.c_int
        L.orc_angle_axis_rotate_point.argtypes = [_f64p, _f64p, _f64p]
        L.orc_evaluate.argtypes = [C.POINTER(OrcProblem), C.c_int, C.c_double, _f64p, _f64p, _f64p]
        L.orc_evaluate.restype = C.c_int
        L.orc_evaluate_ex.argtypes = [C.POINTER(OrcProblem), C.c_int, C.c_double, C.c_int, _f64p, _f64p, _f64p]
        L.orc_evaluate_ex.restype = C.c_int
        L.orc_compose_left.argtypes = [_f64p, _f64p, _f64p]
        L.orc_rig_residual_jacobian.argtypes = [_f64p, _f64p, _f64p, C.POINTER(OrcRig), C.c_int, _f64p, _f64p]
        L.orc_rig_residual_jacobian.restype = C.c_int
        L.orc_se3_compose_left.argtypes = [_f64p, _f64p, _f64p, _f64p]
        L.orc_window_outliers.argtypes = [_f64p, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_ubyte), _i32p, _i32p]
        L.orc_window_outliers.restype = C.c_double
        L.orc_evaluate_rig.argtypes = [C.POINTER(OrcProblem), C.POINTER(OrcRig), C.c_int, C.c_double, _f64p, _f64p,
                                       _f64p]
        L.orc_evaluate_rig.restype = C.c_int
        L.orc_compute_step.argtypes = [C.POINTER(OrcProblem), C.POINTER(OrcOptions), C.c_double, _f64p, _f64p,
                                       C.POINTER(C.c_int)]
        L.orc_compute_step.restype = C.c_int
        L.orc_solve.argtypes = [C.POINTER(OrcProblem), C.POINTER(OrcOptions), C.POINTER(OrcSummary)]
        L.orc_solve.restype = C.c_int
        L.orc_synth_size.argtypes = [C.c_int, C.c_int, C.c_uint64, _i32p, _i32p, _i32p]
        L.orc_synth_size.restype = C.c_int
        L.orc_synth_generate.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int, _i32p, _i32p,
                                         _f64p, _f64p]
        L.orc_synth_generate.restype = C.c_int
        _orc = L
    return _orc


def reference_lib():
    """The reference's own functor / BALProblem compiled by build_ref.sh, or
    None when the reference tree is not available on this machine."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            try:
                ensure_built(reference=True)
            except Exception:
                return None
        if not os.path.exists(REF_LIB):
            return None
        L = C.CDLL(REF_LIB)
        L.ref_residual.argtypes = [_f64p, _f64p, _f64p, _f64p]
        L.ref_residual_jacobian.argtypes = [_f64p, _f64p, _f64p, _f64p, _f64p]
        L.ref_rotate.argtypes = [_f64p, _f64p, _f64p]
        L.ref_aa_to_quat.argtypes = [_f64p, _f64p]
        L.ref_quat_to_aa.argtypes = [_f64p, _f64p]
        L.ref_bal_load.argtypes = [C.c_char_p, C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _f64p, _f64p]
        L.ref_bal_prepare.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_uint, C.c_double, C.c_double, C.c_double,
                                      _f64p]
        L.ref_bal_write.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_bal_write_ply.argtypes = [C.c_char_p, C.c_char_p]
        _ref = L
    return _ref


def f64(a):
    return a.ctypes.data_as(_f64p)


def i32(a):
    return a.ctypes.data_as(_i32p)


def options(**kw) -> OrcOptions:
    o = OrcOptions()
    oracle().orc_options_init(C.byref(o))
    for k, v in kw.items():
        if k == "loss" and isinstance(v, str):
            v = LOSS[v]
        if k == "linear_solver" and isinstance(v, str):
            v = SOLVER[v]
        if k == "camera_update" and isinstance(v, str):
            v = CAMERA_UPDATE[v]
        if k == "lm_policy" and isinstance(v, str):
            v = LM_POLICY[v]
        if k == "pcg_criterion" and isinstance(v, str):
            v = {"residual": 0, "quadratic_model": 1}[v]
        setattr(o, k, v)
    return o


class Problem:
    """Arrays of one BAL problem held for the oracle (parameters copied)."""

    def __init__(self, nc, np_, cam, pt, obs, params):
        self.cam = np.ascontiguousarray(cam, dtype=np.int32)
        self.pt = np.ascontiguousarray(pt, dtype=np.int32)
        self.obs = np.ascontiguousarray(obs, dtype=np.float64).reshape(-1)
        self.params = np.array(params, dtype=np.float64).reshape(-1)
        self.s = OrcProblem(nc, np_, len(self.cam), i32(self.cam), i32(self.pt), f64(self.obs), f64(self.params))

    @classmethod
    def from_bal(cls, b):
        return cls(b.num_cameras(), b.num_points(), b.camera_index(), b.point_index(), b.observations(),
                   b.parameters())

    @classmethod
    def synthetic(cls, config: int, index: int = 0, seed: int = 0) -> "Problem":
        """Benchmark configuration `config`'s seeded problem, generated by the
        oracle's own generator (synth.c; the same bytes as the product's
        gba_synth_generate)."""
        L = oracle()
        nc, np_, no = C.c_int(), C.c_int(), C.c_int()
        if not L.orc_synth_size(config, index, seed, C.byref(nc), C.byref(np_), C.byref(no)):
            raise ValueError(f"oracle synth: bad configuration {config}")
        cam = np.zeros(no.value, np.int32)
        pt = np.zeros(no.value, np.int32)
        obs = np.zeros(2 * no.value)
        par = np.zeros(9 * nc.value + 3 * np_.value)
        if not L.orc_synth_generate(config, index, seed, nc, np_, no, i32(cam), i32(pt), f64(obs), f64(par)):
            raise RuntimeError("oracle synth: generation failed")
        return cls(nc.value, np_.value, cam, pt, obs, par)

    def copy(self) -> "Problem":
        return Problem(self.s.nc, self.s.np, self.cam, self.pt, self.obs, self.params)

    def num_cameras(self) -> int:
        return self.s.nc

    def num_points(self) -> int:
        return self.s.np

    def num_observations(self) -> int:
        return self.s.no


def evaluate(p: Problem, loss="trivial", loss_scale=1.0, camera_update="additive"):
    no = p.s.no
    r = np.zeros(2 * no)
    J = np.zeros(24 * no)
    c = C.c_double()
    ok = oracle().orc_evaluate_ex(C.byref(p.s), LOSS[loss] if isinstance(loss, str) else loss, loss_scale,
                                  CAMERA_UPDATE[camera_update], f64(r), f64(J), C.byref(c))
    return r.reshape(no, 2), J.reshape(no, 2, 12), c.value, bool(ok)


def make_rig(fx, fy, cx, cy, extrinsics, obs_camera):
    """An OrcRig over the given per-observation rig-camera array (kept alive
    on the returned object)."""
    r = OrcRig()
    r.fx, r.fy, r.cx, r.cy = fx, fy, cx, cy
    e = np.asarray(extrinsics, dtype=np.float64).reshape(2, 6)
    for k in range(2):
        for q in range(6):
            r.ext[k][q] = e[k, q]
    oc = np.ascontiguousarray(obs_camera, dtype=np.uint8)
    r._keep = oc
    r.obs_camera = oc.ctypes.data_as(C.POINTER(C.c_ubyte))
    return r


def rig_from_window(w):
    return make_rig(w.fx, w.fy, w.cx, w.cy, w.extrinsics, w.rig_camera)


def window_problem(w):
    """The window as an oracle Problem: poses in 9-slot camera blocks
    (angle-axis, translation, three unused zeros), then the landmarks."""
    nk = w.num_keyframes
    cams = np.zeros((nk, 9))
    cams[:, :6] = np.asarray(w.poses).reshape(nk, 6)
    params = np.concatenate([cams.reshape(-1), np.asarray(w.landmarks, dtype=np.float64).reshape(-1)])
    return Problem(nk, w.num_landmarks, w.keyframe_index, w.landmark_index, w.observations, params)


def evaluate_rig(p: Problem, rig, loss="trivial", loss_scale=1.0):
    no = p.s.no
    r = np.zeros(2 * no)
    J = np.zeros(24 * no)
    c = C.c_double()
    ok = oracle().orc_evaluate_rig(C.byref(p.s), C.byref(rig), LOSS[loss] if isinstance(loss, str) else loss,
                                   loss_scale, f64(r), f64(J), C.byref(c))
    return r.reshape(no, 2), J.reshape(no, 2, 12), c.value, bool(ok)


def se3_compose_left(dw, du, pose):
    out = np.zeros(6)
    oracle().orc_se3_compose_left(f64(np.ascontiguousarray(dw, dtype=np.float64)),
                                  f64(np.ascontiguousarray(du, dtype=np.float64)),
                                  f64(np.ascontiguousarray(pose, dtype=np.float64)), f64(out))
    return out


def window_outliers(chi2, threshold=5.991, max_doublings=5):
    chi2 = np.ascontiguousarray(chi2, dtype=np.float64)
    out = np.zeros(len(chi2), np.uint8)
    ni, no_ = C.c_int(), C.c_int()
    th = oracle().orc_window_outliers(f64(chi2), len(chi2), threshold, max_doublings,
                                      out.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(ni), C.byref(no_))
    return out, ni.value, no_.value, th


def compose_left(dw, w):
    """w' = log(exp(dw) exp(w)) in angle-axis form."""
    a = np.ascontiguousarray(dw, dtype=np.float64)
    b = np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(3)
    oracle().orc_compose_left(f64(a), f64(b), f64(out))
    return out


def compute_step(p: Problem, radius: float, **kw):
    n = p.params.size
    d = np.zeros(n)
    m = C.c_double()
    it = C.c_int()
    ok = oracle().orc_compute_step(C.byref(p.s), C.byref(options(**kw)), radius, f64(d), C.byref(m), C.byref(it))
    return d, m.value, it.value, bool(ok)


def solve(p: Problem, rig=None, **kw):
    """Runs the oracle LM; returns a dict with the summary and the trace."""
    o = options(**kw)
    if rig is not None:
        o.rig = C.pointer(rig)
    cap = max(1, o.max_num_iterations * (G2O_MAX_TRIALS if o.lm_policy == 1 else 1) + 1)
    tc = np.zeros(cap)
    tr = np.zeros(cap)
    tl = np.zeros(cap, np.int32)
    ts = np.zeros(cap, np.int32)
    s = OrcSummary()
    s.trace_capacity = cap
    s.trace_cost, s.trace_radius, s.trace_linear_iterations, s.trace_successful = f64(tc), f64(tr), i32(tl), i32(ts)
    ok = oracle().orc_solve(C.byref(p.s), C.byref(o), C.byref(s))
    n = s.trace_length
    return {
        "ok": bool(ok), "initial_cost": s.initial_cost, "final_cost": s.final_cost,
        "num_iterations": s.num_iterations, "num_successful_steps": s.num_successful_steps,
        "num_unsuccessful_steps": s.num_unsuccessful_steps, "num_invalid_steps": s.num_invalid_steps,
        "num_linear_solver_iterations": s.num_linear_solver_iterations,
        "termination_type": s.termination_type, "termination_reason": s.termination_reason,
        "final_trust_region_radius": s.final_trust_region_radius, "gradient_max_norm": s.gradient_max_norm,
        "trace_cost": tc[:n].copy(), "trace_radius": tr[:n].copy(), "trace_linear_iterations": tl[:n].copy(),
        "trace_successful": ts[:n].copy(), "parameters": p.params.copy(),
    }
