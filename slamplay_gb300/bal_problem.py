"""Python mirror of slamplay::BALProblem (utils/datasets/BALProblem.h:31-119).

Same storage as the reference: one flat ``parameters`` array (9 per camera,
cameras first, then 3 per point), ``camera_index`` / ``point_index`` int32
arrays and interleaved ``observations``.  Accessor names follow the
reference (``num_cameras()``, ``mutable_points()``, ...).  File I/O,
Normalize and Perturb run in libgba's host code, restating
utils/datasets/BALProblem.cpp.
"""
from __future__ import annotations

import numpy as np

from . import _native as N


class BALProblem:
    """BAL problem with the reference's layout and accessors.

    ``BALProblem(filename)`` reads a BAL text file (BALProblem.cpp:78-139);
    ``use_quaternions=True`` switches cameras to the 10-parameter quaternion
    layout as the reference does (BALProblem.cpp:116-138).
    """

    def __init__(self, filename: str | None = None, use_quaternions: bool = False):
        self.use_quaternions = bool(use_quaternions)
        self.camera_index_ = np.zeros(0, np.int32)
        self.point_index_ = np.zeros(0, np.int32)
        self.observations_ = np.zeros(0, np.float64)
        self.parameters_ = np.zeros(0, np.float64)
        self.num_cameras_ = self.num_points_ = self.num_observations_ = 0
        if filename is not None:
            self._read(filename)

    # ---- construction ----------------------------------------------------
    def _read(self, filename: str) -> None:
        L = N.lib()
        nc, np_, no = N.C.c_int32(), N.C.c_int32(), N.C.c_int32()
        N.check(L.gba_bal_read_header(filename.encode(), N.C.byref(nc), N.C.byref(np_), N.C.byref(no)),
                what=f"reading {filename}")
        self._alloc(nc.value, np_.value, no.value)
        v = self._raw_view()
        N.check(L.gba_bal_read(filename.encode(), N.C.byref(v)), what=f"reading {filename}")
        if self.use_quaternions:
            self._to_quaternions()

    def _alloc(self, nc: int, np_: int, no: int) -> None:
        self.num_cameras_, self.num_points_, self.num_observations_ = nc, np_, no
        self.camera_index_ = np.zeros(no, np.int32)
        self.point_index_ = np.zeros(no, np.int32)
        self.observations_ = np.zeros(2 * no, np.float64)
        self.parameters_ = np.zeros(9 * nc + 3 * np_, np.float64)

    @classmethod
    def from_arrays(cls, num_cameras: int, num_points: int, camera_index, point_index, observations,
                    parameters) -> "BALProblem":
        b = cls()
        no = len(camera_index)
        b._alloc(int(num_cameras), int(num_points), int(no))
        b.camera_index_[:] = camera_index
        b.point_index_[:] = point_index
        b.observations_[:] = np.asarray(observations, np.float64).reshape(-1)
        b.parameters_[:] = np.asarray(parameters, np.float64).reshape(-1)
        return b

    @classmethod
    def synthetic(cls, config: int, index: int = 0, seed: int = 0, return_truth: bool = False, **overrides):
        """Seeded synthetic problem of benchmark configuration `config`
        (0 ring, 1 random walk, 2 loops, 3 local-BA window `index`, 4
        serving request `index`).  Keyword overrides patch the generator spec
        (e.g. num_points=500)."""
        L = N.lib()
        spec = N.SynthSpec()
        N.check(L.gba_synth_preset(int(config), int(index), int(seed), N.C.byref(spec)), what="synth preset")
        for k, v in overrides.items():
            setattr(spec, k, v)
        nc, np_, no = N.C.c_int32(), N.C.c_int32(), N.C.c_int32()
        N.check(L.gba_synth_size(N.C.byref(spec), N.C.byref(nc), N.C.byref(np_), N.C.byref(no)), what="synth size")
        b = cls()
        b._alloc(nc.value, np_.value, no.value)
        truth = np.zeros_like(b.parameters_)
        v = b._raw_view()
        N.check(L.gba_synth_generate(N.C.byref(spec), N.C.byref(v), N.f64p(truth)), what="synth generate")
        return (b, truth) if return_truth else b

    # ---- reference accessors (BALProblem.h:55-98) -----------------------
    def camera_block_size(self) -> int:
        return 10 if self.use_quaternions else 9

    def point_block_size(self) -> int:
        return 3

    def num_cameras(self) -> int:
        return self.num_cameras_

    def num_points(self) -> int:
        return self.num_points_

    def num_observations(self) -> int:
        return self.num_observations_

    def num_parameters(self) -> int:
        return self.parameters_.size

    def point_index(self) -> np.ndarray:
        return self.point_index_

    def camera_index(self) -> np.ndarray:
        return self.camera_index_

    def observations(self) -> np.ndarray:
        return self.observations_

    def parameters(self) -> np.ndarray:
        return self.parameters_

    def cameras(self) -> np.ndarray:
        return self.parameters_[: self.camera_block_size() * self.num_cameras_]

    def points(self) -> np.ndarray:
        return self.parameters_[self.camera_block_size() * self.num_cameras_:]

    def mutable_cameras(self) -> np.ndarray:
        return self.cameras()

    def mutable_points(self) -> np.ndarray:
        return self.points()

    def camera_for_observation(self, i: int) -> np.ndarray:
        b = self.camera_block_size()
        c = int(self.camera_index_[i])
        return self.parameters_[b * c: b * c + b]

    def point_for_observation(self, i: int) -> np.ndarray:
        j = int(self.point_index_[i])
        o = self.camera_block_size() * self.num_cameras_
        return self.parameters_[o + 3 * j: o + 3 * j + 3]

    mutable_camera_for_observation = camera_for_observation
    mutable_point_for_observation = point_for_observation

    # ---- views -----------------------------------------------------------
    def _raw_view(self) -> N.ProblemView:
        v = N.ProblemView()
        v.num_cameras = self.num_cameras_
        v.num_points = self.num_points_
        v.num_observations = self.num_observations_
        v.camera_index = N.i32p(self.camera_index_)
        v.point_index = N.i32p(self.point_index_)
        v.observations = N.f64p(self.observations_)
        v.parameters = N.f64p(self.parameters_)
        return v

    def view(self, allow_quaternions: bool = False) -> N.ProblemView:
        """gba_problem_view over this problem's arrays: the angle-axis layout,
        or the quaternion one (10 per camera) for a solver created with
        camera_layout='quaternion' (allow_quaternions)."""
        if self.use_quaternions and not allow_quaternions:
            raise ValueError("this entry point takes the 9-parameter angle-axis camera layout "
                             "(SnavelyReprojectionError.h:89-92); convert with to_angle_axis(), or solve with "
                             "camera_layout='quaternion'")
        for a in (self.camera_index_, self.point_index_):
            assert a.dtype == np.int32 and a.flags.c_contiguous
        for a in (self.observations_, self.parameters_):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        return self._raw_view()

    # ---- I/O and preparation (BALProblem.cpp) ---------------------------
    def WriteToFile(self, filename: str) -> None:
        p = self._angle_axis_copy()
        N.check(N.lib().gba_bal_write(filename.encode(), N.C.byref(p._raw_view())), what=f"writing {filename}")

    def WriteToPLYFile(self, filename: str) -> None:
        p = self._angle_axis_copy()
        N.check(N.lib().gba_bal_write_ply(filename.encode(), N.C.byref(p._raw_view())), what=f"writing {filename}")

    def Normalize(self) -> None:
        self._with_angle_axis(lambda v: N.check(N.lib().gba_bal_normalize(N.C.byref(v)), what="Normalize"))

    def Perturb(self, rotation_sigma: float, translation_sigma: float, point_sigma: float, seed: int = 0) -> None:
        """seed = 0 draws from the C library's rand() as the reference does."""
        self._with_angle_axis(lambda v: N.check(
            N.lib().gba_bal_perturb(N.C.byref(v), rotation_sigma, translation_sigma, point_sigma, seed),
            what="Perturb"))

    # ---- quaternion layout ------------------------------------------------
    def _to_quaternions(self) -> None:
        nc = self.num_cameras_
        old = self.parameters_
        new = np.zeros(10 * nc + 3 * self.num_points_)
        L = N.lib()
        for i in range(nc):
            aa = np.ascontiguousarray(old[9 * i: 9 * i + 3])
            q = np.zeros(4)
            L.gba_angle_axis_to_quaternion(N.f64p(aa), N.f64p(q))
            new[10 * i: 10 * i + 4] = q
            new[10 * i + 4: 10 * i + 10] = old[9 * i + 3: 9 * i + 9]
        new[10 * nc:] = old[9 * nc:]
        self.parameters_ = new

    def _angle_axis_copy(self) -> "BALProblem":
        if not self.use_quaternions:
            return self
        b = BALProblem()
        b._alloc(self.num_cameras_, self.num_points_, self.num_observations_)
        b.camera_index_[:] = self.camera_index_
        b.point_index_[:] = self.point_index_
        b.observations_[:] = self.observations_
        b.parameters_[:] = self.to_angle_axis_parameters()
        return b

    def to_angle_axis_parameters(self) -> np.ndarray:
        if not self.use_quaternions:
            return self.parameters_.copy()
        nc = self.num_cameras_
        out = np.zeros(9 * nc + 3 * self.num_points_)
        L = N.lib()
        for i in range(nc):
            q = np.ascontiguousarray(self.parameters_[10 * i: 10 * i + 4])
            aa = np.zeros(3)
            L.gba_quaternion_to_angle_axis(N.f64p(q), N.f64p(aa))
            out[9 * i: 9 * i + 3] = aa
            out[9 * i + 3: 9 * i + 9] = self.parameters_[10 * i + 4: 10 * i + 10]
        out[9 * nc:] = self.parameters_[10 * nc:]
        return out

    def _with_angle_axis(self, fn) -> None:
        if not self.use_quaternions:
            fn(self._raw_view())
            return
        p = self._angle_axis_copy()
        fn(p._raw_view())
        self.parameters_ = p.parameters_
        self.use_quaternions = False
        self._to_quaternions()
        self.use_quaternions = True

    def copy(self) -> "BALProblem":
        b = BALProblem()
        b.use_quaternions = self.use_quaternions
        b.num_cameras_, b.num_points_, b.num_observations_ = self.num_cameras_, self.num_points_, self.num_observations_
        b.camera_index_ = self.camera_index_.copy()
        b.point_index_ = self.point_index_.copy()
        b.observations_ = self.observations_.copy()
        b.parameters_ = self.parameters_.copy()
        return b
