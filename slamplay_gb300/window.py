"""Local bundle-adjustment windows: the problem full_slam's backend hands to
g2o (full_slam/src/backend.cpp:67-199): the active keyframes' poses T_cw
(SE3, updated on the left, g2o_types.h:48-66), the active landmarks, and one
edge per feature (EdgeProjection, g2o_types.h:127-175) seen by the left or
the right camera of a stereo rig that shares one K (backend.cpp:99-101).

A pose is stored as angle-axis (3) and translation (3): X_cam = R(w) X + t.
A rig camera's extrinsic E_k (Camera::pose(), body -> camera) is stored the
same way.
"""
from __future__ import annotations

import numpy as np

# KITTI-like stereo rig: slambook2-style cameras (E_0 = identity, E_1 a pure
# baseline translation), K of the left camera for both
KITTI_K = (718.856, 718.856, 607.1928, 185.2157)
KITTI_BASELINE = 0.537


def _rotate(w, x):
    """Rodrigues rotation of the rows of x by the angle-axis vectors w."""
    w = np.asarray(w, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    th = np.linalg.norm(w, axis=-1, keepdims=True)
    safe = np.where(th > 0, th, 1.0)
    k = w / safe
    c, s = np.cos(th), np.sin(th)
    kx = np.cross(k, x)
    kd = np.sum(k * x, axis=-1, keepdims=True)
    out = x * c + kx * s + k * kd * (1 - c)
    return np.where(th > 0, out, x + np.cross(w, x))


class LocalBAWindow:
    """One window: arrays in the layout of gba_window_view."""

    def __init__(self, keyframe_index, landmark_index, rig_camera, observations, poses, landmarks,
                 fx, fy, cx, cy, extrinsics):
        self.keyframe_index = np.ascontiguousarray(keyframe_index, dtype=np.int32)
        self.landmark_index = np.ascontiguousarray(landmark_index, dtype=np.int32)
        rc = np.asarray(rig_camera)
        if rc.size and (not np.all(np.isfinite(rc)) or rc.min() < 0 or rc.max() > 1 or np.any(rc != np.round(rc))):
            raise ValueError("rig_camera must be 0 (left) or 1 (right)")
        self.rig_camera = np.ascontiguousarray(rc, dtype=np.uint8)
        self.observations = np.ascontiguousarray(observations, dtype=np.float64).reshape(-1)
        self.poses = np.array(poses, dtype=np.float64).reshape(-1)
        self.landmarks = np.array(landmarks, dtype=np.float64).reshape(-1)
        self.fx, self.fy, self.cx, self.cy = float(fx), float(fy), float(cx), float(cy)
        self.extrinsics = np.array(extrinsics, dtype=np.float64).reshape(2, 6)
        no = self.keyframe_index.size
        if self.landmark_index.size != no or self.rig_camera.size != no or self.observations.size != 2 * no:
            raise ValueError("keyframe_index, landmark_index, rig_camera and observations must describe the same "
                             "observations (observations: 2 per observation)")
        if self.poses.size % 6 or self.landmarks.size % 3:
            raise ValueError("poses are 6 numbers per keyframe, landmarks 3 per landmark")
        if no and (self.keyframe_index.min() < 0 or self.keyframe_index.max() >= self.num_keyframes or
                   self.landmark_index.min() < 0 or self.landmark_index.max() >= self.num_landmarks):
            raise ValueError("keyframe or landmark index out of range")
        if no and self.rig_camera.max() > 1:
            raise ValueError("rig_camera must be 0 (left) or 1 (right)")

    @property
    def num_keyframes(self) -> int:
        return self.poses.size // 6

    @property
    def num_landmarks(self) -> int:
        return self.landmarks.size // 3

    @property
    def num_observations(self) -> int:
        return self.keyframe_index.size

    def copy(self) -> "LocalBAWindow":
        return LocalBAWindow(self.keyframe_index, self.landmark_index, self.rig_camera, self.observations,
                             self.poses.copy(), self.landmarks.copy(), self.fx, self.fy, self.cx, self.cy,
                             self.extrinsics)

    def project(self, poses=None, landmarks=None):
        """Pixel of every observation (K (E_k (T X)), divided by depth) and
        the depth."""
        P = np.asarray(self.poses if poses is None else poses).reshape(-1, 6)
        L = np.asarray(self.landmarks if landmarks is None else landmarks).reshape(-1, 3)
        T = P[self.keyframe_index]
        X = L[self.landmark_index]
        pc = _rotate(T[:, :3], X) + T[:, 3:]
        E = self.extrinsics[self.rig_camera]
        q = _rotate(E[:, :3], pc) + E[:, 3:]
        u = (self.fx * q[:, 0] + self.cx * q[:, 2]) / q[:, 2]
        v = (self.fy * q[:, 1] + self.cy * q[:, 2]) / q[:, 2]
        return np.stack([u, v], axis=1), q[:, 2]

    @classmethod
    def synthetic(cls, seed=0, num_keyframes=7, num_landmarks=600, right_fraction=0.5, pixel_noise=1.0,
                  outlier_fraction=0.05, rotation_noise=0.01, translation_noise=0.05, landmark_noise=0.1,
                  image_size=(1241, 376), return_truth=False):
        """A forward-moving stereo window (full_slam's 7 active keyframes by
        default): landmarks in front of the rig, one left-image feature per
        visible (keyframe, landmark) pair and a right-image one with
        probability right_fraction, Gaussian pixel noise, a fraction of
        gross outliers (20-60 px), and a perturbed initial estimate."""
        rng = np.random.default_rng(seed)
        nk = num_keyframes
        poses = np.zeros((nk, 6))
        for k in range(nk):
            # body moves along +z in the world; T_cw maps the world into the body
            yaw = 0.02 * k + rng.normal() * 0.005
            w = np.array([rng.normal() * 0.005, yaw, rng.normal() * 0.005])
            c = np.array([0.05 * rng.normal(), 0.02 * rng.normal(), 1.0 * k])
            poses[k, :3] = -w
            poses[k, 3:] = -_rotate(-w, c)
        lm = np.stack([rng.uniform(-12, 12, num_landmarks), rng.uniform(-3, 3, num_landmarks),
                       rng.uniform(6, 40, num_landmarks) + nk * 0.5], axis=1)
        ext = np.zeros((2, 6))
        ext[1, 3] = -KITTI_BASELINE
        fx, fy, cx, cy = KITTI_K
        kf, li, rc = [], [], []
        for k in range(nk):
            pc = _rotate(np.repeat(poses[k:k + 1, :3], num_landmarks, 0), lm) + poses[k, 3:]
            for side in (0, 1):
                q = pc + ext[side, 3:]
                u = fx * q[:, 0] / q[:, 2] + cx
                v = fy * q[:, 1] / q[:, 2] + cy
                vis = (q[:, 2] > 1.0) & (u > 0) & (u < image_size[0]) & (v > 0) & (v < image_size[1])
                if side == 1:
                    vis &= rng.random(num_landmarks) < right_fraction
                for j in np.nonzero(vis)[0]:
                    kf.append(k), li.append(j), rc.append(side)
        kf, li, rc = np.array(kf, np.int32), np.array(li, np.int32), np.array(rc, np.uint8)
        # landmarks seen fewer than twice are dropped (they do not constrain)
        counts = np.bincount(li, minlength=num_landmarks)
        keep_lm = np.nonzero(counts >= 2)[0]
        remap = -np.ones(num_landmarks, np.int64)
        remap[keep_lm] = np.arange(keep_lm.size)
        sel = remap[li] >= 0
        kf, li, rc = kf[sel], remap[li[sel]].astype(np.int32), rc[sel]
        lm = lm[keep_lm]
        truth = cls(kf, li, rc, np.zeros(2 * kf.size), poses, lm, fx, fy, cx, cy, ext)
        uv, _ = truth.project()
        uv = uv + rng.normal(size=uv.shape) * pixel_noise
        nout = int(round(outlier_fraction * kf.size))
        if nout:
            idx = rng.choice(kf.size, nout, replace=False)
            ang = rng.uniform(0, 2 * np.pi, nout)
            mag = rng.uniform(20, 60, nout)
            uv[idx, 0] += mag * np.cos(ang)
            uv[idx, 1] += mag * np.sin(ang)
        p0 = poses.copy()
        p0[1:, :3] += rng.normal(size=(nk - 1, 3)) * rotation_noise
        p0[1:, 3:] += rng.normal(size=(nk - 1, 3)) * translation_noise
        l0 = lm + rng.normal(size=lm.shape) * landmark_noise
        w = cls(kf, li, rc, uv, p0, l0, fx, fy, cx, cy, ext)
        if return_truth:
            truth.observations = w.observations.copy()
            return w, truth
        return w
