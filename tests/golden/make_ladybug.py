"""Writes tests/golden/ladybug49_prepared.npz: the reference's own main()
input path for backend/slam_ba_simple_g2o_ceres
(test_bundle_adjustment_ceres.cpp:48-50) on the one BAL file the reference
ships (data/bal/ladybug49.txt), computed by the reference's own
utils/datasets/BALProblem.cpp compiled into oracle/_ref (oracle/build_ref.sh):

  camera_index, point_index, observations, parameters_raw -- BALProblem's
      parse of the file (BALProblem.cpp:78-139);
  parameters_prepared -- after Normalize() and Perturb(0.1, 0.5, 0.5) with
      the C library's rand() in its initial state (main() never seeds it:
      srand(1)).

A machine that runs the GPU tests need not have the reference tree, so the
fixture carries these arrays to the tests there.  Run from the repository root where the reference tree is
present: python tests/golden/make_ladybug.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402


def main():
    root = O.reference_root()
    if not root:
        raise SystemExit("the reference tree is not present on this machine")
    ref = O.reference_lib()
    path = os.path.join(root, "data", "bal", "ladybug49.txt").encode()
    nc, np_, no, npar = (O.C.c_int() for _ in range(4))
    ref.ref_bal_load(path, 0, O.C.byref(nc), O.C.byref(np_), O.C.byref(no), O.C.byref(npar), None, None, None, None)
    cam = np.zeros(no.value, np.int32)
    pt = np.zeros(no.value, np.int32)
    obs = np.zeros(2 * no.value)
    raw = np.zeros(npar.value)
    ref.ref_bal_load(path, 0, O.C.byref(nc), O.C.byref(np_), O.C.byref(no), O.C.byref(npar), O.i32(cam), O.i32(pt),
                     O.f64(obs), O.f64(raw))
    prepared = np.zeros(npar.value)
    ref.ref_bal_prepare(path, 1, 1, 1, 0.1, 0.5, 0.5, O.f64(prepared))
    out = os.path.join(ROOT, "tests", "golden", "ladybug49_prepared.npz")
    np.savez_compressed(out, num_cameras=nc.value, num_points=np_.value, camera_index=cam, point_index=pt,
                        observations=obs, parameters_raw=raw, parameters_prepared=prepared)
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
