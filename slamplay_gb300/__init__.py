"""slamplay_gb300 — GB300-native bundle adjustment, a drop-in for the Ceres
SPARSE_SCHUR solve of slamplay's backend/slam_ba_simple_g2o_ceres path.

The compute lives in libgba.so (C++ host + sm_103a CUDA kernels behind the C
ABI of include/gba.h); this package is its Python face, mirroring the
reference's BALProblem and SolveBA.
"""
from ._native import GBAError
from .bal_problem import BALProblem
from .solver import G2O_VARIANT, LOCAL_BA, Solver, SolveSummary, estimate_footprint, make_options, solve_ba
from .window import LocalBAWindow

__all__ = ["BALProblem", "Solver", "SolveSummary", "solve_ba", "make_options", "estimate_footprint", "G2O_VARIANT",
           "LOCAL_BA", "LocalBAWindow",
           "GBAError"]
