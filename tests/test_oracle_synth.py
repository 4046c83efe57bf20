"""The oracle's own generator of the benchmark configurations (oracle/synth.c)
gives the same bytes as the product library's (gba_synth_generate): the CPU
baseline builds its input with the former, so that it never loads the
product library, and solves the same problem as the GPU arm."""
import numpy as np
import pytest

from oracle import oracle_py as O
from slamplay_gb300 import BALProblem


@pytest.mark.parametrize("config,index", [(0, 0), (1, 0), (3, 0), (3, 7), (3, 1023), (4, 0), (4, 5)])
def test_oracle_synth_matches_library(config, index):
    o = O.Problem.synthetic(config, index=index, seed=0)
    b = BALProblem.synthetic(config, index=index, seed=0)
    assert (o.num_cameras(), o.num_points(), o.num_observations()) == \
        (b.num_cameras(), b.num_points(), b.num_observations())
    assert np.array_equal(o.cam, b.camera_index())
    assert np.array_equal(o.pt, b.point_index())
    assert o.obs.tobytes() == np.ascontiguousarray(b.observations(), np.float64).reshape(-1).tobytes()
    assert o.params.tobytes() == np.ascontiguousarray(b.parameters(), np.float64).reshape(-1).tobytes()


def test_oracle_synth_seed_changes_problem():
    a = O.Problem.synthetic(0, seed=0)
    b = O.Problem.synthetic(0, seed=1)
    assert a.params.tobytes() != b.params.tobytes()


def test_oracle_synth_rejects_unknown_configuration():
    with pytest.raises(ValueError):
        O.Problem.synthetic(9)
