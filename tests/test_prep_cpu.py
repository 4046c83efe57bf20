"""Host logic of the problem preparation (prep.cpp), checked against brute
force by a small C++ program compiled here: the explicit Schur complement's
structure (blocks, transposes, observation pairs in point order, built by
host threads for large problems) and the chunks' stable camera order."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "slamplay_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers are missing")
    out = str(tmp_path_factory.mktemp("prep") / "check_prep")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                    "-I", CUDA_INC, os.path.join(ROOT, "tests", "cpu", "check_prep.cpp"),
                    os.path.join(CSRC, "prep.cpp"), "-o", out], check=True)
    return out


@pytest.mark.parametrize("nc,np_,seed", [(9, 60, 1), (5, 400, 2), (40, 20000, 3)])
def test_prep_matches_brute_force(checker, nc, np_, seed):
    # the last case has ~80k observations: the structure is built on several
    # host threads
    r = subprocess.run([checker, str(nc), str(np_), str(seed)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr


def test_prep_is_the_same_under_concurrency_and_fork(tmp_path):
    """Prepares from several host threads at once (the thread pool busy),
    a shuffled input and a forked child all give the single-thread layout."""
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers are missing")
    out = str(tmp_path / "prep_stress")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                    "-I", CUDA_INC, os.path.join(ROOT, "tests", "cpu", "prep_stress.cpp"),
                    os.path.join(CSRC, "prep.cpp"), "-o", out], check=True)
    r = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
