"""World-size-2 gloo tests of the replica policy (CPU only): problems are
split across ranks with no data-path collective, results gathered on the
host; a rank that dies between steps is detected by the survivor through a
short process-group timeout, with no GPU involved."""
import datetime
import os
import socket

import numpy as np
import pytest

from slamplay_gb300.replicas import shard_range

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def test_shard_range_partitions():
    for n in (0, 1, 5, 1024):
        for w in (1, 2, 3, 8):
            seen = []
            for r in range(w):
                rr = shard_range(n, r, w)
                seen.extend(rr)
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _solve_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    from oracle import oracle_py as O
    from slamplay_gb300 import BALProblem
    from slamplay_gb300.replicas import solve_sharded

    probs = [BALProblem.synthetic(3, index=i, seed=4, num_points=150) for i in range(5)]

    def one(b):
        r = O.solve(O.Problem.from_bal(b), max_num_iterations=5, linear_solver="dense_schur")
        return r["final_cost"]

    res = solve_sharded(probs, rank, world, one, gather=dist.all_gather_object)
    if rank == 0:
        np.save(os.path.join(out_dir, "costs.npy"), np.array(res))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_solve_world2(tmp_path):
    mp.start_processes(_solve_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(tmp_path / "costs.npy")
    from oracle import oracle_py as O
    from slamplay_gb300 import BALProblem

    want = [O.solve(O.Problem.from_bal(BALProblem.synthetic(3, index=i, seed=4, num_points=150)),
                    max_num_iterations=5, linear_solver="dense_schur")["final_cost"] for i in range(5)]
    assert np.array_equal(got, np.array(want))


def _dying_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=3))
    dist.barrier()
    if rank == 1:
        os._exit(0)  # leaves between steps, without joining the next collective
    try:
        dist.barrier()
        status = "no-error"
    except Exception as e:  # noqa: BLE001
        status = "detected:" + type(e).__name__
    with open(os.path.join(out_dir, "rank0.txt"), "w") as f:
        f.write(status)


def test_dead_rank_detected_by_timeout(tmp_path):
    ctx = mp.start_processes(_dying_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=False,
                             start_method="spawn")
    for p in ctx.processes:
        p.join(60)
    status = (tmp_path / "rank0.txt").read_text()
    assert status.startswith("detected"), status
