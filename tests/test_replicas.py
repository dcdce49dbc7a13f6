"""The multi-GPU form (replicas): two gloo ranks on the CPU agree on the job's time
(the slowest rank's) and throughput (all ranks' units), as bench.py computes them."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gudni_gb300 import replicas as R  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    r, w, local = R.ranks()
    R.init(w, "gloo")
    R.barrier(w)
    seconds = R.max_over_ranks(0.010 * (r + 1), w)  # rank r took (r + 1) * 10 ms
    rate = R.job_rate(1000.0, w, seconds)
    R.barrier(w)
    with open(os.path.join(out_dir, f"rank{r}.txt"), "w") as f:
        f.write(f"{r} {w} {local} {seconds!r} {rate!r}\n")
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_time_and_rate(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    rows = sorted(open(tmp_path / f"rank{r}.txt").read().split() for r in range(world))
    for r, row in enumerate(rows):
        rank, w, local, seconds, rate = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        assert (rank, w, local) == (r, world, r)
        assert seconds == pytest.approx(0.020)       # the slowest rank's time
        assert rate == pytest.approx(2 * 1000.0 / 0.020)  # every rank's units over it


def test_single_rank_needs_no_process_group():
    assert R.max_over_ranks(3.5, 1) == 3.5
    assert R.job_rate(10.0, 1, 2.0) == 5.0
