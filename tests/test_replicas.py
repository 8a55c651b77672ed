"""bench.py's multi-GPU path is independent replicas: only the timing scalars
cross ranks.  Two gloo ranks on the CPU check the whole-job rate (steps of
all ranks / the slowest rank's time) and the barrier."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    bench.replica_barrier(world)
    steps, t, rate = bench.job_rate(100 + rank, 1.0 + rank, world)
    with open(os.path.join(out, f"rank{rank}.txt"), "w") as fh:
        fh.write(f"{steps} {t} {rate}\n")
    dist.destroy_process_group()


def test_two_replicas_job_rate(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        steps, t, rate = open(tmp_path / f"rank{r}.txt").read().split()
        assert int(steps) == 201 and float(t) == 2.0 and float(rate) == 100.5


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(7, 0.5, 1) == (7, 0.5, 14.0)
