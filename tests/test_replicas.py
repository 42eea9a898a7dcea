"""The multi-GPU path is replicas only (each rank advances its own copy of
the workload, no collective on the data path); the bench's whole-job timing
takes the slowest rank and counts every replica's cells.  Checked with two
gloo ranks on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench
    t = bench.max_over_ranks(1.0 + rank, world)
    v = bench.whole_job_value(1000, 10, world, t)
    q.put((rank, t, v))
    dist.destroy_process_group()


def test_two_rank_timing_takes_the_slowest_and_counts_every_replica():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]            # the slowest rank's time on both
    assert [o[2] for o in out] == [1000 * 10 * 2 / 2.0] * 2
