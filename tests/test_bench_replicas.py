"""bench.py --gpus N runs N independent replicas (the path does not shard): the job's time is
the slowest rank's, and its seconds per iteration are that time over the iterations of all
ranks.  Checked with two gloo ranks on the CPU (the same all-reduce the NCCL run makes)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    q.put((rank, bench.replica_aggregate(100.0 * (rank + 1), 120.0 + rank, 10, world, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        mx, me, s, e = out[r]
        assert (mx, me) == (200.0, 121.0)                  # the slowest rank's totals on every rank
        assert s == pytest.approx(0.2 / 20) and e == pytest.approx(0.121 / 20)


def test_replica_aggregate_one_rank_is_plain_average():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replica_aggregate(50.0, 60.0, 5, 1, "cpu") == (50.0, 60.0, 0.01, 0.012)
