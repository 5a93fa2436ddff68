"""bench.py's multi-GPU form is replicas only (independent skeletons per rank, no data
exchange): the job's time is the slowest rank's, and the rate counts every rank's
skeletons. Two gloo ranks on the CPU check the aggregation."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.argv = ["bench.py"]
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    total = bench.max_over_ranks(mine, dist, "cpu")
    q.put((rank, total, bench.replica_rate(world, 10, total / 1e3)))
    dist.destroy_process_group()


def test_max_over_ranks_and_rate_with_two_gloo_ranks():
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
    assert [o[1] for o in out] == [150.0, 150.0]            # both ranks see the slowest time
    assert out[0][2] == pytest.approx(2 * 10 / 0.150)       # 20 skeletons in 150 ms


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.replica_rate(1, 10, 2.0) == 5.0
