"""The N > 1 bench path on CPU: two gloo ranks, each with its own replicas,
combined as the bench combines them (all ranks' trials over the slowest
rank's time). No GPU and no data-path collective: the path only shards."""
import multiprocessing as mp
import os
import socket
import sys

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    trials, secs = 1000 * (rank + 1), 2.0 + rank
    n, t = bench.reduce_sum_max(dist, trials, secs, "cpu")
    rate = bench.reduce_rate(bench.job_dist(), trials, secs, "cpu")
    q.put((rank, n, t, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, n, t, rate in out:
        assert n == 3000.0 and t == 3.0            # sum of trials, slowest rank's time
        assert rate == 1000.0


def test_one_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_dist() is None
    assert bench.reduce_rate(None, 500, 2.0, "cpu") == 250.0
