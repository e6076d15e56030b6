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


def test_bench_gpus_n_starts_n_ranks():
    """bench.py --gpus 2 started by hand launches its own two ranks (the
    reference arm: rank 0 runs the host path after every rank has joined a
    gloo group) and reports n_gpus 2."""
    import json
    import subprocess
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "rpm800", "--gpus", "2",
                        "--steps", "1", "--warmup", "1", "--ref-seconds", "0.3"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["impl"] == "reference" and d["value"] > 0


def test_bench_refuses_a_rank_count_other_than_gpus():
    import subprocess
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", WORLD_SIZE="3", RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "running with 3 ranks" in r.stderr
