"""The host side of several GPUs, on the CPU: the cost-balanced partition of
sweep points, and the rank-ordered exchange, the any-over-ranks decision and
the max-over-ranks timing between two gloo processes (127.0.0.1)."""
import datetime
import os
import socket

import numpy as np
import pytest

from spp_gb300 import configs, replicas


def test_partition_by_cost_covers_and_balances():
    pts = configs.sweep_points(n_points=64)
    costs = [p.n for p in pts]
    for world in (1, 2, 3, 8):
        shards = replicas.partition_by_cost(costs, world)
        allidx = np.concatenate(shards)
        assert np.array_equal(np.sort(allidx), np.arange(len(pts)))
        loads = np.array([sum(costs[i] for i in s) for s in shards])
        # largest-first greedy: no shard exceeds the mean by more than the largest item
        assert loads.max() <= loads.mean() + max(costs)
        assert all(np.all(np.diff(s) > 0) for s in shards)
        assert [list(s) for s in shards] == [list(s) for s in replicas.partition_by_cost(costs, world)]


def test_single_process_exchange_is_identity():
    ex = replicas.Exchange()
    a, b = ex([np.arange(3), np.ones(2)])
    assert np.array_equal(a, np.arange(3)) and np.array_equal(b, np.ones(2))
    assert ex.any(True) and not ex.any(False)
    assert replicas.max_over_ranks(2.5) == 2.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        ex = replicas.Exchange(dist)
        # rank r contributes r + 1 items; the result is in rank order on every rank
        a, b = ex([np.full(rank + 1, rank), np.arange(rank + 1, dtype=np.float64) * 10])
        anyflag = ex.any(rank == 1)
        noflag = ex.any(False)
        mx = replicas.max_over_ranks(1.5 + rank, dist)
        out.put((rank, a.tolist(), b.tolist(), anyflag, noflag, mx))
    finally:
        dist.destroy_process_group()


def test_exchange_and_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, a, b, anyflag, noflag, mx in res:
        assert a == [0, 1, 1]
        assert b == [0.0, 0.0, 10.0]
        assert anyflag is True and noflag is False
        assert mx == 2.5


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference launched as two ranks: rank 0 alone times
    the CPU path and prints one JSON line; the other rank exits 0."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["value"] == d["value"]
