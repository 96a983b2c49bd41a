"""A sweep sharded over two ranks: two processes share the one GPU and talk
through gloo on the host (no kernel waits on another rank).  The plain sweep
gives every point bit for bit what the single-process sweep gives, and the
surrogate sweep, whose rounds exchange training points and residuals, ends
on every rank together and answers every point."""
import datetime
import os
import socket

import numpy as np
import pytest

from spp_gb300 import configs, replicas, surrogate

pytestmark = pytest.mark.gpu

KW = dict(max_steps=4000, window=500, seed=4, chunk=1000)


def _points():
    return configs.sweep_points(n_points=256, n_min=256, n_max=1024, seed=4)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, use_surrogate, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=300))
    try:
        ex = replicas.Exchange(dist)
        ans, full, ret, res = replicas.run_sweep_sharded(_points(), rank, world, ex,
                                                         use_surrogate=use_surrogate, **KW)
        out.put((rank, ans, full, ret, int(res.rounds)))
    finally:
        dist.destroy_process_group()


def _run_two(use_surrogate):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, use_surrogate, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=900) for _ in range(2)), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    return res


def test_sharded_plain_sweep_matches_single_process(gpu_lib):
    single = surrogate.run_sweep(_points(), use_surrogate=False, **KW)
    res = _run_two(False)
    for rank, ans, full, ret, _ in res:
        assert np.array_equal(full, single.p_full), rank
        assert np.array_equal(ans, single.p_full) and not ret.any()


def test_sharded_surrogate_sweep_answers_every_point(gpu_lib):
    single = surrogate.run_sweep(_points(), use_surrogate=False, **KW)
    (r0, a0, f0, t0, n0), (r1, a1, f1, t1, n1) = _run_two(True)
    # both ranks hold the same global answers and went through the same rounds
    assert np.array_equal(a0, a1) and np.array_equal(t0, t1) and n0 == n1
    assert np.all(np.isfinite(a0))
    ran = np.isfinite(f0)
    assert np.array_equal(f0[ran], single.p_full[ran])
    assert t0.sum() > 0 and np.all(ran | t0)
    assert np.median(np.abs(a0[t0] - single.p_full[t0])) <= 0.02
