"""Independent systems on several GPUs (one process per GPU).

The reference runs one realisation per MPI rank and farms sweep points over
the ranks (serial/mpi-main.cpp:157-176).  Here a rank holds whole systems:
nothing on the data path crosses GPUs.  The host-side pieces that do cross
ranks live here:
  - the environment of a torchrun launch (WORLD_SIZE, RANK, LOCAL_RANK);
  - the maximum of a timing over ranks (the slowest rank sets the wall time);
  - a partition of sweep points over ranks balanced by their cost (particles
    x steps, largest first onto the least-loaded rank);
  - an exchange that concatenates per-rank numpy arrays in rank order, used
    to fit the sweep surrogate on every rank's completed points and to put
    the answers of a sharded sweep back into point order.
All of it works on any torch.distributed backend (NCCL between GPUs, gloo on
CPU for tests)."""
import os

import numpy as np


def dist_env():
    """(world size, rank, local rank) of a torchrun launch; (1, 0, 0) alone."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value, dist=None):
    """The largest value over all ranks (value itself without a process
    group).  Floats travel as float64 on the backend's device."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def partition_by_cost(costs, world):
    """Index arrays (ascending) of `world` shards of the items with the given
    costs: largest first, each onto the shard with the least cost so far
    (ties to the lowest rank).  Deterministic, so every rank computes the
    same partition."""
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    owner = np.empty(costs.size, np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [np.flatnonzero(owner == r) for r in range(world)]


class Exchange:
    """Concatenates per-rank arrays in rank order (all_gather_object), so that
    every rank sees the same global arrays.  Without a process group it
    returns the arrays unchanged."""

    def __init__(self, dist=None):
        self.dist = dist if dist is not None and dist.is_initialized() else None

    @property
    def world(self):
        return 1 if self.dist is None else self.dist.get_world_size()

    def __call__(self, arrays):
        if self.dist is None or self.world == 1:
            return [np.asarray(a) for a in arrays]
        out = [None] * self.world
        self.dist.all_gather_object(out, [np.asarray(a) for a in arrays])
        return [np.concatenate([out[r][k] for r in range(self.world)]) for k in range(len(arrays))]

    def any(self, flag):
        """True when flag is true on some rank (a collective: every rank calls it)."""
        return bool(np.any(self([np.array([bool(flag)])])[0]))


def run_sweep_sharded(points, rank, world, exchange, **kw):
    """The sweep over `points` split by cost over `world` ranks: this rank
    runs its shard (surrogate fits on every rank's completed points through
    `exchange`), and every rank returns the per-point answers in the original
    order: (p_answer, p_full, retired, local SweepResult)."""
    from .surrogate import run_sweep
    shards = partition_by_cost([p.n for p in points], world)
    mine = shards[rank]
    res = run_sweep([points[i] for i in mine], exchange=exchange, **kw)
    idx, ans, full, ret = exchange([mine, res.p_answer, res.p_full, res.retired.astype(np.int8)])
    n = len(points)
    p_answer = np.full(n, np.nan)
    p_full = np.full(n, np.nan)
    retired = np.zeros(n, bool)
    p_answer[idx] = ans
    p_full[idx] = full
    retired[idx] = ret.astype(bool)
    return p_answer, p_full, retired, res
