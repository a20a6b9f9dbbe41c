"""Multi-process runs: one process per GPU, trajectories sharded across
ranks, readouts gathered on the host.

The reference has no distributed code (its README lists multi-GPU as
future work).  Trajectories are independent, so a sweep shards by
contiguous trajectory ranges with no data-path collective; the only
exchange is a host-side gather of readouts (and, for timing, a barrier and
a max over ranks).  Rendezvous comes from the usual torchrun environment
(RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT); with WORLD_SIZE unset or 1
everything degrades to the single-process case.
"""
import os

import numpy as np


def world():
    """(rank, world_size) from the environment."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def init(backend=None):
    """Initialise torch.distributed when WORLD_SIZE > 1 (nccl with a GPU,
    gloo otherwise).  Returns (rank, world_size)."""
    rank, size = world()
    if size > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend=backend)
    return rank, size


def shard(n, rank, size):
    """Contiguous [begin, end) of n items owned by `rank` (the first n % size
    ranks take one extra)."""
    base, extra = divmod(n, size)
    begin = rank*base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(x):
    """Max of a float over ranks (the job's wall time is its slowest rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    on_gpu = dist.get_backend() == "nccl"
    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_rows(local, n_total):
    """Host-side gather of each rank's trajectory rows (contiguous shards)
    into the full (n_total, ...) array on every rank."""
    import torch.distributed as dist
    local = np.ascontiguousarray(local)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local
    parts = [None]*dist.get_world_size()
    dist.all_gather_object(parts, local)
    out = np.concatenate(parts, axis=0)
    assert out.shape[0] == n_total
    return out


def run_sharded(runner, n_total, gather=True):
    """Run this rank's contiguous share [begin, end) of n_total trajectories
    through runner(begin, end), which returns a dict of arrays whose leading
    dimension is its trajectories (other values pass through unchanged),
    and, with gather, assemble every such array over the ranks in
    trajectory order.  Single process: runner(0, n_total)."""
    rank, size = world()
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        rank, size = 0, 1
    begin, end = shard(n_total, rank, size)
    out = runner(begin, end)
    if not gather or size == 1:
        return out
    res = {}
    for k, v in out.items():
        if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == end - begin and \
                k not in ("time",):
            res[k] = gather_rows(v, n_total)
        else:
            res[k] = v
    return res
