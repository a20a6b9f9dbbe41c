"""Multi-process host logic on CPU (gloo, world size 2): sharding covers
every trajectory once, the max over ranks is the slowest rank, and a
host-side gather of per-rank results reassembles the full sweep."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

from superspinsim_gb300 import replicas  # noqa: E402


def test_shard_partitions():
    for n in (0, 1, 5, 1024, 1025):
        for size in (1, 2, 3, 8):
            got = [replicas.shard(n, r, size) for r in range(size)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(size - 1))
            assert max(e - b for b, e in got) - min(e - b for b, e in got) <= 1


def _worker(rank, size, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    r, s = replicas.init(backend="gloo")
    assert (r, s) == (rank, size)
    n = 11
    b, e = replicas.shard(n, r, s)
    # stand-in for a rank's share of a sweep: row i of the result is i*[1, 2, 3]
    local = np.arange(b, e)[:, None]*np.array([1.0, 2.0, 3.0])
    full = replicas.gather_rows(local, n)
    replicas.barrier()
    mx = replicas.max_over_ranks(10.0 + rank)
    out[rank] = (full.tolist(), mx)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_gloo_gather_and_max():
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    want = (np.arange(11)[:, None]*np.array([1.0, 2.0, 3.0])).tolist()
    for rank in range(2):
        full, mx = out[rank]
        assert full == want
        assert mx == 11.0
