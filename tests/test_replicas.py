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


def _sharded_worker(rank, size, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    replicas.init(backend="gloo")
    progs, rho, kw = _spin1_sweep()
    from oracle import oracle

    def runner(b, e):
        # this rank's trajectories through the CPU oracle (the stand-in for
        # the batched GPU run on a CPU-only test)
        if e <= b:
            return {"states": np.zeros((0,) + kw["shape"])}
        _, st = oracle.simulate(kw["gens"], np.stack([rho]*(e - b)), 0.0, kw["tf"], kw["dt"],
                                progs[b:e], K=2, W=kw["W"], nodes=kw["nodes"], F=kw["F"],
                                vectorisation_map=kw["vm"], mode="vector", flat_out=True)
        return {"states": st, "rank_of_row": np.full(e - b, rank)}

    res = replicas.run_sharded(runner, progs.shape[0])
    out[rank] = (res["states"].tolist(), res["rank_of_row"].tolist())
    import torch.distributed as dist
    dist.destroy_process_group()


def _spin1_sweep():
    """Seven spin-1 ODMR trajectories (the C1 model), 3 samples of 1 ns, F = 10."""
    from conftest import load_case, quadrature
    c = load_case("spin1_c1")
    W, nodes = quadrature(2)
    progs = np.repeat(c["program"][None], 7, axis=0)
    progs[:, 0, 0, 3] = 2.870e9 + 28.025e9*0.01 + np.linspace(-20e6, 20e6, 7)
    kw = {"gens": c["generators"], "vm": c["vectorisation_map"], "W": W, "nodes": nodes,
          "F": 10, "dt": 1e-9, "tf": 3e-9 + 1e-13, "shape": (3, c["generators"].shape[1])}
    return progs, c["rho0"], kw


def test_two_rank_sharded_sweep_equals_single_process():
    """Each of two gloo ranks runs its contiguous share of a sweep (3 and 4
    of 7 trajectories); the gathered states equal the single-process run and
    keep trajectory order."""
    from oracle import oracle
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_sharded_worker, args=(2, port, out), nprocs=2, join=True,
                       start_method="spawn")
    progs, rho, kw = _spin1_sweep()
    _, want = oracle.simulate(kw["gens"], np.stack([rho]*7), 0.0, kw["tf"], kw["dt"], progs, K=2,
                              W=kw["W"], nodes=kw["nodes"], F=kw["F"],
                              vectorisation_map=kw["vm"], mode="vector", flat_out=True)
    for rank in range(2):
        states, owner = out[rank]
        assert np.array_equal(np.array(states), want)
        assert owner == [0]*4 + [1]*3
